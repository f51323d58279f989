"""Batched solves (include/cc_batch.h): every graph's local canonical labels
equal the plain one-graph solve and the oracle, bit for bit, whatever the
schedule."""
from __future__ import annotations

import numpy as np
import pytest

import components_gb300 as cc
import oracle
from components_gb300 import _lib
from components_gb300 import batch as B

pytestmark = pytest.mark.gpu


def _want(batch: B.Batch) -> np.ndarray:
    out = []
    for i in range(batch.k):
        g = batch.graph(i)
        out.append(oracle.uf_labels(g) if g.n else np.zeros(0, np.uint64))
    return np.concatenate(out).astype(np.uint32) if out else np.zeros(0, np.uint32)


@pytest.fixture(scope="module")
def mixed():
    # sizes from 2^6 to 2^17: every shared-memory bucket and the grid-wide path
    return B.gen_batch(96, 6, 17, 0.5, 8.0, seed=3)


def test_batch_matches_oracle_all_placements(cuda, mixed):
    want = _want(mixed)
    D = mixed.to_device("cuda:0")
    for use_graph in (0, 1):
        t = B.default_tuning()
        t.use_graph = use_graph
        for _ in range(2):  # the second run replays the recorded CUDA graph
            got = B.batch_run(D, tuning=t).cpu().numpy().view(np.uint32)
            assert np.array_equal(got, want), use_graph
    got = B.batch_run(mixed)  # host arrays in and out
    assert np.array_equal(got, want)
    got = B.batch_run(mixed.pinned())
    assert np.array_equal(np.asarray(got), want)


def test_batch_equals_plain_path(cuda):
    bt = B.gen_batch(24, 8, 14, 0.5, 8.0, seed=9)
    D = bt.to_device("cuda:0")
    got = B.batch_run(D).cpu().numpy().view(np.uint32)
    v, _, _ = bt.numpy()
    for i in range(bt.k):
        g = bt.graph(i)
        plain = cc.find_components(g, "exp")
        assert np.array_equal(got[int(v[i]):int(v[i + 1])], plain), i


@pytest.mark.parametrize("bucket_edge_par", [0, 1])
@pytest.mark.parametrize("threads", [128, 512])
def test_batch_schedules(cuda, mixed, bucket_edge_par, threads):
    want = _want(mixed)
    D = mixed.to_device("cuda:0")
    t = B.default_tuning()
    for b in range(B.BUCKETS):
        t.threads[b] = threads
        t.edge_parallel[b] = bucket_edge_par
    t.hub_degree = 16
    assert np.array_equal(B.batch_run(D, tuning=t).cpu().numpy().view(np.uint32), want)
    t.smem_max_n[3] = 0  # largest bucket sent to the grid-wide path
    t.smem_max_n[0] = 0
    assert np.array_equal(B.batch_run(D, tuning=t).cpu().numpy().view(np.uint32), want)


def test_autotune_keeps_labels(cuda, mixed):
    D = mixed.to_device("cuda:0")
    t = B.autotune(D, reps=1)
    d = t.as_dict()
    assert all(x in (128, 256, 512) for x in d["threads"])
    assert np.array_equal(B.batch_run(D, tuning=t).cpu().numpy().view(np.uint32), _want(mixed))


def test_batch_edge_cases(cuda):
    graphs = [cc.from_edges(0, []), cc.from_edges(1, []), cc.from_edges(5, []),
              cc.from_edges(4, [(0, 3)]), cc.from_edges(3000, [(9, i) for i in range(3000) if i != 9]),
              cc.from_edges(70000, [(i, i + 1) for i in range(0, 69999, 2)])]
    bt = B.Batch.pack(graphs)
    want = _want(bt)
    assert np.array_equal(B.batch_run(bt.to_device("cuda:0")).cpu().numpy().view(np.uint32), want)


def test_batch_bad_local_id_is_reported(cuda):
    bt = B.Batch.pack([cc.from_edges(4, [(0, 1)]), cc.from_edges(3, [(0, 2)])])
    v, r, c = bt.numpy()
    c = c.copy()
    c[-1] = 7  # local id >= n of its graph
    bad = B.Batch(v, r, c)
    with pytest.raises(_lib.CCError) as ei:
        B.batch_run(bad.to_device("cuda:0"))
    assert ei.value.status == _lib.CC_ERR_INVALID


def test_batch_4096_config_scale(cuda):
    """The batched configuration itself: 4096 G(n, m) graphs, n log-uniform in
    [2^8, 2^18], average degree uniform in [0.5, 8].  Batched labels equal the
    plain path (one cc_ctx_run per graph, looped in C++) and the oracle."""
    import torch
    bt = B.gen_batch(4096, 8, 18, 0.5, 8.0, seed=1)
    want = _want(bt)
    D = bt.to_device("cuda:0")
    ctx = cc.Context(0)
    tune = B.autotune(D, ctx, reps=1)
    got = B.batch_run(D, ctx, tune).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, want)
    plain = torch.full((bt.total_n,), -1, dtype=torch.int32, device="cuda:0")
    B.plain_run(D, ctx, plain, "exp", cc.Config(seed=1001))
    assert np.array_equal(plain.cpu().numpy().view(np.uint32), want)
    ctx.close()


def test_batch_large_graphs_sampled_linking(cuda):
    """Graphs above the shared-memory sizes go through sampled linking with a
    giant root per graph: a large graph whose hub row (more entries than the
    hub threshold) lies outside its giant component, a large graph without a
    giant component (average degree below one), and a large graph of
    isolated vertices, between small graphs; labels equal the oracle's."""
    n = 70000
    path = [(v, v + 1) for v in range(0, 60000)]  # the giant component
    star = [(60001, w) for w in range(60002, 60300)]  # a hub outside it
    bridge = [(60400, 60401), (60401, 60402)]
    hub_graph = cc.from_edges(n, path + star + bridge)
    sparse = cc.gen_gnm(80000, 24000, seed=11)  # average degree 0.6
    empty = cc.from_edges(52000, [])
    small = [cc.gen_gnm(500, 900, seed=s) for s in range(3)]
    bt = B.Batch.pack([small[0], hub_graph, small[1], sparse, empty, small[2]])
    want = _want(bt)
    t = B.default_tuning()
    t.hub_degree = 32
    got = B.batch_run(bt.to_device("cuda:0"), tuning=t).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, want)
