"""GPU parity at the full benchmark sizes: G(n=2^20, m=2^22) with 64-bit ids,
the 8192 x 8192 bond-percolation grid (p = 0.5) with 32-bit ids and the
random hyperbolic graph of 2^26 vertices (d = 16, gamma = 2.6, 32-bit ids,
about 1.1e9 directed entries: the headline configuration).  The
oracle's union-find still finishes in seconds at these sizes, so labels are
compared entry for entry; size-independent checks (every label is a
component minimum, labels constant along every edge) run beside it."""
from __future__ import annotations

import numpy as np
import pytest

import components_gb300 as cc
import oracle

pytestmark = pytest.mark.gpu


def _solve_dev(G, algo, P, conf):
    import torch
    D = G.to_device("cuda:0").with_parts(P)
    dt = torch.int32 if G.id_bytes == 4 else torch.int64
    lab = torch.empty(G.n, dtype=dt, device="cuda:0")
    cc.SOLVERS[algo](conf, 0, P).FindComponents(D, lab)
    out = lab.cpu().numpy()
    return out.view(np.uint32 if G.id_bytes == 4 else np.uint64).astype(np.uint64)


def _properties(G, lab):
    rp, col = G.numpy()
    src = np.repeat(np.arange(G.n, dtype=np.uint64), np.diff(rp).astype(np.int64))
    assert np.array_equal(lab[src], lab[col]), "label differs across an edge"
    assert np.all(lab <= np.arange(G.n, dtype=np.uint64)), "label above its own id"
    roots = lab == np.arange(G.n, dtype=np.uint64)
    assert np.all(roots[lab.astype(np.int64)]), "label is not a root"


@pytest.fixture(scope="module")
def gnm():
    G = cc.gen_gnm(1 << 20, 1 << 22, seed=1, id_bytes=8)
    return G, oracle.uf_labels(G)


@pytest.fixture(scope="module")
def grid():
    G = cc.gen_grid(8192, 8192, 0.5, seed=1, id_bytes=4)
    return G, oracle.uf_labels(G)


@pytest.mark.parametrize("algo", ["exp", "local", "shortcuts", "labels", "allreduce"])
def test_gnm_full_size(cuda, gnm, algo):
    G, want = gnm
    for P in (1, 16):
        got = _solve_dev(G, algo, P, cc.Config(seed=1001))
        assert np.array_equal(got, want), (algo, P)
    _properties(G, got)


@pytest.mark.parametrize("algo,P", [("exp", 1), ("exp", 16), ("exp", 152), ("allreduce", 1),
                                    ("shortcuts", 1)])
def test_grid_full_size(cuda, grid, algo, P):
    G, want = grid
    got = _solve_dev(G, algo, P, cc.Config(seed=1001))
    assert np.array_equal(got, want), (algo, P)


def test_grid_exp_ldd_path(cuda, grid):
    """-seq 0 forces the decomposition levels on the grid's cut graph."""
    G, want = grid
    got = _solve_dev(G, "exp", 64, cc.Config(seed=1002, sequential_limit=0))
    assert np.array_equal(got, want)
    _properties(G, got)


@pytest.fixture(scope="module")
def rhg26():
    G = cc.gen_rhg(1 << 26, 16.0, 2.6, seed=1, id_bytes=4)
    return G, oracle.uf_labels(G)


def test_rhg_2_26_device_generator(cuda, rhg26):
    """The GPU arm of the benchmark builds the headline graph on the device;
    it is the host generator's graph (the one the CPU arm solves) bit for bit."""
    G, _ = rhg26
    D = cc.gen_rhg_device(1 << 26, 16.0, 2.6, seed=1, id_bytes=4)
    assert D.m == G.m
    assert np.array_equal(D.row_ptr.cpu().numpy().view(np.uint64), np.asarray(G.row_ptr))
    assert np.array_equal(D.col.cpu().numpy().view(np.uint32), np.asarray(G.col))


def test_rhg_2_26_full_size(cuda, rhg26):
    """Labels of the headline graph equal the union-find's for exp_contraction
    with one rank and with 16 virtual ranks, and for all_reduce."""
    import torch
    G, want = rhg26
    D = G.to_device("cuda:0")
    lab = torch.empty(G.n, dtype=torch.int32, device="cuda:0")
    for algo, P in (("exp", 1), ("exp", 16), ("allreduce", 1)):
        lab.fill_(-1)
        cc.SOLVERS[algo](cc.Config(seed=1001), 0, P).FindComponents(D.with_parts(P), lab)
        got = lab.cpu().numpy().view(np.uint32).astype(np.uint64)
        assert np.array_equal(got, want), (algo, P)
    del D, lab
    torch.cuda.empty_cache()
