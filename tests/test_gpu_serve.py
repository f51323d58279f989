"""Continuous-batching server (include/cc_serve.h): every request's labels are
the same alone (cc_gpu_run) and in the mix, under budget pressure, with
requests arriving while earlier batches run."""
from __future__ import annotations

import threading
import time

import numpy as np
import pytest

import components_gb300 as cc
import oracle
from components_gb300 import _lib
from components_gb300.serve import Server

pytestmark = pytest.mark.gpu


def _mix(count: int, seed: int):
    """Seeded requests from the three families, sizes spread over the
    shared-memory and grid-wide paths."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        kind = i % 3
        n = int(2 ** rng.uniform(6, 17))
        d = float(rng.uniform(1, 16))
        if kind == 0:
            out.append(cc.gen_gnm(n, max(1, int(n * d / 2)), seed=seed * 1000 + i,
                                  id_bytes=4 if i % 2 else 8))
        elif kind == 1:
            side = max(2, int(np.sqrt(n)))
            out.append(cc.gen_grid(side, side, 0.5, seed=seed * 1000 + i))
        else:
            out.append(cc.gen_rhg(max(n, 64), d, 2.6, seed=seed * 1000 + i))
    return out


def test_results_alone_and_in_the_mix(cuda):
    graphs = _mix(60, 1)
    alone = [cc.find_components(G, "exp") for G in graphs]
    for G, a in zip(graphs[:12], alone[:12]):
        assert np.array_equal(a.astype(np.uint64), oracle.uf_labels(G))
    with Server(max_batch=16, window_us=3000) as srv:
        tickets = {}
        rng = np.random.default_rng(2)

        def producer():
            for i, G in enumerate(graphs):  # Poisson-like arrivals
                tickets[i] = srv.submit(G)
                time.sleep(float(rng.exponential(0.0005)))

        th = threading.Thread(target=producer)
        th.start()
        th.join()
        batches = set()
        for i in range(len(graphs)):
            lab, info = srv.wait(tickets[i], timeout_s=120)
            assert np.array_equal(lab, alone[i]), i
            assert info["submit_s"] <= info["admit_s"] <= info["done_s"]
            batches.add(info["batch_id"])
        st = srv.stats()
        assert st["completed"] == st["collected"] == len(graphs)
        assert st["batches"] == len(batches) and st["batches"] < len(graphs)  # coalesced
        assert st["bytes_in_use"] == 0


def test_budget_admission(cuda):
    graphs = _mix(30, 3)
    need = [8 * (G.n + 1) + G.id_bytes * G.m + 4 * (G.n + 1) for G in graphs]
    budget = int(3 * max(need) + (64 << 20))
    alone = [cc.find_components(G, "exp") for G in graphs]
    with Server(budget_bytes=budget, max_batch=8) as srv:
        ts = [srv.submit(G) for G in graphs]
        # collect in reverse order: the budget frees only as results are taken
        for i in reversed(range(len(graphs))):
            lab, _ = srv.wait(ts[i], timeout_s=120)
            assert np.array_equal(lab, alone[i])
        st = srv.stats()
        assert st["peak_bytes_in_use"] <= budget
        assert st["waiting"] == 0 and st["bytes_in_use"] == 0


def test_poll_and_oversize(cuda):
    G = cc.gen_grid(100, 100, 0.6, seed=4)
    with Server(budget_bytes=1 << 20) as srv:
        big = cc.gen_gnm(200000, 400000, seed=1, id_bytes=4)
        with pytest.raises(_lib.CCError) as ei:
            srv.submit(big)
        assert ei.value.status == _lib.CC_ERR_BUSY
        t = srv.submit(G)
        res = None
        for _ in range(20000):
            res = srv.poll(t)
            if res is not None:
                break
            time.sleep(0.0005)
        assert res is not None
        assert np.array_equal(res[0], cc.find_components(G, "exp"))


def test_invalid_request_is_reported(cuda):
    from conftest import csr_from_rows
    bad = csr_from_rows([[1], [0, 7], [3], [2]])
    good = cc.gen_gnm(500, 600, seed=3, id_bytes=4)
    with Server() as srv:
        tb, tg = srv.submit(bad), srv.submit(good)
        with pytest.raises(_lib.CCError) as ei:
            srv.wait(tb, timeout_s=60)
        assert ei.value.status == _lib.CC_ERR_INVALID
        lab, _ = srv.wait(tg, timeout_s=60)
        assert np.array_equal(lab, cc.find_components(good, "exp"))


def test_thousand_requests_from_two_hundred_graphs(cuda):
    """A serving stream at scale: 1,200 requests drawn from 240 distinct seeded
    graphs (the three families, n log-uniform in [2^10, 2^18], degree uniform
    in [1, 16]) arriving as a Poisson stream; every request's labels equal
    the graph solved alone (the plain path, itself checked against the
    oracle)."""
    rng = np.random.default_rng(17)
    pool = []
    for i in range(240):
        kind = i % 3
        n = int(2 ** rng.uniform(10, 18))
        d = float(rng.uniform(1, 16))
        if kind == 0:
            pool.append(cc.gen_gnm(n, max(1, int(n * d / 2)), seed=7000 + i, id_bytes=4))
        elif kind == 1:
            side = max(2, int(round(np.sqrt(n))))
            pool.append(cc.gen_grid(side, side, 0.5, seed=7000 + i))
        else:
            pool.append(cc.gen_rhg(n, d, 2.6, seed=7000 + i))
    alone = [cc.find_components(G, "exp") for G in pool]
    for j in range(0, len(pool), 8):
        assert np.array_equal(alone[j].astype(np.uint64), oracle.uf_labels(pool[j])), j
    picks = rng.integers(0, len(pool), 1200)
    gaps = rng.exponential(0.0002, len(picks))
    with Server() as srv:
        tickets = []

        def producer():
            for j, g in zip(picks, gaps):
                tickets.append(srv.submit(pool[int(j)]))
                time.sleep(float(g))

        th = threading.Thread(target=producer)
        th.start()
        th.join()
        for t, j in zip(tickets, picks):
            lab, _ = srv.wait(t, timeout_s=300)
            assert np.array_equal(lab, alone[int(j)]), int(j)
        st = srv.stats()
        assert st["completed"] == st["collected"] == len(picks)
        assert st["batches"] < len(picks) and st["bytes_in_use"] == 0
