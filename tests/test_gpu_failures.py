"""Failure paths, reached from the host without faulting the GPU.

* A round loop that runs out of rounds: a test hook lowers the context's round
  cap (cc_debug_set_round_cap), the solve returns CC_ERR_NO_CONVERGENCE, and
  the same context then solves correctly.  The reference has no error path
  here: it exits the process (lib/contraction/dynamic_contraction.h:437-438).
* A served request that cannot be staged (as if its device allocation failed)
  or launched: a test hook makes one chosen request fail
  (cc_serve_debug_fail_next); that request reports the failure and every
  other request of the stream completes with its correct labels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import components_gb300 as cc
import oracle
from components_gb300 import _lib

pytestmark = pytest.mark.gpu


def _path(n):
    return cc.from_edges(n, [(i, i + 1) for i in range(n - 1)])


# (local_contraction has no round loop: two sweeps per level, levels bounded)
@pytest.mark.parametrize("algo,P,seq", [("labels", 1, 1), ("shortcuts", 1, 1), ("exp", 4, 0)])
def test_round_cap_gives_no_convergence_then_context_recovers(cuda, algo, P, seq):
    import torch
    G = _path(4096)
    D = G.to_device("cuda:0").with_parts(P)
    ctx = cc.Context(0)
    lab = torch.empty(G.n, dtype=torch.int32, device="cuda:0")
    solver = cc.SOLVERS[algo](cc.Config(seed=1001, sequential_limit=seq), 0, P, ctx)
    assert _lib.gpu().cc_debug_set_round_cap(ctx.handle, 1) == _lib.CC_OK
    with pytest.raises(_lib.CCError) as e:
        solver.FindComponents(D, lab)
    assert e.value.status == _lib.CC_ERR_NO_CONVERGENCE
    assert _lib.gpu().cc_debug_set_round_cap(ctx.handle, 0) == _lib.CC_OK
    lab.fill_(-1)
    solver.FindComponents(D, lab)
    assert np.array_equal(lab.cpu().numpy().view(np.uint32).astype(np.uint64), oracle.uf_labels(G))
    ctx.close()


def test_served_request_failures_are_reported_alone(cuda):
    from components_gb300.serve import Server
    graphs = []
    for i in range(24):
        if i % 4 == 3:  # above the one-CTA size: solved by the grid-wide path
            graphs.append(cc.gen_gnm(60_000, 120_000, seed=500 + i, id_bytes=4))
        else:
            graphs.append(cc.gen_gnm(2000 + 37 * i, 3000, seed=500 + i, id_bytes=4))
    want = [oracle.uf_labels(G).astype(np.uint32) for G in graphs]
    inject = {5: 1, 7: 2, 10: 1, 15: 2}  # request -> staging (1) or launch (2) failure
    with Server(budget_bytes=8 << 30) as srv:
        tickets = []
        for i, G in enumerate(graphs):
            if i in inject:
                assert _lib.gpu().cc_serve_debug_fail_next(srv._h, inject[i]) == _lib.CC_OK
            tickets.append(srv.submit(G))
        for i, t in enumerate(tickets):
            if i in inject:
                with pytest.raises(_lib.CCError) as e:
                    srv.wait(t, timeout_s=60.0)
                assert e.value.status == (_lib.CC_ERR_OOM if inject[i] == 1 else _lib.CC_ERR_CUDA)
            else:
                got, _ = srv.wait(t, timeout_s=60.0)
                assert np.array_equal(got, want[i]), i
        # the server keeps serving after the failures
        t = srv.submit(graphs[7])
        got, _ = srv.wait(t, timeout_s=60.0)
        assert np.array_equal(got, want[7])
        st = srv.stats()
        assert st["bytes_in_use"] == 0
