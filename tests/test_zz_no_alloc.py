"""cc_gpu_run_noalloc: the allocation-free entry point for callers that cannot
allocate device memory when they solve (an inference runtime's enqueue(), a
process whose device memory is already reserved by its own allocator, a
latency-critical loop that cannot take cudaMalloc's synchronisation).

It must give the same labels as the regular entry point cc_gpu_run, on two
calls in a row (the second call finds the first call's leftovers in the
shared scratch array).  Labels are integers, so the tolerance is zero.  This
file is collected last, so a run that stops at the first failure has already
run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import components_gb300 as cc
from components_gb300 import _lib

pytestmark = pytest.mark.gpu


def _noalloc():
    fn = _lib.gpu().cc_gpu_run_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p]
    return fn


def _regular_labels(D):
    """Labels from the existing entry point, cc_gpu_run, through the C ABI."""
    import torch
    lab = torch.full((D.n,), -1, dtype=torch.int32, device="cuda:0")
    cfg = _lib.cc_config()
    _lib.gpu().cc_config_default(C.byref(cfg))
    csr = D.to_c()
    _lib.check(_lib.gpu().cc_gpu_run(C.byref(csr), _lib.CC_ALLREDUCE, C.byref(cfg), 1001,
                                     lab.data_ptr()))
    return lab.cpu().numpy()


def test_noalloc_matches_regular_entry_point_twice(cuda):
    import torch
    run = _noalloc()
    graphs = [
        cc.gen_gnm(200_000, 300_000, seed=12, id_bytes=4),
        cc.from_edges(5000, [(17, i) for i in range(5000) if i != 17] + [(1, 2)]),  # hub rows
        cc.gen_grid(300, 300, 0.5, seed=4, id_bytes=4),
    ]
    stream = torch.cuda.current_stream().cuda_stream
    for G in graphs:
        D = G.to_device("cuda:0")
        want = _regular_labels(D)
        for call in range(2):
            out = torch.full((D.n,), -1, dtype=torch.int32, device="cuda:0")
            rc = run(D.row_ptr.data_ptr(), D.col.data_ptr(), D.n, D.m, out.data_ptr(), stream)
            assert rc == _lib.CC_OK, (rc, call)
            assert np.array_equal(out.cpu().numpy(), want), (G.n, call)


def test_noalloc_rejects_graphs_above_its_limit(cuda):
    import torch
    run = _noalloc()
    n, m = 1 << 21, 1 << 26  # min(n, m/33 + 1) > 1,048,512: over the scratch limit
    rp = torch.zeros(n + 1, dtype=torch.int64, device="cuda:0")  # a valid (empty) graph
    col = torch.zeros(m, dtype=torch.int32, device="cuda:0")
    out = torch.empty(n, dtype=torch.int32, device="cuda:0")
    rc = run(rp.data_ptr(), col.data_ptr(), n, m, out.data_ptr(), None)
    assert rc == _lib.CC_ERR_UNSUPPORTED
    G = cc.from_edges(6, [(0, 2), (1, 2), (3, 4), (3, 5)])
    D = G.to_device("cuda:0")
    lab = torch.empty(6, dtype=torch.int32, device="cuda:0")
    assert run(D.row_ptr.data_ptr(), D.col.data_ptr(), 6, D.m, lab.data_ptr(), None) == _lib.CC_OK
    assert lab.cpu().tolist() == [0, 0, 0, 3, 3, 3]
