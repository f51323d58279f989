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
    # refused from n and m_dir alone, before any pointer is read: small buffers suffice
    rp = torch.zeros(2, dtype=torch.int64, device="cuda:0")
    col = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    out = torch.empty(1, dtype=torch.int32, device="cuda:0")
    rc = run(rp.data_ptr(), col.data_ptr(), n, m, out.data_ptr(), None)
    assert rc == _lib.CC_ERR_UNSUPPORTED
    G = cc.from_edges(6, [(0, 2), (1, 2), (3, 4), (3, 5)])
    D = G.to_device("cuda:0")
    lab = torch.empty(6, dtype=torch.int32, device="cuda:0")
    assert run(D.row_ptr.data_ptr(), D.col.data_ptr(), 6, D.m, lab.data_ptr(), None) == _lib.CC_OK
    assert lab.cpu().tolist() == [0, 0, 0, 3, 3, 3]


def test_noalloc_reports_bad_input_then_recovers(cuda):
    """A bad id (the kernels check it and skip the access) or non-monotone
    offsets give CC_ERR_INVALID; the next valid call, which finds that error
    word in the shared scratch, clears it and returns CC_OK with the regular
    entry point's labels."""
    import torch
    run = _noalloc()
    G = cc.gen_gnm(3000, 6000, seed=21, id_bytes=4)
    D = G.to_device("cuda:0")
    want = _regular_labels(D)
    rp_h, col_h = G.numpy()
    deg = np.diff(rp_h)
    v = int(np.argmax(deg >= 2))  # a row with a second entry
    u = int(np.flatnonzero(deg >= 1)[-1])  # another non-empty row
    bad_col = D.col.clone()
    bad_col[int(rp_h[v]) + 1] = G.n + 1000  # not its row's first entry
    bad_col[int(rp_h[u])] = G.n + 7  # a row's first entry
    bad_rp = D.row_ptr.clone()
    bad_rp[5] = bad_rp[6] + 1  # offsets decrease
    out = torch.full((G.n,), -1, dtype=torch.int32, device="cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    for rp_t, col_t in ((D.row_ptr, bad_col), (bad_rp, D.col)):
        assert run(rp_t.data_ptr(), col_t.data_ptr(), G.n, G.m, out.data_ptr(), stream) == \
            _lib.CC_ERR_INVALID
        out.fill_(-1)
        assert run(D.row_ptr.data_ptr(), D.col.data_ptr(), G.n, G.m, out.data_ptr(), stream) == \
            _lib.CC_OK
        assert np.array_equal(out.cpu().numpy(), want)


def test_noalloc_on_a_side_stream(cuda):
    """The solve runs on the caller's stream, here not torch's current one."""
    import torch
    run = _noalloc()
    G = cc.gen_grid(200, 150, 0.55, seed=8, id_bytes=4)
    D = G.to_device("cuda:0")
    want = _regular_labels(D)
    side = torch.cuda.Stream()
    out = torch.full((G.n,), -1, dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    assert run(D.row_ptr.data_ptr(), D.col.data_ptr(), G.n, G.m, out.data_ptr(),
               side.cuda_stream) == _lib.CC_OK
    assert np.array_equal(out.cpu().numpy(), want)
