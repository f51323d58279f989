"""Batched solves: many independent graphs in one launch sequence
(include/cc_batch.h).

`Batch` holds the segmented CSR: vertex offsets `voff` (k+1), global row
offsets `row_ptr` (total_n+1) and LOCAL uint32 neighbour ids `col`.  Labels
come back as local canonical labels, the same values cc_gpu_run() gives each
graph alone.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .graph import StaticGraph, _is_torch, _ptr


class cc_batch(C.Structure):
    _fields_ = [("k", C.c_uint32), ("where", C.c_uint32), ("total_n", C.c_uint64),
                ("total_m", C.c_uint64), ("voff", C.c_void_p), ("row_ptr", C.c_void_p),
                ("col", C.c_void_p)]


BUCKETS = 4


class cc_batch_tuning(C.Structure):
    _fields_ = [("smem_max_n", C.c_uint32 * BUCKETS), ("threads", C.c_uint32 * BUCKETS),
                ("edge_parallel", C.c_uint32 * BUCKETS), ("hub_degree", C.c_uint32),
                ("use_graph", C.c_uint32)]

    def as_dict(self) -> dict:
        return {"smem_max_n": list(self.smem_max_n), "threads": list(self.threads),
                "edge_parallel": list(self.edge_parallel), "hub_degree": self.hub_degree,
                "use_graph": self.use_graph}


class cc_host_batch(C.Structure):
    _fields_ = [("k", C.c_uint32), ("pad_", C.c_uint32), ("total_n", C.c_uint64),
                ("total_m", C.c_uint64), ("voff", C.c_void_p), ("row_ptr", C.c_void_p),
                ("col", C.c_void_p)]


_BOUND = False


def _bind():
    global _BOUND
    if _BOUND:
        return
    g = _lib.gpu()
    P = C.c_void_p
    for name, res, args in [
        ("cc_batch_tuning_default", None, [C.POINTER(cc_batch_tuning)]),
        ("cc_batch_run", C.c_int, [P, C.POINTER(cc_batch), C.POINTER(cc_batch_tuning), P, C.c_uint32]),
        ("cc_batch_autotune", C.c_int, [P, C.POINTER(cc_batch), C.c_int, C.POINTER(cc_batch_tuning)]),
        ("cc_batch_run_plain", C.c_int, [P, C.POINTER(cc_batch), C.c_int, C.POINTER(_lib.cc_config),
                                         C.c_uint64, P]),
    ]:
        fn = getattr(g, name)
        fn.restype, fn.argtypes = res, args
    ge = _lib.gen()
    ge.cc_gen_batch.restype = C.c_int
    ge.cc_gen_batch.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_uint64, C.POINTER(cc_host_batch)]
    ge.cc_host_batch_free.restype = None
    ge.cc_host_batch_free.argtypes = [C.POINTER(cc_host_batch)]
    _BOUND = True


@dataclass
class Batch:
    voff: object
    row_ptr: object
    col: object

    @property
    def k(self) -> int:
        return int(self.voff.shape[0]) - 1

    @property
    def total_n(self) -> int:
        return int(self.row_ptr.shape[0]) - 1

    @property
    def total_m(self) -> int:
        return int(self.col.shape[0])

    @property
    def on_device(self) -> bool:
        return _is_torch(self.voff) and self.voff.is_cuda

    def to_c(self) -> cc_batch:
        b = cc_batch()
        b.k = self.k
        b.where = _lib.CC_DEVICE if self.on_device else _lib.CC_HOST
        b.total_n = self.total_n
        b.total_m = self.total_m
        b.voff = _ptr(self.voff)
        b.row_ptr = _ptr(self.row_ptr)
        b.col = _ptr(self.col) if self.total_m else None
        return b

    def numpy(self):
        f = (lambda x: x.cpu().numpy()) if _is_torch(self.voff) else np.asarray
        return (f(self.voff).view(np.uint64), f(self.row_ptr).view(np.uint64),
                f(self.col).view(np.uint32))

    def to_device(self, device="cuda"):
        import torch
        v, r, c = self.numpy()
        return Batch(torch.from_numpy(v.view(np.int64)).to(device),
                     torch.from_numpy(r.view(np.int64)).to(device),
                     torch.from_numpy(c.view(np.int32)).to(device))

    def pinned(self):
        import torch
        v, r, c = self.numpy()
        return Batch(torch.from_numpy(v.view(np.int64)).pin_memory(),
                     torch.from_numpy(r.view(np.int64)).pin_memory(),
                     torch.from_numpy(c.view(np.int32)).pin_memory())

    def graph(self, i: int) -> StaticGraph:
        """Graph i alone (local ids), as host arrays."""
        v, r, c = self.numpy()
        a, b = int(v[i]), int(v[i + 1])
        rp = r[a:b + 1] - r[a]
        return StaticGraph(rp.astype(np.uint64), c[int(r[a]):int(r[b])].copy())

    @staticmethod
    def pack(graphs: list[StaticGraph]) -> "Batch":
        voff = [0]
        rps, cols = [], []
        e = 0
        for G in graphs:
            rp, col = G.numpy()
            rps.append(rp[:-1] + np.uint64(e))
            cols.append(col.astype(np.uint32))
            e += G.m
            voff.append(voff[-1] + G.n)
        rp_all = np.concatenate(rps + [np.array([e], np.uint64)]) if rps else np.zeros(1, np.uint64)
        col_all = np.concatenate(cols) if cols else np.zeros(0, np.uint32)
        return Batch(np.array(voff, np.uint64), rp_all.astype(np.uint64), col_all)


def gen_batch(k: int = 4096, log2_nmin: float = 8, log2_nmax: float = 18, dmin: float = 0.5,
              dmax: float = 8.0, seed: int = 1) -> Batch:
    """The batched G(n, m) workload: k graphs, n log-uniform, degree uniform."""
    _bind()
    hb = cc_host_batch()
    _lib.check(_lib.gen().cc_gen_batch(k, log2_nmin, log2_nmax, dmin, dmax, seed, C.byref(hb)))
    try:
        v = np.ctypeslib.as_array(C.cast(hb.voff, C.POINTER(C.c_uint64)), (k + 1,)).copy()
        r = np.ctypeslib.as_array(C.cast(hb.row_ptr, C.POINTER(C.c_uint64)), (hb.total_n + 1,)).copy()
        c = (np.ctypeslib.as_array(C.cast(hb.col, C.POINTER(C.c_uint32)), (hb.total_m,)).copy()
             if hb.total_m else np.zeros(0, np.uint32))
    finally:
        _lib.gen().cc_host_batch_free(C.byref(hb))
    return Batch(v, r, c)


def default_tuning() -> cc_batch_tuning:
    _bind()
    t = cc_batch_tuning()
    _lib.gpu().cc_batch_tuning_default(C.byref(t))
    return t


def batch_run(batch: Batch, ctx=None, tuning: cc_batch_tuning | None = None, labels=None):
    """Local canonical labels of every graph in `batch` (uint32, total_n)."""
    _bind()
    from .solvers import default_context
    ctx = ctx or default_context()
    if labels is None:
        if batch.on_device:
            import torch
            labels = torch.empty(batch.total_n, dtype=torch.int32, device=batch.voff.device)
        else:
            labels = np.empty(batch.total_n, np.uint32)
    where = _lib.CC_DEVICE if (_is_torch(labels) and labels.is_cuda) else _lib.CC_HOST
    b = batch.to_c()
    _lib.check(_lib.gpu().cc_batch_run(ctx.handle, C.byref(b), C.byref(tuning) if tuning else None,
                                       _ptr(labels), where))
    return labels


def autotune(batch: Batch, ctx=None, reps: int = 3) -> cc_batch_tuning:
    _bind()
    from .solvers import default_context
    ctx = ctx or default_context()
    b = batch.to_c()
    t = cc_batch_tuning()
    _lib.check(_lib.gpu().cc_batch_autotune(ctx.handle, C.byref(b), reps, C.byref(t)))
    return t


def plain_run(batch: Batch, ctx, labels, algo: str = "exp", conf=None) -> None:
    """The plain path: one cc_ctx_run per graph, looped in C++
    (cc_batch_run_plain); device batch and device labels (total_n int32)."""
    from .config import Config
    _bind()
    if not batch.on_device:
        raise ValueError("plain_run takes a device batch")
    conf = conf or Config()
    b = batch.to_c()
    _lib.check(_lib.gpu().cc_batch_run_plain(ctx.handle, C.byref(b), _lib.ALGOS[algo],
                                             C.byref(conf.to_c()), int(conf.seed), labels.data_ptr()))
