"""Continuous-batching server (include/cc_serve.h) from Python.

    srv = Server(budget_bytes=120 << 30)
    t = srv.submit(G)            # host StaticGraph; keep G alive until collected
    labels, info = srv.wait(t)   # canonical labels, timestamps

Requests are admitted under the HBM budget as they arrive, copied while
earlier batches run, coalesced into batched launches, and collected in any
order.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .graph import StaticGraph


class cc_serve_config(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_batch_graphs", C.c_uint32),
                ("compute_streams", C.c_uint32), ("smem_max_n", C.c_uint32),
                ("batch_window_us", C.c_uint32)]


class cc_serve_ticket_info(C.Structure):
    _fields_ = [("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("batch_id", C.c_uint32), ("batch_size", C.c_uint32)]

    def as_dict(self) -> dict:
        return {"submit_s": self.submit_s, "admit_s": self.admit_s, "done_s": self.done_s,
                "batch_id": self.batch_id, "batch_size": self.batch_size}


class cc_serve_stats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("collected", C.c_uint64),
                ("batches", C.c_uint64), ("bytes_in_use", C.c_uint64),
                ("peak_bytes_in_use", C.c_uint64), ("waiting", C.c_uint64)]


_BOUND = False


def _bind():
    global _BOUND
    if _BOUND:
        return
    g = _lib.gpu()
    P = C.c_void_p
    for name, res, args in [
        ("cc_serve_config_default", None, [C.POINTER(cc_serve_config)]),
        ("cc_serve_create", C.c_int, [C.POINTER(P), C.c_int, C.POINTER(cc_serve_config)]),
        ("cc_serve_destroy", C.c_int, [P]),
        ("cc_serve_submit", C.c_int, [P, C.POINTER(_lib.cc_csr), C.POINTER(C.c_uint64)]),
        ("cc_serve_poll", C.c_int, [P, C.c_uint64, P, C.POINTER(C.c_int),
                                    C.POINTER(cc_serve_ticket_info)]),
        ("cc_serve_wait", C.c_int, [P, C.c_uint64, P, C.c_double, C.POINTER(cc_serve_ticket_info)]),
        ("cc_serve_get_stats", C.c_int, [P, C.POINTER(cc_serve_stats)]),
        ("cc_serve_now", C.c_double, []),
    ]:
        fn = getattr(g, name)
        fn.restype, fn.argtypes = res, args
    _BOUND = True


def now() -> float:
    _bind()
    return float(_lib.gpu().cc_serve_now())


class Server:
    def __init__(self, device: int = 0, budget_bytes: int | None = None, max_batch: int = 0,
                 streams: int = 0, smem_max_n: int = 0, window_us: int = 0):
        _bind()
        cfg = cc_serve_config()
        _lib.gpu().cc_serve_config_default(C.byref(cfg))
        if budget_bytes is not None:
            cfg.hbm_budget_bytes = int(budget_bytes)
        if max_batch:
            cfg.max_batch_graphs = max_batch
        if streams:
            cfg.compute_streams = streams
        if smem_max_n:
            cfg.smem_max_n = smem_max_n
        cfg.batch_window_us = window_us
        self._h = C.c_void_p()
        _lib.check(_lib.gpu().cc_serve_create(C.byref(self._h), device, C.byref(cfg)))
        self._graphs: dict[int, StaticGraph] = {}

    def submit(self, G: StaticGraph) -> int:
        if G.on_device:
            raise ValueError("the server takes host graphs")
        csr = G.to_c()
        t = C.c_uint64()
        _lib.check(_lib.gpu().cc_serve_submit(self._h, C.byref(csr), C.byref(t)))
        self._graphs[t.value] = G  # keep the host arrays alive until collected
        return t.value

    def _out(self, t: int) -> np.ndarray:
        G = self._graphs[t]
        return np.empty(max(G.n, 1), np.uint32 if G.id_bytes == 4 else np.uint64)

    def poll(self, t: int):
        out = self._out(t)
        done = C.c_int()
        info = cc_serve_ticket_info()
        _lib.check(_lib.gpu().cc_serve_poll(self._h, t, out.ctypes.data, C.byref(done), C.byref(info)))
        if not done.value:
            return None
        n = self._graphs.pop(t).n
        return out[:n], info.as_dict()

    def wait(self, t: int, timeout_s: float = 0.0):
        out = self._out(t)
        info = cc_serve_ticket_info()
        rc = _lib.gpu().cc_serve_wait(self._h, t, out.ctypes.data, timeout_s, C.byref(info))
        if rc != _lib.CC_ERR_TIMEOUT:  # any other outcome retires the ticket
            n = self._graphs.pop(t).n
        _lib.check(rc)
        return out[:n], info.as_dict()

    def stats(self) -> dict:
        s = cc_serve_stats()
        _lib.check(_lib.gpu().cc_serve_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in cc_serve_stats._fields_}

    def close(self) -> None:
        if self._h:
            _lib.gpu().cc_serve_destroy(self._h)
            self._h = C.c_void_p()
            self._graphs.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
