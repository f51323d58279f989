"""The reference's solver classes over the C ABI.

    comp = ExponentialContraction(conf, rank, size)
    comp.FindComponents(G, labels)

as in app/exp_contraction.cpp:104-105 (and all_reduce.cpp:97-98,
local_contraction.cpp:114/142, shortcuts.cpp:117/145, labels.cpp:101).  On one
GPU the `size` ranks become virtual ranks: contiguous vertex ranges of the one
device-resident CSR (graph_io.h:308-313), so the partition-local steps of the
algorithms keep their meaning.  `labels` is overwritten with canonical labels
(minimum vertex id of the component) for every vertex.

There is no CPU path: these classes call libccgpu and raise if it is missing
or the call fails.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .config import Config
from .graph import StaticGraph, _is_torch, _ptr


class Context:
    """A libccgpu context: one CUDA stream and one device memory pool."""

    def __init__(self, device: int = 0, stream=None, profiling: bool = False):
        self._h = C.c_void_p()
        s = None
        if stream is not None:
            s = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        _lib.check(_lib.gpu().cc_ctx_create(C.byref(self._h), device, s))
        if profiling:
            self.set_profiling(True, components=True)

    @property
    def handle(self):
        return self._h

    @property
    def stream_handle(self) -> int:
        return _lib.gpu().cc_ctx_stream(self._h) or 0

    def set_tuning(self, hook_mode: int = 0, tile_vertices: int = 0, tile_threads: int = 0,
                   hub_degree: int = 0) -> None:
        """Hook-and-compress schedule (include/cc_gpu.h cc_tuning); 0 keeps a default."""
        t = _lib.cc_tuning(hook_mode, tile_vertices, tile_threads, hub_degree)
        _lib.check(_lib.gpu().cc_ctx_set_tuning(self._h, C.byref(t)))

    def tuning(self) -> dict:
        t = _lib.cc_tuning()
        _lib.check(_lib.gpu().cc_ctx_get_tuning(self._h, C.byref(t)))
        return {"hook_mode": t.hook_mode, "tile_vertices": t.tile_vertices,
                "tile_threads": t.tile_threads, "hub_degree": t.hub_degree}

    def set_host_reads(self, mode: int) -> None:
        """Sampled linking of a host graph in page-locked memory: 1 (True, the
        default) reads it in place, 2 reads the ids in place and copies the
        offsets in chunks, 0 (False) copies its rows in chunks."""
        _lib.check(_lib.gpu().cc_ctx_set_host_reads(self._h, int(mode)))

    def set_profiling(self, on: bool, components: bool = False) -> None:
        """Per-kernel CUDA-event timing; with `components` also the component
        count of each solve (one extra pass over the labels)."""
        flags = (_lib.CC_PROF_KERNELS if on else 0) | (_lib.CC_PROF_COMPONENTS if components else 0)
        _lib.check(_lib.gpu().cc_ctx_set_profiling(self._h, flags))

    def run(self, g: StaticGraph, algo: int, cfg: _lib.cc_config, seed: int, labels) -> None:
        csr = g.to_c()
        where = _lib.CC_DEVICE if (_is_torch(labels) and labels.is_cuda) else _lib.CC_HOST
        _lib.check(_lib.gpu().cc_ctx_run(self._h, C.byref(csr), algo, C.byref(cfg), seed,
                                         _ptr(labels), where))

    def stats(self) -> dict:
        st = _lib.cc_stats()
        _lib.check(_lib.gpu().cc_ctx_stats(self._h, C.byref(st)))
        return st.as_dict()

    def profile_totals(self) -> dict:
        """Sums over the solves since profiling was switched on, plus `solves`."""
        st = _lib.cc_stats()
        n = C.c_uint64()
        _lib.check(_lib.gpu().cc_ctx_profile_totals(self._h, C.byref(st), C.byref(n)))
        d = st.as_dict()
        d["solves"] = int(n.value)
        return d

    def arena_bytes(self) -> int:
        return int(_lib.gpu().cc_ctx_arena_bytes(self._h))

    def close(self) -> None:
        if self._h:
            _lib.gpu().cc_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: dict[int, Context] = {}


def default_context() -> Context:
    dev = 0
    try:
        import torch
        if torch.cuda.is_available():
            dev = torch.cuda.current_device()
    except ImportError:
        pass
    if dev not in _default_ctx:
        _default_ctx[dev] = Context(dev)
    return _default_ctx[dev]


def _check_labels(G: StaticGraph, labels) -> None:
    n = G.n
    if int(labels.shape[0]) < n:
        raise ValueError(f"labels has {labels.shape[0]} entries, graph has {n} vertices")
    isz = labels.element_size() if _is_torch(labels) else labels.itemsize
    if isz != G.id_bytes:
        raise ValueError(f"labels are {isz}-byte, graph ids are {G.id_bytes}-byte")
    if not _is_torch(labels) and not labels.flags["C_CONTIGUOUS"]:
        raise ValueError("labels must be contiguous")
    if _is_torch(labels) and not labels.is_contiguous():
        raise ValueError("labels must be contiguous")


class _Solver:
    ALGO = _lib.CC_EXP

    def __init__(self, conf: Config, rank: int = 0, size: int = 1, context: Context | None = None):
        if rank != 0:
            raise ValueError("one process drives one GPU: rank must be 0 (size = virtual ranks)")
        if size < 1:
            raise ValueError("size must be >= 1")
        self.config_ = conf
        self.rank_ = rank
        self.size_ = size
        self.ctx = context
        self._ran_on: Context | None = None

    @property
    def last_stats(self) -> dict:
        """Statistics of the last solve on this solver's context (read on demand)."""
        return self._ran_on.stats() if self._ran_on is not None else {}

    def FindComponents(self, G: StaticGraph, labels) -> None:
        _check_labels(G, labels)
        ctx = self.ctx or default_context()
        g = G.with_parts(self.size_) if G.num_parts != self.size_ else G
        ctx.run(g, self.ALGO, self.config_.to_c(), int(self.config_.seed), labels)
        self._ran_on = ctx

    # driver statistics (exponential_contraction.h:325-335): no exchange on
    # one device
    def GetCommTime(self) -> float:
        return 0.0

    def GetSendVolume(self) -> int:
        return 0

    def GetReceiveVolume(self) -> int:
        return 0


class ExponentialContraction(_Solver):
    """lib/components/exponential_contraction.h:40"""
    ALGO = _lib.CC_EXP


class LocalContraction(_Solver):
    """lib/components/local_contraction.h:39"""
    ALGO = _lib.CC_LOCAL


class ShortcutPropagation(_Solver):
    """lib/components/shortcut_propagation.h:38"""
    ALGO = _lib.CC_SHORTCUTS


class Propagation(_Solver):
    """lib/components/propagation.h:38"""
    ALGO = _lib.CC_LABELS


class AllReduce(_Solver):
    """lib/components/all_reduce.h:34 (AllReduce<GraphType>)"""
    ALGO = _lib.CC_ALLREDUCE


SOLVERS = {"exp": ExponentialContraction, "local": LocalContraction,
           "shortcuts": ShortcutPropagation, "labels": Propagation, "allreduce": AllReduce}


def find_components(G: StaticGraph, algo: str = "exp", conf: Config | None = None,
                    context: Context | None = None):
    """Convenience: labels (same kind and placement as G's ids) for G."""
    conf = conf or Config()
    if G.on_device:
        import torch
        dt = torch.int32 if G.id_bytes == 4 else torch.int64
        labels = torch.empty(G.n, dtype=dt, device=G.row_ptr.device)
    else:
        labels = np.empty(G.n, np.uint32 if G.id_bytes == 4 else np.uint64)
    SOLVERS[algo](conf, 0, G.num_parts, context).FindComponents(G, labels)
    return labels


def component_sizes(labels, context: Context | None = None):
    """Component-size summary of a label array, computed on the device
    (OutputComponents, static_graph.h:504-591): an (k, 2) uint64 array of
    (size, number of components of that size) rows in ascending size, and the
    number of components with more than one vertex (the reference's
    "NUM COMPONENTS").  `labels`: numpy or torch CUDA array of uint32/uint64
    labels below len(labels), e.g. the output of FindComponents."""
    if _is_torch(labels):
        import torch
        if labels.dtype not in (torch.int32, torch.int64) or not labels.is_contiguous():
            raise ValueError("labels: a contiguous int32/int64 tensor")
        where = _lib.CC_DEVICE if labels.is_cuda else _lib.CC_HOST
        idb, n, ptr = labels.element_size(), labels.numel(), labels.data_ptr()
    else:
        labels = np.ascontiguousarray(labels)
        if labels.dtype.itemsize not in (4, 8) or labels.dtype.kind not in "iu":
            raise ValueError("labels: a 32- or 64-bit integer array")
        where, idb, n, ptr = _lib.CC_HOST, labels.dtype.itemsize, labels.size, labels.ctypes.data
    cap = int(np.sqrt(2.0 * n)) + 2
    pairs = np.zeros((cap, 2), np.uint64)
    k, nc = C.c_uint64(), C.c_uint64()
    h = context.handle if context is not None else None
    _lib.check(_lib.gpu().cc_component_sizes(h, ptr, idb, where, n, pairs.ctypes.data, cap,
                                             C.byref(k), C.byref(nc)))
    return pairs[: min(k.value, cap)].copy(), int(nc.value)

