"""Host and device CSR graphs, the METIS reader and the synthetic generators.

`StaticGraph` plays the part of the reference's StaticGraph
(lib/data_structures/static_graph.h:48-704) for a single rank: a symmetric
CSR with uint64 row offsets and uint32 or uint64 neighbour ids.  Its arrays
are numpy arrays (host) or torch CUDA tensors (device); `to_c()` describes
them to the C ABI without copying.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _ptr(x) -> int:
    if _is_torch(x):
        return x.data_ptr()
    return x.ctypes.data


@dataclass
class StaticGraph:
    row_ptr: object            # (n+1,) uint64 / int64
    col: object                # (m,) uint32/int32 or uint64/int64
    num_parts: int = 1         # virtual ranks P

    @property
    def n(self) -> int:
        return int(self.row_ptr.shape[0]) - 1

    @property
    def m(self) -> int:
        return int(self.col.shape[0])

    @property
    def id_bytes(self) -> int:
        return int(self.col.element_size() if _is_torch(self.col) else self.col.itemsize)

    @property
    def on_device(self) -> bool:
        return _is_torch(self.row_ptr) and self.row_ptr.is_cuda

    # reference accessors used by the drivers
    def GetNumberOfVertices(self) -> int:
        return self.n

    def GetNumberOfEdges(self) -> int:
        return self.m

    def to_c(self) -> _lib.cc_csr:
        g = _lib.cc_csr()
        g.n = self.n
        g.m_dir = self.m
        g.row_ptr = _ptr(self.row_ptr) if self.n >= 0 else None
        g.col = _ptr(self.col) if self.m > 0 else None
        g.id_bytes = self.id_bytes
        g.num_parts = int(self.num_parts)
        g.where = _lib.CC_DEVICE if self.on_device else _lib.CC_HOST
        g.reserved = 0
        return g

    def to_device(self, device="cuda", pin=False):
        import torch
        rp = torch.from_numpy(np.ascontiguousarray(self.row_ptr).view(np.int64))
        dt = np.int32 if self.id_bytes == 4 else np.int64
        col = torch.from_numpy(np.ascontiguousarray(self.col).view(dt))
        return StaticGraph(rp.to(device), col.to(device), self.num_parts)

    def pinned(self):
        """Host copy in page-locked memory (torch), for timed host->device copies."""
        import torch
        rp = torch.from_numpy(np.ascontiguousarray(self.row_ptr).view(np.int64)).pin_memory()
        dt = np.int32 if self.id_bytes == 4 else np.int64
        col = torch.from_numpy(np.ascontiguousarray(self.col).view(dt)).pin_memory()
        return StaticGraph(rp, col, self.num_parts)

    def with_parts(self, P: int) -> "StaticGraph":
        return StaticGraph(self.row_ptr, self.col, P)

    def numpy(self):
        """(row_ptr uint64, col uint64) host copies."""
        if _is_torch(self.row_ptr):
            rp = self.row_ptr.cpu().numpy().view(np.uint64)
            c = self.col.cpu().numpy()
        else:
            rp, c = np.asarray(self.row_ptr).view(np.uint64), np.asarray(self.col)
        c = c.view(np.uint32 if c.itemsize == 4 else np.uint64).astype(np.uint64)
        return rp, c


def from_edges(n: int, edges, id_bytes: int = 4, num_parts: int = 1) -> StaticGraph:
    """Symmetric CSR from undirected edges; self-loops and duplicates dropped,
    rows sorted (the reference sorts edges for static graphs,
    graph_io.h:140-143)."""
    e = np.asarray(edges, dtype=np.uint64).reshape(-1, 2)
    if e.size:
        e = e[e[:, 0] != e[:, 1]]
        both = np.concatenate([e, e[:, ::-1]])
        keys = np.unique(both[:, 0] * np.uint64(max(n, 1)) + both[:, 1])
        src = keys // np.uint64(max(n, 1))
        dst = keys % np.uint64(max(n, 1))
    else:
        src = dst = np.zeros(0, np.uint64)
    rp = np.zeros(n + 1, np.uint64)
    np.add.at(rp, (src + np.uint64(1)).astype(np.int64), 1)
    rp = np.cumsum(rp).astype(np.uint64)
    col = dst.astype(np.uint32 if id_bytes == 4 else np.uint64)
    return StaticGraph(rp, col, num_parts)


def _read(fn: str, path: str, id_bytes: int, num_parts: int) -> StaticGraph:
    hg = _lib.cc_host_graph()
    _lib.check(getattr(_lib.gen(), fn)(str(path).encode(), id_bytes, C.byref(hg)))
    return _HostGraph(hg).to_static(num_parts)


def read_metis(path: str, id_bytes: int = 4, num_parts: int = 1) -> StaticGraph:
    """METIS text format (GraphIO::ReadMETISFile, graph_io.h:280-382): a header
    `n m`, then one line of 1-based neighbour ids per vertex; `%` lines are
    comments.  The header's m is not trusted (example/simple.graph states 5
    for 4 edges); the adjacency is symmetrised.  Parsed by libccgen."""
    return _read("cc_read_metis", path, id_bytes, num_parts)


def read_edge_list(path: str, id_bytes: int = 4, num_parts: int = 1) -> StaticGraph:
    """Sorted edge file (GraphIO::ReadSortedEdgeFile, graph_io.h:385-670): a
    header `<type> n m`, then `e u w` records with 1-based endpoints."""
    return _read("cc_read_edge_list", path, id_bytes, num_parts)


def read_binary_edges(path: str, id_bytes: int = 4, num_parts: int = 1) -> StaticGraph:
    """Sorted binary file (GraphIO::ReadSortedBinaryFile, graph_io.h:910-1175):
    uint64 n, uint64 m, then m pairs of uint64 1-based endpoints."""
    return _read("cc_read_binary_edges", path, id_bytes, num_parts)


def _read_device(fn: str, path: str, id_bytes: int, num_parts: int, device, context) -> StaticGraph:
    import torch
    f = getattr(_lib.gpu(), fn)
    h = context.handle if context is not None else None
    n, m = C.c_uint64(), C.c_uint64()
    _lib.check(f(h, str(path).encode(), id_bytes, None, None, 0, C.byref(n), C.byref(m)))  # size query
    rp = torch.empty(n.value + 1, dtype=torch.int64, device=device)
    dt = torch.int32 if id_bytes == 4 else torch.int64
    col = torch.empty(max(m.value, 1), dtype=dt, device=device)
    with torch.cuda.device(rp.device):
        _lib.check(f(h, str(path).encode(), id_bytes, rp.data_ptr(), col.data_ptr(), m.value,
                     C.byref(n), C.byref(m)))
    return StaticGraph(rp, col[: m.value].clone(), num_parts)


def read_metis_device(path: str, id_bytes: int = 4, num_parts: int = 1, device="cuda",
                      context=None) -> StaticGraph:
    """read_metis parsed and built on the device (the same CSR, torch CUDA
    tensors): the file's bytes cross the host link once."""
    return _read_device("cc_read_metis_device", path, id_bytes, num_parts, device, context)


def read_binary_edges_device(path: str, id_bytes: int = 4, num_parts: int = 1, device="cuda",
                             context=None) -> StaticGraph:
    """read_binary_edges built on the device (the same CSR, torch CUDA tensors)."""
    return _read_device("cc_read_binary_edges_device", path, id_bytes, num_parts, device, context)


def load_graph(conf, id_bytes: int = 4, num_parts: int = 1) -> StaticGraph:
    """The input of the reference drivers (IOUtility::LoadGraph,
    io_utils.h:33-56) from a parsed Config: `-input file|edgefile|binary -in
    <path>` reads the file (METIS text, sorted edge file, sorted binary file);
    otherwise `-gen gnm_undirected|grid_2d|rhg` with `-n -m -p -d -gamma
    -seed` builds the graph with the seeded generators.  Partitioned edge
    files (one per rank) and the other KaGen models are refused."""
    t = conf.input_type
    if t == "file":
        return read_metis(conf.input_file, id_bytes, num_parts)
    if t == "edgefile":
        return read_edge_list(conf.input_file, id_bytes, num_parts)
    if t == "binary":
        return read_binary_edges(conf.input_file, id_bytes, num_parts)
    if t == "partition":
        raise ValueError("-input partition (one edge file per rank) is not read on one device")
    if conf.gen == "gnm_undirected":
        return gen_gnm(conf.gen_n, conf.gen_m, seed=conf.seed, id_bytes=id_bytes, num_parts=num_parts)
    if conf.gen == "grid_2d":
        if conf.gen_periodic:
            raise ValueError("-periodic grids are not generated")
        return gen_grid(conf.gen_n, conf.gen_m, conf.gen_p, seed=conf.seed, id_bytes=id_bytes,
                        num_parts=num_parts)
    if conf.gen == "rhg":
        return gen_rhg(conf.gen_n, conf.gen_d, conf.gen_gamma, seed=conf.seed, id_bytes=id_bytes,
                       num_parts=num_parts)
    if conf.gen != "null":
        raise ValueError(f"generator {conf.gen} is not supported")
    raise ValueError("I/O type not supported: give -input file|edgefile|binary -in <path>, or -gen")


class _HostGraph:
    """Owns a graph allocated by libccgen; frees it on close."""

    def __init__(self, hg: _lib.cc_host_graph):
        self.hg = hg

    def to_static(self, num_parts=1) -> StaticGraph:
        n, m, idb = self.hg.n, self.hg.m_dir, self.hg.id_bytes
        rp = np.ctypeslib.as_array(C.cast(self.hg.row_ptr, C.POINTER(C.c_uint64)), shape=(n + 1,)).copy()
        ct = C.c_uint32 if idb == 4 else C.c_uint64
        if m:
            col = np.ctypeslib.as_array(C.cast(self.hg.col, C.POINTER(ct)), shape=(m,)).copy()
        else:
            col = np.zeros(0, np.uint32 if idb == 4 else np.uint64)
        _lib.gen().cc_host_graph_free(self.hg)
        return StaticGraph(rp, col, num_parts)


def gen_gnm(n: int, m: int, seed: int = 1, id_bytes: int = 8, num_parts: int = 1) -> StaticGraph:
    """G(n, m): KaGen gnm_undirected (-gen gnm_undirected -n log2 n -m log2 m)."""
    hg = _lib.cc_host_graph()
    _lib.check(_lib.gen().cc_gen_gnm(n, m, seed, id_bytes, C.byref(hg)))
    return _HostGraph(hg).to_static(num_parts)


def gen_grid(X: int, Y: int, p: float = 0.5, seed: int = 1, id_bytes: int = 4,
             num_parts: int = 1) -> StaticGraph:
    """2D bond percolation (-gen grid_2d -n X -m Y -p p)."""
    hg = _lib.cc_host_graph()
    _lib.check(_lib.gen().cc_gen_grid(X, Y, p, seed, id_bytes, C.byref(hg)))
    return _HostGraph(hg).to_static(num_parts)


def _device_graph(fill, n: int, cap: int, id_bytes: int, device, num_parts: int) -> StaticGraph:
    import torch
    rp = torch.empty(n + 1, dtype=torch.int64, device=device)
    dt = torch.int32 if id_bytes == 4 else torch.int64
    col = torch.empty(max(cap, 1), dtype=dt, device=device)
    m = C.c_uint64()
    with torch.cuda.device(rp.device):
        st = fill(rp.data_ptr(), col.data_ptr(), cap, C.byref(m))
        if st == _lib.CC_ERR_INVALID and m.value > cap:  # an estimated capacity fell short
            del col
            cap = m.value
            col = torch.empty(max(cap, 1), dtype=dt, device=device)
            st = fill(rp.data_ptr(), col.data_ptr(), cap, C.byref(m))
        _lib.check(st)
    if m.value == cap:
        return StaticGraph(rp, col[: max(cap, 0)], num_parts)
    return StaticGraph(rp, col[: m.value].clone(), num_parts)  # exact-size storage


def gen_grid_device(X: int, Y: int, p: float = 0.5, seed: int = 1, id_bytes: int = 4,
                    num_parts: int = 1, device="cuda") -> StaticGraph:
    """gen_grid built on the device (the same graph, torch CUDA tensors)."""
    return _device_graph(lambda rp, col, cap, m: _lib.gpu().cc_gen_grid_device(
        None, X, Y, p, seed, id_bytes, rp, col, cap, m), X * Y, 2 * ((X - 1) * Y + X * (Y - 1)),
        id_bytes, device, num_parts)


def gen_gnm_device(n: int, m: int, seed: int = 1, id_bytes: int = 8, num_parts: int = 1,
                   device="cuda") -> StaticGraph:
    """gen_gnm built on the device (the same graph, torch CUDA tensors)."""
    return _device_graph(lambda rp, col, cap, mm: _lib.gpu().cc_gen_gnm_device(
        None, n, m, seed, id_bytes, rp, col, cap, mm), n, 2 * m, id_bytes, device, num_parts)


def gen_rhg_device(n: int, avg_deg: float = 16.0, gamma: float = 2.6, seed: int = 1,
                   id_bytes: int = 4, num_parts: int = 1, device="cuda", context=None) -> StaticGraph:
    """gen_rhg built on the device (the same graph bit for bit, torch CUDA
    tensors).  With a profiling context its phases are timed (context.stats())."""
    cap = int(1.25 * n * avg_deg) + 4096
    h = context.handle if context is not None else None
    return _device_graph(lambda rp, col, cp, m: _lib.gpu().cc_gen_rhg_device(
        h, n, avg_deg, gamma, seed, id_bytes, rp, col, cp, m), n, cap, id_bytes, device, num_parts)


def gen_rhg(n: int, avg_deg: float = 16.0, gamma: float = 2.6, seed: int = 1, id_bytes: int = 4,
            num_parts: int = 1) -> StaticGraph:
    """Random hyperbolic graph, threshold model (-gen rhg -n log2 n -d d -gamma g)."""
    hg = _lib.cc_host_graph()
    _lib.check(_lib.gen().cc_gen_rhg(n, avg_deg, gamma, seed, id_bytes, C.byref(hg)))
    return _HostGraph(hg).to_static(num_parts)
