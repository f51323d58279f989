"""CPU oracle - TEST INFRASTRUCTURE ONLY.

A plain-C restatement (cc_oracle.c) of the reference's connected-components
algorithms plus an independent union-find.  Only tests/, the smoke check of
__graft_entry__ and the CPU-baseline legs of bench.py use it, and only as the
answer the GPU labels are compared with or as the timed CPU baseline; the
product (components_gb300) never does.

Parity is pinned to the reference's only fixture (example/simple.graph,
canonical labels [0,0,0,3,3,3]) and to the union-find: connected components
are unique, so canonical labels must agree exactly.
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libccoracle.so"

_U64P = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_SYMS = {
    "or_hash3": (C.c_uint64, [C.c_uint64, C.c_uint64, C.c_uint64]),
    "or_geo_table": (C.c_int, [C.c_double, _U64P, C.c_int]),
    "or_uf_labels": (C.c_int, [C.c_uint64, _U64P, _U64P, _U64P]),
    "or_canonicalize": (None, [C.c_uint64, _U64P]),
    "or_canonicalize_any": (None, [C.c_uint64, _U64P]),
    "or_local_components": (C.c_int, [C.c_uint64, _U64P, _U64P, C.c_uint64, _U64P]),
    "or_contract": (C.c_int, [C.c_uint64, _U64P, _U64P, _U64P, C.c_uint64, C.c_uint64, _U64P,
                              _U64P, _U64P, _U64P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "or_ldd": (C.c_int, [C.c_uint64, _U64P, _U64P, _U64P, C.c_uint64, C.c_uint64, C.c_double,
                         _U64P]),
    "or_local_sweeps": (C.c_int, [C.c_uint64, _U64P, _U64P, _U64P, C.c_uint64, C.c_uint64, _U64P]),
    "or_allreduce": (C.c_int, [C.c_uint64, _U64P, _U64P, _U64P, _U64P]),
    "or_exp_contraction": (C.c_int, [C.c_uint64, _U64P, _U64P, C.c_uint64, C.c_double, C.c_uint64,
                                     C.c_int, C.c_uint64, _U64P, C.POINTER(C.c_uint64)]),
    "or_local_contraction": (C.c_int, [C.c_uint64, _U64P, _U64P, C.c_uint64, C.c_uint64, _U64P]),
    "or_labels": (C.c_int, [C.c_uint64, _U64P, _U64P, _U64P]),
    "or_shortcut": (C.c_int, [C.c_uint64, _U64P, _U64P, _U64P, C.c_uint64]),
}


class _HostGraphC(C.Structure):  # cc_host_graph of include/cc_gen.h
    _fields_ = [("n", C.c_uint64), ("m_dir", C.c_uint64), ("row_ptr", C.c_void_p),
                ("col", C.c_void_p), ("id_bytes", C.c_uint32), ("pad_", C.c_uint32)]


_GEN_SYMS = {
    "or_gen_gnm": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint32, C.POINTER(_HostGraphC)]),
    "or_gen_grid": (C.c_int, [C.c_uint64, C.c_uint64, C.c_double, C.c_uint64, C.c_uint32,
                              C.POINTER(_HostGraphC)]),
    "or_gen_rhg": (C.c_int, [C.c_uint64, C.c_double, C.c_double, C.c_uint64, C.c_uint32,
                             C.POINTER(_HostGraphC)]),
    "or_graph_free": (None, [C.POINTER(_HostGraphC)]),
}
_lib = None


GEN_SRC = HERE.parent / "components_gb300" / "csrc" / "gen.cpp"
GEN_DEPS = [GEN_SRC, HERE.parent / "components_gb300" / "csrc" / "rhg.h",
            HERE.parent / "include" / "cc_gen.h", HERE / "inputs.cpp"]


def _run(cmd: list[str]) -> subprocess.CompletedProcess:
    return subprocess.run(cmd, capture_output=True, text=True)


def build(force: bool = False) -> Path:
    """Compile cc_oracle.c with gcc and the input generators (the library's
    generator source, hidden symbols, plus inputs.cpp) with g++, OpenMP when
    available, into one libccoracle.so."""
    BUILD.mkdir(exist_ok=True)
    src = HERE / "cc_oracle.c"
    deps = [src] + GEN_DEPS
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    cc = shutil.which("gcc") or "gcc"
    cxx = shutil.which("g++") or "g++"
    err = ""
    for omp in (["-fopenmp"], []):
        objs = [BUILD / "cc_oracle.o", BUILD / "gen.o", BUILD / "inputs.o"]
        steps = [
            [cc, "-O2", "-std=c11", "-fPIC", "-ffp-contract=off", *omp, "-c", str(src), "-o", str(objs[0])],
            [cxx, "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", *omp,
             "-c", str(GEN_SRC), "-o", str(objs[1])],
            [cxx, "-O2", "-std=c++17", "-fPIC", "-c", str(HERE / "inputs.cpp"), "-o", str(objs[2])],
        ]
        tmp = LIB.with_suffix(".so.tmp")
        link = [cxx, "-shared", *omp, "-o", str(tmp)] + [str(o) for o in objs] + ["-lm"]
        ok = True
        for cmd in steps + [link]:
            r = _run(cmd)
            if r.returncode != 0:
                err, ok = r.stderr, False
                break
        for o in objs:
            if o.exists():
                o.unlink()
        if ok:
            tmp.replace(LIB)
            return LIB
    raise RuntimeError("oracle build failed:\n" + err)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        for name, (res, args) in list(_SYMS.items()) + list(_GEN_SYMS.items()):
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


class HostCSR:
    """A host CSR (numpy row_ptr uint64, col uint32 or uint64) that the
    oracle's own input path built; numpy() and n / m / id_bytes match the
    library's StaticGraph, so every function here takes either."""

    def __init__(self, row_ptr: np.ndarray, col: np.ndarray):
        self.row_ptr, self.col = row_ptr, col

    @property
    def n(self) -> int:
        return int(self.row_ptr.shape[0]) - 1

    @property
    def m(self) -> int:
        return int(self.col.shape[0])

    @property
    def id_bytes(self) -> int:
        return int(self.col.itemsize)

    def numpy(self):
        return self.row_ptr, self.col.astype(np.uint64)


def _take(fn, *args) -> HostCSR:
    hg = _HostGraphC()
    st = getattr(lib(), fn)(*args, C.byref(hg))
    if st != 0:
        raise RuntimeError(f"{fn}: status {st}")
    try:
        n, m = hg.n, hg.m_dir
        rp = np.ctypeslib.as_array(C.cast(hg.row_ptr, C.POINTER(C.c_uint64)), shape=(n + 1,)).copy()
        ct = C.c_uint32 if hg.id_bytes == 4 else C.c_uint64
        col = (np.ctypeslib.as_array(C.cast(hg.col, C.POINTER(ct)), shape=(m,)).copy() if m
               else np.zeros(0, np.uint32 if hg.id_bytes == 4 else np.uint64))
    finally:
        lib().or_graph_free(C.byref(hg))
    return HostCSR(rp, col)


def gen_rhg(n: int, avg_deg: float = 16.0, gamma: float = 2.6, seed: int = 1,
            id_bytes: int = 4) -> HostCSR:
    """The library's random hyperbolic graph, built on the host by the
    oracle's copy of the generator (no GPU library loaded)."""
    return _take("or_gen_rhg", n, avg_deg, gamma, seed, id_bytes)


def gen_grid(X: int, Y: int, p: float = 0.5, seed: int = 1, id_bytes: int = 4) -> HostCSR:
    return _take("or_gen_grid", X, Y, p, seed, id_bytes)


def gen_gnm(n: int, m: int, seed: int = 1, id_bytes: int = 8) -> HostCSR:
    return _take("or_gen_gnm", n, m, seed, id_bytes)


def induced_prefix(G, k: int) -> HostCSR:
    """The subgraph induced by vertices [0, k) of G (rows 0 .. k-1, entries
    below k kept): a bounded sample of a graph for timing the CPU baseline.
    On an angularly ordered hyperbolic graph it is one contiguous sector."""
    rp, col = G.numpy()
    k = min(int(k), G.n)
    head = col[: int(rp[k])]
    keep = head < k
    cm = np.concatenate([[0], np.cumsum(keep, dtype=np.uint64)]).astype(np.uint64)
    new_rp = cm[rp[: k + 1].astype(np.int64)]
    dt = np.uint32 if G.id_bytes == 4 else np.uint64
    return HostCSR(new_rp.astype(np.uint64), head[keep].astype(dt))


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a), dtype=np.uint64)


def csr_u64(G):
    """(n, row_ptr u64, col u64) of a components_gb300 StaticGraph."""
    rp, col = G.numpy()
    return G.n, _u64(rp), _u64(col)


def uf_labels(G) -> np.ndarray:
    n, rp, col = csr_u64(G)
    out = np.empty(max(n, 1), np.uint64)
    lib().or_uf_labels(n, rp, col, out)
    return out[:n]


def canonical(labels) -> np.ndarray:
    lab = _u64(labels).copy()
    if lab.size:
        lib().or_canonicalize_any(lab.size, lab)
    return lab


def local_components(G, P: int) -> np.ndarray:
    n, rp, col = csr_u64(G)
    out = np.empty(max(n, 1), np.uint64)
    lib().or_local_components(n, rp, col, P, out)
    return out[:n]


def contract(G, cl, ncl: int, cut_parts: int = 0):
    n, rp, col = csr_u64(G)
    cl = _u64(cl)
    rp_o = np.zeros(ncl + 1, np.uint64)
    col_o = np.zeros(max(int(rp[-1]) if n else 0, 1), np.uint64)
    vid_o = np.zeros(max(ncl, 1), np.uint64)
    newid_o = np.zeros(max(ncl, 1), np.uint64)
    nn, mm = C.c_uint64(), C.c_uint64()
    lib().or_contract(n, rp, col, cl, ncl, cut_parts, rp_o, col_o, vid_o, newid_o,
                      C.byref(nn), C.byref(mm))
    k, m = nn.value, mm.value
    return rp_o[: k + 1], col_o[:m], vid_o[:k], newid_o[:ncl]


def ldd(G, vid, seed: int, level: int, beta: float):
    n, rp, col = csr_u64(G)
    out = np.empty(max(n, 1), np.uint64)
    rounds = lib().or_ldd(n, rp, col, _u64(vid), seed, level, beta, out)
    return out[:n], rounds


def local_sweeps(G, vid, seed: int, level: int):
    n, rp, col = csr_u64(G)
    out = np.empty(max(n, 1), np.uint64)
    lib().or_local_sweeps(n, rp, col, _u64(vid), seed, level, out)
    return out[:n]


def allreduce(G, labels_in=None):
    n, rp, col = csr_u64(G)
    lab = _u64(np.arange(n) if labels_in is None else labels_in)
    out = np.empty(max(n, 1), np.uint64)
    lib().or_allreduce(n, rp, col, lab, out)
    return out[:n]


def exp_contraction(G, P: int = 1, beta: float = 0.1, seq: int = 1, fixed_seq: bool = False,
                    seed: int = 1):
    """Raw (reference-style) labels and the number of decomposition levels."""
    n, rp, col = csr_u64(G)
    out = np.empty(max(n, 1), np.uint64)
    rounds = C.c_uint64()
    levels = lib().or_exp_contraction(n, rp, col, P, beta, seq, int(fixed_seq), seed, out,
                                      C.byref(rounds))
    return out[:n], levels


def local_contraction(G, seq: int = 1, seed: int = 1):
    n, rp, col = csr_u64(G)
    out = np.empty(max(n, 1), np.uint64)
    levels = lib().or_local_contraction(n, rp, col, seq, seed, out)
    return out[:n], levels


def labels_propagation(G):
    n, rp, col = csr_u64(G)
    out = np.empty(max(n, 1), np.uint64)
    rounds = lib().or_labels(n, rp, col, out)
    return out[:n], rounds


def shortcut(G, labels=None, hitters: int = 0):
    n, rp, col = csr_u64(G)
    lab = _u64(np.arange(n) if labels is None else labels).copy()
    if lab.size == 0:
        lab = np.zeros(1, np.uint64)
    rounds = lib().or_shortcut(n, rp, col, lab, hitters)
    return lab[:n], rounds


def geo_table(beta: float) -> np.ndarray:
    out = np.zeros(4096, np.uint64)
    k = lib().or_geo_table(beta, out, 4096)
    return out[:k]


def hash3(seed: int, a: int, b: int) -> int:
    return int(lib().or_hash3(seed, a, b))


def solve(G, algo: str, P: int = 1, beta: float = 0.1, seq: int = 1, seed: int = 1,
          fixed_seq: bool = False, hitters: int = 0) -> np.ndarray:
    """Canonical labels from the restatement of `algo`."""
    if algo == "exp":
        raw, _ = exp_contraction(G, P, beta, seq, fixed_seq, seed)
    elif algo == "local":
        raw, _ = local_contraction(G, seq, seed)
    elif algo == "shortcuts":
        raw, _ = shortcut(G, None, hitters)
    elif algo == "labels":
        raw, _ = labels_propagation(G)
    elif algo == "allreduce":
        raw = allreduce(G)
    elif algo == "uf":
        raw = uf_labels(G)
    else:
        raise ValueError(algo)
    return canonical(raw)
