"""ctypes view of the C ABI (include/cc_gpu.h, cc_gpu_debug.h, cc_gen.h).

The native libraries are loaded from components_gb300/_build/.  There is no
fallback: if libccgpu.so is missing or does not load, importing the solver
API raises, so a caller can never silently run anything but the CUDA path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

BUILD = Path(__file__).resolve().parent / "_build"

CC_OK = 0
CC_ERR_INVALID = 1
CC_ERR_OOM = 2
CC_ERR_CUDA = 3
CC_ERR_NO_CONVERGENCE = 4
CC_ERR_TIMEOUT = 5
CC_ERR_UNSUPPORTED = 6
CC_ERR_BUSY = 7

CC_HOST = 0
CC_DEVICE = 1

CC_EXP, CC_LOCAL, CC_SHORTCUTS, CC_LABELS, CC_ALLREDUCE = range(5)
ALGOS = {"exp": CC_EXP, "local": CC_LOCAL, "shortcuts": CC_SHORTCUTS, "labels": CC_LABELS,
         "allreduce": CC_ALLREDUCE}

CC_MAX_LEVELS = 64
CC_MAX_KSTATS = 32
CC_PROF_KERNELS, CC_PROF_COMPONENTS = 1, 2


class cc_csr(C.Structure):
    _fields_ = [("n", C.c_uint64), ("m_dir", C.c_uint64), ("row_ptr", C.c_void_p),
                ("col", C.c_void_p), ("id_bytes", C.c_uint32), ("num_parts", C.c_uint32),
                ("where", C.c_uint32), ("reserved", C.c_uint32)]


class cc_config(C.Structure):
    _fields_ = [("beta", C.c_double), ("seq", C.c_uint32), ("prop_iterations", C.c_uint32),
                ("number_of_hitters", C.c_uint32), ("degree_threshold", C.c_uint32),
                ("degree_limit", C.c_uint32), ("hd_sf", C.c_float), ("fixed_seq", C.c_uint8),
                ("contraction", C.c_uint8), ("direct", C.c_uint8), ("single", C.c_uint8),
                ("bfs", C.c_uint8), ("replicate", C.c_uint8), ("regular", C.c_uint8),
                ("overalloc", C.c_uint8), ("verbose", C.c_uint8), ("pad_", C.c_uint8 * 3)]


class cc_kernel_stat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint32), ("pad_", C.c_uint32),
                ("ms", C.c_double), ("bytes", C.c_uint64)]


class cc_stats(C.Structure):
    _fields_ = [("levels", C.c_uint32), ("rounds_total", C.c_uint32),
                ("rounds", C.c_uint32 * CC_MAX_LEVELS),
                ("level_vertices", C.c_uint64 * CC_MAX_LEVELS),
                ("level_edges", C.c_uint64 * CC_MAX_LEVELS),
                ("bytes_algorithmic", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("num_components", C.c_uint64), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("solve_ms", C.c_double), ("total_ms", C.c_double),
                ("comm_time", C.c_double), ("send_volume", C.c_uint64),
                ("recv_volume", C.c_uint64), ("nkernels", C.c_uint32), ("pad_", C.c_uint32),
                ("kernels", cc_kernel_stat * CC_MAX_KSTATS)]

    def as_dict(self) -> dict:
        L = self.levels
        return {
            "levels": L,
            "rounds_total": self.rounds_total,
            "rounds": list(self.rounds[:L]),
            "level_vertices": list(self.level_vertices[:L]),
            "level_edges": list(self.level_edges[:L]),
            "bytes_algorithmic": self.bytes_algorithmic,
            "kernel_launches": self.kernel_launches,
            "num_components": self.num_components,
            "h2d_bytes": self.h2d_bytes,
            "d2h_bytes": self.d2h_bytes,
            "solve_ms": self.solve_ms,
            "total_ms": self.total_ms,
            "kernels": {k.name.decode(): {"launches": k.launches, "ms": k.ms, "bytes": k.bytes}
                        for k in self.kernels[: self.nkernels]},
        }


class cc_tuning(C.Structure):
    _fields_ = [("hook_mode", C.c_uint32), ("tile_vertices", C.c_uint32),
                ("tile_threads", C.c_uint32), ("hub_degree", C.c_uint32)]


CC_HOOK_AUTO, CC_HOOK_GLOBAL, CC_HOOK_TILED, CC_HOOK_SAMPLED = 0, 1, 2, 3


class cc_host_graph(C.Structure):
    _fields_ = [("n", C.c_uint64), ("m_dir", C.c_uint64), ("row_ptr", C.c_void_p),
                ("col", C.c_void_p), ("id_bytes", C.c_uint32), ("pad_", C.c_uint32)]


_P = C.c_void_p
_U64 = C.c_uint64
_U32 = C.c_uint32

# symbol -> (restype, argtypes); these are exactly the exports of the headers
GPU_SYMBOLS = {
    "cc_config_default": (None, [C.POINTER(cc_config)]),
    "cc_gpu_run": (C.c_int, [C.POINTER(cc_csr), C.c_int, C.POINTER(cc_config), _U64, _P]),
    "cc_gpu_stats": (C.c_int, [C.POINTER(cc_stats)]),
    "cc_gpu_strerror": (C.c_char_p, [C.c_int]),
    "cc_csr_validate": (C.c_int, [C.POINTER(cc_csr), C.c_int]),
    "cc_ctx_create": (C.c_int, [C.POINTER(_P), C.c_int, _P]),
    "cc_ctx_destroy": (C.c_int, [_P]),
    "cc_ctx_run": (C.c_int, [_P, C.POINTER(cc_csr), C.c_int, C.POINTER(cc_config), _U64, _P, _U32]),
    "cc_ctx_stats": (C.c_int, [_P, C.POINTER(cc_stats)]),
    "cc_gen_grid_device": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_double, C.c_uint64, C.c_uint32,
                                     _P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "cc_gen_gnm_device": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint32, _P, _P,
                                    C.c_uint64, C.POINTER(C.c_uint64)]),
    "cc_gen_rhg_device": (C.c_int, [_P, C.c_uint64, C.c_double, C.c_double, C.c_uint64, C.c_uint32,
                                    _P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "cc_read_metis_device": (C.c_int, [_P, C.c_char_p, C.c_uint32, _P, _P, C.c_uint64,
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "cc_read_binary_edges_device": (C.c_int, [_P, C.c_char_p, C.c_uint32, _P, _P, C.c_uint64,
                                              C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "cc_component_sizes": (C.c_int, [_P, _P, C.c_uint32, C.c_uint32, C.c_uint64, _P, C.c_uint64,
                                     C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "cc_ctx_arena_bytes": (_U64, [_P]),
    "cc_ctx_set_profiling": (C.c_int, [_P, C.c_int]),
    "cc_ctx_profile_totals": (C.c_int, [_P, C.POINTER(cc_stats), C.POINTER(C.c_uint64)]),
    "cc_ctx_stream": (_P, [_P]),
    "cc_ctx_set_tuning": (C.c_int, [_P, C.POINTER(cc_tuning)]),
    "cc_ctx_get_tuning": (C.c_int, [_P, C.POINTER(cc_tuning)]),
    "cc_ctx_set_host_reads": (C.c_int, [_P, C.c_int]),
    "cc_debug_geo_table": (C.c_int, [C.c_double, _P, C.c_int]),
    "cc_debug_hash3": (_U64, [_U64, _U64, _U64]),
    "cc_debug_ldd": (C.c_int, [C.POINTER(cc_csr), _P, _U64, _U32, C.c_double, C.c_int, _P, _P]),
    "cc_debug_local_sweeps": (C.c_int, [C.POINTER(cc_csr), _P, _U64, _U32, _P]),
    "cc_debug_contract": (C.c_int, [C.POINTER(cc_csr), _P, _U64, _P, _U32, _P, _P, _P, _P,
                                    C.POINTER(_U64), C.POINTER(_U64)]),
    "cc_debug_local_components": (C.c_int, [C.POINTER(cc_csr), _P]),
    "cc_debug_radix_sort": (C.c_int, [_P, _U64, C.c_int]),
    "cc_debug_shortcut": (C.c_int, [C.POINTER(cc_csr), _P, _U32, _P]),
    "cc_debug_set_round_cap": (C.c_int, [_P, _U32]),
    "cc_serve_debug_fail_next": (C.c_int, [_P, C.c_int]),
}

GEN_SYMBOLS = {
    "cc_gen_gnm": (C.c_int, [_U64, _U64, _U64, _U32, C.POINTER(cc_host_graph)]),
    "cc_gen_grid": (C.c_int, [_U64, _U64, C.c_double, _U64, _U32, C.POINTER(cc_host_graph)]),
    "cc_gen_rhg": (C.c_int, [_U64, C.c_double, C.c_double, _U64, _U32, C.POINTER(cc_host_graph)]),
    "cc_host_graph_free": (None, [C.POINTER(cc_host_graph)]),
    "cc_gen_rhg_radius": (C.c_double, [_U64, C.c_double, C.c_double]),
    "cc_gen_rhg_verify": (_U64, [_U64, C.c_double, C.c_double, _U64, C.POINTER(cc_host_graph)]),
    "cc_read_metis": (C.c_int, [C.c_char_p, _U32, C.POINTER(cc_host_graph)]),
    "cc_read_edge_list": (C.c_int, [C.c_char_p, _U32, C.POINTER(cc_host_graph)]),
    "cc_read_binary_edges": (C.c_int, [C.c_char_p, _U32, C.POINTER(cc_host_graph)]),
}

_gpu = None
_gen = None


def _bind(lib, table):
    for name, (res, args) in table.items():
        fn = getattr(lib, name)  # AttributeError: symbol missing -> loud failure
        fn.restype = res
        fn.argtypes = args
    return lib


def gpu_lib_path() -> Path:
    return BUILD / "libccgpu.so"


def gpu() -> C.CDLL:
    """libccgpu.so, loaded once.  Raises if it is not built."""
    global _gpu
    if _gpu is None:
        p = gpu_lib_path()
        if not p.exists():
            raise ImportError(f"{p} is missing: build it with "
                              "`python -c 'import __graft_entry__ as g; g.build()'`")
        _gpu = _bind(C.CDLL(str(p), mode=C.RTLD_GLOBAL), GPU_SYMBOLS)
    return _gpu


def gen() -> C.CDLL:
    global _gen
    if _gen is None:
        p = BUILD / "libccgen.so"
        if not p.exists():
            raise ImportError(f"{p} is missing: build the package first")
        _gen = _bind(C.CDLL(str(p)), GEN_SYMBOLS)
    return _gen


class CCError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[cc status {status}] {msg}")
        self.status = status


def check(status: int) -> None:
    if status != CC_OK:
        msg = gpu().cc_gpu_strerror(status)
        raise CCError(status, msg.decode() if msg else "error")
