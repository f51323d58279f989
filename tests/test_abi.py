"""CPU tests of the boundary: the libraries load and export every function the
headers declare; struct layouts and defaults; the Config/ParseParameters
mirror.  No GPU work is launched here."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from components_gb300 import _lib
from components_gb300.config import Config, parse_parameters

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    return built


def _declared(header: str) -> set[str]:
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(cc_[a-z0-9_]+)\s*\(", text))


def _exported(lib: Path) -> set[str]:
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True,
                         check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_gpu_library_exports_every_declared_symbol():
    declared = set()
    for h in ("cc_gpu.h", "cc_gpu_debug.h", "cc_batch.h", "cc_serve.h"):
        declared |= _declared(h)
    exported = _exported(_lib.gpu_lib_path())
    missing = declared - exported
    assert not missing, missing
    _lib.gpu()  # binds every symbol with its signature


def test_gen_library_exports_every_declared_symbol():
    declared = _declared("cc_gen.h")
    exported = _exported(_lib.BUILD / "libccgen.so")
    assert not (declared - exported)
    _lib.gen()


def test_struct_layouts():
    assert C.sizeof(_lib.cc_csr) == 48
    assert C.sizeof(_lib.cc_config) == 48
    assert C.sizeof(_lib.cc_kernel_stat) == 56
    assert _lib.cc_stats.kernels.offset == 1376


def test_config_defaults_match_parse_parameters():
    c = _lib.cc_config()
    _lib.gpu().cc_config_default(C.byref(c))
    assert c.beta == 0.1 and c.seq == 1 and c.prop_iterations == 3
    assert c.number_of_hitters == 0 and c.degree_threshold == 16 and c.degree_limit == 100
    assert abs(c.hd_sf - 0.5) < 1e-7
    assert c.contraction == c.single == c.bfs == c.replicate == 0
    d = Config().to_c()
    assert d.beta == c.beta and d.seq == c.seq


def test_parse_parameters_like_reference():
    c = parse_parameters(["-gen", "gnm_undirected", "-n", "20", "-m", "22", "-seed", "3",
                          "-beta", "0.2", "-contraction", "-seq", "0", "-heavy-hitters", "4"])
    assert c.gen == "gnm_undirected" and c.gen_n == 1 << 20 and c.gen_m == 1 << 22
    assert c.seed == 3 and c.beta == 0.2 and c.use_contraction and c.sequential_limit == 0
    assert c.number_of_hitters == 4 and not c.use_bfs
    g = parse_parameters(["-gen", "grid_2d", "-n", "8192", "-m", "8192", "-p", "0.5"])
    assert g.gen_n == 8192 and g.gen_m == 8192 and g.gen_p == 0.5  # exact for grid_2d
    big = parse_parameters(["-n", "33"])
    assert big.gen_n == 1 << 33  # 64-bit shift (the reference's int shift overflows)
    flag = parse_parameters(["-verbose", "-bfs"])
    assert flag.print_verbose and flag.use_bfs


def test_strerror_and_invalid_args_need_no_gpu():
    lib = _lib.gpu()
    assert lib.cc_gpu_strerror(0) == b"ok"
    assert lib.cc_gpu_strerror(4).startswith(b"iteration cap")
    # argument checks happen before any device call
    g = _lib.cc_csr()
    g.n, g.m_dir, g.id_bytes, g.num_parts, g.where = 4, 0, 3, 1, 0
    assert lib.cc_csr_validate(C.byref(g), 0) == _lib.CC_ERR_INVALID
    g.id_bytes, g.num_parts = 4, 0
    assert lib.cc_csr_validate(C.byref(g), 0) == _lib.CC_ERR_INVALID


def test_misaligned_device_arrays_are_rejected_before_any_device_call():
    lib = _lib.gpu()
    g = _lib.cc_csr(2, 2, 0x1000, 0x2002, 4, 1, _lib.CC_DEVICE, 0)  # col 2 bytes past a word
    assert lib.cc_csr_validate(C.byref(g), 0) == _lib.CC_ERR_INVALID
    g = _lib.cc_csr(2, 2, 0x1004, 0x2000, 4, 1, _lib.CC_DEVICE, 0)  # offsets not 8-byte aligned
    assert lib.cc_csr_validate(C.byref(g), 0) == _lib.CC_ERR_INVALID
    g = _lib.cc_csr(2, 2, 0x1000, 0x2004, 8, 1, _lib.CC_DEVICE, 0)  # 64-bit ids 4 bytes off
    assert lib.cc_csr_validate(C.byref(g), 0) == _lib.CC_ERR_INVALID


def test_size_limits_are_reported_before_any_device_call():
    """Labels are 32-bit inside: n >= 2^32 - 1 is refused up front, as is a
    G(n, m) draw of 2^32 or more directed entries and a grid of 2^30 vertices
    on the device generators (their offsets use a 32-bit scan)."""
    lib = _lib.gpu()
    g = _lib.cc_csr(1 << 32, 0, 0x1000, 0, 4, 1, _lib.CC_DEVICE, 0)
    assert lib.cc_csr_validate(C.byref(g), 0) == _lib.CC_ERR_UNSUPPORTED
    m = C.c_uint64()
    assert lib.cc_gen_gnm_device(None, 1 << 20, 1 << 31, 1, 4, 0x1000, 0x2000, 1, C.byref(m)) == \
        _lib.CC_ERR_UNSUPPORTED
    assert lib.cc_gen_grid_device(None, 1 << 15, 1 << 15, 0.5, 1, 4, 0x1000, 0x2000, 1, C.byref(m)) == \
        _lib.CC_ERR_UNSUPPORTED
    # bad model parameters are refused before any device call
    assert lib.cc_gen_rhg_device(None, 1 << 32, 16.0, 2.6, 1, 4, 0x1000, 0x2000, 1, C.byref(m)) == \
        _lib.CC_ERR_INVALID
    assert lib.cc_gen_rhg_device(None, 1 << 10, 16.0, 1.9, 1, 4, 0x1000, 0x2000, 1, C.byref(m)) == \
        _lib.CC_ERR_INVALID


def test_host_validation():
    lib = _lib.gpu()
    rp = np.array([0, 1, 2], np.uint64)
    col = np.array([1, 0], np.uint32)
    g = _lib.cc_csr(2, 2, rp.ctypes.data, col.ctypes.data, 4, 1, 0, 0)
    assert lib.cc_csr_validate(C.byref(g), 1) == 0
    bad = np.array([1, 5], np.uint32)
    g.col = bad.ctypes.data
    assert lib.cc_csr_validate(C.byref(g), 0) == _lib.CC_ERR_INVALID
    asym = np.array([1, 1], np.uint32)
    g.col = asym.ctypes.data
    assert lib.cc_csr_validate(C.byref(g), 1) == _lib.CC_ERR_INVALID


def test_library_geo_table_equals_oracle():
    import oracle
    for beta in (0.1, 0.33, 2.0):
        buf = np.zeros(4096, np.uint64)
        k = _lib.gpu().cc_debug_geo_table(beta, buf.ctypes.data, 4096)
        assert np.array_equal(buf[:k], oracle.geo_table(beta))
    for a in [(1, 0, 0), (1001, 77, 3), (2**63 + 1, 2**40, 9)]:
        assert _lib.gpu().cc_debug_hash3(*a) == oracle.hash3(*a)
