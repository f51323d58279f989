"""The C++ drop-in header (include/components_gb300.hpp) used the way the
reference drivers use their solver classes, compiled with g++ and run."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import components_gb300 as cc
import oracle
from components_gb300 import _lib

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_cpp_dropin_solvers(cuda, tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ missing")
    exe = tmp_path / "dropin"
    lib = _lib.gpu_lib_path()
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "dropin_main.cpp"), "-o", str(exe),
                    str(lib), f"-Wl,-rpath,{lib.parent}"], check=True)
    rng = np.random.default_rng(5)
    n = 400
    edges = [(int(a), int(b)) for a, b in rng.integers(0, n, (300, 2)) if a != b]
    text = f"{n} {len(edges)}\n" + "\n".join(f"{a} {b}" for a, b in edges) + "\n"
    out = subprocess.run([str(exe)], input=text, capture_output=True, text=True, check=True).stdout
    want = oracle.uf_labels(cc.from_edges(n, edges))
    lines = out.strip().splitlines()
    summary, lines = lines[5:], lines[:5]
    assert [ln.split()[0] for ln in lines] == ["exp", "local", "shortcuts", "labels", "allreduce"]
    # OutputComponents: size distribution in ascending size, components of more than one vertex
    sizes, counts = np.unique(np.unique(want, return_counts=True)[1], return_counts=True)
    assert summary[0] == "COMPONENTS [ " + "".join(f"size={s} (num={c}) " for s, c in zip(sizes, counts)) + "]"
    assert summary[1] == f"NUM COMPONENTS {int(counts[sizes != 1].sum())}"
    for ln in lines:
        toks = ln.split()
        labels = np.array([int(t) for t in toks[1:1 + n]], np.uint64)
        assert np.array_equal(labels, want), toks[0]
        assert toks[1 + n:] == ["comm=0", "send=0", "recv=0"]
