"""The host thread pool that encodes streamed input (csrc/hostpool.h),
compiled with g++ and run on the CPU: every part exactly once per run."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_hostpool_runs_every_part_once(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ missing")
    cuda_inc = Path("/usr/local/cuda/include")
    if not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("CUDA headers missing")
    exe = tmp_path / "hostpool_main"
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-I", str(ROOT / "components_gb300" / "csrc"),
                    "-I", str(cuda_inc), str(ROOT / "tests" / "cpp" / "hostpool_main.cpp"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok"
