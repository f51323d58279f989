"""In-tree build of the native libraries.

libccgpu.so   CUDA kernels + C ABI (nvcc, sm_103a only)
libccgen.so   seeded graph generators (host C++)

Both land in components_gb300/_build/.  Translation units compile in
parallel; nothing here needs cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
CUDA_SOURCES = ["uf.cu", "sortcsr.cu", "ldd.cu", "prop.cu", "api.cu", "batch.cu", "serve.cu", "gen_dev.cu",
                "load_dev.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libccgpu")
    return cand


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _openmp_flag(cxx: str) -> list[str]:
    probe = BUILD / "_omp_probe.c"
    probe.write_text("#include <omp.h>\nint main(){return omp_get_max_threads()>0?0:1;}\n")
    r = subprocess.run([cxx, "-fopenmp", str(probe), "-o", str(BUILD / "_omp_probe")],
                       capture_output=True)
    for f in (probe, BUILD / "_omp_probe"):
        if f.exists():
            f.unlink()
    return ["-fopenmp"] if r.returncode == 0 else []


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_gpu(force: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libccgpu.so"
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    srcs = [CSRC / s for s in CUDA_SOURCES]
    if not force and not _stale(out, srcs + headers):
        return out
    nv = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "-I", str(ROOT / "include")]

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        _run([nv] + common + ["-c", str(src), "-o", str(obj)])
        return obj

    with ThreadPoolExecutor(max_workers=jobs or len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = out.with_suffix(".so.tmp")
    _run([nv] + ARCH + ["-shared", "-cudart", "static", "-o", str(tmp)] + [str(o) for o in objs])
    os.replace(tmp, out)
    return out


def build_gen(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libccgen.so"
    srcs = [CSRC / "gen.cpp", CSRC / "rhg.h", ROOT / "include" / "cc_gen.h"]
    if not force and not _stale(out, srcs):
        return out
    cxx = shutil.which("g++") or "g++"
    tmp = out.with_suffix(".so.tmp")
    _run([cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off"] + _openmp_flag(cxx)
         + ["-o", str(tmp), str(CSRC / "gen.cpp")])
    os.replace(tmp, out)
    return out


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        fg = ex.submit(build_gen, force)
        fc = ex.submit(build_gpu, force)
        fg.result()
        fc.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", BUILD)
