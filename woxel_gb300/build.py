"""Build the woxel_gb300 shared library (sm_103a CUDA + C++ host code).

The library is built in-tree as ``woxel_gb300/libwoxel_gb300.so``; object
files go to ``woxel_gb300/_build/``. Translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libwoxel_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no FMA contraction on the march (bit-exact FP32 op order);
# IEEE division and square root are nvcc's defaults and are requested explicitly.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread"]

CU_SOURCES = ["kernels.cu", "sdf.cu"]
CXX_SOURCES = ["api.cpp", "server.cpp", "topology.cpp", "scene.cpp", "vdbio.cpp"]
CUDA_INC = ["-I", "/usr/local/cuda/include"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _run(cmd: list[str]) -> str:
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"command failed ({p.returncode}): {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    return p.stdout + p.stderr


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every translation unit and link libwoxel_gb300.so. Returns its path."""
    BUILD.mkdir(exist_ok=True)
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append([_nvcc(), *ARCH, *NVCC_FLAGS, *inc, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append(["g++", *CXX_FLAGS, *inc, *CUDA_INC, "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            print(o)
    if force or _stale(LIB, objs):
        _run([_nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"])
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) via its Makefile."""
    out = _run(["make", "-s", "-C", str(ROOT / "oracle")])
    if verbose and out.strip():
        print(out)
    return ROOT / "oracle" / "liboracle.so"


if __name__ == "__main__":
    import sys

    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
    print(build_oracle())
