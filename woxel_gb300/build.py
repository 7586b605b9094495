"""Build the woxel_gb300 shared library (sm_103a CUDA + C++ host code).

The library is built in-tree as ``woxel_gb300/libwoxel_gb300.so``; object
files go to ``woxel_gb300/_build/``. Translation units compile in parallel.
``build(checked=True)`` builds ``libwoxel_gb300_checked.so`` with WX_BOUNDS_CHECK
(every pool index and pixel the raycast kernels use is range-checked and counted,
see wx_bounds_violations) from objects in ``woxel_gb300/_build/checked/``.
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
LIB_CHECKED = PKG / "libwoxel_gb300_checked.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no FMA contraction on the march (bit-exact FP32 op order);
# IEEE division and square root are nvcc's defaults and are requested explicitly.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread"]

CU_SOURCES = ["kernels.cu", "sdf.cu"]
CXX_SOURCES = ["api.cpp", "server.cpp", "topology.cpp", "scene.cpp", "vdbio.cpp", "inflate.cpp"]
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


def build(verbose: bool = False, force: bool = False, checked: bool = False) -> Path:
    """Compile every translation unit and link libwoxel_gb300.so (or, checked, the
    bounds-checked libwoxel_gb300_checked.so). Returns its path."""
    out_dir = BUILD / "checked" if checked else BUILD
    lib = LIB_CHECKED if checked else LIB
    defs = ["-DWX_BOUNDS_CHECK"] if checked else []
    out_dir.mkdir(parents=True, exist_ok=True)
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC), *defs]
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = out_dir / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append([_nvcc(), *ARCH, *NVCC_FLAGS, *inc, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = out_dir / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append(["g++", *CXX_FLAGS, *inc, *CUDA_INC, "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            print(o)
    if force or _stale(lib, objs):
        _run([_nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lpthread"])
    return lib


def build_oracle(verbose: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) via its Makefile."""
    out = _run(["make", "-s", "-C", str(ROOT / "oracle")])
    if verbose and out.strip():
        print(out)
    return ROOT / "oracle" / "liboracle.so"


if __name__ == "__main__":
    import sys

    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv, checked=True))
    print(build_oracle())
