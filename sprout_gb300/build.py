"""Builds the engine's shared library, sprout_gb300/libsprout_gpu.so, for sm_103a.

Every translation unit is compiled by nvcc in parallel (one -gencode: compute_103a ->
sm_103a) and linked into one C-ABI shared library. The CUDA code is compiled with
-fmad=false so that every float operation rounds the way the source spells it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libsprout_gpu.so"
SOURCES = ["draw.cu", "particles.cu", "admission.cu", "grid.cu", "pressure.cu", "viscosity.cu", "sim.cu", "params.cpp", "scene.cpp",
           "pacer.cpp", "raster.cu", "emit.cu", "optics.cpp", "optics.cu", "spray.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build sprout_gb300")
    return exe


def _flags(src: str) -> list[str]:
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", str(CSRC)]
    if src.endswith(".cu"):
        return ARCH + common + ["-lineinfo", "-fmad=false", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
    return common + ["-x", "c++"]


def _compile(src: str, verbose: bool) -> Path:
    obj = BUILD / (src.replace(".", "_") + ".o")
    s = CSRC / src
    deps = [s] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.inc")) + [PKG.parent / "include" / "sprout_gpu.h"]
    if obj.exists() and obj.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return obj
    cmd = [nvcc(), "-c", str(s), "-o", str(obj)] + _flags(src)
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and verbose:
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    if force:
        for o in BUILD.glob("*.o"):
            o.unlink()
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
