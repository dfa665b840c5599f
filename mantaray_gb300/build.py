"""Builds libmantaray_gpu.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into
mantaray_gb300/lib/libmantaray_gpu.so (static CUDA runtime, C ABI only).
Run `python -m mantaray_gb300.build` or call `build()`.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libmantaray_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]

# Translation units and their extra flags.  The integrators are compiled with
# -fmad=false: the plain kernel because the reference (Rust) never contracts
# a*b+c, the batched kernel so that its explicit fmaf calls are its only
# fused operations (same bits for every launch shape).  Its single-scenario
# builds (rk4_f32_one.cu) also flush FP32 subnormals (-ftz=true; the file
# says why).
UNITS = {
    "rk4_f64.cu": ["-fmad=false"],
    "api.cu": [],
    "netcdf3.cpp": [],
    "diag.cu": [],
    "rk4_f32.cu": ["-fmad=false"],
    "rk4_f32_one.cu": ["-fmad=false", "-ftz=true"],
    "batch_api.cu": [],
    "batch_static.cu": [],
    "diff.cu": [],
    "order.cu": [],
    "seed.cu": ["-fmad=false"],
}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mantaray_gb300")
    return path


def _sources_newer_than(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    for root in (CSRC, INCLUDE):
        for name in os.listdir(root):
            if os.path.getmtime(os.path.join(root, name)) > t:
                return True
    return os.path.getmtime(__file__) > t


def _compile(src: str, flags: list[str], verbose: bool) -> str:
    obj = os.path.join(OBJ, src + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout + res.stderr, file=sys.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles every CUDA/C++ unit for sm_103a and links the shared library."""
    if not force and not _sources_newer_than(LIB):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as pool:
        objs = list(pool.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
