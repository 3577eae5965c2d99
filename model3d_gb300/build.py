"""Builds libmcgpu.so in-tree (model3d_gb300/libmcgpu.so) for sm_103a.

Three translation units compiled in parallel: the CUDA kernels + C ABI
(nvcc), the device GroupTriangles (nvcc) and the host lowering (g++ with
-ffp-contract=off, so the float64 constants it precomputes are rounded
exactly as the reference rounds them).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libmcgpu.so")
BUILD = os.path.join(HERE, "_build")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmcgpu.so")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cpp", ".cuh", ".h"))] + [
        os.path.join(HERE, "..", "include", "mcgpu.h")]


def up_to_date() -> bool:
    if not os.path.exists(OUT):
        return False
    t = os.path.getmtime(OUT)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return OUT
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    cus = [os.path.join(CSRC, f) for f in ("mc_kernels.cu", "mc_group.cu")]
    cpp = os.path.join(CSRC, "mc_lower.cpp")
    cu_os = [os.path.join(BUILD, os.path.basename(f)[:-3] + ".o") for f in cus]
    cpp_o = os.path.join(BUILD, "mc_lower.o")
    cmds = [
        [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v" if verbose else "-O3",
         "-c", cu, "-o", cu_o] for cu, cu_o in zip(cus, cu_os)
    ] + [
        ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-Wall", "-pthread",
         "-c", cpp, "-o", cpp_o],
    ]

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    with ThreadPoolExecutor(len(cmds)) as ex:
        logs = list(ex.map(run, cmds))
    if verbose:
        sys.stderr.write("".join(logs))
    tmp = OUT + ".tmp"
    run([nvcc, ARCH, "-shared", "-cudart", "static", *cu_os, cpp_o, "-o", tmp])
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(OUT)
