"""Builds the CUDA library in-tree: dustyshock3d_gb300/_build/libdustyshock3d_gb300.so.

nvcc, one -gencode (sm_103a), translation units compiled in parallel.  The FP64
kernels that must follow the reference's operation order (ds_cells.cu,
ds_sweep64.cu) are compiled with -fmad=false so nvcc does not contract a*b+c
into FMAs; so are the FP32 sweeps (ds_sweep32.cu), whose multiply-adds are
written out, so that a pair's bits do not depend on the kernel that
evaluates it; the initial-condition generator (ds_ic.cu) also keeps the host
compiler from contracting its plan arithmetic.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdustyshock3d_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "ds_api.cu": [],
    "ds_sort.cu": [],
    "ds_cells.cu": ["-fmad=false"],
    "ds_sweep64.cu": ["-fmad=false"],
    "ds_sweep32.cu": ["-fmad=false"],
    "ds_ic.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "ds_inittxt.cu": [],
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "dustyshock3d_gb300.h"))
    deps.append(__file__)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", CSRC]
    if ptxas_v:
        common += ["-Xptxas", "-v"]

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc] + common + SOURCES[src] + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose or ptxas_v:
        for obj, err in results:
            if err:
                print(err)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, ptxas_v="-v" in sys.argv))
