"""ctypes wrapper for ref_gpu.c: the reference's own CUDA kernels on this GPU.

BASELINE AND TEST INFRASTRUCTURE.  Only bench.py (the reference-GPU baseline)
and tests/ import this module; the product never does.

The kernels are the reference's (kernel.cu with IDIC.h, compiled unmodified
into oracle/_ref/ref_kernels.cubin by oracle/build_ref_gpu.sh where the
reference tree exists); ref_gpu.c restates the reference's host loop
(kernel.cu:1929-2523) around them.  The cubin is built from the reference's
sources, which only the machine holding the reference tree has: where it is
absent, available() says why and nothing here runs.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

from . import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(oracle.BUILD_DIR, "libref_gpu.so")
CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")

# rg_phase_seconds' order: host cell lists, kernels (launch + synchronize),
# blocking copies, host IDIC averages and solve
PHASES = ("host_lists", "kernels", "copies", "host_idic")

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile ref_gpu.c into oracle/_build/libref_gpu.so (gcc; libcuda is opened at run time)."""
    os.makedirs(oracle.BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "ref_gpu.c")
    if (not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(os.path.join(HERE, "oracle.h"))):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", src, "-o", tmp,
                    "-ldl", "-lm"], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def available() -> str | None:
    """None when the reference's kernels can run here, else the reason they cannot."""
    if not os.path.isfile(CUBIN):
        return ("the reference's kernels are not built: oracle/build_ref_gpu.sh compiles them from the "
                "reference tree (DS_REFERENCE_DIR), which this machine does not hold")
    return None


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            L.rg_open.argtypes = [ctypes.c_char_p]
            L.rg_open.restype = ctypes.c_int
            L.rg_run.argtypes = [ctypes.POINTER(oracle.OrcParams), ctypes.POINTER(oracle.OrcSpecies), ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
            L.rg_run.restype = ctypes.c_int
            L.rg_last_error.argtypes = []
            L.rg_last_error.restype = ctypes.c_char_p
            L.rg_phase_seconds.argtypes = [ctypes.POINTER(ctypes.c_double)]
            L.rg_phase_seconds.restype = None
            _lib = L
    return _lib


class RefGPU:
    """The reference's loop on the GPU, over copies of (gas, dust 1, dust 2) in
    the reference's two-species layout (equal counts).  Reference mode only:
    the reference's kernels have no periodic images, per-particle h or CFL."""

    def __init__(self, params, species):
        why = available()
        if why:
            raise RuntimeError(why)
        self.state = oracle.OracleState(params, species)
        if self.state.P.flags & ~(oracle.ORC_REF_INDEX_COUPLING | oracle.ORC_REF_EPS_GUARD | oracle.ORC_REF_SOLVE2
                                  | oracle.ORC_DUST_RHO):
            raise ValueError("the reference's kernels run the reference's step only (reference mode)")
        L = lib()
        if L.rg_open(CUBIN.encode()) != 0:
            raise RuntimeError("reference kernels: " + L.rg_last_error().decode())
        self.step_s: list[float] = []
        # wall time of the steps by kind of work, summed over step() calls
        self.phase_s = {k: 0.0 for k in PHASES}

    @property
    def species(self):
        return self.state.species

    @property
    def Tm(self):
        return self.state.Tm

    def step(self, n: int = 1):
        if n <= 0:
            return self
        L = lib()
        Tm = ctypes.c_double(self.state.Tm)
        times = np.zeros(n, dtype=np.float64)
        st = L.rg_run(ctypes.byref(self.state.P), self.state._arr, int(n), ctypes.byref(Tm),
                      times.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if st != 0:
            raise RuntimeError("reference kernels: " + L.rg_last_error().decode())
        self.state.Tm = Tm.value
        self.step_s.extend(float(t) for t in times)
        ph = np.zeros(len(PHASES), dtype=np.float64)
        L.rg_phase_seconds(ph.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        for k, v in zip(PHASES, ph):
            self.phase_s[k] += float(v)
        return self
