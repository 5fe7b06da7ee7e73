"""ctypes wrapper for the FP64 CPU oracle (oracle.c).

TEST INFRASTRUCTURE.  The oracle is the checker for the CUDA path and the timed
CPU baseline; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
and reference-arm legs import this module.  It restates kernel.cu:1929-2523 and
the IDIC.h kernels of the reference (see oracle.c for line-by-line citations).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
MAX_DUST = 4

ORC_PERIODIC_Y = 0x0001
ORC_PERIODIC_Z = 0x0002
ORC_H_PER_PARTICLE = 0x0004
ORC_TSTOP_CONST = 0x0008
ORC_GAS_ACCEL_PARTICLE = 0x0010
ORC_REF_INDEX_COUPLING = 0x0020
ORC_REF_EPS_GUARD = 0x0040
ORC_REF_SOLVE2 = 0x0080
ORC_CFL = 0x0100
ORC_DUST_RHO = 0x0200
ORC_GRID_PROPER = 0x0400
ORC_IDIC_PROPER = 0x0800


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("X_min", ctypes.c_double), ("X_max", ctypes.c_double),
        ("Y_min", ctypes.c_double), ("Y_max", ctypes.c_double),
        ("Z_min", ctypes.c_double), ("Z_max", ctypes.c_double),
        ("Type_of_state", ctypes.c_int), ("flags", ctypes.c_int),
        ("h", ctypes.c_double), ("tau", ctypes.c_double), ("T_end", ctypes.c_double),
        ("alpha", ctypes.c_double), ("beta", ctypes.c_double), ("eps", ctypes.c_double),
        ("Gam_g", ctypes.c_double), ("Speed_of_sound_gas", ctypes.c_double),
        ("cell_w", ctypes.c_double), ("idic_w", ctypes.c_double),
        ("cfl", ctypes.c_double), ("t_empty", ctypes.c_double),
        ("n_dust", ctypes.c_int), ("stencil", ctypes.c_int),
        ("mass_ratio", ctypes.c_double * MAX_DUST), ("R_dust", ctypes.c_double * MAX_DUST),
        ("t_stop_const", ctypes.c_double * MAX_DUST), ("eps_empty", ctypes.c_double * MAX_DUST),
    ]


_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)


class OrcSpecies(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("pad_", ctypes.c_int)] + [
        (f, _DP) for f in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h", "ts")
    ] + [("ind", _IP)]


_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile oracle.c into oracle/_build/liboracle.so (gcc, OpenMP, no FP contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(os.path.join(HERE, "oracle.h"))):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
           src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            L.orc_step.argtypes = [ctypes.POINTER(OrcParams), ctypes.POINTER(OrcSpecies),
                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
            L.orc_step.restype = ctypes.c_int
            L.orc_step_density.argtypes = [ctypes.POINTER(OrcParams), ctypes.POINTER(OrcSpecies),
                                           ctypes.POINTER(ctypes.c_double)]
            L.orc_step_density.restype = ctypes.c_int
            L.orc_step_complete.argtypes = [ctypes.POINTER(OrcParams), ctypes.POINTER(OrcSpecies),
                                            ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                                            ctypes.POINTER(ctypes.c_double)]
            L.orc_step_complete.restype = ctypes.c_int
            L.orc_build_list.argtypes = [ctypes.POINTER(OrcParams), ctypes.POINTER(OrcSpecies), _IP, _IP]
            L.orc_build_list.restype = ctypes.c_int
            for name in ("orc_cell_keys", "orc_idic_keys"):
                getattr(L, name).argtypes = [ctypes.POINTER(OrcParams), ctypes.POINTER(OrcSpecies), _IP]
                getattr(L, name).restype = None
            L.orc_neighbour_counts.argtypes = [ctypes.POINTER(OrcParams), ctypes.POINTER(OrcSpecies), _IP, _IP]
            L.orc_neighbour_counts.restype = None
            L.orc_grid_info.argtypes = [ctypes.POINTER(OrcParams), _IP]
            L.orc_grid_info.restype = None
            L.orc_idic_solve_cell.argtypes = [ctypes.c_int, _DP, _DP, ctypes.c_double, _DP, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_int, _DP, _DP]
            L.orc_idic_solve_cell.restype = None
            for name in ("orc_kernel_W", "orc_kernel_dW"):
                getattr(L, name).argtypes = [ctypes.c_double, ctypes.c_double]
                getattr(L, name).restype = ctypes.c_double
            _lib = L
    return _lib


# --------------------------------------------------------------------------
# Conversion from the host-side parameter / particle containers
# --------------------------------------------------------------------------

def to_orc_params(P) -> OrcParams:
    """Translate a dustyshock3d_gb300.Params into the oracle's struct."""
    o = OrcParams()
    for f in ("X_min", "X_max", "Y_min", "Y_max", "Z_min", "Z_max", "h", "tau", "T_end",
              "alpha", "beta", "eps", "Gam_g", "Speed_of_sound_gas", "cfl", "t_empty"):
        setattr(o, f, float(getattr(P, f)))
    o.Type_of_state = int(P.Type_of_state)
    o.cell_w = float(P.cell_width())
    o.idic_w = float(P.idic_width())
    o.n_dust = int(P.n_dust)
    o.stencil = int(getattr(P, "stencil", 1) or 1)
    f = 0
    m = P.mode
    if m.periodic_y: f |= ORC_PERIODIC_Y
    if m.periodic_z: f |= ORC_PERIODIC_Z
    if m.h_per_particle: f |= ORC_H_PER_PARTICLE
    if m.tstop_const: f |= ORC_TSTOP_CONST
    if m.gas_accel_particle: f |= ORC_GAS_ACCEL_PARTICLE
    if m.ref_index_coupling: f |= ORC_REF_INDEX_COUPLING
    if m.ref_eps_guard: f |= ORC_REF_EPS_GUARD
    if m.ref_solve2: f |= ORC_REF_SOLVE2
    if m.cfl: f |= ORC_CFL
    if m.dust_rho: f |= ORC_DUST_RHO
    if m.grid_proper: f |= ORC_GRID_PROPER
    if m.idic_proper: f |= ORC_IDIC_PROPER
    o.flags = f
    for k in range(MAX_DUST):
        o.mass_ratio[k] = float(P.mass_ratio[k]) if k < len(P.mass_ratio) else 0.0
        o.R_dust[k] = float(P.R_dust[k]) if k < len(P.R_dust) else 0.0
        o.t_stop_const[k] = float(P.t_stop_const[k]) if k < len(P.t_stop_const) else 0.0
        o.eps_empty[k] = float(P.eps_empty[k]) if k < len(P.eps_empty) else 0.0
    return o


_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h", "ts")


def _orc_species(sp, keep):
    s = OrcSpecies()
    s.n = sp.n
    for f in _FIELDS:
        a = getattr(sp, f)
        assert a is not None and a.dtype == np.float64 and a.flags.c_contiguous, f
        keep.append(a)
        setattr(s, f, a.ctypes.data_as(_DP))
    ind = sp.ind
    assert ind.dtype == np.int32 and ind.flags.c_contiguous
    keep.append(ind)
    s.ind = ind.ctypes.data_as(_IP)
    return s


class OracleState:
    """Owns contiguous float64 copies of every species and steps them on the CPU."""

    def __init__(self, params, species):
        self.params = params
        self.P = to_orc_params(params)
        self.species = [sp.copy() for sp in species]
        for sp in self.species:
            sp.fill_missing()
        self._keep = []
        self._arr = (OrcSpecies * len(self.species))()
        for i, sp in enumerate(self.species):
            self._arr[i] = _orc_species(sp, self._keep)
        self.Tm = 0.0
        self.last_status = 0

    def step(self, n: int = 1):
        L = lib()
        Tm = ctypes.c_double(self.Tm)
        dt = ctypes.c_double(0.0)
        for _ in range(n):
            # the reference's loop runs while Tm < T_end (kernel.cu:1929, 2566): a
            # step after the end time does nothing (and reports dt = 0, as the
            # GPU does)
            if Tm.value >= self.P.T_end:
                dt.value = 0.0
                continue
            st = L.orc_step(ctypes.byref(self.P), self._arr, ctypes.byref(Tm), ctypes.byref(dt))
            if st < 0:
                raise ValueError("oracle: a periodic axis has fewer cells than its stencil needs")
            self.last_status |= st
        self.Tm = Tm.value
        self.last_dt = dt.value
        return self

    def lists(self, s: int):
        L = lib()
        info = self.grid_info()
        head = np.empty(info[3] + 1, dtype=np.int32)
        nxt = np.empty(max(self.species[s].n, 1), dtype=np.int32)
        L.orc_build_list(ctypes.byref(self.P), ctypes.byref(self._arr[s]),
                         head.ctypes.data_as(_IP), nxt.ctypes.data_as(_IP))
        return head, nxt[: self.species[s].n]

    def cell_keys(self, s: int):
        k = np.empty(max(self.species[s].n, 1), dtype=np.int32)
        lib().orc_cell_keys(ctypes.byref(self.P), ctypes.byref(self._arr[s]), k.ctypes.data_as(_IP))
        return k[: self.species[s].n]

    def idic_keys(self, s: int):
        k = np.empty(max(self.species[s].n, 1), dtype=np.int32)
        lib().orc_idic_keys(ctypes.byref(self.P), ctypes.byref(self._arr[s]), k.ctypes.data_as(_IP))
        return k[: self.species[s].n]

    def neighbour_counts(self, s: int):
        n = max(self.species[s].n, 1)
        nc = np.empty(n, dtype=np.int32)
        nn = np.empty(n, dtype=np.int32)
        lib().orc_neighbour_counts(ctypes.byref(self.P), ctypes.byref(self._arr[s]),
                                   nc.ctypes.data_as(_IP), nn.ctypes.data_as(_IP))
        return nc[: self.species[s].n], nn[: self.species[s].n]

    def grid_info(self):
        out = np.empty(8, dtype=np.int32)
        lib().orc_grid_info(ctypes.byref(self.P), out.ctypes.data_as(_IP))
        return out


def solve_cell(eps, t, vg, vd, psi, tau, ref2=False):
    """One component of the IDIC per-cell solve (kernel.cu:2310-2437)."""
    n = len(eps)
    e = np.ascontiguousarray(eps, dtype=np.float64)
    tt = np.ascontiguousarray(t, dtype=np.float64)
    v = np.ascontiguousarray(vd, dtype=np.float64)
    out = np.zeros(n, dtype=np.float64)
    g = ctypes.c_double(0.0)
    lib().orc_idic_solve_cell(n, e.ctypes.data_as(_DP), tt.ctypes.data_as(_DP), float(vg),
                              v.ctypes.data_as(_DP), float(psi), float(tau), int(bool(ref2)),
                              ctypes.byref(g), out.ctypes.data_as(_DP))
    return g.value, out
