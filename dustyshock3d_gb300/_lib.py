"""ctypes binding of the C ABI in include/dustyshock3d_gb300.h.

This is the same binding a Python host driver of the reference would add; the
library is the in-tree build dustyshock3d_gb300/_build/libdustyshock3d_gb300.so.
There is no fallback: if the library is missing or fails to load, every entry
point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from .params import MAX_DUST, MODE_BITS, Params

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdustyshock3d_gb300.so")

DS_OK = 0
STATUS = {0: "DS_OK", 1: "DS_ERR_ARG", 2: "DS_ERR_CUDA", 3: "DS_ERR_STATE", 4: "DS_ERR_NOMEM",
          5: "DS_ERR_DEVICE", 6: "DS_ERR_UNSUPPORTED", 7: "DS_ERR_IO"}
DS_NPHASE = 4


class DsParams(ctypes.Structure):
    _fields_ = [
        ("X_min", ctypes.c_double), ("X_max", ctypes.c_double), ("Y_min", ctypes.c_double),
        ("Y_max", ctypes.c_double), ("Z_min", ctypes.c_double), ("Z_max", ctypes.c_double),
        ("Type_of_state", ctypes.c_int), ("Maximum_particle", ctypes.c_int),
        ("Particle_on_length", ctypes.c_double), ("h", ctypes.c_double), ("Coeff_h_dust_cell", ctypes.c_double),
        ("tau", ctypes.c_double), ("T_end", ctypes.c_double), ("T_out", ctypes.c_double),
        ("alpha", ctypes.c_double), ("beta", ctypes.c_double), ("eps", ctypes.c_double),
        ("Gam_g", ctypes.c_double), ("Speed_of_sound_gas", ctypes.c_double),
        ("n_dust", ctypes.c_int), ("mode", ctypes.c_int), ("precision", ctypes.c_int), ("stencil", ctypes.c_int),
        ("cell_w", ctypes.c_double), ("idic_w", ctypes.c_double), ("cfl", ctypes.c_double),
        ("t_empty", ctypes.c_double), ("list_depth", ctypes.c_int), ("force_list", ctypes.c_int),
        ("mass_ratio", ctypes.c_double * MAX_DUST), ("R_dust", ctypes.c_double * MAX_DUST),
        ("t_stop_const", ctypes.c_double * MAX_DUST), ("eps_empty", ctypes.c_double * MAX_DUST),
        ("list_skin", ctypes.c_double), ("persistent", ctypes.c_int), ("idic_lanes", ctypes.c_int),
    ]


# ds_ic: initial conditions generated on the device (kinds DS_IC_*)
IC_KINDS = {"sod_x_dust": 1, "sod_x_mas": 2, "dusty_sod": 3}
IC_FIELDS = ("dx_left", "Ly", "Lz", "eps", "t_s", "rho_L", "p_L", "rho_R", "p_R", "gamma", "h_factor", "x0", "x1",
             "wall", "lattice_offset", "t_end", "cfl", "alpha", "beta", "av_eps", "idic_cells", "fixed_tau")


class DsIc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("reserved", ctypes.c_int)] + [(f, ctypes.c_double) for f in IC_FIELDS]


_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_VP = ctypes.c_void_p

# name -> (argtypes, restype); every symbol declared in include/dustyshock3d_gb300.h
SIGNATURES = {
    "ds_params_init": ([ctypes.POINTER(DsParams)], ctypes.c_int),
    "ds_params_read_init_txt": ([ctypes.c_char_p, ctypes.POINTER(DsParams)], ctypes.c_int),
    "ds_ic_init": ([ctypes.POINTER(DsIc), ctypes.c_int], ctypes.c_int),
    "ds_ic_read_init_txt": ([ctypes.c_char_p, ctypes.POINTER(DsIc)], ctypes.c_int),
    "ds_ic_plan": ([ctypes.POINTER(DsIc), ctypes.POINTER(DsParams), ctypes.POINTER(DsParams), _IP], ctypes.c_int),
    "ds_init_tube": ([_VP, ctypes.c_int, ctypes.POINTER(DsIc)], ctypes.c_int),
    "ds_create": ([ctypes.POINTER(DsParams), ctypes.POINTER(_VP)], ctypes.c_int),
    "ds_create_batch": ([ctypes.c_int, ctypes.POINTER(DsParams), ctypes.POINTER(_VP)], ctypes.c_int),
    "ds_set_gas": ([_VP, ctypes.c_int, ctypes.c_int] + [_DP] * 14 + [_IP], ctypes.c_int),
    "ds_set_dust": ([_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int] + [_DP] * 10 + [_IP], ctypes.c_int),
    "ds_copy_tube": ([_VP, ctypes.c_int, _VP, ctypes.c_int], ctypes.c_int),
    "ds_upload_gas": ([_VP, ctypes.c_int] + [_DP] * 14 + [_IP], ctypes.c_int),
    "ds_upload_dust": ([_VP, ctypes.c_int, ctypes.c_int] + [_DP] * 10 + [_IP], ctypes.c_int),
    "ds_step": ([_VP, ctypes.c_int], ctypes.c_int),
    "ds_step_async": ([_VP, ctypes.c_int], ctypes.c_int),
    "ds_synchronize": ([_VP], ctypes.c_int),
    "ds_bind_host": ([_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_DP), _IP], ctypes.c_int),
    "ds_step_host": ([_VP, ctypes.c_int], ctypes.c_int),
    "ds_get_gas": ([_VP, ctypes.c_int] + [_DP] * 12 + [_IP], ctypes.c_int),
    "ds_get_dust": ([_VP, ctypes.c_int, ctypes.c_int] + [_DP] * 8 + [_IP], ctypes.c_int),
    "ds_download_gas": ([_VP] + [_DP] * 12 + [_IP], ctypes.c_int),
    "ds_download_dust": ([_VP, ctypes.c_int] + [_DP] * 8 + [_IP], ctypes.c_int),
    "ds_get_time": ([_VP, ctypes.c_int, _DP, _DP, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "ds_debug_cells": ([_VP, ctypes.c_int, ctypes.c_int, _IP, _IP, _IP, _IP, _IP, _IP], ctypes.c_int),
    "ds_debug_idic": ([_VP, ctypes.c_int, ctypes.c_int, _IP, _DP, _IP], ctypes.c_int),
    "ds_conservation": ([_VP, ctypes.c_int, _DP], ctypes.c_int),
    "ds_step_timed": ([_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)],
                      ctypes.c_int),
    "ds_kernels_per_step": ([_VP, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "ds_dust_density": ([_VP], ctypes.c_int),
    "ds_step_lists": ([_VP, ctypes.c_int, ctypes.c_int, _IP, _IP, _IP], ctypes.c_int),
    "ds_get_fields": ([_VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_DP), _IP], ctypes.c_int),
    "ds_save_tube": ([_VP, ctypes.c_int, ctypes.c_char_p], ctypes.c_int),
    "ds_checkpoint_params": ([ctypes.c_char_p, ctypes.POINTER(DsParams)], ctypes.c_int),
    "ds_load_tube": ([_VP, ctypes.c_int, ctypes.c_char_p], ctypes.c_int),
    "ds_memory_bytes": ([_VP, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "ds_last_error": ([_VP, _IP, ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
    "ds_list_stats": ([_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
                      ctypes.c_int),
    "ds_debug_force_lists": ([_VP, ctypes.c_int, ctypes.c_int, _IP, _IP], ctypes.c_int),
    "ds_step_density": ([_VP], ctypes.c_int),
    "ds_get_cfl_min": ([_VP, ctypes.c_int, _DP], ctypes.c_int),
    "ds_set_cfl_min": ([_VP, ctypes.c_int, ctypes.c_double], ctypes.c_int),
    "ds_set_gas_hydro": ([_VP, ctypes.c_int, ctypes.c_int, _IP, _DP, _DP], ctypes.c_int),
    "ds_step_complete": ([_VP], ctypes.c_int),
    "ds_set_time": ([_VP, ctypes.c_int, ctypes.c_double, ctypes.c_longlong], ctypes.c_int),
    "ds_idic_columns": ([ctypes.POINTER(DsParams), ctypes.c_int, _DP, _IP], ctypes.c_int),
    "ds_cell_lists_noalloc": ([ctypes.POINTER(DsParams), ctypes.c_int, _VP, _VP, _VP, _VP, _VP, ctypes.c_int,
                               _VP, _VP], ctypes.c_int),
    "ds_host_alloc": ([ctypes.POINTER(_VP), ctypes.c_longlong], ctypes.c_int),
    "ds_host_free": ([_VP], ctypes.c_int),
    "ds_destroy": ([_VP], None),
    "ds_version": ([], ctypes.c_char_p),
}

_lock = threading.Lock()
_lib = None


class DsError(RuntimeError):
    pass


def load(path: str = LIB_PATH):
    """Load the CUDA library (build it first with dustyshock3d_gb300.build.build())."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise DsError(f"CUDA extension not built: {path} is missing "
                              "(run python -c 'import __graft_entry__ as g; g.build()')")
            L = ctypes.CDLL(path)
            for name, (args, res) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = res
            _lib = L
    return _lib


def params_to_c(P: Params) -> DsParams:
    c = DsParams()
    for f in ("X_min", "X_max", "Y_min", "Y_max", "Z_min", "Z_max", "Particle_on_length", "h",
              "Coeff_h_dust_cell", "tau", "T_end", "T_out", "alpha", "beta", "eps", "Gam_g",
              "Speed_of_sound_gas", "cell_w", "idic_w", "cfl", "t_empty"):
        setattr(c, f, float(getattr(P, f)))
    c.Type_of_state = int(P.Type_of_state)
    c.Maximum_particle = int(min(P.Maximum_particle, 2 ** 31 - 1))
    c.n_dust = int(P.n_dust)
    mode = 0
    for name, bit in MODE_BITS.items():
        if getattr(P.mode, name):
            mode |= bit
    c.mode = mode
    c.precision = 1 if str(P.precision).lower() in ("fp32", "1") else 0
    c.stencil = int(getattr(P, "stencil", 1) or 1)
    c.list_depth = int(getattr(P, "list_depth", 0) or 0)
    c.force_list = int(getattr(P, "force_list", 0) or 0)
    c.list_skin = float(getattr(P, "list_skin", 0.0) or 0.0)
    c.persistent = int(getattr(P, "persistent", 0) or 0)
    c.idic_lanes = int(getattr(P, "idic_lanes", 0) or 0)
    for k in range(MAX_DUST):
        c.mass_ratio[k] = float(P.mass_ratio[k]) if k < len(P.mass_ratio) else 0.0
        c.R_dust[k] = float(P.R_dust[k]) if k < len(P.R_dust) else 0.0
        c.t_stop_const[k] = float(P.t_stop_const[k]) if k < len(P.t_stop_const) else 0.0
        c.eps_empty[k] = float(P.eps_empty[k]) if k < len(P.eps_empty) else 0.0
    return c


def params_from_c(c: DsParams) -> Params:
    """Inverse of params_to_c."""
    P = Params()
    for f in ("X_min", "X_max", "Y_min", "Y_max", "Z_min", "Z_max", "Particle_on_length", "h",
              "Coeff_h_dust_cell", "tau", "T_end", "T_out", "alpha", "beta", "eps", "Gam_g",
              "Speed_of_sound_gas", "cell_w", "idic_w", "cfl", "t_empty"):
        setattr(P, f, float(getattr(c, f)))
    P.Type_of_state = int(c.Type_of_state)
    P.Maximum_particle = int(c.Maximum_particle)
    P.n_dust = int(c.n_dust)
    for name, bit in MODE_BITS.items():
        setattr(P.mode, name, bool(c.mode & bit))
    P.precision = "fp32" if c.precision == 1 else "fp64"
    P.stencil = int(c.stencil)
    P.list_depth = int(c.list_depth)
    P.force_list = int(c.force_list)
    P.list_skin = float(c.list_skin)
    P.persistent = int(c.persistent)
    P.idic_lanes = int(c.idic_lanes)
    P.mass_ratio = [float(c.mass_ratio[k]) for k in range(P.n_dust)]
    P.R_dust = [float(c.R_dust[k]) for k in range(P.n_dust)]
    P.t_stop_const = [float(c.t_stop_const[k]) for k in range(P.n_dust)]
    P.eps_empty = [float(c.eps_empty[k]) for k in range(P.n_dust)]
    return P


def check(L, ctx, status: int, what: str):
    if status != DS_OK:
        msg = ctypes.create_string_buffer(512)
        flags = ctypes.c_int(0)
        if ctx:
            L.ds_last_error(ctx, ctypes.byref(flags), msg, 512)
        raise DsError(f"{what}: {STATUS.get(status, status)} {msg.value.decode(errors='replace')}"
                      f"{' flags=%d' % flags.value if flags.value else ''}")
