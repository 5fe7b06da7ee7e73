"""Host-side mirror of the reference's step driver over the C ABI.

``Solver`` plays the part of the reference's ``main`` between set-up and output
(kernel.cu:1929-2566): it uploads the SoA particle arrays once, advances them on
the device and downloads them at output times.  A ``Solver`` built from several
``Params`` advances that many independent tubes together (batched launches, one
CUDA graph per step).
"""
from __future__ import annotations

import ctypes
from typing import List, Sequence

import numpy as np

from . import _lib
from .params import Params
from .species import Species

_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)


def _dp(a):
    return None if a is None else a.ctypes.data_as(_DP)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_IP)


def _f64(a, n):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    assert a.shape == (n,), (a.shape, n)
    return a


def idic_columns(P: Params, x) -> np.ndarray:
    """The IDIC cell column (x index) of each position as the step computes it
    for P's precision (ds_idic_columns, host-side)."""
    L = _lib.load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    col = np.empty(max(len(x), 1), dtype=np.int32)
    cp = _lib.params_to_c(P)
    _lib.check(L, None, L.ds_idic_columns(ctypes.byref(cp), len(x), _dp(x), _ip(col)), "ds_idic_columns")
    return col[: len(x)]


class Solver:
    def __init__(self, params):
        self.L = _lib.load()
        plist: List[Params] = list(params) if isinstance(params, (list, tuple)) else [params]
        self.params = plist
        arr = (_lib.DsParams * len(plist))(*[_lib.params_to_c(p) for p in plist])
        self._cparams = arr
        ctx = ctypes.c_void_p()
        st = self.L.ds_create_batch(len(plist), arr, ctypes.byref(ctx))
        _lib.check(self.L, None, st, "ds_create_batch")
        self.ctx = ctx
        self.n = [[None] * (1 + p.n_dust) for p in plist]
        self._pinned = []  # host buffers from ds_host_alloc, freed with the solver

    # -- upload -------------------------------------------------------------
    def set_species(self, tube: int, s: int, sp: Species):
        n = sp.n
        g = lambda f: _f64(getattr(sp, f), n)  # noqa: E731
        ind = np.ascontiguousarray(sp.ind if sp.ind is not None else np.zeros(n, np.int32), dtype=np.int32)
        keep = {f: g(f) for f in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h", "ts")}
        if s == 0:
            st = self.L.ds_set_gas(self.ctx, tube, n, *[_dp(keep[f]) for f in
                                                        ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho",
                                                         "p", "e", "m", "h")], _ip(ind))
        else:
            st = self.L.ds_set_dust(self.ctx, tube, s, n, *[_dp(keep[f]) for f in
                                                            ("x", "y", "z", "vx", "vy", "vz", "rho", "m", "ts",
                                                             "h")], _ip(ind))
        _lib.check(self.L, self.ctx, st, f"set species {s} of tube {tube}")
        self.n[tube][s] = n

    def copy_tube_from(self, tube: int, src: "Solver", src_tube: int):
        """Carry a running tube of ``src`` into ``tube`` (device to device, at the first step)."""
        _lib.check(self.L, self.ctx, self.L.ds_copy_tube(self.ctx, tube, src.ctx, src_tube), "ds_copy_tube")
        self.n[tube] = list(src.n[src_tube])

    def set_tube(self, tube: int, species: Sequence[Species]):
        for s, sp in enumerate(species):
            self.set_species(tube, s, sp.copy().fill_missing())

    def init_tube(self, tube: int, spec):
        """Generate the tube's particles on the device (ds_init_tube); spec is an
        ic.DeviceIC whose plan gave this tube's parameters."""
        _lib.check(self.L, self.ctx, self.L.ds_init_tube(self.ctx, tube, ctypes.byref(spec.to_c())),
                   f"ds_init_tube({spec.kind})")
        _, counts = spec.plan(self.params[tube])
        self.n[tube] = list(counts)

    # -- stepping -----------------------------------------------------------
    def step(self, n: int = 1):
        _lib.check(self.L, self.ctx, self.L.ds_step(self.ctx, int(n)), "ds_step")

    def step_async(self, n: int = 1):
        _lib.check(self.L, self.ctx, self.L.ds_step_async(self.ctx, int(n)), "ds_step_async")

    def synchronize(self):
        _lib.check(self.L, self.ctx, self.L.ds_synchronize(self.ctx), "ds_synchronize")

    # -- split step (slab decomposition) -------------------------------------
    def step_density(self):
        """First part of one step: sort, gas density, EOS (ds_step_density)."""
        _lib.check(self.L, self.ctx, self.L.ds_step_density(self.ctx), "ds_step_density")

    def cfl_min(self, tube: int = 0) -> float:
        v = ctypes.c_double(0.0)
        _lib.check(self.L, self.ctx, self.L.ds_get_cfl_min(self.ctx, tube, ctypes.byref(v)), "ds_get_cfl_min")
        return v.value

    def set_cfl_min(self, tube: int, dtmin: float):
        _lib.check(self.L, self.ctx, self.L.ds_set_cfl_min(self.ctx, tube, float(dtmin)), "ds_set_cfl_min")

    def set_gas_hydro(self, tube: int, idx, rho, p):
        """Density and pressure of gas particles (caller indices idx) between
        the two parts of a step (ds_set_gas_hydro)."""
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        n = len(idx)
        rho, p = _f64(rho, n), _f64(p, n)
        _lib.check(self.L, self.ctx, self.L.ds_set_gas_hydro(self.ctx, tube, n, _ip(idx), _dp(rho), _dp(p)),
                   "ds_set_gas_hydro")

    def step_complete(self):
        """Second part of the step begun by step_density (ds_step_complete)."""
        _lib.check(self.L, self.ctx, self.L.ds_step_complete(self.ctx), "ds_step_complete")

    def set_time(self, tube: int, Tm: float, nsteps: int):
        _lib.check(self.L, self.ctx, self.L.ds_set_time(self.ctx, tube, float(Tm), int(nsteps)), "ds_set_time")

    # -- host arrays as the state of record ----------------------------------
    def pinned(self, n: int, dtype=np.float64) -> np.ndarray:
        """A numpy array in pinned host memory (ds_host_alloc), freed with the solver."""
        dtype = np.dtype(dtype)
        ptr = ctypes.c_void_p()
        nbytes = max(1, n * dtype.itemsize)
        _lib.check(self.L, None, self.L.ds_host_alloc(ctypes.byref(ptr), nbytes), "ds_host_alloc")
        self._pinned.append(ptr)
        buf = (ctypes.c_char * nbytes).from_address(ptr.value)
        return np.frombuffer(buf, dtype=dtype, count=n)

    def bind_host(self, tube: int, s: int, arrays, ind=None):
        """Bind pinned arrays (field name -> float64 array, the names of
        Species; ind int32) to species s of a tube (ds_bind_host); arrays None
        unbinds it."""
        names = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h", "ts")
        if arrays is None:
            _lib.check(self.L, self.ctx, self.L.ds_bind_host(self.ctx, tube, s, 0, None, None), "ds_bind_host")
            return
        n = self.n[tube][s]
        for f, a in arrays.items():
            assert f in names and a.dtype == np.float64 and a.shape == (n,), f
        assert ind is None or (ind.dtype == np.int32 and ind.shape == (n,))
        self._bound = getattr(self, "_bound", {})
        self._bound[(tube, s)] = (arrays, ind)  # keep the arrays alive while bound
        ptrs = (_DP * len(names))(*[_dp(arrays.get(f)) for f in names])
        _lib.check(self.L, self.ctx, self.L.ds_bind_host(self.ctx, tube, s, n, ptrs, _ip(ind)), "ds_bind_host")

    def step_host(self, n: int = 1):
        _lib.check(self.L, self.ctx, self.L.ds_step_host(self.ctx, int(n)), "ds_step_host")

    def step_timed(self, n: int = 1):
        """(total ms, per-phase ms) of n steps with their kernels launched one by
        one and events between phases (ds_step_timed)."""
        tot = ctypes.c_float(0)
        ph = (ctypes.c_float * _lib.DS_NPHASE)()
        _lib.check(self.L, self.ctx, self.L.ds_step_timed(self.ctx, int(n), ctypes.byref(tot), ph), "ds_step_timed")
        return tot.value, list(ph)

    def step_timed_graph(self, n: int = 1) -> float:
        """Device ms of n steps as ds_step runs them (graph replays between two
        events; ds_step_timed with no phase split)."""
        tot = ctypes.c_float(0)
        _lib.check(self.L, self.ctx, self.L.ds_step_timed(self.ctx, int(n), ctypes.byref(tot), None),
                   "ds_step_timed")
        return tot.value

    # -- download -----------------------------------------------------------
    def get_species(self, tube: int, s: int, template: Species = None) -> Species:
        """Every field of one species in caller order (ds_get_fields).  template
        is accepted for older callers and not needed: m and h come back too."""
        n = self.n[tube][s]
        names = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h", "ts")
        out = {f: np.empty(n, np.float64) for f in names}
        ind = np.empty(n, np.int32)
        ptrs = (_DP * len(names))(*[_dp(out[f]) for f in names])
        _lib.check(self.L, self.ctx, self.L.ds_get_fields(self.ctx, tube, s, ptrs, _ip(ind)),
                   f"get species {s} of tube {tube}")
        return Species(ind=ind, **out)

    def step_lists(self, tube: int, s: int):
        """(head, next) of the cell lists the last step built (ds_step_lists)."""
        n = self.n[tube][s]
        nc = ctypes.c_int(0)
        _lib.check(self.L, self.ctx, self.L.ds_step_lists(self.ctx, tube, s, None, None, ctypes.byref(nc)),
                   "ds_step_lists")
        head = np.empty(nc.value + 1, np.int32)
        nxt = np.empty(max(n, 1), np.int32)
        _lib.check(self.L, self.ctx, self.L.ds_step_lists(self.ctx, tube, s, _ip(head), _ip(nxt), ctypes.byref(nc)),
                   "ds_step_lists")
        return head, nxt[:n]

    def write_snapshot(self, directory: str, num: int, tube: int = 0):
        """The reference's snapshot files (Data_out / Data_out_dust) for one
        tube, with the Nn columns from the last step's cell lists."""
        from . import snapshot
        P = self.params[tube]
        species = [self.get_species(tube, s) for s in range(1 + P.n_dust)]
        nexts = [self.step_lists(tube, s)[1] for s in range(1 + P.n_dust)]
        snapshot.write(directory, num, self.time(tube)[0], P.tau, P.h, species, nexts)

    def time(self, tube: int = 0):
        Tm, dt = ctypes.c_double(), ctypes.c_double()
        ns = ctypes.c_longlong()
        _lib.check(self.L, self.ctx, self.L.ds_get_time(self.ctx, tube, ctypes.byref(Tm), ctypes.byref(dt),
                                                        ctypes.byref(ns)), "ds_get_time")
        return Tm.value, dt.value, ns.value

    def debug_cells(self, tube: int, s: int):
        n = self.n[tube][s]
        nc = ctypes.c_int(0)
        # first call for ncells
        key = np.empty(max(n, 1), np.int32)
        nxt = np.empty(max(n, 1), np.int32)
        cand = np.empty(max(n, 1), np.int32)
        nnb = np.empty(max(n, 1), np.int32)
        _lib.check(self.L, self.ctx, self.L.ds_debug_cells(self.ctx, tube, s, None, None, None, None, None,
                                                           ctypes.byref(nc)), "ds_debug_cells")
        head = np.empty(nc.value + 1, np.int32)
        _lib.check(self.L, self.ctx, self.L.ds_debug_cells(self.ctx, tube, s, _ip(key), _ip(head), _ip(nxt),
                                                           _ip(cand), _ip(nnb), ctypes.byref(nc)), "ds_debug_cells")
        return dict(cell_key=key[:n], head=head, next=nxt[:n], ncand=cand[:n], nnb=nnb[:n], ncells=nc.value)

    def debug_idic(self, tube: int, s: int):
        n = ctypes.c_int(0)
        _lib.check(self.L, self.ctx, self.L.ds_debug_idic(self.ctx, tube, s, None, None, ctypes.byref(n)),
                   "ds_debug_idic")
        cnt = np.empty(n.value, np.int32)
        cells = np.empty((12, n.value), np.float64)
        _lib.check(self.L, self.ctx, self.L.ds_debug_idic(self.ctx, tube, s, _ip(cnt), _dp(cells), ctypes.byref(n)),
                   "ds_debug_idic")
        return cnt, cells

    def conservation(self, tube: int = 0):
        out = np.zeros(6, np.float64)
        _lib.check(self.L, self.ctx, self.L.ds_conservation(self.ctx, tube, _dp(out)), "ds_conservation")
        return out

    def save(self, tube: int, path: str):
        """Binary checkpoint of one tube (ds_save_tube)."""
        _lib.check(self.L, self.ctx, self.L.ds_save_tube(self.ctx, tube, path.encode()), "ds_save_tube")

    def load(self, tube: int, path: str):
        """Restore one tube's particles and clock from a checkpoint (ds_load_tube)."""
        st = self.L.ds_load_tube(self.ctx, tube, path.encode())
        _lib.check(self.L, self.ctx, st, "ds_load_tube")
        ps = _lib.DsParams()
        _lib.check(self.L, None, self.L.ds_checkpoint_params(path.encode(), ctypes.byref(ps)), "ds_checkpoint_params")
        self.n[tube] = [None] * (1 + int(ps.n_dust))
        with open(path, "rb") as f:  # particle counts, from the file's species records
            f.seek(8 + ctypes.sizeof(_lib.DsParams) + 3 * 8)
            nsp = int(np.frombuffer(f.read(4), np.int32)[0])
            for s in range(nsp):
                n = int(np.frombuffer(f.read(8), np.int64)[0])
                self.n[tube][s] = n
                f.seek(n * (15 * 8 + 4), 1)

    @classmethod
    def from_checkpoint(cls, path: str) -> "Solver":
        """A one-tube solver with the checkpoint's parameters, particles and clock."""
        L = _lib.load()
        ps = _lib.DsParams()
        _lib.check(L, None, L.ds_checkpoint_params(path.encode(), ctypes.byref(ps)), "ds_checkpoint_params")
        S = cls(_lib.params_from_c(ps))
        S.load(0, path)
        return S

    def device_flags(self) -> int:
        """Sticky device flags of the context (DS_FLAG_* bits of the ABI):
        1 IDIC index out of range, 2 dust index beyond the gas count,
        4 a non-finite velocity, position or energy, 8 a cut-off beyond the
        stencil's cells (proper grid)."""
        flags = ctypes.c_int(0)
        msg = ctypes.create_string_buffer(512)
        _lib.check(self.L, self.ctx, self.L.ds_last_error(self.ctx, ctypes.byref(flags), msg, 512), "ds_last_error")
        return flags.value

    def dust_density(self):
        """Dust self-density of every tube at the current positions (the
        reference's output-only sweep, kernel.cu:2029-2043), on demand."""
        _lib.check(self.L, self.ctx, self.L.ds_dust_density(self.ctx), "ds_dust_density")

    def list_stats(self, tube: int = 0):
        """(steps that re-sorted and recorded the neighbour lists, steps taken)."""
        r, n = ctypes.c_longlong(0), ctypes.c_longlong(0)
        _lib.check(self.L, self.ctx, self.L.ds_list_stats(self.ctx, tube, ctypes.byref(r), ctypes.byref(n)),
                   "ds_list_stats")
        return int(r.value), int(n.value)

    def debug_force_lists(self, tube: int = 0, cap: int = 512):
        """The recorded force lists of the tube's gas by caller index: (count,
        nbr) with count[i] = entries of particle i (-1: its warp walks) and
        nbr[i, :count[i]] their caller indices."""
        n = self.n[tube][0]
        count = np.zeros(max(n, 1), dtype=np.int32)
        nbr = np.full((max(n, 1), cap), -1, dtype=np.int32)
        _lib.check(self.L, self.ctx, self.L.ds_debug_force_lists(self.ctx, tube, cap, _ip(count), _ip(nbr)),
                   "ds_debug_force_lists")
        return count[:n], nbr[:n]

    def kernels_per_step(self):
        k = ctypes.c_int(0)
        _lib.check(self.L, self.ctx, self.L.ds_kernels_per_step(self.ctx, ctypes.byref(k)), "ds_kernels_per_step")
        return k.value

    def memory_bytes(self):
        b = ctypes.c_longlong(0)
        _lib.check(self.L, self.ctx, self.L.ds_memory_bytes(self.ctx, ctypes.byref(b)), "ds_memory_bytes")
        return b.value

    def close(self):
        if getattr(self, "ctx", None):
            self.L.ds_destroy(self.ctx)
            self.ctx = None
        for ptr in getattr(self, "_pinned", []):
            self.L.ds_host_free(ptr)
        self._pinned = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
