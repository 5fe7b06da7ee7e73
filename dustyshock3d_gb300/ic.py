"""Initial conditions.

``init_sod_x_dust`` restates the reference's active generator
(kernel.cu:1391-1582) so that a reference run can be replayed from identical
FP64 inputs, including its quirks:

* the ``Ind`` flag is assigned outside the accept test (kernel.cu:1441-1448,
  1481-1488), so a rejected lattice point overwrites the flag of the last
  accepted particle;
* the interior test uses ``X_cube`` for y (kernel.cu:1441, 1481);
* ``Coeff_h_dust_cell`` is forced to 0.5 (kernel.cu:1498).

A rejected point before the first accepted one makes the reference write
``Ind_gas[-1]``; that is undefined behaviour there and rejected here.

``dusty_sod_tube`` builds the dusty Sod shock tube of the benchmark
configurations (no reference counterpart): two cubic lattices with equal
particle mass, dust on the same lattices offset by half a spacing, h = 1.3
local spacing, periodic y/z, frozen walls at the x ends.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from .params import Mode, Params
from .species import Species


def _eq_state(rho, e, type_of_state, gam, cs):
    """kernel.cu:92-97."""
    if type_of_state == 1:
        return cs * cs * rho
    return rho * e * (gam - 1)


def _lattice(x0, sign, dl, Im, Y_min, Jm, Z_min, Km):
    i, j, k = np.meshgrid(np.arange(Im + 1, dtype=np.float64), np.arange(Jm + 1, dtype=np.float64),
                          np.arange(Km + 1, dtype=np.float64), indexing="ij")
    i = i.ravel(); j = j.ravel(); k = k.ravel()
    if sign < 0:
        x = 0.0 - (i * dl)
    else:
        x = dl + (i * dl)
    y = Y_min + (j * dl)
    z = Z_min + (k * dl)
    return x, y, z


def _eq_state1(p, e, type_of_state, gam, cs):
    """kernel.cu:99-103."""
    if type_of_state == 1:
        return p / (cs * cs)
    return p / (e * (gam - 1))


def _reference_lattices(P: Params, e_lr, p_lr, rho_lr, cube, inner, before_first: str = "error") -> Species:
    """The gas of the reference's two-lattice generators (kernel.cu:938-1042,
    1391-1495): left lattice x = 0 - i dl, right x = dl + i dl, points accepted
    in ``cube``, Ind from the ``inner`` thresholds with the reference's quirk.

    before_first: lattice points before the first accepted one make the
    reference write Ind_gas[-1], outside its array (kernel.cu:1441-1448;
    undefined behaviour).  "error" refuses such a box; "skip" drops those
    writes, which change no particle -- the reference's own default Init.txt
    (a box of [-2, 2]^3 around the accept cube) is such a box."""
    h = P.h
    mas_particle = 1.0 / (P.Particle_on_length * P.Particle_on_length * P.Particle_on_length)
    dlh = [math.pow(mas_particle / rho_lr[0], 1 / 3.0), math.pow(mas_particle / rho_lr[1], 1 / 3.0)]
    parts = []
    Im = int((0.0 - P.X_min) / dlh[0]) + 1
    Jm = int((P.Y_max - P.Y_min) / dlh[0]) + 1
    Km = int((P.Z_max - P.Z_min) / dlh[0]) + 1
    xl, yl, zl = _lattice(0.0, -1, dlh[0], Im, P.Y_min, Jm, P.Z_min, Km)
    parts.append((xl, yl, zl, e_lr[0], p_lr[0], rho_lr[0]))
    Im = int((P.X_max - 0.0) / dlh[1]) + 1
    Jm = int((P.Y_max - P.Y_min) / dlh[1]) + 1
    Km = int((P.Z_max - P.Z_min) / dlh[1]) + 1
    xr, yr, zr = _lattice(0.0, +1, dlh[1], Im, P.Y_min, Jm, P.Z_min, Km)
    parts.append((xr, yr, zr, e_lr[1], p_lr[1], rho_lr[1]))

    X = np.concatenate([q[0] for q in parts])
    Y = np.concatenate([q[1] for q in parts])
    Z = np.concatenate([q[2] for q in parts])
    E = np.concatenate([np.full(len(q[0]), q[3]) for q in parts])
    PP = np.concatenate([np.full(len(q[0]), q[4]) for q in parts])
    R = np.concatenate([np.full(len(q[0]), q[5]) for q in parts])
    acc = (np.abs(X) <= cube[0]) & (np.abs(Y) <= cube[1]) & (np.abs(Z) <= cube[2])
    interior = (np.abs(X) <= inner[0]) & (np.abs(Y) <= inner[1]) & (np.abs(Z) <= inner[2])
    pidx = np.cumsum(acc) - 1  # index of the last accepted particle at each lattice point
    if len(pidx) and pidx[0] < 0:
        if before_first != "skip":
            raise ValueError("first lattice point rejected: the reference writes Ind_gas[-1] here "
                             "(undefined behaviour); choose Y_min, Z_min inside the accept cube")
        keep = pidx >= 0
        pidx, interior = pidx[keep], interior[keep]
    N = int(acc.sum())
    if N > P.Maximum_particle:
        raise ValueError(f"{N} gas particles exceed Maximum_particle={P.Maximum_particle} "
                         "(the reference would overrun its arrays, kernel.cu:1751)")
    # Ind[p] takes the interior flag of the LAST lattice point that saw p as current
    last = np.full(N, -1, dtype=np.int64)
    np.maximum.at(last, pidx, np.arange(len(pidx)))
    ind = np.where(interior[last], 0, 1).astype(np.int32)

    sel = np.nonzero(acc)[0]
    n = len(sel)
    return Species(x=X[sel].copy(), y=Y[sel].copy(), z=Z[sel].copy(),
                   vx=np.zeros(n), vy=np.zeros(n), vz=np.zeros(n),
                   ax=np.zeros(n), ay=np.zeros(n), az=np.zeros(n),
                   rho=R[sel].copy(), p=PP[sel].copy(), e=E[sel].copy(),
                   m=np.full(n, mas_particle), h=np.full(n, h), ts=np.zeros(n), ind=ind)


def _dust_on_gas(P: Params, gas: Species) -> List[Species]:
    """Dust species 1..n_dust on the gas sites (kernel.cu:1505-1548)."""
    n = gas.n
    dust = []
    for k in range(P.n_dust):
        mr, Rd = P.mass_ratio[k], P.R_dust[k]
        # Eq_t_stop, kernel.cu:43-46
        ts = Rd / (np.sqrt(P.Gam_g * gas.p / gas.rho) * gas.rho)
        dust.append(Species(x=gas.x.copy(), y=gas.y.copy(), z=gas.z.copy(),
                            vx=np.zeros(n), vy=np.zeros(n), vz=np.zeros(n),
                            ax=np.zeros(n), ay=np.zeros(n), az=np.zeros(n),
                            rho=gas.rho * mr, p=np.zeros(n), e=np.zeros(n),
                            m=gas.m * mr, h=np.full(n, P.h), ts=ts, ind=gas.ind.copy()))
    return dust


def init_sod_x_dust(P: Params, before_first: str = "error") -> Tuple[Params, List[Species]]:
    """kernel.cu:1391-1582: gas on two lattices (e 2.5 | 2.0, rho 1 | 1) and two
    dust species copied onto the gas positions.  Returns (params, [gas, d1, d2]).
    before_first: see _reference_lattices ("skip" runs the reference's default
    Init.txt box)."""
    P = P.copy()
    border_length = 2.5 * P.h
    X_cube, Y_cube, Z_cube = 1.0, 0.8, 0.8
    e_lr, rho_lr = (2.5, 2.0), (1.0, 1.0)
    p_lr = tuple(_eq_state(rho_lr[s], e_lr[s], P.Type_of_state, 1.4, 1.0) for s in range(2))
    # the interior test compares |y| with X_cube (kernel.cu:1441, 1481)
    inner = (X_cube - border_length, X_cube - border_length, Z_cube - border_length)
    gas = _reference_lattices(P, e_lr, p_lr, rho_lr, (X_cube, Y_cube, Z_cube), inner, before_first)
    # kernel.cu:1497-1502
    P.Coeff_h_dust_cell = 0.5
    P.n_dust = 2
    P.mass_ratio = [0.75, 0.5]
    P.R_dust = [0.01, 1.0]
    P.mode = Mode.reference()
    return P, [gas] + _dust_on_gas(P, gas)


def init_sod_x_mas(P: Params) -> Tuple[Params, List[Species]]:
    """The equal-mass lattices of kernel.cu:938-1042 (p 1 | 0.1, e 2.5 | 2.0, rho
    from Eq_State1, accepted in |x|, |y|, |z| <= 1) with P.n_dust dust species on
    the gas sites as init_Sod_X_Dust places them (kernel.cu:1505-1548, using
    P.mass_ratio and P.R_dust).  Returns (params, [gas, dust...])."""
    P = P.copy()
    border_length = 2.5 * P.h
    p_lr, e_lr = (1.0, 0.1), (2.5, 2.0)
    rho_lr = tuple(_eq_state1(p_lr[s], e_lr[s], P.Type_of_state, 1.4, 1.0) for s in range(2))
    inner = (1.0 - border_length,) * 3
    gas = _reference_lattices(P, e_lr, p_lr, rho_lr, (1.0, 1.0, 1.0), inner)
    return P, [gas] + _dust_on_gas(P, gas)


def dusty_sod_tube(dx_left: float, Ly: float, Lz: float = None, eps: float = 1.0, t_s: float = 1e-3,
                   rho_L: float = 1.0, p_L: float = 1.0, rho_R: float = 0.125, p_R: float = 0.1,
                   gamma: float = 1.4, h_factor: float = 1.3, x_range=(-0.5, 0.5), wall: float = 2.5,
                   t_end: float = 0.2, cfl: float = 0.3, alpha: float = 1.0, beta: float = 2.0,
                   av_eps: float = 0.01, idic_cells_per_right_spacing: float = 2.0,
                   fixed_tau: float = None, lattice_offset: float = 0.25) -> Tuple[Params, List[Species]]:
    """Dusty Sod tube on [x0, x1] x [0, Ly] x [0, Lz], periodic in y and z.

    The left state sits on a cubic lattice of spacing ``dx_left``; the right
    lattice has n_R = round(L/(dx_left*(rho_L/rho_R)^(1/3))) sites across each
    periodic side and the same particle mass per x-slab (spacing 2 dx_left for
    the classical density ratio 8).  One dust species sits on each lattice
    offset by half a spacing in x, y and z, with mass eps x the gas mass.
    Particles within ``wall`` smoothing lengths of either x end are frozen
    (Ind = 1), like the reference's border particles (kernel.cu:1396, 1441).

    Gas sites sit at (i + lattice_offset) spacings from the lower faces and
    dust sites half a spacing further.  With the default 0.25 no particle
    starts on a face of the IDIC grid (width 2 right spacings = 4 left
    spacings, origin at the lower box corner): a lattice on the faces would
    put whole columns of dust exactly on them, and rounding-level motion would
    then move a column between cells and change the cells' eps at once.
    """
    Lz = Ly if Lz is None else Lz
    x0, x1 = x_range
    xm = 0.5 * (x0 + x1)

    def side(rho, p, xa, xb, dxy_target, left):
        ny = max(1, int(round(Ly / dxy_target)))
        nz = max(1, int(round(Lz / dxy_target)))
        dy, dz = Ly / ny, Lz / nz
        m = rho_L * dx_left ** 3
        dx = m / (rho * dy * dz)
        nx = max(1, int(round((xb - xa) / dx)))
        dx = (xb - xa) / nx
        mass = rho * dx * dy * dz
        hloc = h_factor * (dx * dy * dz) ** (1.0 / 3.0)
        i, j, k = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64),
                              np.arange(nz, dtype=np.float64), indexing="ij")
        gx = xa + (i.ravel() + lattice_offset) * dx
        gy = (j.ravel() + lattice_offset) * dy
        gz = (k.ravel() + lattice_offset) * dz
        # dust: offset by half a spacing (y, z wrap onto the periodic lattice)
        dxp = gx + 0.5 * dx
        dyp = np.mod(gy + 0.5 * dy, Ly)
        dzp = np.mod(gz + 0.5 * dz, Lz)
        e = p / ((gamma - 1.0) * rho)
        return dict(gx=gx, gy=gy, gz=gz, dxp=dxp, dyp=dyp, dzp=dzp, mass=mass, h=hloc, rho=rho, p=p, e=e,
                    dx=dx)

    L = side(rho_L, p_L, x0, xm, dx_left, True)
    R = side(rho_R, p_R, xm, x1, dx_left * (rho_L / rho_R) ** (1.0 / 3.0), False)

    def build(key_x, key_y, key_z, dust):
        xs, ys, zs, ms, hs, rs, ps, es = [], [], [], [], [], [], [], []
        for S in (L, R):
            n = len(S[key_x])
            xs.append(S[key_x]); ys.append(S[key_y]); zs.append(S[key_z])
            ms.append(np.full(n, S["mass"] * (eps if dust else 1.0)))
            hs.append(np.full(n, S["h"]))
            rs.append(np.full(n, S["rho"] * (eps if dust else 1.0)))
            ps.append(np.full(n, 0.0 if dust else S["p"]))
            es.append(np.full(n, 0.0 if dust else S["e"]))
        x = np.concatenate(xs); n = len(x)
        h = np.concatenate(hs)
        ind = ((x < x0 + wall * h) | (x > x1 - wall * h)).astype(np.int32)
        return Species(x=x, y=np.concatenate(ys), z=np.concatenate(zs), vx=np.zeros(n), vy=np.zeros(n),
                       vz=np.zeros(n), ax=np.zeros(n), ay=np.zeros(n), az=np.zeros(n),
                       rho=np.concatenate(rs), p=np.concatenate(ps), e=np.concatenate(es),
                       m=np.concatenate(ms), h=h, ts=np.full(n, t_s) if dust else np.zeros(n), ind=ind)

    gas = build("gx", "gy", "gz", False)
    dust = build("dxp", "dyp", "dzp", True)
    h_max = max(L["h"], R["h"])
    P = Params(X_min=x0, X_max=x1, Y_min=0.0, Y_max=Ly, Z_min=0.0, Z_max=Lz, Type_of_state=0,
               Maximum_particle=gas.n, Particle_on_length=1.0 / dx_left, h=h_max, Coeff_h_dust_cell=0.5,
               tau=fixed_tau if fixed_tau else 1e-4, T_end=t_end, T_out=t_end, alpha=alpha, beta=beta,
               eps=av_eps, Gam_g=gamma, Speed_of_sound_gas=1.0, n_dust=1, mass_ratio=[eps], R_dust=[0.0],
               t_stop_const=[t_s], eps_empty=[eps], t_empty=t_s, cell_w=1.001 * h_max, stencil=2,
               idic_w=idic_cells_per_right_spacing * R["dx"], cfl=cfl, mode=Mode.baseline())
    if fixed_tau:
        P.mode.cfl = False
    return P, [gas, dust]


def uneven_tube_kwargs(N_gas: float, rho_ratio: float, p_ratio: float, eps: float, t_s: float, t_end: float = 0.2,
                       n_across: int = 24, x_range=(-0.5, 0.5)) -> dict:
    """dusty_sod_tube arguments of a tube with about N_gas gas particles (and as
    many dust), left state (rho 1, p 1), right state (1/rho_ratio, 1/p_ratio),
    n_across left lattice sites across the periodic cross-section."""
    L = x_range[1] - x_range[0]
    dx_left = 0.5 * L * n_across * n_across * (1.0 + 1.0 / rho_ratio) / N_gas
    return dict(dx_left=dx_left, Ly=n_across * dx_left, eps=eps, t_s=t_s, rho_R=1.0 / rho_ratio,
                p_R=1.0 / p_ratio, t_end=t_end, x_range=x_range)


def uneven_tube(N_gas: float, rho_ratio: float, p_ratio: float, eps: float, t_s: float, t_end: float = 0.2,
                n_across: int = 24, x_range=(-0.5, 0.5)) -> Tuple[Params, List[Species]]:
    """The tube of uneven_tube_kwargs, generated on the host."""
    return dusty_sod_tube(**uneven_tube_kwargs(N_gas, rho_ratio, p_ratio, eps, t_s, t_end, n_across, x_range))


def draw_tube_params(rng, n_range=(2.0e4, 1.0e6)):
    """One tube of the uneven-batch distributions: particle count per phase
    log-uniform in n_range, density ratio U[4, 16], pressure ratio U[5, 20],
    eps log-U[0.01, 10], t_s log-U[1e-4, 1e-1]."""
    lo, hi = np.log(n_range[0]), np.log(n_range[1])
    return dict(N_gas=float(np.exp(rng.uniform(lo, hi))), rho_ratio=float(rng.uniform(4.0, 16.0)),
                p_ratio=float(rng.uniform(5.0, 20.0)), eps=float(np.exp(rng.uniform(np.log(0.01), np.log(10.0)))),
                t_s=float(np.exp(rng.uniform(np.log(1e-4), np.log(1e-1)))))


def batch_tubes(seed: int = 2026, n_tubes: int = 64, n_range=(2.0e4, 1.0e6), t_end: float = 0.2):
    """The seeded batch of uneven tubes: a list of (params, species)."""
    rng = np.random.default_rng(seed)
    return [uneven_tube(t_end=t_end, **draw_tube_params(rng, n_range)) for _ in range(n_tubes)]


# ---------------------------------------------------------------------------
# Initial conditions generated on the device (ds_ic / ds_init_tube)
# ---------------------------------------------------------------------------
@dataclass
class DeviceIC:
    """A generator run on the device by ``Solver.init_tube`` (the C ABI's
    ds_ic; defaults are ds_ic_init's).  ``kind``: "sod_x_dust"
    (kernel.cu:1391-1582), "sod_x_mas" (kernel.cu:938-1042 with dust on the gas
    sites) or "dusty_sod" (``dusty_sod_tube``; the remaining fields are its
    arguments: ``x0, x1`` = ``x_range``, ``idic_cells`` =
    ``idic_cells_per_right_spacing``, ``Lz`` 0 = ``Ly``, ``fixed_tau`` 0 =
    none).  The particles equal the host generators' bit for bit."""

    kind: str = "sod_x_dust"
    dx_left: float = 0.0
    Ly: float = 0.0
    Lz: float = 0.0
    eps: float = 1.0
    t_s: float = 1e-3
    rho_L: float = 1.0
    p_L: float = 1.0
    rho_R: float = 0.125
    p_R: float = 0.1
    gamma: float = 1.4
    h_factor: float = 1.3
    x0: float = -0.5
    x1: float = 0.5
    wall: float = 2.5
    lattice_offset: float = 0.25
    t_end: float = 0.2
    cfl: float = 0.3
    alpha: float = 1.0
    beta: float = 2.0
    av_eps: float = 0.01
    idic_cells: float = 2.0
    fixed_tau: float = 0.0

    @staticmethod
    def dusty_sod(dx_left: float, Ly: float, Lz: float = None, x_range=(-0.5, 0.5),
                  idic_cells_per_right_spacing: float = 2.0, fixed_tau: float = None, **kw) -> "DeviceIC":
        """The device twin of ``dusty_sod_tube`` (same keyword arguments)."""
        return DeviceIC(kind="dusty_sod", dx_left=dx_left, Ly=Ly, Lz=0.0 if Lz is None else Lz,
                        x0=x_range[0], x1=x_range[1], idic_cells=idic_cells_per_right_spacing,
                        fixed_tau=fixed_tau or 0.0, **kw)

    @staticmethod
    def uneven(**kw) -> "DeviceIC":
        """The device twin of ``uneven_tube``."""
        return DeviceIC.dusty_sod(**uneven_tube_kwargs(**kw))

    def to_c(self):
        from . import _lib
        c = _lib.DsIc()
        c.kind = _lib.IC_KINDS[self.kind]
        for f in _lib.IC_FIELDS:
            setattr(c, f, float(getattr(self, f)))
        return c

    def plan(self, init: Params = None) -> Tuple[Params, List[int]]:
        """(run parameters, particles per species) of this generator, computed by
        the library on the host (ds_ic_plan).  init: the Init.txt parameters the
        reference generators read."""
        import ctypes

        from . import _lib
        L = _lib.load()
        out = _lib.DsParams()
        counts = (ctypes.c_int * (1 + 4))()
        cinit = _lib.params_to_c(init) if init is not None else None
        st = L.ds_ic_plan(ctypes.byref(self.to_c()), ctypes.byref(cinit) if cinit is not None else None,
                          ctypes.byref(out), counts)
        _lib.check(L, None, st, f"ds_ic_plan({self.kind})")
        P = _lib.params_from_c(out)
        return P, [int(counts[s]) for s in range(1 + P.n_dust)]


def parse_ic_init_txt(text: str) -> DeviceIC:
    """The ``ic = <kind>`` and ``ic.<field> = value`` extension lines of an
    Init.txt (no ``ic`` line: the reference's generator, sod_x_dust)."""
    kv = []
    for line in text.splitlines()[18:]:
        body = line.split("//", 1)[0].strip()
        if not body or "=" not in body:
            continue
        key, val = (t.strip() for t in body.split("=", 1))
        kv.append((key, val))
    kind = "sod_x_dust"
    for key, val in kv:
        if key == "ic":
            if val.lower() not in ("sod_x_dust", "sod_x_mas", "dusty_sod"):
                raise ValueError(f"unknown initial-condition kind {val!r}")
            kind = val.lower()
    spec = DeviceIC(kind=kind)
    names = {f.name for f in dataclasses.fields(DeviceIC)} - {"kind"}
    for key, val in kv:
        if key.startswith("ic."):
            if key[3:] not in names:
                raise ValueError(f"unknown initial-condition field {key!r}")
            setattr(spec, key[3:], float(val))
    return spec
