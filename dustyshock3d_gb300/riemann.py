"""Exact solutions of the shock-tube problems the dusty Sod tube reduces to.

The reference has no exact-solution check: its runs were judged by eye from
the snapshot files (kernel.cu:250-265).  This module gives the two limits in
which the dusty shock tube has a closed-form answer, so that a run can be
scored against the physics rather than against another run:

* ``euler_riemann`` -- the exact solution of the Riemann problem of the 1-D
  Euler equations for an ideal gas, by the method of E. F. Toro, *Riemann
  Solvers and Numerical Methods for Fluid Dynamics* (3rd ed., Springer 2009),
  chapter 4: the star-region pressure is the root of the pressure function
  f(p) = f_L(p) + f_R(p) + (u_R - u_L), where f_K is the shock branch (a
  Rankine-Hugoniot curve) for p > p_K and the rarefaction branch (an
  isentrope) otherwise; it is found by Newton-Raphson from the
  primitive-variable guess, clipped to a small positive pressure; the star
  velocity follows, and the self-similar solution is sampled at x / t.

* the gas-only limit, dust-to-gas ratio eps -> 0: the gas is the classical
  Sod problem (``euler_riemann`` on the gas states);

* the perfectly coupled limit, stopping time t_s -> 0 with a uniform dust-to-
  gas ratio eps (``dusty_sod_coupled``): gas and dust move with one velocity,
  so the mixture obeys the Euler equations with density (1 + eps) rho_g, the
  gas pressure, the same gamma (the dust carries no pressure and no heat), and
  total energy 1/2 (1 + eps) rho_g v^2 + p / (gamma - 1) -- the ideal-gas form
  with the mixture density.  Its sound speed is c_s / sqrt(1 + eps).  The gas
  density is the mixture's divided by 1 + eps; gas and dust velocities are the
  mixture's.

``l1_against_exact`` scores particle fields against a profile: the mean over
the chosen particles of |q_i - q_exact(x_i, t)|.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, Tuple

import numpy as np


@dataclass(frozen=True)
class RiemannState:
    rho: float
    u: float
    p: float


@dataclass(frozen=True)
class StarRegion:
    p: float      # star pressure
    u: float      # star (contact) velocity
    rho_L: float  # density left of the contact
    rho_R: float  # density right of the contact


def _sound(s: RiemannState, gamma: float) -> float:
    return float(np.sqrt(gamma * s.p / s.rho))


def _pressure_branch(p: float, s: RiemannState, gamma: float) -> Tuple[float, float]:
    """f_K(p) and its derivative (Toro 2009, eqs. 4.6-4.7 and 4.37)."""
    c = _sound(s, gamma)
    if p > s.p:  # shock: Rankine-Hugoniot
        A = 2.0 / ((gamma + 1.0) * s.rho)
        B = (gamma - 1.0) / (gamma + 1.0) * s.p
        q = np.sqrt(A / (p + B))
        return (p - s.p) * q, q * (1.0 - 0.5 * (p - s.p) / (B + p))
    # rarefaction: isentrope
    e = (gamma - 1.0) / (2.0 * gamma)
    r = p / s.p
    return 2.0 * c / (gamma - 1.0) * (r ** e - 1.0), r ** (-(gamma + 1.0) / (2.0 * gamma)) / (s.rho * c)


def star_region(L: RiemannState, R: RiemannState, gamma: float, tol: float = 1e-14,
                max_iter: int = 100) -> StarRegion:
    """Star-region pressure and velocity (Toro 2009, section 4.3.1), and the
    densities on either side of the contact (eqs. 4.50, 4.53, 4.57, 4.60)."""
    cL, cR = _sound(L, gamma), _sound(R, gamma)
    if 2.0 * (cL + cR) / (gamma - 1.0) <= R.u - L.u:
        raise ValueError("the initial states generate vacuum")
    # primitive-variable (linearised) guess, clipped positive
    p = max(0.5 * (L.p + R.p) - 0.125 * (R.u - L.u) * (L.rho + R.rho) * (cL + cR), 1e-12 * max(L.p, R.p))
    for _ in range(max_iter):
        fL, dL = _pressure_branch(p, L, gamma)
        fR, dR = _pressure_branch(p, R, gamma)
        p_new = max(p - (fL + fR + R.u - L.u) / (dL + dR), 1e-12 * max(L.p, R.p))
        change = abs(p_new - p) / (0.5 * (p_new + p))
        p = p_new
        if change < tol:
            break
    else:
        raise RuntimeError("Newton iteration for the star pressure did not converge")
    fL, _ = _pressure_branch(p, L, gamma)
    fR, _ = _pressure_branch(p, R, gamma)
    u = 0.5 * (L.u + R.u) + 0.5 * (fR - fL)
    g1 = (gamma - 1.0) / (gamma + 1.0)

    def rho_star(s: RiemannState) -> float:
        r = p / s.p
        if p > s.p:
            return s.rho * (r + g1) / (g1 * r + 1.0)
        return s.rho * r ** (1.0 / gamma)

    return StarRegion(p=p, u=u, rho_L=rho_star(L), rho_R=rho_star(R))


@dataclass(frozen=True)
class SodWaves:
    """Wave speeds of a problem whose left wave is a rarefaction and right
    wave a shock (the Sod family): positions are x0 + speed * t."""
    head: float     # rarefaction head
    tail: float     # rarefaction tail
    contact: float
    shock: float
    star: StarRegion


def sod_waves(L: RiemannState, R: RiemannState, gamma: float) -> SodWaves:
    """Speeds of the four wave fronts (Toro 2009, eqs. 4.55, 4.58 and 4.59)."""
    st = star_region(L, R, gamma)
    if not (st.p <= L.p and st.p > R.p):
        raise ValueError("not a left-rarefaction / right-shock problem")
    cL, cR = _sound(L, gamma), _sound(R, gamma)
    c_star = cL * (st.p / L.p) ** ((gamma - 1) / (2 * gamma))
    shock = R.u + cR * np.sqrt((gamma + 1) / (2 * gamma) * st.p / R.p + (gamma - 1) / (2 * gamma))
    return SodWaves(head=L.u - cL, tail=st.u - c_star, contact=st.u, shock=float(shock), star=st)


def euler_riemann(x: np.ndarray, t: float, L: RiemannState, R: RiemannState, gamma: float,
                  x0: float = 0.0) -> Dict[str, np.ndarray]:
    """The exact solution at positions x and time t > 0 for the discontinuity
    initially at x0 (Toro 2009, section 4.5, sampling in x / t).  Returns
    rho, u, p as arrays shaped like x."""
    x = np.asarray(x, dtype=np.float64)
    if t <= 0:
        raise ValueError("t must be positive")
    st = star_region(L, R, gamma)
    S = (x - x0) / t
    rho = np.empty_like(x)
    u = np.empty_like(x)
    p = np.empty_like(x)
    g = gamma
    for side, K, sgn, rho_star in ((0, L, 1.0, st.rho_L), (1, R, -1.0, st.rho_R)):
        # sgn = +1 for the left wave family (speeds measured to the left), -1 for the right
        c = _sound(K, g)
        mask = (S <= st.u) if side == 0 else (S > st.u)
        Sm = S[mask]
        r = np.empty_like(Sm)
        v = np.empty_like(Sm)
        q = np.empty_like(Sm)
        if st.p > K.p:  # shock
            speed = K.u - sgn * c * np.sqrt((g + 1) / (2 * g) * st.p / K.p + (g - 1) / (2 * g))
            outside = (Sm <= speed) if side == 0 else (Sm >= speed)
            r[:] = rho_star
            v[:] = st.u
            q[:] = st.p
            r[outside], v[outside], q[outside] = K.rho, K.u, K.p
        else:  # rarefaction
            head = K.u - sgn * c
            c_star = c * (st.p / K.p) ** ((g - 1) / (2 * g))
            tail = st.u - sgn * c_star
            if side == 0:
                outside, star = Sm <= head, Sm >= tail
            else:
                outside, star = Sm >= head, Sm <= tail
            fan = ~(outside | star)
            r[outside], v[outside], q[outside] = K.rho, K.u, K.p
            r[star], v[star], q[star] = rho_star, st.u, st.p
            # inside the fan (Toro eqs. 4.56 / 4.63)
            a = 2.0 / (g + 1) + sgn * (g - 1) / ((g + 1) * c) * (K.u - Sm[fan])
            r[fan] = K.rho * a ** (2.0 / (g - 1))
            v[fan] = 2.0 / (g + 1) * (sgn * c + (g - 1) / 2 * K.u + Sm[fan])
            q[fan] = K.p * a ** (2.0 * g / (g - 1))
        rho[mask], u[mask], p[mask] = r, v, q
    return {"rho": rho, "u": u, "p": p}


def sod_gas(x: np.ndarray, t: float, rho_L: float = 1.0, p_L: float = 1.0, rho_R: float = 0.125,
            p_R: float = 0.1, gamma: float = 1.4, x0: float = 0.0) -> Dict[str, np.ndarray]:
    """The gas of the dusty tube with eps -> 0: the classical Sod problem."""
    return euler_riemann(x, t, RiemannState(rho_L, 0.0, p_L), RiemannState(rho_R, 0.0, p_R), gamma, x0)


def dusty_sod_coupled(x: np.ndarray, t: float, eps: float, rho_L: float = 1.0, p_L: float = 1.0,
                      rho_R: float = 0.125, p_R: float = 0.1, gamma: float = 1.4,
                      x0: float = 0.0) -> Dict[str, np.ndarray]:
    """The dusty tube with t_s -> 0 and uniform dust-to-gas ratio eps: the
    mixture (density (1 + eps) rho_g, gas pressure, same gamma) solved as one
    ideal gas.  Returns the gas density rho, the common velocity u (gas and
    dust) and the pressure p."""
    f = 1.0 + eps
    sol = euler_riemann(x, t, RiemannState(f * rho_L, 0.0, p_L), RiemannState(f * rho_R, 0.0, p_R), gamma, x0)
    sol["rho"] = sol["rho"] / f
    return sol


def dusty_sod_coupled_waves(eps: float, rho_L: float = 1.0, p_L: float = 1.0, rho_R: float = 0.125,
                            p_R: float = 0.1, gamma: float = 1.4) -> SodWaves:
    """Wave speeds of the perfectly coupled mixture (star densities are the
    mixture's; divide by 1 + eps for the gas)."""
    f = 1.0 + eps
    return sod_waves(RiemannState(f * rho_L, 0.0, p_L), RiemannState(f * rho_R, 0.0, p_R), gamma)


def l1_against_exact(x: np.ndarray, q: np.ndarray, q_exact: np.ndarray, mask: np.ndarray = None) -> float:
    """Mean of |q_i - q_exact_i| over the particles in mask (all by default)."""
    x = np.asarray(x)
    if mask is None:
        mask = np.ones(x.shape, bool)
    return float(np.mean(np.abs(np.asarray(q)[mask] - np.asarray(q_exact)[mask])))


def score_dusty_sod(gas, dust, t: float, eps: float, limit: str, x_window: float = 0.4,
                    gamma: float = 1.4, rho_L: float = 1.0, p_L: float = 1.0, rho_R: float = 0.125,
                    p_R: float = 0.1, x0: float = 0.0) -> Dict[str, float]:
    """Scores one tube against the exact solution of a limit.

    gas, dust: objects with x, vx arrays (gas also rho, p, ind); limit "gas"
    (eps -> 0: Sod on the gas states) or "coupled" (t_s -> 0: the mixture).
    Particles with |x - x0| < x_window that are not frozen (ind == 0) count.

    Returns the L1 errors (mean |q - q_exact| per particle) of the gas density,
    gas and dust velocity and pressure; the shock position error (where the
    gas density, averaged over bins 0.01 wide, last crosses midway between the post- and pre-shock densities,
    minus the exact position); the relative errors of the mean gas density,
    velocity and pressure over the middle 40 % of the post-shock plateau
    between contact and shock; and the L1 of the gas velocity over the fan's
    leading part (10 % to 35 % of the way from its head to its tail).
    """
    if limit == "gas":
        f = 1.0
    elif limit == "coupled":
        f = 1.0 + eps
    else:
        raise ValueError("limit is 'gas' or 'coupled'")
    Ls, Rs = RiemannState(f * rho_L, 0.0, p_L), RiemannState(f * rho_R, 0.0, p_R)
    w = sod_waves(Ls, Rs, gamma)

    def exact(x):
        s = euler_riemann(x, t, Ls, Rs, gamma, x0)
        s["rho"] = s["rho"] / f
        return s

    xg = np.asarray(gas.x)
    free = np.asarray(gas.ind) == 0 if getattr(gas, "ind", None) is not None else np.ones(xg.shape, bool)
    mg = free & (np.abs(xg - x0) < x_window)
    xd = np.asarray(dust.x)
    dfree = np.asarray(dust.ind) == 0 if getattr(dust, "ind", None) is not None else np.ones(xd.shape, bool)
    md = dfree & (np.abs(xd - x0) < x_window)
    eg, ed = exact(xg), exact(xd)
    out = {
        "l1_rho_gas": l1_against_exact(xg, gas.rho, eg["rho"], mg),
        "l1_v_gas": l1_against_exact(xg, gas.vx, eg["u"], mg),
        "l1_v_dust": l1_against_exact(xd, dust.vx, ed["u"], md),
        "l1_p_gas": l1_against_exact(xg, gas.p, eg["p"], mg),
    }
    # shock position from the binned gas density
    rho_post = w.star.rho_R / f
    mid = 0.5 * (rho_post + rho_R)
    edges = np.arange(x0 + w.contact * t, x0 + x_window + 1e-12, 0.01)
    idx = np.digitize(xg[mg], edges)
    crossing = np.nan
    for b in range(len(edges) - 1, 0, -1):
        sel = idx == b
        if sel.any() and np.mean(np.asarray(gas.rho)[mg][sel]) > mid:
            crossing = 0.5 * (edges[b - 1] + edges[b])
            break
    out["shock_dx"] = float(crossing - (x0 + w.shock * t))
    # post-shock plateau means
    a = x0 + t * (w.contact + 0.3 * (w.shock - w.contact))
    b = x0 + t * (w.shock - 0.3 * (w.shock - w.contact))
    sel = mg & (xg > a) & (xg < b)
    out["plateau_rho_rel"] = float(np.mean(np.asarray(gas.rho)[sel]) / rho_post - 1.0)
    out["plateau_v_rel"] = float(np.mean(np.asarray(gas.vx)[sel]) / w.star.u - 1.0)
    out["plateau_p_rel"] = float(np.mean(np.asarray(gas.p)[sel]) / w.star.p - 1.0)
    # leading part of the fan
    a = x0 + t * (w.head + 0.10 * (w.tail - w.head))
    b = x0 + t * (w.head + 0.35 * (w.tail - w.head))
    sel = mg & (xg > a) & (xg < b)
    out["fan_l1_v_gas"] = l1_against_exact(xg, gas.vx, eg["u"], sel)
    return out
