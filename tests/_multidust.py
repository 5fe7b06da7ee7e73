"""Dusty Sod tubes with several dust species, for the GPU and oracle tests."""
import numpy as np

from dustyshock3d_gb300 import ic

EPS = (1.0, 0.5, 2.0, 0.1)
T_S = (1e-3, 1e-2, 3e-4, 1e-1)


def multi_dust_tube(eps, t_s, shift=True):
    """The small dusty Sod tube with one dust lattice per (eps_k, t_k),
    species k shifted by k/10 of a local spacing in y (periodic), or all on
    the same sites when shift is False."""
    P, (gas, dust) = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=t_s[0], x_range=(-0.25, 0.25))
    P = P.copy()
    n = len(eps)
    P.n_dust = n
    P.mass_ratio = list(eps)
    P.R_dust = [0.0] * n
    P.t_stop_const = list(t_s)
    P.eps_empty = list(eps)
    spacing = (dust.m / dust.rho) ** (1.0 / 3.0)  # local lattice spacing (mass / density = volume)
    out = [gas]
    for k in range(n):
        d = dust.copy().fill_missing()
        if shift:
            d.y = np.mod(d.y + 0.1 * k * spacing, P.Y_max - P.Y_min)
        d.m = dust.m * eps[k]
        d.rho = dust.rho * eps[k]
        d.ts = np.full(d.n, t_s[k])
        out.append(d)
    return P, out
