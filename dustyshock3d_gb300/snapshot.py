"""Snapshot files in the reference's text format (Data_out, kernel.cu:232-295;
Data_out_dust, kernel.cu:434-496 and 635-687): the files the reference writes
at each output time, byte for byte in its layout, so a host's post-processing
reads them unchanged.

Per output number `num` (7-digit zero-padded names, kernel.cu:242-248):
  Data/G{num}.dat        every gas particle: x y z r mas rho p Vx Vy Vy V e Ind Nn
  Data/L_X{num}.dat      gas with y^2 + z^2 <= h^2: ... Vx Vy Vy V Ax Ay Az e Ind
  Data/D-k-{num}.dat     every dust-k particle: x y z r mas rho t_stop Vx Vy Vy V Ind Nn
  Data/D-k-L_X{num}.dat  dust-k with y^2 + z^2 <= h^2: ... Vx Vy Vy V Ax Ay Az t_stop Ind
for the first two dust species (the reference writes D-1 and D-2).  The
reference prints Vy where a Vz column is announced (kernel.cu:262) and labels
the dust line files' t_stop column "Ind"; both are kept, so that files written
here and there are interchangeable.  Dust accelerations are not state of the
step: the reference prints its host arrays, which it never fills; here they
are zero.
"""
from __future__ import annotations

import math
import os
from typing import Optional, Sequence

import numpy as np

from .species import Species

_F = "%10.8f"


def _name(directory: str, stem: str, num: int) -> str:
    return os.path.join(directory, f"{stem}{num:07d}.dat")


def _header(Tm: float, tau: float, h: float, columns: str) -> str:
    return f"t={Tm:5.3f} \ntau={tau:10.8f} \t h={h:10.8f} \n{columns}\n"


def _row(values, ints) -> str:
    return " \t ".join([_F % v for v in values] + ["%d" % k for k in ints]) + " \n"


def _r_v(q: Species, i: int):
    r = math.sqrt(q.x[i] * q.x[i] + q.y[i] * q.y[i] + q.z[i] * q.z[i])
    v = math.sqrt(q.vx[i] * q.vx[i] + q.vy[i] * q.vy[i] + q.vz[i] * q.vz[i])
    return r, v


def write(directory: str, num: int, Tm: float, tau: float, h: float, species: Sequence[Species],
          nexts: Optional[Sequence[np.ndarray]] = None) -> list:
    """Write the snapshot files of one output time; returns their paths.
    species[0] is the gas, species[1:] the dust; nexts[s] the Nn column of
    species s (the cell lists' next pointers; zeros when absent)."""
    os.makedirs(directory, exist_ok=True)
    paths = []
    eps2 = (1.0 * h) * (1.0 * h)
    g = species[0]
    nn = nexts[0] if nexts is not None else np.zeros(g.n, np.int32)
    with open(_name(directory, "G", num), "w") as f:
        f.write(_header(Tm, tau, h, "x \t y \t z \t r \t mas \t rho \t p \t Vx \t Vy \t Vz \t V \t e \t Ind "))
        for i in range(g.n):
            r, v = _r_v(g, i)
            f.write(_row((g.x[i], g.y[i], g.z[i], r, g.m[i], g.rho[i], g.p[i], g.vx[i], g.vy[i], g.vy[i], v, g.e[i]),
                         (g.ind[i], nn[i])))
    paths.append(_name(directory, "G", num))
    with open(_name(directory, "L_X", num), "w") as f:
        f.write(_header(Tm, tau, h, "x \t y \t z \t r \t mas \t rho \t p \t Vx \t Vy \t Vz \t V \t Ax \t Ay \t Az "
                                    "\t e \t Ind "))
        for i in range(g.n):
            if g.y[i] * g.y[i] + g.z[i] * g.z[i] <= eps2:
                r, v = _r_v(g, i)
                f.write(_row((g.x[i], g.y[i], g.z[i], r, g.m[i], g.rho[i], g.p[i], g.vx[i], g.vy[i], g.vy[i], v,
                              g.ax[i], g.ay[i], g.az[i], g.e[i]), (g.ind[i],)))
    paths.append(_name(directory, "L_X", num))
    for k in range(1, min(len(species), 3)):
        d = species[k]
        nn = nexts[k] if nexts is not None else np.zeros(d.n, np.int32)
        with open(_name(directory, f"D-{k}-", num), "w") as f:
            f.write(_header(Tm, tau, h, "x \t y \t z \t r \t mas \t rho \t t_stop \t Vx \t Vy \t Vz \t V \t Ind "
                                        "\t Nn "))
            for i in range(d.n):
                r, v = _r_v(d, i)
                f.write(_row((d.x[i], d.y[i], d.z[i], r, d.m[i], d.rho[i], d.ts[i], d.vx[i], d.vy[i], d.vy[i], v),
                             (d.ind[i], nn[i])))
        paths.append(_name(directory, f"D-{k}-", num))
        with open(_name(directory, f"D-{k}-L_X", num), "w") as f:
            f.write(_header(Tm, tau, h, "x \t y \t z \t r \t mas \t rho \t Vx \t Vy \t Vz \t V \t Ax \t Ay \t Az "
                                        "\t Ind "))
            for i in range(d.n):
                if d.y[i] * d.y[i] + d.z[i] * d.z[i] <= eps2:
                    r, v = _r_v(d, i)
                    f.write(_row((d.x[i], d.y[i], d.z[i], r, d.m[i], d.rho[i], d.vx[i], d.vy[i], d.vy[i], v,
                                  0.0, 0.0, 0.0, d.ts[i]), (d.ind[i],)))
        paths.append(_name(directory, f"D-{k}-L_X", num))
    return paths
