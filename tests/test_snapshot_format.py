"""The snapshot writer's rows and headers are what C's printf makes of the
reference's format strings (kernel.cu:250-265, 452-467; no GPU needed)."""
import ctypes
import ctypes.util

import numpy as np

from dustyshock3d_gb300 import snapshot
from dustyshock3d_gb300.species import Species


def _c(fmt, *args):
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    buf = ctypes.create_string_buffer(4096)
    cargs = [ctypes.c_double(a) if isinstance(a, float) else ctypes.c_int(a) for a in args]
    libc.snprintf(buf, 4096, fmt.encode(), *cargs)
    return buf.value.decode()


def test_rows_and_headers_match_printf(tmp_path):
    rng = np.random.default_rng(3)
    n = 40
    vals = lambda: rng.normal(0, 3, n) * 10.0 ** rng.integers(-9, 4, n)  # noqa: E731
    g = Species(x=vals(), y=rng.uniform(-1, 1, n), z=rng.uniform(-1, 1, n), vx=vals(), vy=vals(), vz=vals(),
                ax=vals(), ay=vals(), az=vals(), rho=np.abs(vals()), p=np.abs(vals()), e=np.abs(vals()),
                m=np.abs(vals()), h=np.full(n, 0.2), ts=np.zeros(n), ind=rng.integers(0, 2, n).astype(np.int32))
    d = Species(**{f: getattr(g, f).copy() for f in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho",
                                                      "p", "e", "m", "h", "ind")}, ts=np.abs(vals()))
    nn = rng.integers(-1, n, n).astype(np.int32)
    snapshot.write(str(tmp_path), 3, 0.0123456, 5e-3, 0.2, [g, d, d], [nn, nn, nn])
    G = open(tmp_path / "G0000003.dat").read().splitlines(True)
    assert G[0] == _c("t=%5.3f \n", 0.0123456)
    assert G[1] == _c("tau=%10.8lf \t h=%10.8lf \n", 5e-3, 0.2)
    assert G[2] == "x \t y \t z \t r \t mas \t rho \t p \t Vx \t Vy \t Vz \t V \t e \t Ind \n"
    fmt = " \t ".join(["%10.8lf"] * 12 + ["%d", "%d"]) + " \n"
    for i in range(n):
        r = float(np.sqrt(g.x[i] ** 2 + g.y[i] ** 2 + g.z[i] ** 2))
        v = float(np.sqrt(g.vx[i] ** 2 + g.vy[i] ** 2 + g.vz[i] ** 2))
        want = _c(fmt, float(g.x[i]), float(g.y[i]), float(g.z[i]), r, float(g.m[i]), float(g.rho[i]),
                  float(g.p[i]), float(g.vx[i]), float(g.vy[i]), float(g.vy[i]), v, float(g.e[i]), int(g.ind[i]),
                  int(nn[i]))
        assert G[3 + i] == want
    D = open(tmp_path / "D-2-0000003.dat").read().splitlines(True)
    assert D[2] == "x \t y \t z \t r \t mas \t rho \t t_stop \t Vx \t Vy \t Vz \t V \t Ind \t Nn \n"
    L = open(tmp_path / "L_X0000003.dat").read().splitlines(True)
    inside = [i for i in range(n) if g.y[i] ** 2 + g.z[i] ** 2 <= 0.2 * 0.2]
    assert len(L) == 3 + len(inside)
