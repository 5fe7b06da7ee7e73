"""Known-answer tests of the oracle's building blocks, from mathematics."""
import math

import numpy as np
import pytest

from oracle import oracle as orc

PI_REF = 3.14159265  # the reference's truncated constant (kernel.cu:14)


def test_W_normalisation():
    """The M4 spline with 1/(pi h^3) integrates to 1; the reference's truncated
    pi makes it 1 + O(4e-9)."""
    L = orc.lib()
    h = 0.37
    r = np.linspace(0.0, 2.0 * h, 200001)
    w = np.array([L.orc_kernel_W(float(x), h) for x in r[::50]])
    integral = np.trapezoid(4 * np.pi * r[::50] ** 2 * w, r[::50])
    assert abs(integral - math.pi / PI_REF) < 1e-6


def test_dW_is_derivative_of_W():
    L = orc.lib()
    h = 0.21
    for r in np.linspace(0.01 * h, 1.99 * h, 37):
        d = 1e-7 * h
        fd = (L.orc_kernel_W(r + d, h) - L.orc_kernel_W(r - d, h)) / (2 * d)
        assert abs(L.orc_kernel_dW(r, h) - fd) < 1e-5 * abs(L.orc_kernel_W(0.0, h)) / h


@pytest.mark.parametrize("eps,t,tau", [(1.0, 1e-3, 4e-4), (0.01, 0.1, 4e-4), (10.0, 1e-4, 1e-3)])
def test_idic_one_species_closed_form(eps, t, tau):
    """N = 1: x_new = (x + tau Psi)/(1 + tau (1 + eps)/t_s); v_g = (y_new + eps x_new)/(1+eps)."""
    vg, vd, psi = 0.3, -0.2, 1.7
    g, d = orc.solve_cell([eps], [t], vg, [vd], psi, tau)
    x = vg - vd
    y = vg + eps * vd
    xn = (x + tau * psi) / (1 + tau * (1 + eps) / t)
    yn = y + tau * psi
    assert g == pytest.approx((yn + eps * xn) / (1 + eps), rel=1e-12)
    assert d[0] == pytest.approx((yn - xn) / (1 + eps), rel=1e-12)


def test_idic_two_species_reference_order_equals_sherman_morrison():
    rng = np.random.default_rng(3)
    for _ in range(200):
        eps = rng.uniform(0.01, 5, 2)
        t = 10 ** rng.uniform(-4, 0, 2)
        vg, psi, tau = rng.normal(), rng.normal(), 10 ** rng.uniform(-4, -2)
        vd = rng.normal(size=2)
        g1, d1 = orc.solve_cell(eps, t, vg, vd, psi, tau, ref2=True)
        g2, d2 = orc.solve_cell(eps, t, vg, vd, psi, tau, ref2=False)
        assert g1 == pytest.approx(g2, rel=1e-9, abs=1e-12)
        assert np.allclose(d1, d2, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_idic_solve_equals_the_implicit_system(n):
    """The per-cell solve is the implicit drag step of every species at once:
    v_g' = v_g + tau Psi - tau sum_k eps_k (v_g' - v_k') / t_k and
    v_k' = v_k + tau (v_g' - v_k') / t_k, solved here directly as an
    (N+1) x (N+1) linear system for random cells."""
    rng = np.random.default_rng(100 + n)
    for _ in range(200):
        eps = rng.uniform(0.01, 5, n)
        t = 10 ** rng.uniform(-4, 0, n)
        vg, psi, tau = rng.normal(), rng.normal(), 10 ** rng.uniform(-4, -2)
        vd = rng.normal(size=n)
        A = np.zeros((n + 1, n + 1))
        b = np.zeros(n + 1)
        A[0, 0] = 1 + tau * np.sum(eps / t)
        A[0, 1:] = -tau * eps / t
        b[0] = vg + tau * psi
        for k in range(n):
            A[k + 1, 0] = -tau / t[k]
            A[k + 1, k + 1] = 1 + tau / t[k]
            b[k + 1] = vd[k]
        x = np.linalg.solve(A, b)
        g, d = orc.solve_cell(eps, t, vg, vd, psi, tau)
        scale = np.abs(x).max()
        assert abs(g - x[0]) <= 1e-12 * scale
        assert np.abs(np.asarray(d) - x[1:]).max() <= 1e-12 * scale


def test_idic_conserves_cell_momentum():
    """Without Psi the drag only exchanges momentum: v_g + sum eps_k v_k is kept."""
    eps, t = [0.7, 2.0, 0.1], [1e-3, 3e-2, 1e-4]
    vg, vd = 0.5, [0.1, -0.4, 0.9]
    g, d = orc.solve_cell(eps, t, vg, vd, 0.0, 5e-4)
    assert g + np.dot(eps, d) == pytest.approx(vg + np.dot(eps, vd), rel=1e-12)


def test_step_flags_a_cutoff_past_the_stencil():
    """Proper grid, stencil 2 over cells of 1.001 h_max: an h just inside the
    reach (stencil x cell width / 2) raises nothing, one past it raises flag 8
    (the library's DS_FLAG_REACH); the reference grid raises it for no h."""
    from dustyshock3d_gb300 import ic
    from tests import _golden
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25))
    assert P.stencil == 2
    q = int(np.nonzero(sp[0].ind == 0)[0][0])
    for factor, want in ((0.999, 0), (1.05, 8)):
        g = sp[0].copy().fill_missing()
        g.h[q] = factor * P.cell_w
        O = orc.OracleState(P, [g, sp[1].copy().fill_missing()]).step(1)
        assert O.last_status & 8 == want, factor
    _, R, rsp = _golden.setup("refB")
    g = rsp[0].copy().fill_missing()
    g.h[:] = 3.0 * R.h
    O = orc.OracleState(R, [g] + [d.copy().fill_missing() for d in rsp[1:]]).step(1)
    assert O.last_status & 8 == 0


def test_split_species_moves_the_gas_as_one():
    """Three dust species on the same sites with one stopping time and mass
    ratios summing to 1 drag the gas as one species of ratio 1 does: with
    equal t_k the implicit solve sees the species only through sum_k eps_k."""
    from tests._multidust import multi_dust_tube
    P1, sp1 = multi_dust_tube((1.0,), (2e-3,), shift=False)
    P3, sp3 = multi_dust_tube((0.2, 0.3, 0.5), (2e-3,) * 3, shift=False)
    A = orc.OracleState(P1, sp1).step(4)
    B = orc.OracleState(P3, sp3).step(4)
    for f in ("x", "vx", "rho", "e"):
        a, b = getattr(A.species[0], f), getattr(B.species[0], f)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max(), f
    for k in (1, 2, 3):
        assert np.abs(B.species[k].vx - A.species[1].vx).max() <= 1e-12 * np.abs(A.species[1].vx).max(), k


def test_cfl_step_is_the_smallest_signal_crossing_time():
    """CFL step (extension; the reference steps by a fixed tau): tau = cfl x
    min over free gas particles of h_i / (c_i + |v_i|), with c from the step's
    own density and pressure and v from the step's start, clamped to T_end."""
    from dustyshock3d_gb300 import ic
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25))
    assert P.mode.cfl
    g0 = sp[0].copy().fill_missing()
    rng = np.random.default_rng(5)
    g0.vx = rng.normal(scale=0.3, size=g0.n)  # velocities that matter against c
    species = [g0, sp[1].copy().fill_missing()]
    O = orc.OracleState(P, species).step(1)
    g1 = O.species[0]
    free = g0.ind == 0
    c = np.sqrt(P.Gam_g * g1.p[free] / g1.rho[free])
    v = np.sqrt(g0.vx[free] ** 2 + g0.vy[free] ** 2 + g0.vz[free] ** 2)
    want = P.cfl * np.min(g0.h[free] / (c + v))
    assert O.last_dt == pytest.approx(want, rel=1e-14)
    assert O.Tm == O.last_dt
    P2 = P.copy()
    P2.T_end = 0.5 * want  # the first step stops at T_end
    O2 = orc.OracleState(P2, species).step(1)
    assert O2.last_dt == P2.T_end and O2.Tm == P2.T_end
