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


def test_idic_conserves_cell_momentum():
    """Without Psi the drag only exchanges momentum: v_g + sum eps_k v_k is kept."""
    eps, t = [0.7, 2.0, 0.1], [1e-3, 3e-2, 1e-4]
    vg, vd = 0.5, [0.1, -0.4, 0.9]
    g, d = orc.solve_cell(eps, t, vg, vd, 0.0, 5e-4)
    assert g + np.dot(eps, d) == pytest.approx(vg + np.dot(eps, vd), rel=1e-12)
