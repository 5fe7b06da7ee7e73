"""The exact Riemann solver (dustyshock3d_gb300/riemann.py) checked from the
mathematics: the star state is a root of the pressure function, the jumps obey
the Rankine-Hugoniot conditions, the fan keeps its Riemann invariant and
entropy, the sampled solution conserves mass, momentum and energy over the
tube, and the coupled dusty limit is the Euler solution of the mixture."""
import numpy as np
import pytest

from dustyshock3d_gb300 import riemann as R

G = 1.4
L0 = R.RiemannState(1.0, 0.0, 1.0)
R0 = R.RiemannState(0.125, 0.0, 0.1)


def test_sod_star_state():
    st = R.star_region(L0, R0, G)
    # the classical value of Sod's problem
    assert st.p == pytest.approx(0.30313, abs=5e-6)
    assert st.u == pytest.approx(0.92745, abs=5e-6)
    # root of f_L(p) + f_R(p) + u_R - u_L
    fL, _ = R._pressure_branch(st.p, L0, G)
    fR, _ = R._pressure_branch(st.p, R0, G)
    assert abs(fL + fR) < 1e-13


def test_shock_obeys_rankine_hugoniot():
    w = R.sod_waves(L0, R0, G)
    st = w.star
    S = w.shock
    # in the shock's frame: mass, momentum and energy fluxes equal on both sides
    def flux(rho, u, p):
        v = u - S
        E = p / (G - 1) + 0.5 * rho * v * v
        return np.array([rho * v, rho * v * v + p, v * (E + p)])

    a = flux(R0.rho, R0.u, R0.p)
    b = flux(st.rho_R, st.u, st.p)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-12)


def test_fan_keeps_riemann_invariant_and_entropy():
    w = R.sod_waves(L0, R0, G)
    t = 0.2
    x = np.linspace(w.head * t + 1e-6, w.tail * t - 1e-6, 101)
    s = R.sod_gas(x, t)
    c = np.sqrt(G * s["p"] / s["rho"])
    inv = s["u"] + 2 * c / (G - 1)
    assert np.allclose(inv, 2 * np.sqrt(G) / (G - 1), rtol=1e-12)
    assert np.allclose(s["p"] / s["rho"] ** G, 1.0, rtol=1e-12)
    # the fan is continuous with the star state and the left state
    assert s["u"][0] == pytest.approx(0.0, abs=1e-4) and s["u"][-1] == pytest.approx(w.star.u, rel=1e-4)


@pytest.mark.parametrize("eps", [0.0, 1.0, 10.0])
def test_exact_solution_conserves_mass_momentum_energy(eps):
    """Over [-0.5, 0.5] before any wave reaches an end, the walls push with p_L
    and p_R: mass and energy stay fixed and momentum grows at p_L - p_R."""
    t = 0.2
    x = np.linspace(-0.5, 0.5, 2_000_001)
    dx = x[1] - x[0]
    s = R.dusty_sod_coupled(x, t, eps)
    rho_mix = (1 + eps) * s["rho"]
    E = s["p"] / (G - 1) + 0.5 * rho_mix * s["u"] ** 2

    def integral(q):
        return float(np.sum(0.5 * (q[1:] + q[:-1])) * dx)

    assert integral(rho_mix) == pytest.approx(0.5 * (1 + eps) * (1 + 0.125), rel=1e-5)
    assert integral(rho_mix * s["u"]) == pytest.approx((1.0 - 0.1) * t, rel=1e-4)
    assert integral(E) == pytest.approx(0.5 * (1.0 + 0.1) / (G - 1), rel=1e-5)


def test_coupled_limit_is_the_mixture_problem():
    eps = 1.0
    x = np.linspace(-0.5, 0.5, 1001)
    a = R.dusty_sod_coupled(x, 0.2, eps)
    b = R.euler_riemann(x, 0.2, R.RiemannState(2.0, 0, 1.0), R.RiemannState(0.25, 0, 0.1), G)
    assert np.array_equal(a["rho"], b["rho"] / 2) and np.array_equal(a["u"], b["u"])
    # slower waves: sound speed c / sqrt(1 + eps)
    w0, w1 = R.sod_waves(L0, R0, G), R.dusty_sod_coupled_waves(eps)
    assert w1.head == pytest.approx(w0.head / np.sqrt(1 + eps), rel=1e-12)
    assert w1.star.p == pytest.approx(w0.star.p, rel=1e-12)  # same star pressure
    assert w1.star.u == pytest.approx(w0.star.u / np.sqrt(1 + eps), rel=1e-12)


def test_symmetric_collision_and_vacuum_guard():
    st = R.star_region(R.RiemannState(1, 1, 0.4), R.RiemannState(1, -1, 0.4), G)
    assert st.u == pytest.approx(0.0, abs=1e-14) and st.p > 0.4
    with pytest.raises(ValueError):
        R.star_region(R.RiemannState(1, -20, 0.4), R.RiemannState(1, 20, 0.4), G)
