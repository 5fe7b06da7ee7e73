"""The benchmark physics pinned to exact solutions.

The dusty Sod tube of 45,000 + 45,000 particles (left spacing 1/200, right
1/100, cross-section 0.1 x 0.1, periodic in y and z, h = 1.3 local spacing,
CFL 0.3, IDIC cells of 2 right spacings), run to t = 0.2 on the FP64 path, on
the FP32 path and on the oracle, and scored against the two limits that have a
closed-form answer (dustyshock3d_gb300/riemann.py, Toro's exact Riemann
solver):

* eps -> 0 (eps = 1e-6): the gas is the classical Sod problem;
* t_s -> 0 (t_s = 1e-4, eps = 1): gas and dust move as one ideal gas of
  density (1 + eps) rho_g, sound speed c_s / sqrt(1 + eps).

The scores (per-particle L1 of the gas density, gas and dust velocity and
pressure over |x| < 0.4; shock position; post-shock plateau means; the fan's
leading part) measure the scheme, not the arithmetic: the reference's SPH
(its force and energy sums, IDIC.h:183-260) on a lattice with a density jump
of 8 leaves a spurious plateau at the rarefaction's tail, and its gas relaxation
to the cell's dust solution (IDIC.h:287-315) diffuses momentum across IDIC
cells when dt >> t_s.  The bounds are those of the FP64 path with a stated
margin.  The FP32 path must score within a stated factor of the FP64 path:
its error against the physics is the FP64 path's, although FP32 and FP64 runs
differ from each other at t = 0.2 (the scheme amplifies rounding-level
differences once the shock has formed).

The FP32 path keeps an FP64 state of record; a third run rounds its
integrated state (positions, velocities, internal energy) to FP32 after every
step, as an FP32 state of record would hold it, and must score within the
same factor of the FP64 path (measured: gas_sod L1 rho 0.0345 against 0.0356,
coupled 0.0596 against 0.0599).

Conservation over the run: the mass is fixed; the x momentum of all species
grows as the frozen end walls push with p_L and p_R, (p_L - p_R) A t exactly
for the exact solution; the total energy (gas internal + kinetic of all
species) stays constant in the exact solution and drifts here only by the
scheme's dissipation.
"""
import numpy as np
import pytest

from dustyshock3d_gb300 import ic, riemann
from dustyshock3d_gb300.solver import Solver
from oracle.oracle import OracleState

pytestmark = pytest.mark.gpu

CASES = {
    # name: (eps, t_s, limit)
    "gas_sod": (1e-6, 1e-3, "gas"),
    "coupled": (1.0, 1e-4, "coupled"),
}

# Bounds on the FP64 path (= the oracle): its measured scores with a margin of
# about 25 % (measured: gas_sod L1 rho 0.0356, v 0.0644, v_dust 0.0610, p 0.0398,
# shock -0.010, plateau -2.2 %, -2.2 %, -2.4 %, fan 0.088; coupled L1 rho 0.0599,
# v 0.0674, v_dust 0.0676, p 0.0729, shock -0.052, plateau -17 %, -25 %, -26 %,
# fan 0.037).
BOUNDS = {
    "gas_sod": dict(l1_rho_gas=0.045, l1_v_gas=0.080, l1_v_dust=0.077, l1_p_gas=0.050, shock_dx=0.02,
                    plateau=0.035, fan_l1_v_gas=0.11),
    "coupled": dict(l1_rho_gas=0.075, l1_v_gas=0.085, l1_v_dust=0.085, l1_p_gas=0.091, shock_dx=0.07,
                    plateau=0.32, fan_l1_v_gas=0.05),
}
# The FP32 path's L1 scores may exceed the FP64 path's by this factor (plus 1e-3).
# Measured: FP32 / FP64 = 0.986 to 1.000 on every score of both cases.
FP32_FACTOR = 1.05

_runs = {}


def _tube(name):
    eps, t_s, _ = CASES[name]
    return ic.dusty_sod_tube(dx_left=1 / 200, Ly=0.1, eps=eps, t_s=t_s)


def _totals(P, species):
    """mass, x momentum, gas internal energy, kinetic energy: FP64 sums."""
    g = species[0]
    M = sum(float(np.sum(s.m)) for s in species)
    px = sum(float(np.sum(s.m * s.vx)) for s in species)
    U = float(np.sum(g.m * g.e))
    K = sum(float(np.sum(0.5 * s.m * (s.vx ** 2 + s.vy ** 2 + s.vz ** 2))) for s in species)
    return np.array([M, px, U, K])


def _run(name, engine):
    key = (name, engine)
    if key in _runs:
        return _runs[key]
    P, sp = _tube(name)
    before = _totals(P, sp)
    if engine == "oracle":
        O = OracleState(P, sp)
        while O.Tm < P.T_end:
            O.step(20)
        out, Tm = O.species, O.Tm
    elif engine == "fp32_state":
        # the FP32 path with its integrated state (x, v and the gas's e) rounded
        # to FP32 after every step, as an FP32 state of record would keep it
        # (absolute coordinates: coarser than FP32 offsets from a cell origin)
        P.precision = "fp32"
        with Solver(P) as S:
            S.set_tube(0, sp)
            Tm = 0.0
            while Tm < P.T_end:
                S.step(1)
                Tm = S.time(0)[0]
                for s in range(2):
                    q = S.get_species(0, s)
                    for f in ("x", "y", "z", "vx", "vy", "vz") + (("e",) if s == 0 else ()):
                        setattr(q, f, getattr(q, f).astype(np.float32).astype(np.float64))
                    S.set_species(0, s, q)
            out = [S.get_species(0, s) for s in range(2)]
            assert S.device_flags() & ~0x4 == 0
    else:
        P.precision = engine
        with Solver(P) as S:
            S.set_tube(0, sp)
            Tm = 0.0
            while Tm < P.T_end:
                S.step(20)
                Tm = S.time(0)[0]
            out = [S.get_species(0, s) for s in range(2)]
            assert S.device_flags() & ~0x4 == 0
    eps, _, limit = CASES[name]
    scores = riemann.score_dusty_sod(out[0], out[1], Tm, eps, limit)
    A = (P.Y_max - P.Y_min) * (P.Z_max - P.Z_min)
    res = dict(species=out, Tm=Tm, scores=scores, before=before, after=_totals(P, out), area=A)
    _runs[key] = res
    print(f"{name} {engine}: t={Tm:.6f} " + " ".join(f"{k}={v:.4f}" for k, v in scores.items()))
    return res


def _check_bounds(name, s, ref=None):
    b = BOUNDS[name]
    for k in ("l1_rho_gas", "l1_v_gas", "l1_v_dust", "l1_p_gas"):
        lim = b[k] if ref is None else FP32_FACTOR * ref[k] + 1e-3
        assert s[k] <= lim, f"{name}: {k} = {s[k]:.4f} > {lim:.4f}"
    assert abs(s["shock_dx"]) <= b["shock_dx"], f"{name}: shock off by {s['shock_dx']:.4f}"
    for k in ("plateau_rho_rel", "plateau_v_rel", "plateau_p_rel"):
        assert abs(s[k]) <= b["plateau"], f"{name}: {k} = {s[k]:.3f}"
    assert s["fan_l1_v_gas"] <= b["fan_l1_v_gas"], f"{name}: fan L1 {s['fan_l1_v_gas']:.4f}"


@pytest.mark.parametrize("name", list(CASES))
def test_fp64_path_against_the_exact_solution(name):
    _check_bounds(name, _run(name, "fp64")["scores"])


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_is_the_fp64_path_to_t_end(name):
    """The oracle runs the same 150-220 steps: same clock, same particles, so
    its scores are the FP64 path's."""
    a, o = _run(name, "fp64"), _run(name, "oracle")
    assert a["Tm"] == o["Tm"]
    for s in range(2):
        for f in ("x", "vx", "rho"):
            x, y = getattr(a["species"][s], f), getattr(o["species"][s], f)
            assert np.max(np.abs(x - y)) <= 1e-9 * max(1.0, float(np.max(np.abs(y)))), (name, s, f)
    _check_bounds(name, o["scores"])


@pytest.mark.parametrize("name", list(CASES))
def test_fp32_path_scores_like_the_fp64_path(name):
    r32, r64 = _run(name, "fp32"), _run(name, "fp64")
    _check_bounds(name, r32["scores"], ref=r64["scores"])


@pytest.mark.parametrize("name", list(CASES))
def test_fp32_state_of_record_scores_like_the_fp64_path(name):
    """Whether the FP32 path needs its FP64 state of record: the same run with
    the integrated state rounded to FP32 after every step scores against the
    exact solution as the FP64 path does (same bounds as the FP32 path)."""
    r, r64 = _run(name, "fp32_state"), _run(name, "fp64")
    _check_bounds(name, r["scores"], ref=r64["scores"])


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("engine", ["fp64", "fp32", "fp32_state"])
def test_conservation_over_the_run(name, engine):
    r = _run(name, engine)
    M0, px0, U0, K0 = r["before"]
    M1, px1, U1, K1 = r["after"]
    assert M1 == M0
    expected_px = (1.0 - 0.1) * r["area"] * r["Tm"]
    assert abs(px1 - expected_px) <= 0.01 * expected_px, (px1, expected_px)  # measured -0.38 %
    # total energy: conserved by the exact solution; the scheme's own loss here
    rel = (U1 + K1) / (U0 + K0) - 1.0
    assert abs(rel) <= ENERGY_DRIFT[name], f"{name} {engine}: energy drift {rel:.2e}"


# measured on the FP64 path: +4.1e-3 (gas_sod), -4.6e-3 (coupled)
ENERGY_DRIFT = {"gas_sod": 6e-3, "coupled": 7e-3}
