"""Several dust species (needs a GPU).  The reference runs two; the step takes
up to DS_MAX_DUST = 4, each with its own mass ratio and stopping time, coupled
to the gas through one implicit drag solve per IDIC cell (the general-N
Sherman-Morrison form of the reference's 2-species solve: cell eps at
kernel.cu:2196-2210, velocity updates in V_dustKernel_IDIC / V_gasKernel_IDIC,
IDIC.h:264-315).

  * the FP64 path equals the oracle bit for bit with 1..4 species;
  * the FP32 path tracks the oracle within the FP32 tolerance of the parity
    tests (gas rho relative L1 <= 1e-5, velocities <= 1e-4 of their scale);
  * splitting one species into three with the same stopping time and the same
    positions (mass ratios summing to the original) moves the gas as the one
    species does, up to rounding: the drag solve depends on the species only
    through sum_k eps_k / (t_k + tau) when the t_k agree."""
import numpy as np
import pytest

from oracle.oracle import OracleState
from tests._multidust import EPS, T_S, multi_dust_tube
from tests.test_gpu_parity import compare_exact, run_gpu

pytestmark = pytest.mark.gpu

@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_multi_species_fp64_bitexact(n):
    P, sp = multi_dust_tube(EPS[:n], T_S[:n])
    gpu, (Tm, dt, _) = run_gpu(P, sp, 6)
    O = OracleState(P, sp).step(6)
    assert Tm == O.Tm and dt == O.last_dt
    compare_exact(gpu, O.species, f"{n} dust species")
    # every species was dragged: its velocities are no longer all zero
    for k in range(1, n + 1):
        assert np.abs(gpu[k].vx).max() > 0.0, k


@pytest.mark.parametrize("n", [3, 4])
def test_multi_species_fp32_tracks_the_oracle(n):
    P, sp = multi_dust_tube(EPS[:n], T_S[:n])
    P32 = P.copy()
    P32.precision = "fp32"
    gpu, _ = run_gpu(P32, sp, 10)
    O = OracleState(P, sp).step(10)
    g, o = gpu[0], O.species[0]
    assert np.abs(g.rho - o.rho).sum() / np.abs(o.rho).sum() < 1e-5
    vscale = np.abs(o.vx).max()
    assert np.abs(g.vx - o.vx).mean() / vscale < 1e-4
    for k in range(1, n + 1):
        assert np.abs(gpu[k].vx - O.species[k].vx).mean() / vscale < 1e-4, k


def test_split_species_moves_the_gas_as_one():
    P1, sp1 = multi_dust_tube((1.0,), (2e-3,), shift=False)
    P3, sp3 = multi_dust_tube((0.2, 0.3, 0.5), (2e-3,) * 3, shift=False)
    one, (Tm1, _, _) = run_gpu(P1, sp1, 6)
    three, (Tm3, _, _) = run_gpu(P3, sp3, 6)
    assert abs(Tm1 - Tm3) <= 1e-12 * Tm1
    g1, g3 = one[0], three[0]
    for f in ("x", "vx", "vy", "rho", "e"):
        a, b = getattr(g1, f), getattr(g3, f)
        scale = max(np.abs(a).max(), 1e-300)
        assert np.abs(a - b).max() <= 1e-10 * scale, f
    vscale = np.abs(one[1].vx).max()
    for k in (1, 2, 3):  # the three species move as the one species
        assert np.abs(three[k].vx - one[1].vx).max() <= 1e-10 * vscale, k
