"""One behaviour switch at a time on the small dusty Sod tube (needs a GPU).

The benchmark physics (Mode.baseline()) and the reference's own step
(Mode.reference()) are covered by the parity tests; here each switch of the
mode word, and the isothermal equation of state (Type_of_state 1,
kernel.cu:95-96), is flipped alone from the benchmark physics and from the
reference's step.  Every variant from the benchmark physics:
the FP64 path equals the oracle bit for bit after 4 steps, and the FP32 path
tracks the oracle within the parity tests' FP32 tolerance after 10."""
import numpy as np
import pytest

from dustyshock3d_gb300 import ic
from oracle.oracle import OracleState
from tests._multidust import multi_dust_tube
from tests.test_gpu_parity import compare_exact, run_gpu

pytestmark = pytest.mark.gpu


def _flip(name):
    """(params, species) of the small benchmark tube with one switch flipped."""
    if name == "ref_solve2":  # the reference's 2-species operation order needs two species
        P, sp = multi_dust_tube((1.0, 0.5), (1e-3, 1e-2))
    else:
        P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
        P = P.copy()
    m = P.mode
    if name == "periodic_off":  # open y and z faces, with a frozen layer of one h on them
        m.periodic_y = m.periodic_z = False
        for s in sp:          # (as the reference freezes its border particles, kernel.cu:1396, 1441)
            near = ((s.y < P.Y_min + s.h) | (s.y > P.Y_max - s.h) |
                    (s.z < P.Z_min + s.h) | (s.z > P.Z_max - s.h))
            s.ind = np.where(near, 1, s.ind).astype(np.int32)
    elif name == "isothermal":
        P.Type_of_state = 1
        for s in sp[:1]:
            s.p = P.Speed_of_sound_gas ** 2 * s.rho  # p = c^2 rho (kernel.cu:96)
    elif name == "tstop_const":  # t_stop = R / (c_s rho) of the gas at the same index (kernel.cu:43-46)
        m.tstop_const = False
        P.R_dust = [1e-3]
    else:
        setattr(m, name, not getattr(m, name))
    return P, sp


SWITCHES = ["periodic_off", "h_per_particle", "tstop_const", "gas_accel_particle", "ref_index_coupling",
            "ref_eps_guard", "ref_solve2", "cfl", "dust_rho", "idic_proper", "isothermal"]


@pytest.mark.parametrize("name", SWITCHES)
def test_switch_fp64_bitexact(name):
    P, sp = _flip(name)
    gpu, (Tm, dt, _) = run_gpu(P, sp, 4)
    O = OracleState(P, sp).step(4)
    assert O.last_status == 0
    assert Tm == O.Tm and dt == O.last_dt
    compare_exact(gpu, O.species, name)
    assert np.abs(gpu[0].vx).max() > 0.0  # the gas moved


@pytest.mark.parametrize("name", SWITCHES)
def test_switch_fp32_tracks_the_oracle(name):
    P, sp = _flip(name)
    P32 = P.copy()
    P32.precision = "fp32"
    gpu, _ = run_gpu(P32, sp, 10)
    O = OracleState(P, sp).step(10)
    g, o = gpu[0], O.species[0]
    assert np.abs(g.rho - o.rho).sum() / np.abs(o.rho).sum() < 1e-5
    vscale = np.abs(o.vx).max()
    assert np.abs(g.vx - o.vx).mean() / vscale < 1e-4
    for k in range(1, len(sp)):
        assert np.abs(gpu[k].vx - O.species[k].vx).mean() / vscale < 1e-4, k


REF_SWITCHES = ["h_per_particle", "tstop_const", "gas_accel_particle", "ref_index_coupling",
                "ref_eps_guard", "ref_solve2", "cfl", "dust_rho", "grid_proper", "idic_proper", "isothermal"]


@pytest.mark.parametrize("name", REF_SWITCHES)
def test_reference_step_with_one_switch_fp64_bitexact(name):
    """The same from the reference's own step (case refB: gas and two dust
    species on the reference's aliasing grid): every switch flipped alone,
    FP64 path = oracle bit for bit after 5 steps.  (Periodic axes need the
    proper grid: refused at ds_create on this one.)"""
    from tests import _golden
    _, P, sp = _golden.setup("refB")
    P = P.copy()
    m = P.mode
    if name == "isothermal":
        P.Type_of_state = 1
    elif name == "tstop_const":
        m.tstop_const = True
        P.t_stop_const = [1e-3, 1e-2]
    elif name == "cfl":
        m.cfl = True
        P.cfl = 0.3
    else:
        setattr(m, name, not getattr(m, name))
    gpu, (Tm, dt, _) = run_gpu(P, sp, 5)
    O = OracleState(P, sp).step(5)
    assert O.last_status == 0
    assert Tm == O.Tm and dt == O.last_dt
    compare_exact(gpu, O.species, name)


@pytest.mark.parametrize("stencil,cell_factor", [(3, 0.6673), (4, 0.5005)])
def test_one_h_with_small_cells_fp32(stencil, cell_factor):
    """One h for every pair on cells of h / 1.5 and h / 2 (3 and 4 cells each
    side): the FP32 path tracks the oracle on its own grid."""
    P, sp = _flip("h_per_particle")
    P32 = P.copy()
    P32.precision = "fp32"
    P32.stencil = stencil
    P32.cell_w = cell_factor * P.h
    gpu, _ = run_gpu(P32, sp, 10)
    O = OracleState(P, sp).step(10)
    g, o = gpu[0], O.species[0]
    assert np.abs(g.rho - o.rho).sum() / np.abs(o.rho).sum() < 1e-5
    vscale = np.abs(o.vx).max()
    assert np.abs(g.vx - o.vx).mean() / vscale < 1e-4
