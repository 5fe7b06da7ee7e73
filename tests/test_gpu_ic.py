"""Initial conditions generated on the device (ds_init_tube) equal the host
generators bit for bit: the reference's init_Sod_X_Dust (kernel.cu:1391-1582,
pinned to the reference program by the golden snapshots), init_Sod_X_mas
(kernel.cu:938-1042) with dust on the gas sites, and the dusty Sod tube; a
generated tube then steps exactly like an uploaded one."""
import numpy as np
import pytest

from dustyshock3d_gb300 import ic, params
from dustyshock3d_gb300.solver import Solver

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h", "ts", "ind")

REF_BOXES = [
    dict(X_min=-1.2, X_max=1.2, Y_min=-0.8, Y_max=1.0, Z_min=-0.8, Z_max=1.0, Type_of_state=0,
         Particle_on_length=10, h=0.2),
    dict(X_min=-1.05, X_max=1.15, Y_min=-0.65, Y_max=0.85, Z_min=-0.72, Z_max=0.78, Type_of_state=1,
         Particle_on_length=10, h=0.23),
    dict(X_min=-1.5, X_max=1.5, Y_min=-0.5, Y_max=1.5, Z_min=-0.3, Z_max=2.0, Type_of_state=0,
         Particle_on_length=40, h=0.1),  # 180k gas particles, 4 x 180k in all
]

TUBES = [
    dict(dx_left=1 / 200, Ly=0.1),
    dict(dx_left=1 / 97, Ly=0.15, Lz=0.12, eps=0.3, t_s=2e-2, rho_R=0.2, p_R=0.15, lattice_offset=0.0,
         wall=1.5, x_range=(-0.3, 0.45), fixed_tau=2e-4, h_factor=1.2, idic_cells_per_right_spacing=3.0),
    ic.uneven_tube_kwargs(N_gas=3.1e4, rho_ratio=9.3, p_ratio=12.0, eps=0.05, t_s=3e-3),
    dict(dx_left=1 / 800, Ly=0.05),  # the 720k + 720k benchmark tube
]


def _init(**kw):
    P = params.Params()
    P.Maximum_particle = 10 ** 7
    for k, v in kw.items():
        setattr(P, k, v)
    return P


def _assert_species_equal(got, want, what):
    assert got.n == want.n, what
    for f in FIELDS:
        a, b = getattr(got, f), getattr(want, f)
        # NaN where both have NaN (the refA box goes NaN at step 3, as the reference does)
        assert np.array_equal(a, b, equal_nan=a.dtype.kind == "f"), f"{what}: {f} differs at {np.nonzero(a != b)[0][:5]}"


def _generated(spec, P):
    S = Solver(P)
    S.init_tube(0, spec)
    return S


@pytest.mark.parametrize("box", range(len(REF_BOXES)))
@pytest.mark.parametrize("kind", ["sod_x_dust", "sod_x_mas"])
def test_reference_generators_on_device(box, kind):
    P0 = _init(**REF_BOXES[box])
    if kind == "sod_x_mas":
        P0.n_dust, P0.mass_ratio, P0.R_dust = 3, [0.75, 0.5, 2.0], [0.01, 1.0, 0.3]
    spec = ic.DeviceIC(kind=kind)
    Pp, counts = spec.plan(P0)
    Ph, host = (ic.init_sod_x_dust if kind == "sod_x_dust" else ic.init_sod_x_mas)(P0)
    with _generated(spec, Pp) as S:
        for s in range(1 + Pp.n_dust):
            _assert_species_equal(S.get_species(0, s), host[s], f"{kind} box {box} species {s}")


@pytest.mark.parametrize("case", range(len(TUBES)))
def test_dusty_sod_tube_on_device(case):
    kw = TUBES[case]
    spec = ic.DeviceIC.dusty_sod(**kw)
    Pp, counts = spec.plan()
    Ph, host = ic.dusty_sod_tube(**kw)
    with _generated(spec, Pp) as S:
        for s in range(2):
            _assert_species_equal(S.get_species(0, s), host[s], f"tube {case} species {s}")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_generated_tube_steps_like_an_uploaded_one(precision):
    spec = ic.DeviceIC.dusty_sod(**TUBES[0])
    P, _ = spec.plan()
    P.precision = precision
    _, host = ic.dusty_sod_tube(**TUBES[0])
    with Solver(P) as A, Solver(P) as B:
        A.init_tube(0, spec)
        B.set_tube(0, host)
        A.step(4)
        B.step(4)
        assert A.time() == B.time()
        for s in range(2):
            _assert_species_equal(A.get_species(0, s), B.get_species(0, s), f"{precision} species {s}")


def test_reference_mode_generated_run_equals_uploaded_run():
    P0 = _init(**REF_BOXES[1])
    spec = ic.DeviceIC(kind="sod_x_dust")
    P, _ = spec.plan(P0)
    _, host = ic.init_sod_x_dust(P0)
    with Solver(P) as A, Solver(P) as B:
        A.init_tube(0, spec)
        B.set_tube(0, host)
        A.step(3)
        B.step(3)
        for s in range(3):
            _assert_species_equal(A.get_species(0, s), B.get_species(0, s), f"species {s}")


def test_resident_tube_regenerated_and_mixed_batch():
    """A batch of a generated and an uploaded tube; then the generated tube is
    generated again into its resident segments (same counts)."""
    spec = ic.DeviceIC.dusty_sod(**TUBES[2])
    P, _ = spec.plan()
    P2, host2 = ic.dusty_sod_tube(**TUBES[0])
    _, host = ic.dusty_sod_tube(**TUBES[2])
    with Solver([P, P2]) as S:
        S.init_tube(0, spec)
        S.set_tube(1, host2)
        S.step(2)
        with Solver(P2) as alone:
            alone.set_tube(0, host2)
            alone.step(2)
            for s in range(2):
                _assert_species_equal(S.get_species(1, s), alone.get_species(0, s), f"uploaded tube {s}")
        S.init_tube(0, spec)
        for s in range(2):
            _assert_species_equal(S.get_species(0, s), host[s], f"regenerated species {s}")
        S.step(1)
