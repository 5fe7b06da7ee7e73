"""Ragged and empty inputs on the GPU (needs a GPU): a batch mixing a normal
tube, a tube of five gas particles without dust, and a tube whose gas is all
frozen.  Every tube must equal its own run alone and the oracle (FP64 path:
bit for bit)."""
import numpy as np
import pytest

from dustyshock3d_gb300 import ic
from dustyshock3d_gb300.solver import Solver
from dustyshock3d_gb300.species import Species
from oracle.oracle import OracleState

pytestmark = pytest.mark.gpu


def _sub(s: Species, idx) -> Species:
    f = {k: getattr(s, k)[idx].copy() for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e",
                                                  "m", "h", "ts", "ind")}
    return Species(**f)


def _tubes():
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
    g, d = sp
    mid = np.nonzero((g.ind == 0) & (np.abs(g.x) < 0.05))[0][:5]
    tiny = [_sub(g, mid), _sub(d, np.arange(0))]            # 5 gas, no dust
    frozen_g = _sub(g, np.arange(g.n))
    frozen_g.ind[:] = 1                                      # nothing moves
    frozen = [frozen_g, _sub(d, np.arange(d.n))]
    return P, [sp, tiny, frozen]


def _run(Ps, tubes, steps):
    with Solver(Ps) as S:
        for t, sp in enumerate(tubes):
            S.set_tube(t, sp)
        S.step(steps)
        return [[S.get_species(t, s, template=sp[s]) for s in range(2)] for t, sp in enumerate(tubes)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ragged_batch_with_empty_and_tiny_tubes(precision):
    P, tubes = _tubes()
    P.precision = precision
    batched = _run([P] * len(tubes), tubes, 4)
    for t, sp in enumerate(tubes):
        alone = _run([P], [sp], 4)[0]
        for s in range(2):
            for f in ("x", "vx", "rho"):
                assert np.array_equal(getattr(batched[t][s], f), getattr(alone[s], f)), (t, s, f)
    # the oracle on the FP64 path
    if precision == "fp64":
        for t, sp in enumerate(tubes):
            O = OracleState(P, sp).step(4)
            for s in range(2):
                for f in ("x", "vx", "rho"):
                    assert np.array_equal(getattr(batched[t][s], f), getattr(O.species[s], f)), (t, s, f)
    # frozen tube: positions unchanged
    assert np.array_equal(batched[2][0].x, tubes[2][0].x)


def test_species_beyond_the_list_entry_limit_is_refused_before_allocating():
    """A list entry holds a slot in 24 bits on the FP32 path (25 on the FP64
    path): a species of more particles is DS_ERR_UNSUPPORTED at the first step,
    before any device memory is taken.  A 19.4M-gas tube, generated on the
    device, so no host arrays either."""
    from dustyshock3d_gb300 import _lib
    spec = ic.DeviceIC.dusty_sod(dx_left=1 / 2400, Ly=0.05)
    P, counts = spec.plan()
    assert counts[0] > 2 ** 24
    P.precision = "fp32"
    with Solver(P) as S:
        S.init_tube(0, spec)
        with pytest.raises(_lib.DsError, match="DS_ERR_UNSUPPORTED"):
            S.step(1)
        assert S.memory_bytes() == 0


def test_particle_outside_the_grid_flags_and_matches_the_oracle():
    """A free gas particle outside the box: its neighbour key falls off the grid
    (dropped from the lists, still moved: kernel.cu:1950) and its IDIC cell index
    is out of range, where the reference writes out of bounds (kernel.cu:2116);
    here the particle is left unrelaxed and DS_FLAG_IDIC_RANGE is raised, which
    fails ds_step with DS_ERR_DEVICE.  The state equals the oracle's bit for bit."""
    from dustyshock3d_gb300 import _lib
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
    g = sp[0].copy().fill_missing()
    free = np.nonzero(g.ind == 0)[0]
    q = free[len(free) // 2]
    g.x[q] = P.X_max + 0.25  # beyond the last IDIC cell (the grid has int(L / w) + 1 cells per axis)
    species = [g, sp[1].copy().fill_missing()]
    with Solver(P) as S:
        S.set_tube(0, species)
        with pytest.raises(_lib.DsError, match="DS_ERR_DEVICE"):
            S.step(1)
        assert S.device_flags() & 1
        gpu = [S.get_species(0, s) for s in range(2)]
    O = OracleState(P, species).step(1)
    assert O.last_status & 1
    for s in range(2):
        for f in ("x", "y", "z", "vx", "vy", "vz", "rho"):
            a, b = getattr(gpu[s], f), getattr(O.species[s], f)
            assert np.array_equal(a, b, equal_nan=True), (s, f, np.nonzero(a != b)[0][:5])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_cutoff_beyond_the_stencil_is_flagged(precision):
    """Proper cell grid, stencil 2 over cells of 1.001 h_max: a particle whose
    cut-off 2h reaches past the two cells each side would lose partners (the
    walks search the stencil's cells at most), so DS_FLAG_REACH is raised and
    ds_step fails with DS_ERR_DEVICE.  h just inside the reach steps cleanly."""
    from dustyshock3d_gb300 import _lib
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
    P.precision = precision
    assert P.stencil == 2
    g = sp[0].copy().fill_missing()
    free = np.nonzero(g.ind == 0)[0]
    q = free[len(free) // 3]
    for factor, flagged in ((0.999, False), (1.05, True)):
        g2 = g.copy()
        g2.h[q] = factor * P.cell_w  # reach = stencil x cell width / 2 = cell_w
        with Solver(P) as S:
            S.set_tube(0, [g2, sp[1].copy().fill_missing()])
            if flagged:
                with pytest.raises(_lib.DsError, match="DS_ERR_DEVICE"):
                    S.step(1)
                assert S.device_flags() & 8
            else:
                S.step(1)
                assert S.device_flags() == 0


def test_cutoff_beyond_the_cell_on_the_reference_grid_is_not_flagged():
    """The reference grid searches its 27 cells of width 2h whatever a
    particle's h field holds (kernel.cu:2014-2016): an oversize h there is the
    reference's behaviour, not an error.  No flag, and the step equals the
    oracle's bit for bit."""
    from tests import _golden
    _, P, sp = _golden.setup("refB")
    assert not P.mode.grid_proper
    g = sp[0].copy().fill_missing()
    free = np.nonzero(g.ind == 0)[0]
    g.h[free[len(free) // 2]] = 1.5 * P.h
    species = [g] + [d.copy().fill_missing() for d in sp[1:]]
    with Solver(P) as S:
        S.set_tube(0, species)
        S.step(1)
        assert S.device_flags() & 8 == 0
        gpu = [S.get_species(0, s) for s in range(len(species))]
    O = OracleState(P, species).step(1)
    for s in range(len(species)):
        for f in ("x", "vx", "rho"):
            assert np.array_equal(getattr(gpu[s], f), getattr(O.species[s], f), equal_nan=True), (s, f)


def test_lattice_on_the_cell_faces_fp64_bitexact():
    """Gas and dust lattices starting exactly on the faces of the IDIC cells
    (a quarter of the gas sits on an x face): the cell of such a particle is
    decided by the rounding of (x - origin) / width, done as the oracle does it,
    so the FP64 path still equals the oracle bit for bit after 6 steps."""
    from tests.test_gpu_parity import compare_exact, run_gpu
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25),
                              lattice_offset=0.0)
    fx = (sp[0].x - P.X_min) / P.idic_w
    assert np.sum(np.abs(fx - np.round(fx)) < 1e-12) > sp[0].n // 8
    gpu, (Tm, dt, _) = run_gpu(P, sp, 6)
    O = OracleState(P, sp).step(6)
    assert Tm == O.Tm and dt == O.last_dt
    compare_exact(gpu, O.species, "lattice on the faces")
