"""The timing entry points advance the tubes exactly as ds_step does, and the
autotuner keeps the fastest candidate it timed."""
import numpy as np
import pytest

from dustyshock3d_gb300 import ic, tune
from dustyshock3d_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _tube():
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25))
    P.precision = "fp32"
    return P, sp


def test_timed_steps_equal_plain_steps():
    P, sp = _tube()
    with Solver(P) as A, Solver(P) as B:
        A.set_tube(0, sp)
        B.set_tube(0, sp)
        A.step(1)
        ms = A.step_timed_graph(3)   # the graphs ds_step replays, between two events
        tot, ph = A.step_timed(2)    # kernels one by one, events between phases
        B.step(6)
        assert ms > 0 and tot > 0
        assert len(ph) == 4 and all(p >= 0 for p in ph)
        assert abs(sum(ph) - tot) <= 0.05 * tot + 0.02  # the phases cover the steps
        assert A.time() == B.time() and A.time()[2] == 6
        for s in range(2):
            a, b = A.get_species(0, s), B.get_species(0, s)
            for f in ("x", "y", "z", "vx", "vy", "vz", "rho", "e"):
                assert np.array_equal(getattr(a, f), getattr(b, f)), (s, f)


def test_autotuner_keeps_the_fastest_candidate():
    rng = np.random.default_rng(7)
    tubes = [ic.uneven_tube(**ic.draw_tube_params(rng, (2.0e4, 4.0e4))) for _ in range(2)]
    best, log = tune.tune(tubes, sample=2, warmup=1, steps=2,
                          candidates=[(2, 1.001, 32), (1, 2.002, 32), (4, 0.5005, 32)], skin_candidates=())
    timed = [row for row in log if row[6] is not None]
    assert timed, log
    assert best.ms_per_step == min(row[6] for row in timed)
    assert best.list_skin == 0.0
    assert (best.stencil, best.cell_factor, best.persistent, best.idic_lanes) in \
        [(row[0], row[1], row[3], row[4]) for row in timed]
    # the launch shapes were tried for the winning grid
    assert {(row[3], row[4]) for row in timed} >= set(tune.LAUNCH_CANDIDATES)


def test_autotuner_times_the_skins_for_the_winner():
    rng = np.random.default_rng(11)
    tubes = [ic.uneven_tube(**ic.draw_tube_params(rng, (2.0e4, 4.0e4))) for _ in range(2)]
    best, log = tune.tune(tubes, sample=2, warmup=1, steps=2, candidates=[(2, 1.001, 32)],
                          launch_candidates=[(0, 4)], skin_steps=6)
    skin_rows = log[-(1 + len(tune.SKIN_CANDIDATES)):]
    assert [row[5] for row in skin_rows] == [0.0] + list(tune.SKIN_CANDIDATES)
    assert all(row[6] is not None for row in skin_rows)
    fastest = min(skin_rows, key=lambda row: row[6])
    assert (best.list_skin, best.ms_per_step) == (fastest[5], fastest[6])


@pytest.mark.parametrize("persistent,lanes", [(1, 4), (0, 2), (1, 8)])
def test_launch_shapes_keep_the_results(persistent, lanes):
    """Persistent sweeps give the same results bit for bit (a chunk's work does
    not depend on the block that claims it); the threads per IDIC cell change
    only the cell sums' rounding (FP32 path bounds)."""
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
    P.precision = "fp32"
    out = []
    for q in (P, tune.apply(P, P.stencil, P.cell_w / P.h, P.list_depth, persistent, lanes)):
        with Solver(q) as S:
            S.set_tube(0, sp)
            S.step(8)
            out.append([S.get_species(0, s) for s in range(2)])
    for s in range(2):
        for f in ("x", "vx", "rho"):
            a, b = getattr(out[1][s], f), getattr(out[0][s], f)
            if lanes == 4:
                assert np.array_equal(a, b), (s, f)
            else:  # the FP32 path's bounds: relative L1 1e-5
                assert np.abs(a - b).sum() <= 1e-5 * np.abs(b).sum(), (s, f)
