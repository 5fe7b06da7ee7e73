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
                          candidates=[(2, 1.001, 32), (1, 2.002, 32), (4, 0.5005, 32)])
    timed = [row for row in log if row[3] is not None]
    assert timed, log
    assert best.ms_per_step == min(row[3] for row in timed)
    assert (best.stencil, best.cell_factor) in [(row[0], row[1]) for row in timed]
