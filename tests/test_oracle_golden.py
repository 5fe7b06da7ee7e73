"""The oracle against the reference program's own snapshots (golden fixtures).

The fixtures were printed by the unmodified reference (tests/golden/make_golden.py)
with %10.8lf, so floats agree to the printed rounding (5e-9) and the linked-list
next pointers and Ind flags agree exactly.
"""
import numpy as np
import pytest

from oracle.oracle import OracleState
from tests._golden import NAMES, assert_close_nan, setup, snapshot_steps

ATOL = 1.0e-8  # half a unit in the 8th printed decimal, plus rounding of the parse


@pytest.mark.parametrize("name", NAMES)
def test_initial_conditions_match_reference(name):
    g, P, sp = setup(name)
    assert sp[0].n == len(g["ind"])
    assert (sp[0].ind == g["ind"]).all(), "Ind flags (incl. the reference's overwrite quirk)"
    assert np.abs(sp[0].x - g["x0"]).max() <= ATOL


@pytest.mark.parametrize("name", NAMES)
def test_oracle_replays_reference_snapshots(name):
    g, P, sp = setup(name)
    nsnap = len(g["snap_times"])
    steps = snapshot_steps(P, nsnap)
    O = OracleState(P, sp)
    interior = g["ind"] == 0
    step = 0
    for s, target in enumerate(steps, start=1):
        while step < target:
            nexts = [O.lists(k)[1].copy() for k in range(3)]
            O.step(1)
            step += 1
        gas = O.species[0]
        assert (nexts[0] == g[f"s{s}_gas_Nn"]).all(), f"snapshot {s}: gas list order"
        for col, arr in (("x", gas.x), ("y", gas.y), ("z", gas.z), ("rho", gas.rho), ("p", gas.p),
                         ("Vx", gas.vx), ("Vy", gas.vy), ("e", gas.e)):
            assert_close_nan(arr[interior], g[f"s{s}_gas_{col}"], ATOL, f"{name} s{s} gas {col}")
        for k in (1, 2):
            d = O.species[k]
            assert (nexts[k] == g[f"s{s}_d{k}_Nn"]).all(), f"snapshot {s}: dust {k} list order"
            for col, arr in (("x", d.x), ("y", d.y), ("z", d.z), ("rho", d.rho), ("t_stop", d.ts),
                             ("Vx", d.vx), ("Vy", d.vy)):
                assert_close_nan(arr[interior], g[f"s{s}_d{k}_{col}"], ATOL, f"{name} s{s} dust{k} {col}")


def test_refA_nan_onset_is_the_reference_defect():
    """refA's NaN at step 3 comes from the eps_2 guard testing species 1's count
    (kernel.cu:2203): a cell holding gas and dust 1 but no dust 2 gets eps_2 = 0."""
    g, P, sp = setup("refA")
    nan3 = np.isnan(g["s3_gas_Vx"])
    assert nan3.sum() > 0 and not np.isnan(g["s2_gas_Vx"]).any()
