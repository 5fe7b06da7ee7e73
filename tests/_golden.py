"""Helpers shared by the tests that replay the golden reference snapshots."""
import os

import numpy as np

from dustyshock3d_gb300 import ic, parse_init_txt

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
NAMES = ("refA", "refB", "refC")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def setup(name):
    """Reference-mode parameters and initial particles of one golden run."""
    g = load(name)
    P = parse_init_txt(str(g["init_txt"]))
    P, species = ic.init_sod_x_dust(P)
    return g, P, species


def snapshot_steps(P, nsnap):
    """Steps after which the reference wrote snapshots 1..nsnap: it adds tau to
    Tm at the top of each step and writes when Tm >= out_num * T_out
    (kernel.cu:1931, 2528)."""
    Tm, out_num, step, steps = 0.0, 1, 0, []
    while len(steps) < nsnap:
        Tm = Tm + P.tau
        step += 1
        if Tm >= out_num * P.T_out:
            steps.append(step)
            out_num += 1
    return steps


def assert_close_nan(a, b, atol, what):
    na, nb = np.isnan(a), np.isnan(b)
    assert (na == nb).all(), f"{what}: NaN pattern differs at {np.nonzero(na != nb)[0][:10]}"
    f = ~na
    if f.any():
        err = np.abs(a[f] - b[f]).max()
        assert err <= atol, f"{what}: max |diff| {err:.3e} > {atol:.1e}"
