"""Init.txt handling mirrors the reference's reader (kernel.cu:1705-1723)."""
import os

import pytest

from dustyshock3d_gb300 import Params, parse_init_txt, write_init_txt
from tests._golden import load


def test_parse_reference_style_init():
    g = load("refB")
    P = parse_init_txt(str(g["init_txt"]))
    assert (P.X_min, P.X_max, P.Type_of_state, P.Particle_on_length, P.h, P.tau) == (-1.05, 1.15, 0, 12.0, 0.19, 3e-3)


def test_roundtrip_with_extensions():
    P = Params(h=0.05, n_dust=1, mass_ratio=[2.0], precision="fp32", list_skin=0.2, persistent=1, idic_lanes=8)
    P.mode.periodic_y = True
    Q = parse_init_txt(write_init_txt(P))
    assert Q == P


def test_short_file_rejected():
    with pytest.raises(ValueError):
        parse_init_txt("title\n1\n2\n")
