"""Initial conditions and the Init.txt extension on the CPU: the library's
host-side plan (ds_ic_plan) against the host generators, the ds_ic defaults and
layout, and the C Init.txt reader against params.py (no GPU needed)."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from dustyshock3d_gb300 import _lib, ic, params
from dustyshock3d_gb300 import build as dsbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Init.txt boxes of the golden reference runs (first lattice point inside the
# accept cube) and two more shapes
REF_BOXES = [
    dict(X_min=-1.2, X_max=1.2, Y_min=-0.8, Y_max=1.0, Z_min=-0.8, Z_max=1.0, Type_of_state=0,
         Particle_on_length=10, h=0.2),
    dict(X_min=-1.05, X_max=1.15, Y_min=-0.65, Y_max=0.85, Z_min=-0.72, Z_max=0.78, Type_of_state=0,
         Particle_on_length=12, h=0.19),
    dict(X_min=-1.05, X_max=1.15, Y_min=-0.65, Y_max=0.85, Z_min=-0.72, Z_max=0.78, Type_of_state=1,
         Particle_on_length=10, h=0.23),
    dict(X_min=-0.4, X_max=0.3, Y_min=-0.5, Y_max=0.2, Z_min=-0.3, Z_max=0.1, Type_of_state=0,
         Particle_on_length=20, h=0.05),
]

TUBES = [
    dict(dx_left=1 / 200, Ly=0.1),
    dict(dx_left=1 / 97, Ly=0.15, Lz=0.12, eps=0.3, t_s=2e-2, rho_R=0.2, p_R=0.15, lattice_offset=0.0,
         wall=1.5, x_range=(-0.3, 0.45), fixed_tau=2e-4, h_factor=1.2, idic_cells_per_right_spacing=3.0),
    ic.uneven_tube_kwargs(N_gas=3.1e4, rho_ratio=9.3, p_ratio=12.0, eps=0.05, t_s=3e-3),
]


def _params(**kw):
    P = params.Params()
    P.Maximum_particle = 10 ** 7
    for k, v in kw.items():
        setattr(P, k, v)
    return P


def _same_params(a, b):
    ca, cb = _lib.params_to_c(a), _lib.params_to_c(b)
    diffs = []
    for f, _ in _lib.DsParams._fields_:
        va, vb = getattr(ca, f), getattr(cb, f)
        if hasattr(va, "__len__"):
            va, vb = list(va), list(vb)
        if va != vb:
            diffs.append((f, va, vb))
    assert not diffs, diffs
    assert bytes(ca) == bytes(cb)


@pytest.mark.parametrize("box", range(len(REF_BOXES)))
@pytest.mark.parametrize("kind", ["sod_x_dust", "sod_x_mas"])
def test_plan_matches_reference_generators(box, kind):
    P = _params(**REF_BOXES[box])
    host = ic.init_sod_x_dust if kind == "sod_x_dust" else ic.init_sod_x_mas
    Ph, species = host(P)
    Pp, counts = ic.DeviceIC(kind=kind).plan(P)
    assert counts == [s.n for s in species]
    _same_params(Pp, Ph)


@pytest.mark.parametrize("case", range(len(TUBES)))
def test_plan_matches_dusty_sod_tube(case):
    kw = dict(TUBES[case])
    Ph, species = ic.dusty_sod_tube(**kw)
    Pp, counts = ic.DeviceIC.dusty_sod(**kw).plan()
    assert counts == [s.n for s in species]
    _same_params(Pp, Ph)


def test_plan_rejects_what_the_host_generators_reject():
    # the reference's own Init.txt: y = -2 at the first lattice point is outside
    # the 0.8 cube, where the reference writes Ind_gas[-1]
    P = _params(Particle_on_length=40, h=0.1)
    with pytest.raises(ValueError):
        ic.init_sod_x_dust(P)
    with pytest.raises(_lib.DsError):
        ic.DeviceIC(kind="sod_x_dust").plan(P)
    P = _params(**REF_BOXES[1])
    P.Maximum_particle = 1000  # kernel.cu:1751
    with pytest.raises(ValueError):
        ic.init_sod_x_dust(P)
    with pytest.raises(_lib.DsError):
        ic.DeviceIC(kind="sod_x_dust").plan(P)
    with pytest.raises(_lib.DsError):
        ic.DeviceIC.dusty_sod(dx_left=0.0, Ly=0.1).plan()
    with pytest.raises(_lib.DsError):
        ic.DeviceIC(kind="sod_x_dust").plan(None)  # the reference generators need Init.txt values


def test_ic_defaults_and_layout_match_the_header():
    L = _lib.load()
    for kind, code in _lib.IC_KINDS.items():
        c = _lib.DsIc()
        assert L.ds_ic_init(ctypes.byref(c), code) == 0
        d = ic.DeviceIC(kind=kind)
        for f in _lib.IC_FIELDS:
            assert getattr(c, f) == getattr(d, f), (kind, f)
    with tempfile.TemporaryDirectory() as dd:
        src = os.path.join(dd, "t.c")
        open(src, "w").write('#include "dustyshock3d_gb300.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                             'int main(){printf("%zu %zu %zu %zu %d %d %d\\n", sizeof(ds_ic), offsetof(ds_ic, dx_left),'
                             ' offsetof(ds_ic, idic_cells), offsetof(ds_ic, fixed_tau), DS_IC_SOD_X_DUST,'
                             ' DS_IC_SOD_X_MAS, DS_IC_DUSTY_SOD);return 0;}\n')
        exe = os.path.join(dd, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    c = _lib.DsIc
    assert out[:4] == [ctypes.sizeof(c), c.dx_left.offset, c.idic_cells.offset, c.fixed_tau.offset]
    assert out[4:] == [_lib.IC_KINDS["sod_x_dust"], _lib.IC_KINDS["sod_x_mas"], _lib.IC_KINDS["dusty_sod"]]
    assert L.ds_ic_init(ctypes.byref(_lib.DsIc()), 9) == 1  # unknown kind: DS_ERR_ARG


def _c_read(path):
    L = _lib.load()
    p = _lib.DsParams()
    assert L.ds_params_init(ctypes.byref(p)) == 0
    st = L.ds_params_read_init_txt(str(path).encode(), ctypes.byref(p))
    return st, p


def _nondefault_params():
    P = _params(X_min=-0.7, X_max=0.9, Y_min=0.0, Y_max=0.05, Z_min=0.0, Z_max=0.05, Type_of_state=1,
                Particle_on_length=123.0, h=0.0123, tau=2.5e-4, T_end=0.15, T_out=0.05, alpha=0.75, beta=1.5,
                eps=0.02)
    P.Maximum_particle = 4321
    P.Gam_g, P.Speed_of_sound_gas, P.t_empty = 5.0 / 3.0, 0.9, 2e-3
    P.cell_w, P.idic_w, P.cfl = 0.031, 0.0125, 0.25
    P.n_dust, P.stencil, P.list_depth, P.force_list = 3, 2, 64, 320
    P.list_skin, P.persistent, P.idic_lanes = 0.25, 1, 2
    P.mass_ratio, P.R_dust = [0.1, 1.0, 10.0], [0.0, 0.5, 2.0]
    P.t_stop_const, P.eps_empty = [1e-4, 1e-3, 1e-2], [0.1, 1.0, 10.0]
    P.precision = "fp32"
    P.mode = params.Mode.baseline()
    P.mode.cfl = False
    return P


def test_c_init_txt_reader_matches_params_py(tmp_path):
    for P in (_nondefault_params(), params.Params()):
        text = params.write_init_txt(P)
        f = tmp_path / "Init.txt"
        f.write_text(text)
        st, c = _c_read(f)
        assert st == 0
        assert bytes(c) == bytes(_lib.params_to_c(params.parse_init_txt(text)))
    # the plain reference file (17 values, no extensions) keeps the other defaults
    text = params.write_init_txt(params.Params(), extensions=False)
    f.write_text(text)
    st, c = _c_read(f)
    assert st == 0 and bytes(c) == bytes(_lib.params_to_c(params.parse_init_txt(text)))


def test_init_txt_extension_syntax(tmp_path):
    base = params.write_init_txt(params.Params(), extensions=False)
    extra = ("\n// a comment line\nmass_ratio = 0.5, 2.0   // comma separated\nmode.cfl = yes\nmode.dust_rho = off\n"
             "h = 0.2\nMaximum_particle = 777.9\nprecision = FP32\nno equals sign here\n"
             "ic = dusty_sod\nic.dx_left = 0.01\n")
    f = tmp_path / "Init.txt"
    f.write_text(base + extra)
    st, c = _c_read(f)
    P = params.parse_init_txt(base + extra)
    assert st == 0 and bytes(c) == bytes(_lib.params_to_c(P))
    assert P.mass_ratio == [0.5, 2.0] and P.mode.cfl and not P.mode.dust_rho and P.h == 0.2
    assert c.Maximum_particle == 777 and c.precision == 1
    for bad in ("mode.no_such_switch = 1\n", "n_dust = 2.5\n", "no_such_field = 3\n", "h = abc\n"):
        f.write_text(base + bad)
        assert _c_read(f)[0] == 1, bad
        with pytest.raises(ValueError):
            params.parse_init_txt(base + bad)


def test_ic_lines_of_init_txt(tmp_path):
    L = _lib.load()
    base = params.write_init_txt(params.Params())
    cases = {
        "": ic.DeviceIC(kind="sod_x_dust"),
        "ic = sod_x_mas\n": ic.DeviceIC(kind="sod_x_mas"),
        "ic.Ly = 0.05\nic = dusty_sod\nic.dx_left = 0.00125 // left spacing\nic.x1 = 0.75\nic.fixed_tau = 1e-4\n":
            ic.DeviceIC(kind="dusty_sod", Ly=0.05, dx_left=0.00125, x1=0.75, fixed_tau=1e-4),
    }
    for extra, want in cases.items():
        text = base + extra
        f = tmp_path / "Init.txt"
        f.write_text(text)
        c = _lib.DsIc()
        assert L.ds_ic_read_init_txt(str(f).encode(), ctypes.byref(c)) == 0
        got = ic.parse_ic_init_txt(text)
        assert got == want
        assert bytes(c) == bytes(want.to_c())
        # the parameter reader skips the ic lines
        assert _c_read(f)[0] == 0
    for bad in ("ic = nowhere\n", "ic.no_field = 1\n"):
        f = tmp_path / "Init.txt"
        f.write_text(base + bad)
        assert L.ds_ic_read_init_txt(str(f).encode(), ctypes.byref(_lib.DsIc())) == 1
        with pytest.raises(ValueError):
            ic.parse_ic_init_txt(base + bad)


def test_library_builds_the_generator_without_contraction():
    # ds_ic.cu's plan arithmetic must not be fused into FMAs by the host compiler
    assert "-ffp-contract=off" in dsbuild.SOURCES["ds_ic.cu"]
    assert "-fmad=false" in dsbuild.SOURCES["ds_ic.cu"]
