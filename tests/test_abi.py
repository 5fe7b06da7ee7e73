"""The C-ABI library builds, loads and exports every symbol of include/*.h (no GPU needed)."""
import ctypes
import os
import re

from dustyshock3d_gb300 import _lib
from dustyshock3d_gb300 import build as dsbuild
from dustyshock3d_gb300.params import MODE_BITS

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dustyshock3d_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ds_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    dsbuild.build()
    L = ctypes.CDLL(dsbuild.LIB)
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert set(syms) == set(_lib.SIGNATURES), set(syms) ^ set(_lib.SIGNATURES)


def test_params_struct_layout_matches_header():
    # sizeof(ds_params): 6+1 doubles... computed by the compiler in a tiny TU
    import subprocess, tempfile
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        open(src, "w").write('#include "dustyshock3d_gb300.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                             'int main(){printf("%zu %zu %zu %zu\\n", sizeof(ds_params), offsetof(ds_params, n_dust),'
                             ' offsetof(ds_params, cell_w), offsetof(ds_params, eps_empty));return 0;}\n')
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    c = _lib.DsParams
    assert [int(x) for x in out] == [ctypes.sizeof(c), c.n_dust.offset, c.cell_w.offset, c.eps_empty.offset]


def test_mode_bits_match_header():
    text = open(HEADER).read()
    hdr = {m.group(1).lower(): int(m.group(2), 16) for m in re.finditer(r"#define DS_MODE_([A-Z_0-9]+) (0x[0-9a-f]+)", text)}
    for name, bit in MODE_BITS.items():
        assert hdr[name] == bit, name


def test_params_init_and_init_txt_reader(tmp_path):
    L = _lib.load()
    p = _lib.DsParams()
    assert L.ds_params_init(ctypes.byref(p)) == 0
    assert p.Gam_g == 1.4 and p.n_dust == 2 and p.mass_ratio[1] == 0.5
    f = tmp_path / "Init.txt"
    f.write_text("// Initial parameters\n-1.5\t// X_min\n1.5\n-0.5\n0.5\n-0.25\n0.75\n1\t// eos\n5000\n20\n0.07\n0.5\n"
                 "2.5e-3\n0.3\n0.05\n0.5\n1.5\n0.02\n")
    assert L.ds_params_read_init_txt(str(f).encode(), ctypes.byref(p)) == 0
    assert (p.X_min, p.Z_max, p.Type_of_state, p.Maximum_particle, p.h, p.tau, p.eps) == \
        (-1.5, 0.75, 1, 5000, 0.07, 2.5e-3, 0.02)


def test_version_string():
    assert b"sm_103a" in _lib.load().ds_version()


def test_checkpoint_params_reads_the_header_and_rejects_bad_files(tmp_path):
    """ds_checkpoint_params (file I/O only, no GPU): a file that starts with the
    magic and a ds_params gives those parameters back; a missing, foreign or
    truncated file gives DS_ERR_IO (7)."""
    L = _lib.load()
    P = _lib.DsParams()
    assert L.ds_params_init(ctypes.byref(P)) == 0
    P.h = 0.0123
    P.n_dust = 1
    good = tmp_path / "good.ckpt"
    good.write_bytes(b"DSCKPT01" + bytes(P))
    Q = _lib.DsParams()
    assert L.ds_checkpoint_params(str(good).encode(), ctypes.byref(Q)) == 0
    assert Q.h == 0.0123 and Q.n_dust == 1
    for name, data in (("foreign", b"NOTACKPT" + bytes(P)), ("short", b"DSCKPT01" + bytes(P)[:10])):
        f = tmp_path / name
        f.write_bytes(data)
        assert L.ds_checkpoint_params(str(f).encode(), ctypes.byref(Q)) == 7, name
    assert L.ds_checkpoint_params(str(tmp_path / "missing").encode(), ctypes.byref(Q)) == 7


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    """No fallback: without the built library every entry point raises."""
    import pytest
    from dustyshock3d_gb300 import params
    from dustyshock3d_gb300 import solver as solver_mod
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(_lib.DsError, match="not built"):
        _lib.load(str(tmp_path / "libdustyshock3d_gb300.so"))
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libdustyshock3d_gb300.so"))
    monkeypatch.setattr(_lib.load, "__defaults__", (str(tmp_path / "libdustyshock3d_gb300.so"),))
    with pytest.raises(_lib.DsError):
        solver_mod.Solver(params.Params())


def test_extreme_grids_are_refused_before_any_device_work():
    """Box extents and cell widths are checked in double before the grid's int
    sizes are formed: NaN or negative extents, zero widths and grids beyond 2^28
    cells are DS_ERR_ARG from ds_create (no CUDA call is made before the check)."""
    L = _lib.load()
    base = _lib.DsParams()
    assert L.ds_params_init(ctypes.byref(base)) == 0
    cases = [dict(X_max=float("nan")), dict(X_max=-5.0), dict(cell_w=1e-9), dict(X_min=-1e12, X_max=1e12),
             dict(idic_w=0.0, Coeff_h_dust_cell=0.0), dict(idic_w=1e-9)]
    for kw in cases:
        p = _lib.DsParams.from_buffer_copy(base)
        for k, v in kw.items():
            setattr(p, k, v)
        ctx = ctypes.c_void_p()
        assert L.ds_create(ctypes.byref(p), ctypes.byref(ctx)) == 1, kw
        assert not ctx.value


def test_unsupported_combinations_are_refused_before_any_device_work():
    """Combinations the step does not implement are DS_ERR_UNSUPPORTED from
    ds_create: periodic axes or the FP32 path on the reference's aliasing grid
    (its rows are not true rows), wide stencils without the proper grid, and
    stencils past 2 cells on the FP64 path."""
    L = _lib.load()
    base = _lib.DsParams()
    assert L.ds_params_init(ctypes.byref(base)) == 0
    proper = 0x0400
    cases = [dict(mode=0x0001), dict(mode=0x0002), dict(precision=1), dict(stencil=2),
             dict(stencil=3, mode=proper)]
    for kw in cases:
        p = _lib.DsParams.from_buffer_copy(base)
        for k, v in kw.items():
            setattr(p, k, v)
        ctx = ctypes.c_void_p()
        assert L.ds_create(ctypes.byref(p), ctypes.byref(ctx)) == 6, kw
        assert not ctx.value
