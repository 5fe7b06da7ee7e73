"""The host loop around the reference's own CUDA kernels (oracle/ref_gpu.c)
builds and loads without a GPU, exports its entry points, and refuses runs it
cannot make (no cubin, a run before the module is loaded, extensions the
reference's kernels lack) with a clear message instead of launching anything."""
import ctypes

import pytest

from oracle import oracle, ref_gpu


def test_library_builds_and_exports():
    L = ctypes.CDLL(ref_gpu.build(force=True))
    for name in ("rg_open", "rg_run", "rg_last_error", "rg_phase_seconds"):
        assert hasattr(L, name), name


def test_run_before_open_is_refused():
    L = ref_gpu.lib()
    P = oracle.OrcParams()
    sp = (oracle.OrcSpecies * 3)()
    Tm = ctypes.c_double(0.0)
    assert L.rg_run(ctypes.byref(P), sp, 1, ctypes.byref(Tm), None) == -1
    assert b"rg_open" in L.rg_last_error()
    assert Tm.value == 0.0


def test_missing_cubin_is_reported(monkeypatch, tmp_path):
    monkeypatch.setattr(ref_gpu, "CUBIN", str(tmp_path / "none.cubin"))
    why = ref_gpu.available()
    assert why and "build_ref_gpu.sh" in why
    from _golden import setup
    _, P, sp = setup("refC")
    with pytest.raises(RuntimeError, match="build_ref_gpu.sh"):
        ref_gpu.RefGPU(P, sp)


def test_extensions_are_refused_before_any_launch(monkeypatch, tmp_path):
    cubin = tmp_path / "k.cubin"
    cubin.write_bytes(b"")
    monkeypatch.setattr(ref_gpu, "CUBIN", str(cubin))
    from dustyshock3d_gb300 import ic
    P, sp = ic.dusty_sod_tube(dx_left=1 / 32, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
    with pytest.raises(ValueError, match="reference mode"):
        ref_gpu.RefGPU(P, sp)
