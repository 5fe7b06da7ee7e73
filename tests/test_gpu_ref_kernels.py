"""The reference's own CUDA kernels on the GPU (oracle/ref_gpu.c loading the
cubin that oracle/build_ref_gpu.sh compiles from kernel.cu and IDIC.h) against
the oracle and against this library's FP64 path, on two small reference-mode
runs.

The reference's kernels are built with nvcc's default floating-point options
(multiply-adds contracted), so they differ from its host build -- and so from
the oracle and the FP64 path, which equal the host build bit for bit -- by
rounding: the bound below is on that rounding, carried through the steps.
The cubin exists only where the reference tree was at build time; without it
the tests skip with the reason.
"""
import numpy as np
import pytest

from _golden import setup

pytestmark = pytest.mark.gpu

# relative to the field's scale, after the steps below
REL_TOL = 1e-9


def _ref_gpu():
    from oracle import ref_gpu
    why = ref_gpu.available()
    if why:
        pytest.skip(why)
    return ref_gpu


def _close(a, b, what):
    scale = max(1.0, float(np.max(np.abs(b))))
    err = float(np.max(np.abs(a - b)))
    assert err <= REL_TOL * scale, f"{what}: max |diff| {err:.3e} > {REL_TOL:.0e} x {scale:.3g}"
    return err / scale


@pytest.mark.parametrize("name,nsteps", [("refB", 10), ("refC", 10)])
def test_reference_kernels_track_the_oracle(name, nsteps):
    ref_gpu = _ref_gpu()
    from oracle.oracle import OracleState
    _, P, sp = setup(name)
    R = ref_gpu.RefGPU(P, sp).step(nsteps)
    O = OracleState(P, sp).step(nsteps)
    assert R.Tm == O.Tm
    for s in range(3):
        a, b = R.species[s], O.species[s]
        fields = ("x", "y", "z", "vx", "vy", "vz", "rho") + (("p", "e", "ax") if s == 0 else ("ts",))
        for f in fields:
            _close(getattr(a, f), getattr(b, f), f"{name} species {s} {f}")
    assert len(R.step_s) == nsteps and min(R.step_s) > 0.0
    assert R.phase_s["kernels"] > 0.0 and sum(R.phase_s.values()) <= sum(R.step_s)


def test_reference_kernels_track_the_fp64_path():
    ref_gpu = _ref_gpu()
    from dustyshock3d_gb300.solver import Solver
    _, P, sp = setup("refC")
    R = ref_gpu.RefGPU(P, sp).step(4)
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(4)
        got = [S.get_species(0, s) for s in range(3)]
    for s in range(3):
        for f in ("x", "vx", "rho"):
            _close(getattr(R.species[s], f), getattr(got[s], f), f"refC species {s} {f}")
    _close(R.species[0].e, got[0].e, "refC gas e")


def test_reference_kernels_refuse_extensions():
    ref_gpu = _ref_gpu()
    from dustyshock3d_gb300 import ic
    P, sp = ic.dusty_sod_tube(dx_left=1 / 32, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
    with pytest.raises(ValueError):
        ref_gpu.RefGPU(P, sp)
