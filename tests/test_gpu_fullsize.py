"""Size-independent properties at the benchmark sizes: the 720k + 720k dusty
Sod tube (1.44M particles) and, where cheap, the 5.76M + 5.76M tube.  The
oracle takes minutes per step there, so these check what must hold at any
size: the FP32 path tracks the FP64 path (itself bit-exact against the oracle
at small sizes), recorded force lists equal the cell walk bit for bit, a tube's
arithmetic does not depend on its batch, a checkpoint resumes bit for bit, the
bound-host step equals separate calls, the interior of a uniform tube stays
at rest, and generated initial conditions equal the host generator.  One
oracle step of the 1.44M tube takes about a second on 16 cores, so the FP64
path is also held bit-exact against the oracle there."""
import numpy as np
import pytest

from dustyshock3d_gb300 import ic
from dustyshock3d_gb300.solver import Solver

pytestmark = pytest.mark.gpu

C2 = dict(dx_left=1 / 800, Ly=0.05)      # 720,000 gas + 720,000 dust
C3 = dict(dx_left=1 / 1600, Ly=0.05)     # 5,760,000 gas + 5,760,000 dust
FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "ts", "ind")


def _solver(kw, precision="fp32", **over):
    spec = ic.DeviceIC.dusty_sod(**kw)
    P, _ = spec.plan()
    P.precision = precision
    for k, v in over.items():
        setattr(P, k, v)
    S = Solver(P)
    S.init_tube(0, spec)
    return S


def _rel_l1(a, b):
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


def _same(A, B, ta=0, tb=0, what=""):
    for s in range(2):
        a, b = A.get_species(ta, s), B.get_species(tb, s)
        for f in FIELDS:
            assert np.array_equal(getattr(a, f), getattr(b, f)), f"{what} species {s} {f}"


def test_fp32_tracks_fp64_at_1_44m():
    with _solver(C2, "fp32") as A, _solver(C2, "fp64") as B:
        A.step(10)
        B.step(10)
        assert A.time()[2] == B.time()[2] == 10
        g32, g64 = A.get_species(0, 0), B.get_species(0, 0)
        d32, d64 = A.get_species(0, 1), B.get_species(0, 1)
        assert _rel_l1(g32.rho, g64.rho) < 1e-5
        assert _rel_l1(g32.vx, g64.vx) < 2e-4
        assert _rel_l1(d32.vx, d64.vx) < 2e-4
        assert np.array_equal(g32.ind, g64.ind)


def test_force_lists_equal_walk_at_1_44m():
    with _solver(C2, force_list=0) as A, _solver(C2, force_list=-1) as B:
        A.step(3)
        B.step(3)
        _same(A, B, what="lists vs walk")


def test_batch_invariance_at_1_44m():
    small = ic.DeviceIC.dusty_sod(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25))
    spec = ic.DeviceIC.dusty_sod(**C2)
    P, _ = spec.plan()
    Ps, _ = small.plan()
    P.precision = Ps.precision = "fp32"
    with Solver([Ps, P]) as A, Solver(P) as B:
        A.init_tube(0, small)
        A.init_tube(1, spec)
        B.init_tube(0, spec)
        A.step(3)
        B.step(3)
        _same(A, B, ta=1, tb=0, what="batched vs alone")


def test_checkpoint_resume_at_1_44m(tmp_path):
    path = str(tmp_path / "c2.ckpt")
    with _solver(C2) as A:
        A.step(2)
        A.save(0, path)
        A.step(2)
        with Solver.from_checkpoint(path) as B:
            assert B.params[0].precision == "fp32"  # the parameters travel in the file
            B.step(2)
            _same(A, B, what="resumed")


def test_bound_host_step_equals_separate_calls_at_1_44m():
    names = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h")
    dnames = ("x", "y", "z", "vx", "vy", "vz", "rho", "m", "ts", "h")
    with _solver(C2) as A, _solver(C2) as B:
        arrs = []
        for s, nm in ((0, names), (1, dnames)):
            cur = A.get_species(0, s)
            a = {f: A.pinned(cur.n) for f in nm}
            for f in nm:
                a[f][:] = getattr(cur, f)
            ind = A.pinned(cur.n, np.int32)
            ind[:] = cur.ind
            A.bind_host(0, s, a, ind)
            arrs.append(a)
        A.step_host(2)
        B.step(2)
        for s, nm in ((0, names), (1, dnames)):
            b = B.get_species(0, s)
            for f in nm:
                assert np.array_equal(arrs[s][f], getattr(b, f)), (s, f)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_uniform_tube_interior_stays_at_rest_at_1_44m(precision):
    """Equal states on both sides make one continuous lattice: away from the
    walls every particle sees the same neighbourhood and every force cancels.
    (At the walls the frozen particles keep rho = 1 while their free neighbours
    sum theirs, a small pressure step that sends a wave in from each end.)"""
    with _solver(dict(C2, rho_R=1.0, p_R=1.0), precision) as S:
        S.step(5)
        vmax = 0.0
        for s in range(2):
            sp = S.get_species(0, s)
            inner = np.abs(sp.x) < 0.4
            for f in ("vx", "vy", "vz"):
                vmax = max(vmax, float(np.abs(getattr(sp, f)[inner]).max()))
        assert vmax < (1e-12 if precision == "fp64" else 1e-6), vmax


def test_fp64_path_bitexact_vs_oracle_at_1_44m():
    """The FP64 path equals the oracle (the reference's algorithm restated on
    the CPU) bit for bit on the full 1.44M-particle tube, two steps."""
    from oracle.oracle import OracleState
    from tests.test_gpu_parity import compare_exact
    P, sp = ic.dusty_sod_tube(**C2)
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(2)
        gpu = [S.get_species(0, s) for s in range(2)]
        Tm, dt, _ = S.time(0)
    O = OracleState(P, sp).step(2)
    assert Tm == O.Tm and dt == O.last_dt
    compare_exact(gpu, O.species, "1.44M tube")


def test_device_initial_conditions_at_11_5m():
    spec = ic.DeviceIC.dusty_sod(**C3)
    P, counts = spec.plan()
    assert counts == [5_760_000, 5_760_000]
    _, host = ic.dusty_sod_tube(**C3)
    with Solver(P) as S:
        S.init_tube(0, spec)
        for s in range(2):
            got = S.get_species(0, s)
            for f in FIELDS + ("m", "h"):
                assert np.array_equal(getattr(got, f), getattr(host[s], f)), (s, f)


def test_fp32_tracks_fp64_at_11_5m():
    with _solver(C3, "fp32") as A, _solver(C3, "fp64") as B:
        A.step(10)
        B.step(10)
        g32, g64 = A.get_species(0, 0), B.get_species(0, 0)
        assert _rel_l1(g32.rho, g64.rho) < 1e-5
        assert _rel_l1(g32.vx, g64.vx) < 2e-4
