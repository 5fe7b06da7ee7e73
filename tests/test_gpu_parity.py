"""CUDA path against the oracle and the reference's own snapshots (needs a GPU).

Bit-exactness claims:
  * cell keys, the reference's linked lists (head / next) and per-particle
    candidate / in-range counts equal the oracle's exactly (integers);
  * the FP64 path equals the oracle bit for bit after N steps (same operation
    and summation order, no FMA contraction) -- floats compared with ==;
  * the FP32 path is compared with a stated tolerance.
"""
import dataclasses

import numpy as np
import pytest

from dustyshock3d_gb300 import ic
from dustyshock3d_gb300.solver import Solver
from oracle.oracle import OracleState
from tests._golden import NAMES, assert_close_nan, setup, snapshot_steps

pytestmark = pytest.mark.gpu

GAS_F = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e")
DUST_F = ("x", "y", "z", "vx", "vy", "vz", "rho", "ts")


def run_gpu(P, species, nsteps):
    with Solver(P) as S:
        S.set_tube(0, species)
        if nsteps:
            S.step(nsteps)
        out = [S.get_species(0, s) for s in range(len(species))]
        t = S.time(0)
    return out, t


def assert_equal_nan(a, b, what):
    a = np.asarray(a); b = np.asarray(b)
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    if not same.all():
        bad = np.nonzero(~same)[0]
        err = np.nanmax(np.abs(a[bad] - b[bad])) if len(bad) else 0
        raise AssertionError(f"{what}: {len(bad)} of {len(a)} differ (max |diff| {err:.3e}), first {bad[:5]}")


def compare_exact(gpu, orc, tag):
    for f in GAS_F:
        assert_equal_nan(getattr(gpu[0], f), getattr(orc[0], f), f"{tag} gas {f}")
    for k in range(1, len(orc)):
        for f in DUST_F:
            assert_equal_nan(getattr(gpu[k], f), getattr(orc[k], f), f"{tag} dust{k} {f}")
    assert (gpu[0].ind == orc[0].ind).all()


@pytest.mark.parametrize("name", NAMES)
def test_lists_and_counts_bitexact(name):
    g, P, sp = setup(name)
    O = OracleState(P, sp)
    with Solver(P) as S:
        S.set_tube(0, sp)
        for s in range(3):
            dbg = S.debug_cells(0, s)
            head, nxt = O.lists(s)
            assert (dbg["cell_key"] == O.cell_keys(s)).all(), f"species {s} cell keys"
            assert dbg["ncells"] + 1 == len(head)
            assert (dbg["head"] == head).all(), f"species {s} list heads"
            assert (dbg["next"] == nxt).all(), f"species {s} next pointers"
            nc, nn = O.neighbour_counts(s)
            assert (dbg["ncand"] == nc).all(), f"species {s} candidate counts"
            assert (dbg["nnb"] == nn).all(), f"species {s} in-range counts"
        # lists again after two steps (particles have moved)
        S.step(2)
        O.step(2)
        for s in range(3):
            dbg = S.debug_cells(0, s)
            head, nxt = O.lists(s)
            assert (dbg["head"] == head).all() and (dbg["next"] == nxt).all()


@pytest.mark.parametrize("name,nsteps", [("refA", 3), ("refB", 10), ("refC", 10)])
def test_reference_mode_fp64_bitexact(name, nsteps):
    g, P, sp = setup(name)
    gpu, (Tm, dt, ns) = run_gpu(P, sp, nsteps)
    O = OracleState(P, sp).step(nsteps)
    assert ns == nsteps
    assert Tm == O.Tm
    compare_exact(gpu, O.species, name)


def test_nonfinite_flag_marks_the_reference_nan_onset():
    """refA turns NaN at its third step (the reference's eps_2 guard defect,
    kernel.cu:2203).  DS_FLAG_NONFINITE is clear while the oracle's moving
    particles stay finite and set from the step where one of their velocities,
    positions or energies first is not."""
    g, P, sp = setup("refA")
    O = OracleState(P, sp)
    seen = False
    with Solver(P) as S:
        S.set_tube(0, sp)
        for _ in range(5):
            S.step(1)
            O.step(1)
            for k, q in enumerate(O.species):
                m = q.ind == 0
                fields = [q.vx, q.vy, q.vz, q.x, q.y, q.z] + ([q.e] if k == 0 else [])
                seen = seen or not all(np.isfinite(f[m]).all() for f in fields)
            assert bool(S.device_flags() & 4) == seen
            if seen:
                break
    assert seen


@pytest.mark.parametrize("name", NAMES)
def test_gpu_replays_reference_snapshots(name):
    """The CUDA path against what the reference program itself printed."""
    g, P, sp = setup(name)
    nsnap = len(g["snap_times"])
    steps = snapshot_steps(P, nsnap)
    interior = g["ind"] == 0
    with Solver(P) as S:
        S.set_tube(0, sp)
        done = 0
        for s, target in enumerate(steps, start=1):
            S.step(target - done)
            done = target
            gas = S.get_species(0, 0)
            for col, arr in (("x", gas.x), ("rho", gas.rho), ("p", gas.p), ("Vx", gas.vx), ("Vy", gas.vy),
                             ("e", gas.e)):
                assert_close_nan(arr[interior], g[f"s{s}_gas_{col}"], 1e-8, f"{name} s{s} gas {col}")
            for k in (1, 2):
                d = S.get_species(0, k)
                for col, arr in (("x", d.x), ("rho", d.rho), ("t_stop", d.ts), ("Vx", d.vx)):
                    assert_close_nan(arr[interior], g[f"s{s}_d{k}_{col}"], 1e-8, f"{name} s{s} dust{k} {col}")


def small_tube(**kw):
    args = dict(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
    args.update(kw)
    return ic.dusty_sod_tube(**args)


@pytest.mark.parametrize("eps,t_s", [(1.0, 1e-3), (0.01, 1e-1), (10.0, 1e-4)])
def test_baseline_mode_fp64_bitexact(eps, t_s):
    P, sp = small_tube(eps=eps, t_s=t_s)
    gpu, (Tm, dt, ns) = run_gpu(P, sp, 6)
    O = OracleState(P, sp).step(6)
    assert Tm == O.Tm and dt == O.last_dt
    compare_exact(gpu, O.species, f"eps={eps} ts={t_s}")


def test_baseline_lists_and_counts_bitexact():
    P, sp = small_tube()
    O = OracleState(P, sp).step(3)
    with Solver(P) as S:
        S.set_tube(0, O.species)
        for s in range(2):
            dbg = S.debug_cells(0, s)
            head, nxt = O.lists(s)
            assert (dbg["cell_key"] == O.cell_keys(s)).all()
            assert (dbg["head"] == head).all() and (dbg["next"] == nxt).all()
            nc, nn = O.neighbour_counts(s)
            assert (dbg["ncand"] == nc).all() and (dbg["nnb"] == nn).all()


@pytest.mark.parametrize("stencil,cell_factor", [(2, 1.001), (3, 0.6673), (4, 0.5005)])
def test_fp32_path_against_fp64_oracle(stencil, cell_factor):
    """FP32 sweeps (Kahan sums, FP32 positions relative to cell / x-block
    origins, row walks) vs the FP64 oracle on its own grid: relative L1 of gas
    density <= 1e-5 after 10 steps, velocities <= 1e-4 of the velocity scale.
    Smaller cells with wider stencils (cells of h_max / 2, up to 9 cells per
    side for the right state's longer cut-off) give the same physics."""
    P, sp = small_tube()
    P32 = P.copy()
    P32.precision = "fp32"
    P32.stencil = stencil
    P32.cell_w = cell_factor * P.h
    gpu, _ = run_gpu(P32, sp, 10)
    O = OracleState(P, sp).step(10)
    g, o = gpu[0], O.species[0]
    l1 = np.abs(g.rho - o.rho).sum() / np.abs(o.rho).sum()
    assert l1 < 1e-5, l1
    vscale = np.abs(o.vx).max()
    assert np.abs(g.vx - o.vx).mean() / vscale < 1e-4
    assert np.abs(gpu[1].vx - O.species[1].vx).mean() / vscale < 1e-4


@pytest.mark.parametrize("cap,stencil", [(0, 2), (100, 2), (8, 2), (0, 4), (100, 4)])
def test_fp32_force_lists_equal_walk(cap, stencil):
    """The FP32 force sweep over the neighbours recorded by the density sweep
    equals the force sweep's own cell walk bit for bit: every chunk listed
    (0 -> 256 entries), listed and walked chunks mixed (100: interior gas has
    ~80 neighbours, gas at the contact and in the shock more), every chunk
    walked (8)."""
    P, sp = small_tube()
    P.precision = "fp32"
    if stencil == 4:
        P.stencil, P.cell_w = 4, 0.5005 * P.h
    Pw = P.copy()
    Pw.force_list = -1
    walk, tw = run_gpu(Pw, sp, 8)
    Pl = P.copy()
    Pl.force_list = cap
    listed, tl = run_gpu(Pl, sp, 8)
    assert tw == tl
    compare_exact(listed, walk, f"force_list={cap}")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_dust_density_on_demand(precision):
    """ds_dust_density after N steps without the per-step dust sweep equals the
    oracle's dust self-density at the same positions (the oracle computes it
    at the start of its next step, from the GPU's state): bit for bit on the
    FP64 path, relative L1 <= 1e-6 on the FP32 path."""
    P, sp = small_tube()
    P.precision = precision
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(5)
        S.dust_density()
        g = S.get_species(0, 0)
        d = S.get_species(0, 1)
    g.m, g.h = sp[0].m, sp[0].h
    d.m, d.h = sp[1].m, sp[1].h
    Q = P.copy()
    Q.precision = "fp64"
    Q.mode = dataclasses.replace(P.mode, dust_rho=True)
    O = OracleState(Q, [g, d]).step(1)
    ref = O.species[1].rho
    if precision == "fp64":
        assert_equal_nan(d.rho, ref, "dust rho")
    else:
        assert np.abs(d.rho - ref).sum() / np.abs(ref).sum() < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_checkpoint_resume(precision, tmp_path):
    """5 steps, checkpoint, a new solver from the file, 5 more steps = 10 steps
    straight: bit for bit on the FP64 path (the step order depends only on the
    caller order), relative L1 <= 1e-6 on the FP32 path (its cells keep their
    previous slot order, which the checkpoint does not carry)."""
    P, sp = small_tube()
    P.precision = precision
    path = str(tmp_path / "tube.ckpt")
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(5)
        S.save(0, path)
        t_saved = S.time(0)
        S.step(5)
        straight = [S.get_species(0, s) for s in range(2)]
        t_straight = S.time(0)
    R = Solver.from_checkpoint(path)
    try:
        t0 = R.time(0)
        assert t0[0] == t_saved[0] and t0[2] == 5
        R.step(5)
        resumed = [R.get_species(0, s) for s in range(2)]
        t_resumed = R.time(0)
    finally:
        R.close()
    assert t_resumed[0] == t_straight[0] and t_resumed[2] == t_straight[2] == 10
    for s in range(2):
        for f in ("x", "vx", "rho"):
            a, b = getattr(resumed[s], f), getattr(straight[s], f)
            if precision == "fp64":
                assert_equal_nan(a, b, f"species {s} {f}")
            else:
                assert np.abs(a - b).sum() / np.abs(b).sum() < 1e-6, (s, f)


def test_checkpoint_with_other_run_parameters_is_refused(tmp_path):
    """A checkpoint saved under other physics (here another stopping time, then
    another h layout) is DS_ERR_ARG, and the tube keeps its own state."""
    P, sp = small_tube()
    path = str(tmp_path / "tube.ckpt")
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(2)
        S.save(0, path)
    for other in (small_tube(t_s=1e-2), small_tube(h_factor=1.2)):
        P2, sp2 = other
        with Solver(P2) as S:
            S.set_tube(0, sp2)
            S.step(1)
            before = [S.get_species(0, s) for s in range(2)]
            assert S.L.ds_load_tube(S.ctx, 0, path.encode()) == 1
            after = [S.get_species(0, s) for s in range(2)]
            for s in range(2):
                for f in ("x", "vx", "rho"):
                    assert_equal_nan(getattr(after[s], f), getattr(before[s], f), f"species {s} {f}")


def test_batched_tubes_equal_single_runs():
    cases = [small_tube(eps=1.0, t_s=1e-3), small_tube(eps=0.1, t_s=1e-2, rho_R=0.25, p_R=0.2),
             small_tube(dx_left=1 / 48, Ly=0.375, eps=3.0, t_s=3e-4)]
    with Solver([c[0] for c in cases]) as S:
        for t, (P, sp) in enumerate(cases):
            S.set_tube(t, sp)
        S.step(5)
        batched = [[S.get_species(t, s) for s in range(2)] for t in range(len(cases))]
    for t, (P, sp) in enumerate(cases):
        alone, _ = run_gpu(P, sp, 5)
        compare_exact(batched[t], alone, f"tube {t}")


def test_time_loop_stops_at_t_end():
    P, sp = small_tube()
    P.T_end = 0.02
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(100)
        Tm, dt, ns = S.time(0)
    assert Tm == pytest.approx(0.02, rel=0, abs=1e-15) and ns < 100


def test_upload_download_roundtrip_preserves_order():
    P, sp = small_tube()
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(1)
        a = S.get_species(0, 0)
        # upload the downloaded state again; one more step must equal two steps straight
        S2 = Solver(P)
        S2.set_tube(0, sp)
        S2.step(2)
        b = S2.get_species(0, 0)
        S2.close()
        a.m, a.h = sp[0].m, sp[0].h
        d = S.get_species(0, 1)
        d.m, d.h = sp[1].m, sp[1].h
        S.set_tube(0, [a, d])
        S.step(1)
        c = S.get_species(0, 0)
    for f in ("x", "vx", "rho", "e"):
        assert_equal_nan(getattr(c, f), getattr(b, f), f)


@pytest.mark.parametrize("source", ["host", "device"])
@pytest.mark.parametrize("name", ["refB", "refC"])
def test_snapshot_files_replay_the_reference_output(name, source, tmp_path):
    """The reference-format snapshot files written from the GPU state at the
    reference's output steps hold what the reference program printed: every
    column of every interior particle to the printed 8 decimals, and its cell
    lists (the Nn column, from the lists of the step) exactly.  source
    "device": the initial particles are generated on the device from the same
    Init.txt (ds_init_tube, init_Sod_X_Dust) instead of uploaded."""
    g, P, sp = setup(name)
    nsnap = len(g["snap_times"])
    steps = snapshot_steps(P, nsnap)
    cols_g = ["x", "y", "z", "r", "mas", "rho", "p", "Vx", "Vy", "Vy2", "V", "e", "Ind", "Nn"]
    cols_d = ["x", "y", "z", "r", "mas", "rho", "t_stop", "Vx", "Vy", "Vy2", "V", "Ind", "Nn"]
    interior = g["ind"] == 0

    def read(path):
        with open(path) as f:
            lines = f.read().splitlines()
        return lines, np.array([[float(v) for v in ln.split()] for ln in lines[3:] if ln.strip()])

    if source == "device":
        from dustyshock3d_gb300 import ic, parse_init_txt
        spec = ic.DeviceIC(kind="sod_x_dust")
        P = spec.plan(parse_init_txt(str(g["init_txt"])))[0]
    with Solver(P) as S:
        if source == "device":
            S.init_tube(0, spec)
        else:
            S.set_tube(0, sp)
        done = 0
        for s, st in enumerate(steps, start=1):
            S.step(st - done)
            done = st
            S.write_snapshot(str(tmp_path), s)
            lines, G = read(tmp_path / f"G{s:07d}.dat")
            assert lines[0] == f"t={g['snap_times'][s - 1]:5.3f} "
            assert (G[:, cols_g.index("Nn")].astype(np.int32) == g[f"s{s}_gas_Nn"]).all()
            for c in ("x", "y", "z", "rho", "p", "Vx", "Vy", "V", "e"):
                assert_close_nan(G[interior, cols_g.index(c)], g[f"s{s}_gas_{c}"], 1.01e-8, f"{name} s{s} G {c}")
            for k in (1, 2):
                _, D = read(tmp_path / f"D-{k}-{s:07d}.dat")
                assert (D[:, cols_d.index("Nn")].astype(np.int32) == g[f"s{s}_d{k}_Nn"]).all()
                for c in ("x", "y", "z", "rho", "t_stop", "Vx", "Vy", "V"):
                    assert_close_nan(D[interior, cols_d.index(c)], g[f"s{s}_d{k}_{c}"], 1.01e-8,
                                     f"{name} s{s} D-{k} {c}")
            assert (tmp_path / f"L_X{s:07d}.dat").exists() and (tmp_path / f"D-2-L_X{s:07d}.dat").exists()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pinned_upload_download_equal_pageable(precision):
    """Pinned (mapped) host buffers take the in-place kernels, pageable ones the
    copy engines; both give the same state bit for bit."""
    import ctypes

    from dustyshock3d_gb300 import _lib
    P, sp = small_tube()
    P.precision = precision
    L = _lib.load()
    keep = []

    def pinned_copy(a):
        ptr = ctypes.c_void_p()
        assert L.ds_host_alloc(ctypes.byref(ptr), a.nbytes) == 0
        keep.append(ptr)
        out = np.frombuffer((ctypes.c_char * a.nbytes).from_address(ptr.value), dtype=a.dtype, count=a.size)
        out[:] = a
        return out

    fields = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h", "ts")
    try:
        results = []
        for pin in (False, True):
            with Solver(P) as S:
                S.set_tube(0, sp)
                S.step(2)
                got = [S.get_species(0, s) for s in range(2)]
                if pin:  # re-upload the state from pinned buffers, then step on
                    for s in range(2):
                        q = got[s]
                        for f in fields:
                            setattr(q, f, pinned_copy(getattr(q, f)))
                        q.ind = pinned_copy(q.ind)
                        S.set_species(0, s, q)
                else:
                    for s in range(2):
                        S.set_species(0, s, got[s])
                S.step(2)
                out = []
                for s in range(2):
                    n = S.n[0][s]
                    bufs = {f: (pinned_copy(np.zeros(n)) if pin else np.zeros(n)) for f in fields}
                    ind = pinned_copy(np.zeros(n, np.int32)) if pin else np.zeros(n, np.int32)
                    ptrs = (ctypes.POINTER(ctypes.c_double) * 15)(
                        *[bufs[f].ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for f in fields])
                    assert L.ds_get_fields(S.ctx, 0, s, ptrs, ind.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == 0
                    out.append({**{f: bufs[f].copy() for f in fields}, "ind": ind.copy()})
                results.append(out)
        for s in range(2):
            for f in fields + ("ind",):
                assert_equal_nan(results[1][s][f], results[0][s][f], f"species {s} {f}")
    finally:
        for p in keep:
            L.ds_host_free(p)


@pytest.mark.parametrize("name", ["refB", "refC"])
def test_fp32_path_with_reference_physics(name):
    """The FP32 path needs the proper cell grid; with it, the reference's other
    semantics (index-coupled t_stop, the species-1 eps guard, the 2-species
    solve order, dust self-density every step) run on it.  After 10 steps it
    is within the FP32 bound of the FP64 oracle on the same grid (relative L1
    of gas rho <= 1e-5, velocities <= 1e-4 of their scale).  On the
    reference's aliasing grid the FP32 path is refused."""
    from dustyshock3d_gb300 import _lib
    g, P, sp = setup(name)
    bad = P.copy()
    bad.precision = "fp32"
    with pytest.raises(_lib.DsError, match="DS_ERR_UNSUPPORTED"):
        Solver(bad)
    P.mode = dataclasses.replace(P.mode, grid_proper=True)
    P32 = P.copy()
    P32.precision = "fp32"
    gpu, _ = run_gpu(P32, sp, 10)
    O = OracleState(P, sp).step(10)
    gg, o = gpu[0], O.species[0]
    assert np.abs(gg.rho - o.rho).sum() / np.abs(o.rho).sum() < 1e-5
    vscale = np.abs(o.vx).max()
    assert np.abs(gg.vx - o.vx).mean() / vscale < 1e-4
    for k in (1, 2):
        assert np.abs(gpu[k].vx - O.species[k].vx).mean() / max(np.abs(O.species[k].vx).max(), 1e-30) < 1e-4
