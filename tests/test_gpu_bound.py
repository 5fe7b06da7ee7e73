"""Host arrays as the state of record (ds_bind_host / ds_step_host): each step
reads the bound arrays and writes back what it changed, with the transfers
overlapped with the step.  Results equal, bit for bit, the plain cycle of
ds_upload_* + ds_step(1) + ds_get_* on the same host arrays."""
import numpy as np
import pytest

from dustyshock3d_gb300 import _lib, ic
from dustyshock3d_gb300.solver import Solver

pytestmark = pytest.mark.gpu

GAS_IN = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h")
DUST_IN = ("x", "y", "z", "vx", "vy", "vz", "rho", "m", "ts", "h")
GAS_OUT = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e")
DUST_OUT = ("x", "y", "z", "vx", "vy", "vz", "rho", "ts")


def _tube(precision):
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25))
    P.precision = precision
    return P, [s.copy().fill_missing() for s in sp]


def _host_state(sp):
    """Plain numpy copies of the arrays a reference host keeps per species."""
    return [{f: getattr(s, f).copy() for f in (GAS_IN if k == 0 else DUST_IN)} | {"ind": s.ind.copy()}
            for k, s in enumerate(sp)]


def _bind(S, state, skip=()):
    """Pinned copies of the host state, bound to tube 0; returns them."""
    pinned = []
    for k, st in enumerate(state):
        arrs = {}
        for f, a in st.items():
            if f == "ind" or f in skip:
                continue
            b = S.pinned(len(a))
            b[:] = a
            arrs[f] = b
        ind = S.pinned(len(st["ind"]), np.int32)
        ind[:] = st["ind"]
        S.bind_host(0, k, arrs, ind)
        pinned.append((arrs, ind))
    return pinned


def _plain_step(S, state, species=(0, 1)):
    """ds_upload_* of the host arrays, one step, ds_get_* of what it changed."""
    from dustyshock3d_gb300.species import Species
    for k in species:
        st = state[k]
        S.set_species(0, k, Species(ind=st["ind"], **{f: a for f, a in st.items() if f != "ind"}).fill_missing())
    S.step(1)
    for k in species:
        got = S.get_species(0, k)
        for f in (GAS_OUT if k == 0 else DUST_OUT):
            state[k][f] = getattr(got, f).copy()


def _assert_state(bound, state, what):
    for k, (arrs, ind) in enumerate(bound):
        for f, a in arrs.items():
            assert np.array_equal(a, state[k][f], equal_nan=True), f"{what}: species {k} {f}"
        assert np.array_equal(ind, state[k]["ind"]), f"{what}: species {k} ind"


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_bound_steps_equal_upload_step_download(precision):
    P, sp = _tube(precision)
    ref = _host_state(sp)
    with Solver(P) as A, Solver(P) as B:
        A.set_tube(0, sp)
        B.set_tube(0, sp)
        bound = _bind(A, _host_state(sp))
        for step in range(5):
            A.step_host(1)
            _plain_step(B, ref)
            _assert_state(bound, ref, f"{precision} step {step + 1}")
        assert A.time() == B.time()
        A.step_host(3)  # several steps in one call
        for _ in range(3):
            _plain_step(B, ref)
        _assert_state(bound, ref, f"{precision} after 3 more")


def test_partial_binding_and_unbound_fields():
    """Only the gas bound (the dust stays resident); and a gas binding without
    ax, ay, az (kept on the device) equals one with them."""
    P, sp = _tube("fp32")
    ref = _host_state(sp)
    with Solver(P) as A, Solver(P) as B, Solver(P) as C:
        for S in (A, B, C):
            S.set_tube(0, sp)
        gas_a = _bind(A, _host_state(sp)[:1])
        gas_c = _bind(C, _host_state(sp)[:1], skip=("ax", "ay", "az"))
        for _ in range(4):
            A.step_host(1)
            C.step_host(1)
            _plain_step(B, ref, species=(0,))
        _assert_state(gas_a, ref[:1], "gas bound")
        for f in GAS_OUT:
            if f not in ("ax", "ay", "az"):
                assert np.array_equal(gas_c[0][0][f], ref[0][f]), f
        for f in DUST_OUT:
            assert np.array_equal(getattr(A.get_species(0, 1), f), getattr(B.get_species(0, 1), f)), f
            assert np.array_equal(getattr(C.get_species(0, 1), f), getattr(B.get_species(0, 1), f)), f


def test_host_changes_between_steps_and_resident_steps_in_between():
    """The host may edit bound arrays between calls; ds_step in between advances
    the device state, which the next bound step overwrites from the host arrays
    (they are the state of record), as the plain cycle would."""
    P, sp = _tube("fp64")
    ref = _host_state(sp)
    with Solver(P) as A, Solver(P) as B:
        A.set_tube(0, sp)
        B.set_tube(0, sp)
        bound = _bind(A, _host_state(sp))
        A.step_host(1)
        _plain_step(B, ref)
        bound[0][0]["vx"][:10] += 0.01
        ref[0]["vx"][:10] += 0.01
        A.step(1)
        B.step(1)
        A.step_host(2)
        _plain_step(B, ref)
        _plain_step(B, ref)
        _assert_state(bound, ref, "after edits and a resident step")
        assert A.time() == B.time()


def test_bind_errors():
    P, sp = _tube("fp32")
    with Solver(P) as S:
        S.set_tube(0, sp)
        with pytest.raises(_lib.DsError, match="DS_ERR_STATE"):
            S.step_host(1)
        with pytest.raises(_lib.DsError, match="pinned"):
            S.bind_host(0, 0, {"x": np.zeros(sp[0].n)})  # pageable numpy memory
        bound = _bind(S, _host_state(sp))
        S.step_host(1)
        S.bind_host(0, 0, None)
        S.bind_host(0, 1, None)
        with pytest.raises(_lib.DsError, match="DS_ERR_STATE"):
            S.step_host(1)
        L = S.L
        import ctypes
        ptrs = (ctypes.POINTER(ctypes.c_double) * 15)()
        assert L.ds_bind_host(S.ctx, 0, 0, sp[0].n + 1, ptrs, None) == 1  # wrong count
        assert L.ds_bind_host(S.ctx, 0, 5, sp[0].n, ptrs, None) == 1      # no such species


def _reuse_tube(skin):
    """A cross-section that holds the periodic stencil of cells widened by the skin."""
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.375, x_range=(-0.25, 0.25))
    P.precision = "fp32"
    P.list_skin = skin
    return P, [s.copy().fill_missing() for s in sp]


def test_bound_steps_with_list_reuse_equal_resident_steps():
    """With list reuse a bound step keeps the recorded lists and the slot order
    when the host's positions allow it, and re-sorts from the previous slot
    order otherwise, exactly as a step on the resident state: bound steps on
    unedited host arrays equal resident steps bit for bit, with the same
    rebuild decisions."""
    P, sp = _reuse_tube(0.15)
    with Solver(P) as A, Solver(P) as B:
        A.set_tube(0, sp)
        B.set_tube(0, sp)
        bound = _bind(B, _host_state(sp))
        for step in range(10):
            A.step(1)
            B.step_host(1)
            for k in range(2):
                got = A.get_species(0, k)
                for f in (GAS_OUT if k == 0 else DUST_OUT):
                    assert np.array_equal(bound[k][0][f], getattr(got, f)), f"step {step + 1} species {k} {f}"
        ra, na = A.list_stats(0)
        rb, nb = B.list_stats(0)
        assert (ra, na) == (rb, nb) and na == 10
        assert 1 <= rb < nb, (rb, nb)  # some steps kept their lists
        assert A.time() == B.time()


@pytest.mark.parametrize("field", ["h", "ind"])
def test_host_edit_of_h_or_ind_forces_a_rebuild(field):
    """The lists' cut-offs and membership assume each particle's h and Ind: a
    bound step whose host arrays changed either re-sorts and records, and its
    results stay within the FP32 path's bounds of the plain upload cycle."""
    P, sp = _reuse_tube(0.45)
    ref = _host_state(sp)
    with Solver(P) as A, Solver(P) as B:
        A.set_tube(0, sp)
        B.set_tube(0, sp)
        bound = _bind(A, _host_state(sp))
        for _ in range(3):
            A.step_host(1)
            _plain_step(B, ref)
        r0, n0 = A.list_stats(0)
        A.step_host(1)
        _plain_step(B, ref)
        r1, n1 = A.list_stats(0)
        assert n1 == n0 + 1 and r1 == r0, "the lists should be kept on an unedited step"
        i = int(np.nonzero(ref[0]["ind"] == 0)[0][len(ref[0]["ind"]) // 2])
        if field == "h":
            bound[0][0]["h"][i] *= 1.0 + 2.0 ** -40
            ref[0]["h"][i] *= 1.0 + 2.0 ** -40
        else:
            bound[0][1][i] = 1
            ref[0]["ind"][i] = 1
        A.step_host(1)
        _plain_step(B, ref)
        r2, n2 = A.list_stats(0)
        assert n2 == n1 + 1 and r2 == r1 + 1, "the edit should force a rebuild"
        for f in ("x", "vx", "rho", "e"):
            a, b = bound[0][0][f], ref[0][f]
            assert np.abs(a - b).sum() <= 1e-5 * np.abs(b).sum() + 1e-30, f


def test_partial_binding_with_list_reuse_equals_resident_steps():
    """With list reuse and only the gas bound (the dust resident), bound steps
    still equal resident steps bit for bit: the unbound dust is gathered in
    caller order with the host's gas, so the test and the sort see every
    species through the resident order."""
    P, sp = _reuse_tube(0.15)
    with Solver(P) as A, Solver(P) as B:
        A.set_tube(0, sp)
        B.set_tube(0, sp)
        gas = _bind(B, _host_state(sp)[:1])
        for step in range(8):
            A.step(1)
            B.step_host(1)
            got = A.get_species(0, 0)
            for f in GAS_OUT:
                assert np.array_equal(gas[0][0][f], getattr(got, f)), f"step {step + 1} gas {f}"
            for f in DUST_OUT:
                assert np.array_equal(getattr(B.get_species(0, 1), f), getattr(A.get_species(0, 1), f)), \
                    f"step {step + 1} dust {f}"
        assert A.list_stats(0) == B.list_stats(0)
        assert B.list_stats(0)[0] < 8
