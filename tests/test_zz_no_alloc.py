"""The allocation-free cell-list entry point (ds_cell_lists_noalloc).

Some callers cannot call cudaMalloc: a host that has handed all device memory
to its own pool allocator, or code running where an allocation would be an
error or would stall the device.  For them the library builds the reference's
cell lists (raw cell key, head and next pointers, kernel.cu:1937-1955) with
its scratch in a static device array instead of allocating.  This test calls
that entry point through the C ABI, twice in a row on the same inputs, and
checks that it reports exactly what the allocating path reports through
ds_debug_cells (integers, so the tolerance is zero).

The test allocates its own input and output buffers with PyTorch; the entry
point itself allocates nothing.  Kept in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

from dustyshock3d_gb300 import _lib, ic
from dustyshock3d_gb300.solver import Solver
from tests._golden import setup

pytestmark = pytest.mark.gpu


def _cases():
    g, P, sp = setup("refB")  # reference grid (aliasing key stride)
    yield "refB", P, sp
    P2, sp2 = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
    yield "periodic", P2, sp2  # proper grid with periodic y, z


@pytest.mark.parametrize("case", ["refB", "periodic"])
def test_noalloc_cell_lists_match_allocating_path(case):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    name, P, sp = next(c for c in _cases() if c[0] == case)
    L = _lib.load()
    with Solver(P) as S:
        S.set_tube(0, sp)
        expected = [S.debug_cells(0, s) for s in range(len(sp))]
    cp = _lib.params_to_c(P)
    for call in range(2):
        for s, species in enumerate(sp):
            n = species.n
            exp = expected[s]
            xs = [torch.tensor(getattr(species, f), dtype=torch.float64, device="cuda") for f in ("x", "y", "z")]
            key = torch.full((n,), -7, dtype=torch.int32, device="cuda")
            nxt = torch.full((n,), -7, dtype=torch.int32, device="cuda")
            head = torch.full((exp["ncells"] + 1,), -7, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            st = L.ds_cell_lists_noalloc(ctypes.byref(cp), n, xs[0].data_ptr(), xs[1].data_ptr(), xs[2].data_ptr(),
                                         key.data_ptr(), head.data_ptr(), exp["ncells"] + 1, nxt.data_ptr(), None)
            torch.cuda.synchronize()
            assert st == 0, f"call {call} species {s}: status {st}"
            assert np.array_equal(key.cpu().numpy(), exp["cell_key"]), f"call {call} species {s}: cell keys"
            assert np.array_equal(head.cpu().numpy(), exp["head"]), f"call {call} species {s}: heads"
            assert np.array_equal(nxt.cpu().numpy(), exp["next"]), f"call {call} species {s}: next pointers"


def test_noalloc_rejects_oversize_and_short_head():
    L = _lib.load()
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25))
    cp = _lib.params_to_c(P)
    too_many = 262144 + 1
    assert L.ds_cell_lists_noalloc(ctypes.byref(cp), too_many, 1, 1, 1, 1, 1, 10 ** 6, 1, None) == 1
    assert L.ds_cell_lists_noalloc(ctypes.byref(cp), 10, 1, 1, 1, 1, 1, 1, 1, None) == 1
