"""The allocation-free cell-list entry point (ds_cell_lists_noalloc).

Some callers cannot call cudaMalloc: a host that has handed all device memory
to its own pool allocator, or code running where an allocation would be an
error or would stall the device.  For them the library builds the reference's
cell lists (raw cell key, head and next pointers, kernel.cu:1937-1955) with
its scratch in a static device array instead of allocating.  These tests call
that entry point through the C ABI, twice in a row on the same inputs, and
check that it reports exactly what the allocating path reports through
ds_debug_cells (integers, so the tolerance is zero); that further calls leave
the device's free memory unchanged; and that the very first call in a fresh
process, which loads the library's device code, works the same.

The tests allocate their own input and output buffers with PyTorch; the entry
point itself allocates nothing.  Kept in its own file, collected last.
"""
import ctypes
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from dustyshock3d_gb300 import _lib, ic
from dustyshock3d_gb300.solver import Solver
from tests._golden import setup

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cases():
    g, P, sp = setup("refB")  # reference grid (aliasing key stride)
    yield "refB", P, sp
    P2, sp2 = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
    yield "periodic", P2, sp2  # proper grid with periodic y, z


def _torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


class _Buffers:
    """Caller-owned device buffers for one species: positions in, lists out."""

    def __init__(self, torch, species, ncells):
        n = species.n
        self.n = n
        self.ncells = ncells
        self.xs = [torch.tensor(getattr(species, f), dtype=torch.float64, device="cuda") for f in ("x", "y", "z")]
        self.key = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        self.nxt = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        self.head = torch.full((ncells + 1,), -7, dtype=torch.int32, device="cuda")

    def call(self, L, cp):
        return L.ds_cell_lists_noalloc(ctypes.byref(cp), self.n, self.xs[0].data_ptr(), self.xs[1].data_ptr(),
                                       self.xs[2].data_ptr(), self.key.data_ptr(), self.head.data_ptr(),
                                       self.ncells + 1, self.nxt.data_ptr(), None)


@pytest.mark.parametrize("case", ["refB", "periodic"])
def test_noalloc_cell_lists_match_allocating_path(case):
    torch = _torch_cuda()
    name, P, sp = next(c for c in _cases() if c[0] == case)
    L = _lib.load()
    with Solver(P) as S:
        S.set_tube(0, sp)
        expected = [S.debug_cells(0, s) for s in range(len(sp))]
    cp = _lib.params_to_c(P)
    bufs = [_Buffers(torch, species, expected[s]["ncells"]) for s, species in enumerate(sp)]
    for call in range(2):
        for s, b in enumerate(bufs):
            for t in (b.key, b.nxt, b.head):
                t.fill_(-7)
            torch.cuda.synchronize()
            st = b.call(L, cp)
            torch.cuda.synchronize()
            exp = expected[s]
            assert st == 0, f"call {call} species {s}: status {st}"
            assert np.array_equal(b.key.cpu().numpy(), exp["cell_key"]), f"call {call} species {s}: cell keys"
            assert np.array_equal(b.head.cpu().numpy(), exp["head"]), f"call {call} species {s}: heads"
            assert np.array_equal(b.nxt.cpu().numpy(), exp["next"]), f"call {call} species {s}: next pointers"
    # Every buffer exists already; further calls must not change the device's free memory.
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        for b in bufs:
            assert b.call(L, cp) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before, "the entry point changed the device's free memory"


# Run in a fresh process: the entry point is the first call of this library on
# the device (its device code and static array are loaded by it), then called
# again; the free device memory must not move across the later calls.
_FRESH = r"""
import ctypes, sys
import numpy as np
import torch
from dustyshock3d_gb300 import _lib, ic
P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))
ncells = int(sys.argv[2])
L = _lib.load()
cp = _lib.params_to_c(P)
g = sp[0]
xs = [torch.tensor(getattr(g, f), dtype=torch.float64, device="cuda") for f in ("x", "y", "z")]
key = torch.full((g.n,), -7, dtype=torch.int32, device="cuda")
nxt = torch.full((g.n,), -7, dtype=torch.int32, device="cuda")
head = torch.full((ncells + 1,), -7, dtype=torch.int32, device="cuda")
def call():
    return L.ds_cell_lists_noalloc(ctypes.byref(cp), g.n, xs[0].data_ptr(), xs[1].data_ptr(), xs[2].data_ptr(),
                                   key.data_ptr(), head.data_ptr(), ncells + 1, nxt.data_ptr(), None)
torch.cuda.synchronize()
st = [call()]
torch.cuda.synchronize()
first = (key.cpu().numpy(), head.cpu().numpy(), nxt.cpu().numpy())
free0 = torch.cuda.mem_get_info()[0]
for _ in range(4):
    st.append(call())
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
np.savez(sys.argv[1], status=np.array(st), key=first[0], head=first[1], next=first[2],
         key2=key.cpu().numpy(), head2=head.cpu().numpy(), next2=nxt.cpu().numpy(), free=np.array([free0, free1]))
"""


def test_noalloc_first_call_in_fresh_process():
    _torch_cuda()
    name, P, sp = next(c for c in _cases() if c[0] == "periodic")
    with Solver(P) as S:
        S.set_tube(0, sp)
        exp = S.debug_cells(0, 0)
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "fresh.npz")
        env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
        r = subprocess.run([sys.executable, "-c", _FRESH, out, str(exp["ncells"])], cwd=ROOT, env=env,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, f"fresh process failed:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}"
        got = dict(np.load(out))
    assert (got["status"] == 0).all(), f"statuses {got['status']}"
    for sfx in ("", "2"):  # the cold first call, and the last of the calls after it
        assert np.array_equal(got["key" + sfx], exp["cell_key"]), f"cell keys{sfx}"
        assert np.array_equal(got["head" + sfx], exp["head"]), f"heads{sfx}"
        assert np.array_equal(got["next" + sfx], exp["next"]), f"next pointers{sfx}"
    assert got["free"][0] == got["free"][1], "the entry point changed the device's free memory"


def test_noalloc_rejects_oversize_and_short_head():
    L = _lib.load()
    P, sp = ic.dusty_sod_tube(dx_left=1 / 64, Ly=0.25, x_range=(-0.25, 0.25))
    cp = _lib.params_to_c(P)
    too_many = 262144 + 1
    assert L.ds_cell_lists_noalloc(ctypes.byref(cp), too_many, 1, 1, 1, 1, 1, 10 ** 6, 1, None) == 1
    assert L.ds_cell_lists_noalloc(ctypes.byref(cp), 10, 1, 1, 1, 1, 1, 1, 1, None) == 1
