"""Slab decomposition on the CUDA library (needs a GPU).

Two or three gloo ranks, each stepping its x-slab of one tube on cuda:0
through the library's split step (ds_step_density, ds_get/set_cfl_min,
ds_set_gas_hydro, ds_step_complete) with dustyshock3d_gb300.slab's
SolverBackend (a fixed-capacity context, unused slots parked past the tube's
end).  The ranks exchange through the host only; no kernel of one rank waits
for another's.  FP64: the slab run equals the single-domain oracle bit for
bit.  FP32: within the FP32 path's own bounds of the single-domain FP32 run."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "ts")
TUBE = dict(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))

RANK_SCRIPT = r"""
import os, sys
import numpy as np
sys.path.insert(0, {root!r})
import torch.distributed as dist
dist.init_process_group("gloo")
from dustyshock3d_gb300 import ic
from dustyshock3d_gb300.slab import SlabTube, SolverBackend, TorchComm
P, sp = ic.dusty_sod_tube(**{tube!r})
P.precision = {precision!r}
for q in sp:
    q.vx = np.where(q.ind == 0, q.vx + {drift!r}, q.vx)
B = SolverBackend(P)
slab = SlabTube(P, sp, B, TorchComm())
slab.step({nsteps})
out = {{}}
for s in range(len(sp)):
    g = slab.gather(s, sp[s].n)
    for f in {fields!r}:
        out[f"{{s}}_{{f}}"] = getattr(g, f)
out["Tm"] = np.array([slab.time()[0]])
out["migrated"] = slab.comm.allreduce_sum(np.array([float(slab.migrated)]))
B.close()
if dist.get_rank() == 0:
    np.savez({path!r}, **out)
dist.barrier()
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_slabs(world, precision, nsteps, drift, path):
    port = _free_port()
    script = RANK_SCRIPT.format(root=ROOT, tube=TUBE, precision=precision, nsteps=nsteps, drift=drift,
                                fields=FIELDS, path=path)
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", script], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    for p in procs:
        out, err = p.communicate(timeout=900)
        assert p.returncode == 0, err[-3000:]
    return dict(np.load(path))


def one_domain(precision, nsteps, drift):
    from dustyshock3d_gb300 import ic
    from dustyshock3d_gb300.solver import Solver
    P, sp = ic.dusty_sod_tube(**TUBE)
    P.precision = precision
    for q in sp:
        q.vx = np.where(q.ind == 0, q.vx + drift, q.vx)
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(nsteps)
        return [S.get_species(0, s) for s in range(len(sp))], S.time(0)[0]


@pytest.mark.parametrize("world,drift", [(2, 0.0), (3, 1.5)])
def test_fp64_slabs_equal_one_domain_bit_for_bit(world, drift, tmp_path):
    nsteps = 8
    got = run_slabs(world, "fp64", nsteps, drift, str(tmp_path / "s.npz"))
    ref, Tm = one_domain("fp64", nsteps, drift)
    assert got["Tm"][0] == Tm
    if drift:
        assert got["migrated"][0] > 0
    for s, g in enumerate(ref):
        for f in FIELDS:
            a, b = got[f"{s}_{f}"], getattr(g, f)
            same = (a == b) | (np.isnan(a) & np.isnan(b))
            assert same.all(), f"species {s} {f}: {np.count_nonzero(~same)} of {len(a)} differ"


def test_fp32_slabs_track_one_domain(tmp_path):
    nsteps = 8
    got = run_slabs(2, "fp32", nsteps, 0.0, str(tmp_path / "s.npz"))
    ref, Tm = one_domain("fp32", nsteps, 0.0)
    assert abs(got["Tm"][0] - Tm) <= 1e-6 * Tm
    g = ref[0]
    l1 = np.abs(got["0_rho"] - g.rho).sum() / np.abs(g.rho).sum()
    assert l1 < 1e-5, l1
    vscale = np.abs(g.vx).max()
    assert np.abs(got["0_vx"] - g.vx).mean() / vscale < 1e-4
    assert np.abs(got["1_vx"] - ref[1].vx).mean() / vscale < 1e-4


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_split_step_equals_one_step_and_refuses_calls_out_of_order(precision):
    """ds_step_density + ds_step_complete with the CFL minimum read and written
    back equal one ds_step bit for bit; calls out of order are refused with
    DS_ERR_STATE and leave the step usable."""
    from dustyshock3d_gb300 import ic
    from dustyshock3d_gb300._lib import DsError
    from dustyshock3d_gb300.solver import Solver
    P, sp = ic.dusty_sod_tube(**TUBE)
    P.precision = precision
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(2)
        ref = [S.get_species(0, s) for s in range(2)], S.time(0)
    with Solver(P) as S:
        S.set_tube(0, sp)
        with pytest.raises(DsError, match="DS_ERR_STATE"):
            S.step_complete()
        for _ in range(2):
            S.step_density()
            with pytest.raises(DsError, match="DS_ERR_STATE"):
                S.step(1)
            with pytest.raises(DsError, match="DS_ERR_STATE"):
                S.step_density()
            with pytest.raises(DsError, match="DS_ERR_STATE"):
                S.set_tube(0, sp)
            dtmin = S.cfl_min(0)
            assert dtmin > 0
            S.set_cfl_min(0, dtmin)
            S.step_complete()
        with pytest.raises(DsError, match="DS_ERR_STATE"):
            S.set_cfl_min(0, 1.0)
        got = [S.get_species(0, s) for s in range(2)], S.time(0)
    assert got[1] == ref[1]
    for s in range(2):
        for f in FIELDS:
            assert np.array_equal(getattr(got[0][s], f), getattr(ref[0][s], f)), (s, f)
