"""Slab decomposition of one tube over gloo ranks on CPU (no GPU).

Each rank steps its x-slab with the CPU oracle's split step
(tests/_slab_oracle.py) through dustyshock3d_gb300.slab: ghosts within
2 h_max before the density, an allreduce(min) of the CFL candidates, the
ghosts' density and pressure from their owners before the force, migration
after the move.  On the FP64 path the slab run equals the single-domain
oracle bit for bit (every sum visits the same partners in the same order);
the conservation sums agree to FP64 rounding."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "ts")

RANK_SCRIPT = r"""
import os, sys
import numpy as np
sys.path.insert(0, {root!r})
sys.path.insert(0, os.path.join({root!r}, "tests"))
import torch.distributed as dist
dist.init_process_group("gloo")
from dustyshock3d_gb300 import ic
from dustyshock3d_gb300.slab import SlabTube, TorchComm
from _slab_oracle import OracleBackend
P, sp = ic.dusty_sod_tube(**{tube!r})
P.tau = {tau!r}
P.mode.cfl = {cfl!r}
for q in sp:
    q.vx = np.where(q.ind == 0, q.vx + {drift!r}, q.vx)
slab = SlabTube(P, sp, OracleBackend(P), TorchComm())
counts = [len(g) for g in slab.gid]
slab.step({nsteps})
out = {{}}
for s in range(len(sp)):
    g = slab.gather(s, sp[s].n)
    for f in {fields!r}:
        out[f"{{s}}_{{f}}"] = getattr(g, f)
out["cons"] = slab.conservation()
out["Tm"] = np.array([slab.time()[0]])
out["counts"] = np.array(counts)
out["migrated"] = slab.comm.allreduce_sum(np.array([float(slab.migrated)]))
if dist.get_rank() == 0:
    np.savez({path!r}, **out)
dist.barrier()
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_slabs(world, tube, nsteps, tau, cfl, drift, path):
    port = _free_port()
    script = RANK_SCRIPT.format(root=ROOT, tube=tube, nsteps=nsteps, tau=tau, cfl=cfl, drift=drift, fields=FIELDS,
                                path=path)
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
        procs.append(subprocess.Popen([sys.executable, "-c", script], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    for p in procs:
        out, err = p.communicate(timeout=600)
        assert p.returncode == 0, err[-3000:]
    return dict(np.load(path))


def single_domain(tube, nsteps, tau, cfl, drift):
    sys.path.insert(0, ROOT)
    from dustyshock3d_gb300 import ic
    from oracle.oracle import OracleState
    P, sp = ic.dusty_sod_tube(**tube)
    P.tau = tau
    P.mode.cfl = cfl
    for q in sp:
        q.vx = np.where(q.ind == 0, q.vx + drift, q.vx)
    O = OracleState(P, sp).step(nsteps)
    cons = np.zeros(5)
    for s, g in enumerate(O.species):
        cons += [g.m.sum(), (g.m * g.vx).sum(), (g.m * g.vy).sum(), (g.m * g.vz).sum(),
                 (0.5 * g.m * (g.vx ** 2 + g.vy ** 2 + g.vz ** 2)).sum() + (g.m * g.e).sum() * (s == 0)]
    return O, cons


TUBE = dict(dx_left=1 / 64, Ly=0.25, eps=1.0, t_s=1e-3, x_range=(-0.25, 0.25))


@pytest.mark.parametrize("world,cfl,drift", [(2, True, 0.0), (3, True, 0.0), (2, False, 0.0), (2, True, 1.5),
                                             (3, False, -1.5)])
def test_slabs_equal_one_domain_bit_for_bit(world, cfl, drift, tmp_path):
    """The dusty Sod tube at rest, and moving bodily (drift added to every free
    particle's vx) so that particles cross the slab bounds."""
    nsteps, tau = 10, 2e-3
    got = run_slabs(world, TUBE, nsteps, tau, cfl, drift, str(tmp_path / "slabs.npz"))
    O, cons = single_domain(TUBE, nsteps, tau, cfl, drift)
    assert len(got["counts"]) == 2 and got["counts"].sum() > 0
    if drift:
        assert got["migrated"][0] > 0, "no particle crossed a slab bound"
    assert got["Tm"][0] == O.Tm
    for s, g in enumerate(O.species):
        for f in FIELDS:
            a, b = got[f"{s}_{f}"], getattr(g, f)
            same = (a == b) | (np.isnan(a) & np.isnan(b))
            assert same.all(), f"species {s} {f}: {np.count_nonzero(~same)} of {len(a)} differ"
    # the whole-tube sums: FP64 per rank, then allreduce(sum)
    assert np.allclose(got["cons"], cons, rtol=1e-12, atol=1e-12 * np.abs(cons).max())


def test_split_columns_give_every_rank_columns():
    sys.path.insert(0, ROOT)
    from dustyshock3d_gb300.slab import split_columns
    cols = np.repeat(np.arange(10), [50, 50, 50, 50, 50, 5, 5, 5, 5, 5])
    for n in (1, 2, 3, 4, 8):
        K = split_columns(cols, n)
        owner = np.searchsorted(K, cols, side="right") - 1
        assert owner.min() == 0 and owner.max() == n - 1
        assert (np.diff(K) > 0).all()
        assert set(np.unique(owner)) == set(range(n))


def test_unsupported_modes_are_refused():
    sys.path.insert(0, ROOT)
    from dustyshock3d_gb300 import ic
    from dustyshock3d_gb300.slab import check_supported
    P, _ = ic.dusty_sod_tube(**TUBE)
    check_supported(P)
    P.mode.tstop_const = False
    with pytest.raises(ValueError, match="constant stopping times"):
        check_supported(P)
