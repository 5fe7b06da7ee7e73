"""Multi-process host logic of bench.py on CPU: two gloo ranks (no GPU).

The path does not exchange data between GPUs: a single tube runs as one
replica per rank, and the batched tubes are split over the ranks.  What the
ranks share is the timing: the slowest rank sets the whole-job rate."""
import json
import os
import socket
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, sys
sys.path.insert(0, {root!r})
import bench
ws, rank, dist = bench.dist_setup()
ms = 10.0 if rank == 0 else 25.0          # rank 1 is the slow one
rate = bench.replica_rate(dist, ws, 1000, 4, ms)
bench.barrier(dist)
print(json.dumps({{"rank": rank, "ws": ws, "rate": rate}}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_take_the_slowest_time():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    # 2 ranks x 1000 particles x 4 steps over the slower rank's 25 ms
    for o in outs:
        assert o["ws"] == 2
        assert o["rate"] == 2 * 1000 * 4 / 25e-3


def test_balanced_shards_partition_the_tubes():
    sys.path.insert(0, ROOT)
    import bench
    rng = np.random.default_rng(5)
    sizes = list(np.exp(rng.uniform(np.log(2e4), np.log(1e6), 64)).astype(int) * 2)
    for ws in (1, 2, 3, 4, 8):
        sh = bench.balanced_shards(sizes, ws)
        assert len(sh) == ws
        flat = sorted(i for s in sh for i in s)
        assert flat == list(range(64))                      # disjoint and complete
        loads = [sum(sizes[i] for i in s) for s in sh]
        # greedy largest-first: no rank above the mean by more than the largest tube
        assert max(loads) <= sum(sizes) / ws + max(sizes)
    assert bench.balanced_shards(sizes, 2) == bench.balanced_shards(sizes, 2)  # deterministic
