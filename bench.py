#!/usr/bin/env python3
"""Benchmark: particle-steps/s of the dusty-gas SPH + IDIC step on one GB300.

Workload (default): the 720k gas + 720k dust dusty Sod shock tube (left
dx = 1/800, cross-section 0.05 x 0.05, eps = 1, t_s = 1e-3, h = 1.3 local dx,
CFL 0.3, periodic y/z), synthetic lattice initial conditions.  A step is one
time step of every particle.  The state (~370 MB resident) is larger than L2,
so no flush is needed between timed steps.

Reported (one JSON line from rank 0):
  value      FP32 path (FP32 neighbour sums, Kahan; FP64 state, IDIC, sums),
             device-resident, CUDA events around exactly --steps replays of
             the step graphs ds_step runs (phases from a second pass)
  fp64       the plain FP64 path (reference operation order) on the same tube
  l1_*       L1 error of the FP32 path against the FP64 path after the run
  e2e        the same metric through the C ABI with host buffers: the pinned
             host arrays are bound once (ds_bind_host) and each step
             (ds_step_host) reads all of them and writes back what the step
             changed; separate_calls: ds_upload_* + ds_step + ds_download_*
  roofline   the gas density sweep (dominant kernel): compulsory bytes / duration
  cpu_baseline  the FP64 CPU oracle (OpenMP, all host cores) on a bounded sample
  reference_gpu the reference's own CUDA kernels (compiled unmodified into a
             cubin where the reference tree exists) under a restatement of its
             host loop, on its default run, beside the FP64 path on that run
  serve      the served stream: 64 Poisson requests, continuous batching,
             p50 / p99 time to solution (--workload serve adds comparators)

--impl reference times the reference algorithm on the host cores (the oracle,
a CPU restatement of the reference's step).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Batched and served workloads (not the default line): 64 seeded uneven tubes,
# and a Poisson stream of such tubes under a 150 GB budget.
EXTRA_WORKLOADS = ("batch64", "serve", "accuracy_720k", "initial_conditions", "reference_init")

WORKLOADS = {
    # name: (dx_left, Ly, description)
    "dusty_sod_720k": (1 / 800, 0.05, "dusty Sod tube, 720k gas + 720k dust (left dx 1/800, 0.05^2 cross-section)"),
    "dusty_sod_45k": (1 / 200, 0.1, "dusty Sod tube, 45k gas + 45k dust (left dx 1/200, 0.1^2 cross-section)"),
    "dusty_sod_5760k": (1 / 1600, 0.05, "dusty Sod tube, 5.76M gas + 5.76M dust (left dx 1/1600, 0.05^2)"),
}
DEFAULT_WORKLOAD = "dusty_sod_720k"
DEFAULT_SKIN = 0.15  # list reuse of the FP32 legs (units of h)
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS) + list(EXTRA_WORKLOADS))
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--rate", type=float, default=4.0, help="serve: mean arrivals per second")
    ap.add_argument("--requests", type=int, default=64, help="serve: number of requests")
    ap.add_argument("--compare", type=int, default=16,
                    help="serve: requests (first by arrival) also served alone and solved one at a time")
    ap.add_argument("--host-ic", action="store_true",
                    help="serve: make initial particles on the host and upload them (default: on the device)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-c3", action="store_true", help="default line: skip the 11.5M-particle tube record")
    ap.add_argument("--no-batch", action="store_true", help="default line: skip the 64-tube batch record")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="default line: skip the reference's own CUDA kernels on its default run")
    ap.add_argument("--no-serve", action="store_true",
                    help="default line: skip the served stream (64 Poisson requests, no comparators)")
    ap.add_argument("--t-end", type=float, default=0.2, help="accuracy_720k: end time of every run")
    ap.add_argument("--list-skin", type=float, default=DEFAULT_SKIN,
                    help="FP32 legs of the default line: reuse the recorded neighbour lists across steps with this "
                         "skin (units of h; 0: off).  0.15 measured fastest on the 720k tube, device-resident and "
                         "end to end")
    return ap.parse_args()


def make_tube(name, ly_scale=1.0):
    from dustyshock3d_gb300 import ic
    dx, Ly, _ = WORKLOADS[name]
    return ic.dusty_sod_tube(dx_left=dx, Ly=Ly * ly_scale, eps=1.0, t_s=1e-3)


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        self.index = index

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        loaded = [v for v in sm if v > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# distributed plumbing (one process per GPU, replicas of the tube)
# ---------------------------------------------------------------------------
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        devs = vis.split(",") if vis else [str(i) for i in range(64)]
        os.environ["CUDA_VISIBLE_DEVICES"] = devs[local]
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return ws, rank, dist
    return 1, 0, None


def dist_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def replica_rate(dist, ws, n, steps, ms):
    """Whole-job particle-steps/s of ws ranks that each advanced n particles
    for `steps` steps in `ms` milliseconds: the slowest rank sets the time."""
    return ws * n * steps / (dist_max(dist, ms) * 1e-3)


def balanced_shards(sizes, ws):
    """Independent tubes split over ws ranks, largest first onto the least
    loaded rank (deterministic; ties to the lower rank).  Returns one sorted
    index list per rank."""
    load = [0] * ws
    out = [[] for _ in range(ws)]
    for i in sorted(range(len(sizes)), key=lambda i: (-sizes[i], i)):
        r = min(range(ws), key=lambda r: (load[r], r))
        load[r] += sizes[i]
        out[r].append(i)
    return [sorted(o) for o in out]


# ---------------------------------------------------------------------------
# CPU: the oracle (reference algorithm restated, FP64, OpenMP)
# ---------------------------------------------------------------------------
def time_cpu(name, steps, budget_s=25.0):
    """Oracle steps on all host cores on one of the benchmark tubes.  Returns
    (particle-steps/s, sample text, particles)."""
    P, sp = make_tube(name, 1.0)
    return time_cpu_params(P, sp, steps, budget_s)


def time_cpu_params(P, sp, steps, budget_s=25.0):
    """Oracle steps on all host cores from the given state: at least one, more
    while they fit the budget.  Returns (particle-steps/s, sample text,
    particles)."""
    from oracle.oracle import OracleState
    O = OracleState(P, sp)
    t0 = time.perf_counter()
    O.step(1)
    t1 = time.perf_counter() - t0
    n = sum(s.n for s in sp)
    done, el = 1, t1
    while done < steps and el + t1 <= budget_s:
        t0 = time.perf_counter()
        O.step(1)
        el += time.perf_counter() - t0
        done += 1
    return n * done / el, f"{done} FP64 step(s) of the full {n}-particle tube from t=0 ({el:.1f} s)", n


def reference_init_tube():
    """The reference's own default run: ds_params_init (the values of its
    Init.txt) and its generator init_Sod_X_Dust (323,584 gas + 2 x 323,584
    dust), in reference mode."""
    import ctypes

    from dustyshock3d_gb300 import _lib, ic
    L = _lib.load()
    c = _lib.DsParams()
    _lib.check(L, None, L.ds_params_init(ctypes.byref(c)), "ds_params_init")
    return ic.init_sod_x_dust(_lib.params_from_c(c), before_first="skip")


def reference_gpu_record(P=None, sp=None, steps=3):
    """The reference's own CUDA kernels on this GPU against this library's FP64
    path, on the reference's default run (both from t = 0, `steps` steps).

    The reference's arm: kernel.cu and IDIC.h compiled unmodified into a cubin
    (oracle/build_ref_gpu.sh, where the reference tree exists), launched by a
    restatement of its host loop (oracle/ref_gpu.c): host cell lists, one
    launch and one device synchronize per stencil offset, host IDIC solve,
    blocking copies -- wall time per step, the median of steps 2.. (the first
    pays first-launch costs).  This library's arm: the FP64 path (the same
    operation order as the reference's host build), one untimed step, then
    steps - 1 graph replays between CUDA events.  Both states are compared
    after the same steps: the reference's kernels contract multiply-adds
    (nvcc's default), so they differ from the FP64 path by rounding only."""
    import numpy as np

    from dustyshock3d_gb300.solver import Solver
    from oracle import ref_gpu
    why = ref_gpu.available()
    if why:
        return {"unavailable": why}
    if P is None:
        P, sp = reference_init_tube()
    n = sum(q.n for q in sp)
    steps = max(2, steps)
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(1)
        ms = S.step_timed_graph(steps - 1)
        ours = [S.get_species(0, s) for s in range(3)]
    R = ref_gpu.RefGPU(P, sp).step(steps)
    ref_s = float(np.median(R.step_s[1:]))
    diff = {}
    for s, tag in ((0, "gas"), (1, "dust1"), (2, "dust2")):
        for f in ("x", "vx", "rho"):
            a, b = getattr(R.species[s], f), getattr(ours[s], f)
            diff[f"{tag}_{f}"] = float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
    ours_v = n * (steps - 1) / (ms * 1e-3)
    return {"workload": "reference_init", "particles": n, "steps": steps,
            "reference_kernels": {"value": n / ref_s, "unit": "particle-steps/s", "ms_per_step": 1e3 * ref_s,
                                  "step_ms": [1e3 * t for t in R.step_s],
                                  "phase_ms_per_step": {k: 1e3 * v / steps for k, v in R.phase_s.items()},
                                  "what": "the reference's CUDA kernels (kernel.cu, IDIC.h compiled unmodified, "
                                          "nvcc -O3, sm_103a) under a restatement of its host loop: host lists, "
                                          "~120 launches each followed by a device synchronize, host IDIC, "
                                          "blocking copies; wall time per step, median of steps 2.."},
            "fp64_path": {"value": ours_v, "unit": "particle-steps/s", "ms_per_step": ms / (steps - 1),
                          "what": "this library's FP64 path, CUDA events around steps - 1 graph replays"},
            "fp64_path_over_reference_kernels": ours_v * ref_s / n,
            "max_rel_diff_after_steps": diff}


def batch64_tubes(seed):
    """The 64 seeded uneven tubes (ic.batch_tubes' draws), as device generators:
    (params, DeviceIC) pairs, so that no particle is made on the host."""
    import numpy as np

    from dustyshock3d_gb300 import ic
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(64):
        spec = ic.DeviceIC.uneven(**ic.draw_tube_params(rng))
        out.append((spec.plan()[0], spec))
    return out


def batch64_record(seed, steps, warmup, shard=None):
    """Batched FP32: the 64 uneven tubes in one context, cell size and list
    depth chosen by the autotuner on the first 8; CUDA events around exactly
    `steps` replays of the step graphs.  Returns (record, n_particles_all)."""
    from dustyshock3d_gb300 import tune
    from dustyshock3d_gb300.solver import Solver
    all_tubes = batch64_tubes(seed)
    sizes = [sum(spec.plan()[1]) for _, spec in all_tubes]
    idx = list(range(64)) if shard is None else shard
    tubes = [all_tubes[i] for i in idx]
    t0 = time.perf_counter()
    choice, log = tune.tune(tubes, sample=8)
    tune_s = time.perf_counter() - t0
    ps = []
    for P, _ in tubes:
        Q = tune.apply(P, choice.stencil, choice.cell_factor, choice.list_depth, choice.persistent,
                       choice.idic_lanes, choice.list_skin)
        Q.precision = "fp32"
        ps.append(Q)
    n = sum(sizes[i] for i in idx)
    with Solver(ps) as S:
        for t, (_, spec) in enumerate(tubes):
            S.init_tube(t, spec)
        S.step(warmup)
        total_ms = S.step_timed_graph(steps)  # the graphs ds_step replays
        _, phase = S.step_timed(steps)         # phase split, after the timed region
        kps = S.kernels_per_step()
        mem = S.memory_bytes()
    rec = {"value": n * steps / (total_ms * 1e-3), "ms_per_step": total_ms / steps, "steps": steps,
           "warmup": warmup, "tubes": len(tubes), "particles": n, "seed": seed,
           "initial_conditions": "generated on the device (ds_init_tube)",
           "autotuned": dataclasses.asdict(choice), "tuning_s": tune_s,
           "tuning_log": [dict(stencil=a, cell_factor=b, list_depth=c, persistent=p, idic_lanes=q, list_skin=k,
                               ms=d) for a, b, c, p, q, k, d in log],
           "device_bytes": mem,
           "phase_ms_per_step": {k: v / steps for k, v in zip(("sort", "density", "force", "idic_update"), phase)},
           "gpu_launches": kps * steps}
    return rec, sum(sizes), total_ms


def device_tube_record(name, steps32=10, steps64=2, warmup=2, skin=0.0):
    """One tube generated on the device, timed on the FP32 (list reuse with
    `skin`) and the FP64 path (CUDA events around the step graphs, after
    warm-up steps)."""
    from dustyshock3d_gb300 import ic
    from dustyshock3d_gb300.solver import Solver
    dx, Ly, desc = WORKLOADS[name]
    spec = ic.DeviceIC.dusty_sod(dx_left=dx, Ly=Ly)
    P, counts = spec.plan()
    n = sum(counts)
    out = {"workload": name, "description": desc, "particles": n, "gas": counts[0]}
    for prec, steps, wu in (("fp32", steps32, warmup), ("fp64", steps64, 1)):
        Q = P.copy()
        Q.precision = prec
        if prec == "fp32":
            Q.list_skin = skin
        with Solver(Q) as S:
            S.init_tube(0, spec)
            S.step(wu)
            ms = S.step_timed_graph(steps)
            rec = {"value": n * steps / (ms * 1e-3), "ms_per_step": ms / steps, "steps": steps, "warmup": wu}
            if prec == "fp32":
                rec["list_skin_h"] = skin
                rec["list_rebuilds_steps"] = list(S.list_stats(0))
                _, phase = S.step_timed(steps)
                rec["phase_ms_per_step"] = {k: v / steps for k, v in
                                            zip(("sort", "density", "force", "idic_update"), phase)}
        out[prec] = rec
    return out


def cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def workload_config(name, n, n_gas, ws):
    """The `config` of a line: what the workload is, the same for both arms."""
    return {"workload": name, "description": WORKLOADS[name][2], "particles": n, "gas": n_gas,
            "parallelism": f"replicas x{ws}" if ws > 1 else "single tube"}


def run_reference(args):
    ws, rank, dist = dist_setup()
    if rank != 0:
        return 0
    from oracle.oracle import OracleState
    name = args.workload
    P, sp = make_tube(name)
    O = OracleState(P, sp)
    n = sum(s.n for s in sp)
    t0 = time.perf_counter()
    O.step(1)
    t_step = time.perf_counter() - t0
    # bounded: warmup + steps must end within ~3 minutes; otherwise time a
    # tube of smaller cross-section (same lattice spacing)
    scale = 1.0
    budget = 180.0
    if t_step * (args.warmup + args.steps) > budget:
        scale = max(0.2, (budget / (t_step * (args.warmup + args.steps))) ** 0.5)
        P, sp = make_tube(name, scale)
        O = OracleState(P, sp)
        n = sum(s.n for s in sp)
    for _ in range(max(0, args.warmup - 1)):
        O.step(1)
    t0 = time.perf_counter()
    O.step(args.steps)
    el = time.perf_counter() - t0
    v = n * args.steps / el
    sample = (f"{args.steps} FP64 oracle steps of a {n}-particle tube"
              + ("" if scale == 1.0 else f" (cross-section scaled by {scale:.2f}^2 to fit the time budget)"))
    line = {"metric": "particle-steps/s", "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": workload_config(name, n, sp[0].n, 1),
            "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": cores(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(path):
    """DRAM bytes per launch of the force sweep from a committed ncu summary."""
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("dram_bytes_per_particle:"):
                    return float(line.split(":")[1])
    except OSError:
        pass
    return None


def density_bytes_per_particle(hpp: bool) -> int:
    """Compulsory bytes of one FP32 gas density launch per gas particle, each
    array read or written once, not counting the recorded force neighbours
    (4 bytes per entry, added by the caller): read pos32, vm32 (32), h (8,
    per-particle h), rho, p, e (24), vx, vy, vz (24, CFL bound), Ind and the
    own cell key (8); write rho, p (16), hyd32 (16), the list count (4)."""
    return 32 + (8 if hpp else 0) + 24 + 24 + 8 + 16 + 16 + 4


def profile_value(path, key):
    """A `key: value` line of a committed ncu summary, or None."""
    try:
        with open(path) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return float(line.split(":")[1])
    except OSError:
        pass
    return None


def sm_count():
    try:
        import torch
        return int(torch.cuda.get_device_properties(0).multi_processor_count)
    except Exception:  # noqa: BLE001 - reported as unknown
        return None


def issue_ceiling(profile, n_gas, launch_ms, clk):
    """The ceiling that binds the density sweep: warp-instruction issue.  Each
    SM issues at most 4 warp instructions per clock (one per sub-partition), so
    a launch of I warp instructions needs I / (4 SMs f) seconds at SM clock f.
    I per launch: the committed ncu capture's count per gas particle times the
    gas particles; f: the median SM clock sampled during this run."""
    per = profile_value(profile, "warp_instructions_per_particle")
    sms = sm_count()
    if per is None or sms is None or not clk or not clk.get("sm_mhz"):
        return None
    inst = per * n_gas
    slots = 4 * sms * clk["sm_mhz"] * 1e6 * launch_ms * 1e-3
    return {"bound": "issue", "warp_instructions_per_launch": inst, "issue_slots_per_launch": slots,
            "frac": inst / slots, "sms": sms, "sm_mhz": clk["sm_mhz"],
            "note": "warp instructions / (4 x SMs x SM clock x launch time); instructions from the ncu capture"}


def batch64_sizes(seed):
    return [sum(spec.plan()[1]) for _, spec in batch64_tubes(seed)]


# Compulsory bytes of one launch of the FP32 force sweep over the recorded
# lists per gas particle, not counting the 4-byte entries: read pos32, vm32,
# hyd32 (48), Ind and the entry count (8); write ax, ay, az and the energy
# rate (32, FP64).
FORCE_LIST_BYTES_PER_PARTICLE = 48 + 8 + 32


def e2e_run(P, sp, steps, warmup, bound=True):
    """The metric end to end through the C ABI with the state on the host.

    bound (the headline): the reference host's arrays, pinned, bound once with
    ds_bind_host; each timed step is one ds_step_host(1) call that reads every
    bound array from host memory, steps, and writes back what the step changed
    (the transfers overlapped with the step's kernels).  Otherwise: per step
    ds_upload_gas / ds_upload_dust from the same pinned arrays, ds_step(1),
    ds_download_gas / ds_download_dust, each call returning before the next."""
    import ctypes

    import numpy as np

    from dustyshock3d_gb300 import _lib
    from dustyshock3d_gb300.solver import Solver
    L = _lib.load()
    S = Solver(P)
    S.set_tube(0, sp)
    g = sp[0].copy().fill_missing()
    ds = [q.copy().fill_missing() for q in sp[1:]]  # every dust species
    GIN = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e", "m", "h")
    DIN = ("x", "y", "z", "vx", "vy", "vz", "rho", "m", "ts", "h")
    GOUT = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "rho", "p", "e")
    DOUT = ("x", "y", "z", "vx", "vy", "vz", "rho", "ts")
    gin = {f: S.pinned(g.n) for f in GIN}
    dins = [{f: S.pinned(d.n) for f in DIN} for d in ds]
    gind = S.pinned(g.n, np.int32)
    dinds = [S.pinned(d.n, np.int32) for d in ds]
    for f, a in gin.items():
        a[:] = getattr(g, f)
    for d, din, dind in zip(ds, dins, dinds):
        for f, a in din.items():
            a[:] = getattr(d, f)
        dind[:] = d.ind
    gind[:] = g.ind
    h2d = (sum(a.nbytes for a in gin.values()) + gind.nbytes
           + sum(sum(a.nbytes for a in din.values()) + dind.nbytes for din, dind in zip(dins, dinds)))
    if bound:  # what ds_step_host writes back (dust rho and t_stop only where the step can change them)
        dout = [f for f in DOUT if (f != "rho" or P.mode.dust_rho) and (f != "ts" or not P.mode.tstop_const)]
    else:
        dout = DOUT
    d2h = sum(gin[f].nbytes for f in GOUT) + sum(din[f].nbytes for din in dins for f in dout)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))  # noqa: E731
    if bound:
        S.bind_host(0, 0, gin, gind)
        for k, (din, dind) in enumerate(zip(dins, dinds)):
            S.bind_host(0, k + 1, din, dind)
        c = S.ctx

        def one():
            _lib.check(L, c, L.ds_step_host(c, 1), "ds_step_host")
    else:
        d2h += gind.nbytes + sum(a.nbytes for a in dinds)  # the downloads return Ind too
        c = S.ctx

        def one():
            _lib.check(L, c, L.ds_upload_gas(c, g.n, *[dp(gin[f]) for f in GIN], ip(gind)), "upload gas")
            for k, (d, din, dind) in enumerate(zip(ds, dins, dinds)):
                _lib.check(L, c, L.ds_upload_dust(c, k + 1, d.n, *[dp(din[f]) for f in DIN], ip(dind)),
                           "upload dust")
            _lib.check(L, c, L.ds_step(c, 1), "step")
            _lib.check(L, c, L.ds_download_gas(c, *[dp(gin[f]) for f in GOUT], ip(gind)), "download gas")
            for k, (din, dind) in enumerate(zip(dins, dinds)):
                _lib.check(L, c, L.ds_download_dust(c, k + 1, *[dp(din[f]) for f in DOUT], ip(dind)),
                           "download dust")

    for _ in range(warmup):
        one()
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    el = time.perf_counter() - t0
    S.close()
    return el, h2d, d2h


def run_ours(args):
    ws, rank, dist = dist_setup()
    import numpy as np

    from dustyshock3d_gb300.solver import Solver
    name = args.workload
    P, sp = make_tube(name)
    n = sum(s.n for s in sp)
    n_gas = sp[0].n
    clocks = ClockSampler(0)
    clocks.start()

    # FP32 path: the headline
    P32 = P.copy()
    P32.precision = "fp32"
    P32.list_skin = args.list_skin
    S = Solver(P32)
    S.set_tube(0, sp)
    S.step(args.warmup)
    barrier(dist)
    # the timed region: the captured graphs ds_step replays, between two CUDA
    # events on the context's stream
    total_ms = S.step_timed_graph(args.steps)
    value = replica_rate(dist, ws, n, args.steps, total_ms)
    total_ms = dist_max(dist, total_ms)
    kps = S.kernels_per_step()
    list_rebuilds, list_steps = S.list_stats(0)
    g32 = S.get_species(0, 0)
    d32 = S.get_species(0, 1)
    t32 = S.time(0)
    # after the timed region: the phase split (the same kernels launched one by
    # one with events between phases), then the recorded force neighbours of
    # the final state (0 < r < 2 max(h_i, h_j), counted by the parity hook)
    _, phase = S.step_timed(args.steps)
    list_rebuilds2, list_steps2 = S.list_stats(0)
    dbg = S.debug_cells(0, 0)
    free = S.get_species(0, 0).ind == 0
    list_entries = int(dbg["nnb"][free].sum())
    # the entries the list kernels stream: the recorded lists (the particle
    # itself and, with a skin, the partners in the skin's shell among them)
    fcount, _ = S.debug_force_lists(0, cap=1)
    streamed_entries = int(fcount[fcount > 0].sum())
    cand_per_pair = {"stencil_cells": float(dbg["ncand"][free].sum() / max(list_entries, 1)),
                     "note": "particles in the cells of each gas particle's stencil per recorded pair "
                             "(0 < r < 2 max(h_i, h_j)); the FP32 walk screens only the x window of each row, "
                             "about 2/3 of these"}
    S.close()

    fp64 = None
    if not args.no_fp64:
        S = Solver(P)
        S.set_tube(0, sp)
        S.step(args.warmup)
        barrier(dist)
        ms64 = S.step_timed_graph(args.steps)
        ms64 = dist_max(dist, ms64)
        g64 = S.get_species(0, 0)
        d64 = S.get_species(0, 1)
        t64 = S.time(0)
        n_ph64 = min(args.steps, 5)
        _, phase64 = S.step_timed(n_ph64)  # phase split, after the comparison state
        S.close()
        fp64 = {"value": ws * n * args.steps / (ms64 * 1e-3), "ms_per_step": ms64 / args.steps,
                "phase_ms_per_step": {k: v / n_ph64 for k, v in zip(("sort", "density", "force", "idic_update"),
                                                                      phase64)}}
        rel = lambda a, b: float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))  # noqa: E731
        fp64["l1_fp32_vs_fp64"] = {"rho_gas": rel(g32.rho, g64.rho), "v_gas": rel(g32.vx, g64.vx),
                                   "v_dust": rel(d32.vx, d64.vx), "t_fp32": t32[0], "t_fp64": t64[0],
                                   "steps": args.warmup + args.steps}
        if not args.no_e2e:  # the same-precision end-to-end number
            barrier(dist)
            el, h2d, d2h = e2e_run(P, sp, args.steps, 1, bound=True)
            el = dist_max(dist, el)
            fp64["e2e"] = {"value": ws * n * args.steps / el, "unit": "particle-steps/s",
                           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * el / args.steps,
                           "path": "as the headline e2e (ds_bind_host + ds_step_host(1) per step), fp64 path"}

    e2e = None
    if not args.no_e2e:
        barrier(dist)
        el, h2d, d2h = e2e_run(P32, sp, args.steps, min(args.warmup, 2), bound=True)
        el = dist_max(dist, el)
        e2e = {"value": ws * n * args.steps / el, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * el / args.steps,
               "path": "pinned host arrays bound once (ds_bind_host); per step ds_step_host(1): every bound "
                       "array read, one step, the changed fields written back; fp32 path"}
        barrier(dist)
        el2, h2d2, d2h2 = e2e_run(P32, sp, args.steps, min(args.warmup, 2), bound=False)
        el2 = dist_max(dist, el2)
        e2e["separate_calls"] = {"value": ws * n * args.steps / el2, "h2d_bytes_per_step": h2d2,
                                 "d2h_bytes_per_step": d2h2, "ms_per_step": 1e3 * el2 / args.steps,
                                 "path": "ds_upload_gas/dust (pinned) + ds_step(1) + ds_download_gas/dust"}
    c3 = None
    if not args.no_c3 and name == DEFAULT_WORKLOAD:
        barrier(dist)
        c3 = device_tube_record("dusty_sod_5760k", skin=args.list_skin)
    batch = None
    if not args.no_batch and name == DEFAULT_WORKLOAD:
        barrier(dist)
        shard = balanced_shards(batch64_sizes(args.seed), ws)[rank] if ws > 1 else None
        batch, n_batch_all, bms = batch64_record(args.seed, 10, 3, shard)
        bms = dist_max(dist, bms)
        batch["value"] = n_batch_all * 10 / (bms * 1e-3)  # whole job: all 64 tubes over the slowest rank
        batch["ms_per_step"] = bms / 10
    ref_gpu_rec = None
    if not args.no_ref_gpu and name == DEFAULT_WORKLOAD and rank == 0:
        ref_gpu_rec = reference_gpu_record()
    serve_rec = None
    if not args.no_serve and name == DEFAULT_WORKLOAD and ws == 1:
        serve_rec = serve_record(args.seed, args.rate, args.requests)
    clk = clocks.stop()

    if rank != 0:
        return 0
    peak, peak_kind = peak_hbm()
    dens_ms = phase[1] / args.steps
    dens_prof = os.path.join(ROOT, "profiles", "density32_dusty_sod_720k.txt")
    dens = {"kernel": "k_density32 (gas density + EOS + force-list record, FP32)",
            "algorithmic_bytes_per_launch": density_bytes_per_particle(P.mode.h_per_particle) * n_gas
            + 4 * list_entries, "list_entries_per_launch": list_entries, "candidates_per_pair": cand_per_pair}
    if args.list_skin > 0:
        # with list reuse the force sweep over the lists runs every step and
        # takes the largest share; the density phase mixes the recording walk
        # (steps that re-sort) and the streamed lists (steps that keep them)
        f_ms = phase[2] / args.steps
        prof = os.path.join(ROOT, "profiles", "force32_list_dusty_sod_720k_skin015.txt")
        alg = FORCE_LIST_BYTES_PER_PARTICLE * n_gas + 4 * streamed_entries
        achieved = alg / (f_ms * 1e-3) / 1e9
        tr = profile_traffic(prof)
        roof = {"kernel": "k_force32_list (force + energy rate over the recorded lists, FP32)", "bound": "hbm",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": None if tr is None else tr * n_gas,
                "algorithmic_bytes_per_launch": alg, "avg_launch_ms": f_ms,
                "list_entries_per_launch": streamed_entries,
                "note": "launch time: the force phase (k_tstop and k_dt, ~0.01 ms, run in it; the overflow walk runs "
                        "beside it on a second stream); algorithmic bytes: 88 per gas particle + 4 per streamed "
                        "entry; traffic from the committed ncu capture of this workload"}
        roof["issue"] = issue_ceiling(prof, n_gas, f_ms, clk)
        dens["phase_ms_per_step"] = dens_ms
        dens["note"] = ("with list reuse the density phase is the recording walk on steps that re-sort and the "
                        "streamed lists (k_density32_lst) on the others")
        roof["density_sweep"] = dens
    else:
        alg = dens["algorithmic_bytes_per_launch"]
        achieved = alg / (dens_ms * 1e-3) / 1e9
        tr = profile_traffic(dens_prof)
        roof = {"kernel": dens["kernel"], "bound": "hbm",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": None if tr is None else tr * n_gas,
                "algorithmic_bytes_per_launch": alg, "avg_launch_ms": dens_ms,
                "list_entries_per_launch": list_entries,
                "note": "issue-bound, not HBM-bound: every particle screens the candidates of 27 (or 125) cells "
                        "in FP32; traffic from the committed ncu capture of this workload"}
        roof["issue"] = issue_ceiling(dens_prof, n_gas, dens_ms, clk)
        roof["candidates_per_pair"] = cand_per_pair
    cpu = None
    if not args.no_cpu_baseline:
        v, sample, _ = time_cpu(name, 3)
        cpu = {"value": v, "unit": "particle-steps/s", "cores": cores(), "kind": "port", "sample": sample}
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(name, n, n_gas, ws),
            "precision": "fp32 neighbour sums (Kahan), fp64 state / IDIC / sums",
            "l2": "inputs larger than L2 (resident state ~%d MB)" % (n * 256 // 2 ** 20),
            "timing": "CUDA events around the step graphs ds_step replays, on the context's stream; "
                      "phase split from a second pass with events between phases",
            "phase_ms_per_step": {k: v / args.steps for k, v in zip(("sort", "density", "force", "idic_update"),
                                                                     phase)},
            "fp64": fp64, "e2e": e2e, "roofline": roof, "cpu_baseline": cpu,
            "dusty_sod_5760k": c3, "batch64": batch, "reference_gpu": ref_gpu_rec, "serve": serve_rec,
            "gpu_launches": kps * args.steps, "clocks": clk}
    if args.list_skin > 0:
        line["list_reuse"] = {"skin_h": args.list_skin, "steps": list_steps, "steps_that_rebuilt": list_rebuilds,
                              "phase_pass": {"steps": list_steps2 - list_steps,
                                             "steps_that_rebuilt": list_rebuilds2 - list_rebuilds}}
    print(json.dumps(line))
    return 0


def run_batch(args):
    """64 uneven tubes (seeded) advanced together, FP32, autotuned, generated on
    the device.  With N ranks the tubes are split over the GPUs (balanced by
    particle count; the tubes are independent, so no collective touches the data
    path)."""
    ws, rank, dist = dist_setup()
    shard = balanced_shards(batch64_sizes(args.seed), ws)[rank] if ws > 1 else None
    clocks = ClockSampler(0)
    clocks.start()
    rec, n_all, total_ms = batch64_record(args.seed, args.steps, args.warmup, shard)
    clk = clocks.stop()
    total_ms = dist_max(dist, total_ms)
    if rank != 0:
        return 0
    value = n_all * args.steps / (total_ms * 1e-3)
    cfg = {"workload": "batch64", "tubes": 64, "particles": n_all, "seed": args.seed,
           "tubes_on_rank0": rec["tubes"], "particles_on_rank0": rec["particles"]}
    for k in ("autotuned", "tuning_s", "tuning_log", "device_bytes", "initial_conditions"):
        cfg[k] = rec[k]
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "strong" if ws > 1 else "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": cfg,
            "phase_ms_per_step": rec["phase_ms_per_step"], "gpu_launches": rec["gpu_launches"], "clocks": clk}
    print(json.dumps(line))
    return 0


def serve_summary(res, wall, rebuilds=None, rebuild_s=None):
    """Throughput and p50 / p99 time to solution of served (or one-at-a-time) results."""
    import numpy as np
    tts = np.array([r.time_to_solution for r in res])
    ps = sum(r.particles * r.steps for r in res)
    out = {"requests": len(res), "wall_s": wall, "particle_steps": ps, "value": ps / wall,
           "p50_time_to_solution_s": float(np.percentile(tts, 50)),
           "p99_time_to_solution_s": float(np.percentile(tts, 99))}
    if rebuilds is not None:
        out.update(rebuilds=rebuilds, rebuild_s=rebuild_s, rebuild_ms_each=1e3 * rebuild_s / max(rebuilds, 1))
    return out


def serve_record(seed, rate=4.0, requests=64):
    """The served stream of the serve workload without its comparators: 64
    Poisson requests of uneven tubes generated on the device at admission,
    continuous batching under 150 GB, epochs of 10 steps."""
    from dustyshock3d_gb300.serve import Server, device_uneven_tube, poisson_requests
    reqs = poisson_requests(rate, requests, seed, device_uneven_tube)
    server = Server(budget_bytes=150e9, epoch_steps=10, precision="fp32")
    t0 = time.perf_counter()
    res = server.run(reqs)
    rec = serve_summary(res, time.perf_counter() - t0, server.rebuilds, server.rebuild_s)
    rec.update(workload="serve", rate_per_s=rate, seed=seed, budget_bytes=150e9, epoch_steps=10,
               note="python bench.py --workload serve adds the comparators (the first 16 requests served alone "
                    "and solved one at a time on FP32 and FP64)")
    return rec


def run_serve(args):
    """Poisson stream of uneven tubes, continuous batching under 150 GB.

    Comparators, all measured: the first --compare requests (by arrival, same
    arrival times) served on their own, then solved one at a time in arrival
    order on the FP32 path and on the plain FP64 path (ds_step of one tube per
    context, a request waiting while the previous one runs)."""
    from dustyshock3d_gb300 import ic
    from dustyshock3d_gb300.serve import Server, device_uneven_tube, one_at_a_time, poisson_requests
    if args.host_ic:  # initial particles made on the host and uploaded at admission
        make = lambda rng: ic.uneven_tube(**ic.draw_tube_params(rng))  # noqa: E731
    else:  # generated on the device at admission (ds_init_tube)
        make = device_uneven_tube
    reqs = poisson_requests(args.rate, args.requests, args.seed, make)

    summary = serve_summary

    clocks = ClockSampler(0)
    clocks.start()
    server = Server(budget_bytes=150e9, epoch_steps=10, precision="fp32")
    t0 = time.perf_counter()
    res = server.run(reqs)
    wall = time.perf_counter() - t0
    full = summary(res, wall, server.rebuilds, server.rebuild_s)
    comp = None
    if args.compare > 0:
        sub = sorted(reqs, key=lambda r: r.arrival)[:args.compare]
        s2 = Server(budget_bytes=150e9, epoch_steps=10, precision="fp32")
        t0 = time.perf_counter()
        r2 = s2.run(sub)
        served = summary(r2, time.perf_counter() - t0, s2.rebuilds, s2.rebuild_s)
        rows = {"served_fp32": served}
        for prec in ("fp32", "fp64"):
            t0 = time.perf_counter()
            rs = one_at_a_time(sub, prec)
            rows[f"one_at_a_time_{prec}"] = summary(rs, time.perf_counter() - t0)
        comp = {"subset": f"the first {len(sub)} requests by arrival ({sum(r.particles for r in sub)} particles), "
                          "same arrival times", **rows}
    clk = clocks.stop()
    line = {"metric": "particle-steps/s", "value": full["value"], "unit": "particle-steps/s", "n_gpus": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "serve", "requests": len(reqs), "rate_per_s": args.rate, "seed": args.seed,
                       "budget_bytes": 150e9, "epoch_steps": 10, "t_end": "U[0.05, 0.2]",
                       "initial_conditions": "host" if args.host_ic else "device"},
            "p50_time_to_solution_s": full["p50_time_to_solution_s"],
            "p99_time_to_solution_s": full["p99_time_to_solution_s"], "wall_s": full["wall_s"],
            "rebuilds": full["rebuilds"], "rebuild_s": full["rebuild_s"], "rebuild_ms_each": full["rebuild_ms_each"],
            "particle_steps": full["particle_steps"], "comparators": comp, "clocks": clk}
    print(json.dumps(line))
    return 0


def run_accuracy(args):
    """The 720k tube to t_end on the FP64 and the FP32 path for
    t_s in {1e-1, 1e-2, 1e-3, 1e-4} x eps in {0.01, 1, 10}: L1 error of the
    FP32 path's gas density, gas and dust x-velocity against the FP64 path
    (sum |a - b| / sum |b|), per particle and of the x profile (means over
    400 bins of the tube's length), and both paths' rates.

    Floor: for t_s = 1e-3, eps = 1 the FP64 path is also run from gas
    positions moved by 1e-10 of the left spacing (seeded normal offsets).  On
    this tube the scheme amplifies differences at the rounding level by orders
    of magnitude once the shock has formed (the M4 kernel at h = 1.3 dx has
    ~74 neighbours, twice that behind the shock, where SPH particle
    arrangements are unstable), so the L1 of that pair of FP64 runs is the
    level below which no comparison of two differently rounded runs falls.

    Against the physics: the runs in a limit with a closed-form answer (eps =
    0.01: Sod on the gas states; t_s = 1e-4: gas and dust as one mixture of
    sound speed c_s / sqrt(1 + eps)) are also scored against the exact Riemann
    solution (dustyshock3d_gb300.riemann, Toro's method), FP32 beside FP64:
    the FP32 path meets the spec accuracy when its error against the
    exact solution is within a stated factor of the FP64 path's."""
    import copy

    import numpy as np

    from dustyshock3d_gb300 import ic, riemann
    from dustyshock3d_gb300.solver import Solver
    ws, rank, dist = dist_setup()
    if rank != 0:
        return 0
    dx, Ly, _ = WORKLOADS["dusty_sod_720k"]
    rel = lambda a, b: float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))  # noqa: E731
    nb = 400

    def prof(q, f, x0, x1):
        b = np.clip(((q.x - x0) / (x1 - x0) * nb).astype(int), 0, nb - 1)
        return np.bincount(b, weights=getattr(q, f), minlength=nb) / np.maximum(np.bincount(b, minlength=nb), 1)

    def run(P, sp, prec):
        Q = P.copy()
        Q.precision = prec
        if prec == "fp32":
            Q.list_skin = args.list_skin  # the default line's FP32 configuration
        with Solver(Q) as S:
            S.set_tube(0, sp)
            ms_tot, groups = 0.0, 0
            while S.time(0)[0] < Q.T_end and groups < 2000:  # bounded: 20000 steps
                ms, _ = S.step_timed(10)
                ms_tot += ms
                groups += 1
            Tm, _, nstep = S.time(0)
            return S.get_species(0, 0), S.get_species(0, 1), Tm, nstep, ms_tot

    def errors(g, d, g0, d0, x0, x1):
        return {"l1_rho_gas": rel(g.rho, g0.rho), "l1_v_gas": rel(g.vx, g0.vx), "l1_v_dust": rel(d.vx, d0.vx),
                "l1_profile_rho_gas": rel(prof(g, "rho", x0, x1), prof(g0, "rho", x0, x1)),
                "l1_profile_v_gas": rel(prof(g, "vx", x0, x1), prof(g0, "vx", x0, x1)),
                "l1_profile_v_dust": rel(prof(d, "vx", x0, x1), prof(d0, "vx", x0, x1))}

    clocks = ClockSampler(0)
    clocks.start()
    rows, floor = [], None
    for t_s in (1e-1, 1e-2, 1e-3, 1e-4):
        for eps in (0.01, 1.0, 10.0):
            P, sp = ic.dusty_sod_tube(dx_left=dx, Ly=Ly, eps=eps, t_s=t_s, t_end=args.t_end)
            n = sum(q.n for q in sp)
            g64, d64, _, n64, ms64 = run(P, sp, "fp64")
            g32, d32, T32, n32, ms32 = run(P, sp, "fp32")
            row = {"t_s": t_s, "eps": eps, "t": T32, "steps_fp32": n32, "steps_fp64": n64,
                   **errors(g32, d32, g64, d64, P.X_min, P.X_max),
                   "fp32_particle_steps_per_s": n * n32 / (ms32 * 1e-3),
                   "fp64_particle_steps_per_s": n * n64 / (ms64 * 1e-3)}
            limit = "gas" if eps <= 0.01 else ("coupled" if t_s <= 1e-4 else None)
            if limit:
                s64 = riemann.score_dusty_sod(g64, d64, T32, eps, limit)
                s32 = riemann.score_dusty_sod(g32, d32, T32, eps, limit)
                row["exact"] = {"limit": limit, "fp64": s64, "fp32": s32,
                                "fp32_over_fp64": {k: s32[k] / s64[k] for k in s64
                                                   if k.startswith("l1_") and s64[k] > 0}}
            rows.append(row)
            print(json.dumps(row), file=sys.stderr, flush=True)
            if t_s == 1e-3 and eps == 1.0:
                moved = [copy.copy(q) for q in sp]
                rng = np.random.default_rng(args.seed)
                moved[0].x = sp[0].x + 1e-10 * dx * rng.standard_normal(sp[0].n) * (sp[0].ind == 0)
                gp, dp, _, _, _ = run(P, moved, "fp64")
                floor = {"t_s": t_s, "eps": eps, "perturbation": "gas x moved by 1e-10 dx_left (normal, seeded)",
                         **errors(gp, dp, g64, d64, P.X_min, P.X_max)}
                print(json.dumps(floor), file=sys.stderr, flush=True)
    clk = clocks.stop()
    keys = ("l1_rho_gas", "l1_v_gas", "l1_v_dust", "l1_profile_rho_gas", "l1_profile_v_gas", "l1_profile_v_dust")
    ratios = [v for r in rows if "exact" in r for v in r["exact"]["fp32_over_fp64"].values()]
    line = {"metric": "l1 error, fp32 path vs fp64 path", "workload": "accuracy_720k", "t_end": args.t_end,
            "fp32_list_skin_h": args.list_skin,
            "particles": n, "rows": rows, "max": {k: max(r[k] for r in rows) for k in keys},
            "exact_fp32_over_fp64": {"min": min(ratios), "max": max(ratios)} if ratios else None,
            "fp64_floor": floor,
            "note": "rates include up to 9 steps after t_end that do no work (steps run in groups of 10)",
            "clocks": clk}
    print(json.dumps(line))
    return 0


def run_reference_init(args):
    """The reference's own default run: ds_params_init (the values of its
    Init.txt: box [-2, 2]^3, 40 particles per unit length, h = 0.1, tau = 5e-3,
    T_end = 0.2), its generator (init_Sod_X_Dust: 323,584 gas + 2 x 323,584
    dust), reference mode -- the reference's grid, index coupling, eps guard,
    2-species solve, dust density every step -- on the FP64 path, which equals
    the oracle (and so the reference program) bit for bit.  Device-resident
    (CUDA events around the step graphs) and end to end through
    ds_bind_host / ds_step_host; the CPU oracle on the host cores beside it.
    The run has 40 steps in all: --warmup steps, then up to --steps of the
    rest are timed.  Beside it, the reference's own CUDA kernels on the same
    input and GPU (reference_gpu_record), and its loops built for the host
    (timed where the reference tree exists, oracle/compare_cpu_baselines.py)."""
    from dustyshock3d_gb300.solver import Solver
    ws, rank, dist = dist_setup()
    if rank != 0:
        return 0
    P, sp = reference_init_tube()
    n = sum(q.n for q in sp)
    total = int(round(P.T_end / P.tau))
    steps = max(1, min(args.steps, total - args.warmup))
    clocks = ClockSampler(0)
    clocks.start()
    with Solver(P) as S:
        S.set_tube(0, sp)
        S.step(args.warmup)
        ms = S.step_timed_graph(steps)
        kps = S.kernels_per_step()
    el, h2d, d2h = e2e_run(P, sp, steps, args.warmup, bound=True)
    clk = clocks.stop()
    refk = None if args.no_ref_gpu else reference_gpu_record(P, sp)
    v, sample, _ = time_cpu_params(P, sp, 1)
    line = {"metric": "particle-steps/s", "value": n * steps / (ms * 1e-3), "unit": "particle-steps/s",
            "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (the reference's own default initial conditions)",
            "config": {"workload": "reference_init", "particles": n, "gas": sp[0].n,
                       "description": "the reference's default Init.txt run, reference mode, FP64 path"},
            "e2e": {"value": n * steps / el, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * el / steps,
                    "path": "ds_bind_host + ds_step_host(1) per step, fp64 path"},
            "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": cores(), "kind": "port",
                             "sample": sample},
            "reference_gpu": refk, "gpu_launches": kps * steps, "clocks": clk}
    print(json.dumps(line))
    return 0


def run_ic(args):
    """Initial conditions of the 720k and 5.76M tubes: made on the host (numpy,
    ic.dusty_sod_tube) and uploaded at the first step, against generated on the
    device (ds_init_tube) at the first step; and the regeneration of a resident
    tube (plan + generator kernels + sync), median of args.steps.  The
    generator writes 15 doubles and 2 ints per particle (128 B): its roofline
    is HBM writes."""
    import numpy as np

    from dustyshock3d_gb300 import ic
    from dustyshock3d_gb300.solver import Solver
    hbm, hbm_kind = peak_hbm()
    clocks = ClockSampler(0)
    clocks.start()
    rows = []
    for name in ("dusty_sod_720k", "dusty_sod_5760k"):
        dx, Ly, desc = WORKLOADS[name]
        kw = dict(dx_left=dx, Ly=Ly)
        spec = ic.DeviceIC.dusty_sod(**kw)
        P, counts = spec.plan()
        P.precision = "fp32"
        n = sum(counts)
        t0 = time.perf_counter()
        _, sp = ic.dusty_sod_tube(**kw)
        t1 = time.perf_counter()
        with Solver(P) as S:
            S.set_tube(0, sp)
            S.step(0)
            t2 = time.perf_counter()
        del sp
        t3 = time.perf_counter()
        with Solver(P) as S:
            S.init_tube(0, spec)
            S.step(0)
            t4 = time.perf_counter()
            for _ in range(max(3, args.warmup)):
                S.init_tube(0, spec)
            regen = []
            for _ in range(max(5, args.steps)):
                a = time.perf_counter()
                S.init_tube(0, spec)
                regen.append(time.perf_counter() - a)
        r = float(np.median(regen))
        rows.append({"workload": name, "particles": n, "host_generate_s": t1 - t0,
                     "host_copies_and_upload_s": t2 - t1, "device_generate_and_setup_s": t4 - t3,
                     "device_regenerate_s": r, "device_particles_per_s": n / r, "write_GBs": n * 128 / r / 1e9})
    clk = clocks.stop()
    big = rows[-1]
    line = {"metric": "particles generated/s", "value": big["device_particles_per_s"], "unit": "particles/s",
            "n_gpus": 1, "steps": max(5, args.steps), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "initial_conditions", "tubes": [r["workload"] for r in rows]},
            "roofline": {"bound": "hbm", "achieved": big["write_GBs"], "peak": hbm, "unit": "GB/s",
                         "frac": big["write_GBs"] / hbm, "traffic": None,
                         "note": f"128 B written per particle; plan, launch and sync inside the time; peak {hbm_kind}"},
            "tubes": rows, "gpu_launches": 2, "clocks": clk}
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch64":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "accuracy_720k":
        return run_accuracy(args)
    if args.workload == "reference_init":
        return run_reference_init(args)
    if args.workload == "initial_conditions":
        return run_ic(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
