"""Times the reference's own step loop built for the host against the oracle.

TEST INFRASTRUCTURE, a measurement recipe: it shows that the oracle (the CPU
restatement of the reference's step that bench.py times as the CPU baseline)
is not slower than the reference's own per-particle loops on the same input.

Both run the reference's default Init.txt (970,752 particles: gas and two dust
species on the init_Sod_X_Dust lattices, kernel.cu:1391-1582), in reference
mode, for N steps of its fixed tau, with the same number of OpenMP threads:

* the reference program itself (kernel.cu + IDIC.h + data.h, unmodified but
  for its launch syntax; oracle/build_ref.sh), whose kernels run as OpenMP
  loops over their blocks and whose list build and IDIC algebra run as written
  on one thread.  Its step-loop time is the run to T_end = N tau minus a run to
  T_end = 0 (start-up, initial conditions and the first snapshot), with no
  snapshot inside the loop (T_out beyond T_end);
* the oracle (oracle.c) on the same particles (ic.init_sod_x_dust with
  before_first="skip": the default box makes the reference write Ind_gas[-1],
  which changes no particle).

Needs the reference tree (DS_REFERENCE_DIR); writes only under a temporary
directory.  Usage:
    DS_REFERENCE_DIR=... python oracle/compare_cpu_baselines.py [steps] [threads]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this folder would shadow the `oracle` package
sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, ROOT)


def main(steps: int = 5, threads: int = 0) -> dict:
    ref = os.environ.get("DS_REFERENCE_DIR")
    if not ref:
        raise SystemExit("DS_REFERENCE_DIR is not set: point it at the reference tree (kernel.cu, IDIC.h, data.h)")
    threads = threads or len(os.sched_getaffinity(0))
    exe = subprocess.run([os.path.join(HERE, "build_ref.sh")], check=True, capture_output=True,
                         text=True).stdout.strip().splitlines()[-1]
    base = open(os.path.join(ref, "Init.txt")).read().splitlines()
    tau = float(base[12].split()[0])

    def init_txt(d, t_end):
        os.makedirs(os.path.join(d, "Data"), exist_ok=True)
        lines = list(base)
        lines[13] = f"{t_end!r}\t\t\t// Time end"
        lines[14] = "1000.0\t\t// Time interval to output in files"
        text = "\n".join(lines) + "\n"
        with open(os.path.join(d, "Init.txt"), "w") as f:
            f.write(text)
        return text

    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    wall = {}
    with tempfile.TemporaryDirectory() as td:
        for tag, t_end in (("setup", 0.0), ("run", steps * tau - 1e-12)):
            d = os.path.join(td, tag)
            init_txt(d, t_end)
            t0 = time.perf_counter()
            subprocess.run([exe], cwd=d, env=env, check=True, stdout=subprocess.DEVNULL)
            wall[tag] = time.perf_counter() - t0
        text = init_txt(os.path.join(td, "port"), 0.2)
    ref_loop = wall["run"] - wall["setup"]

    os.environ["OMP_NUM_THREADS"] = str(threads)
    from dustyshock3d_gb300 import ic, parse_init_txt
    from oracle.oracle import OracleState
    P, sp = ic.init_sod_x_dust(parse_init_txt(text), before_first="skip")
    n = sum(s.n for s in sp)
    O = OracleState(P, sp)
    t0 = time.perf_counter()
    O.step(steps)
    port = time.perf_counter() - t0
    out = {"particles": n, "steps": steps, "threads": threads,
           "reference_host_build_s": ref_loop, "reference_particle_steps_per_s": n * steps / ref_loop,
           "reference_setup_s": wall["setup"],
           "oracle_s": port, "oracle_particle_steps_per_s": n * steps / port,
           "oracle_over_reference_speed": ref_loop / port}
    return out


if __name__ == "__main__":
    import json
    a = [int(x) for x in sys.argv[1:3]]
    print(json.dumps(main(*a)))
