"""Generate the golden fixtures that pin the oracle to the reference program.

Builds the UNMODIFIED reference (kernel.cu, IDIC.h, data.h) for the host CPU
with oracle/build_ref.sh, runs its own ``main`` (its own Init.txt reader,
``init_Sod_X_Dust`` generator, host cell lists, 27-offset sweeps, host IDIC
averaging and solve) on small Init.txt files, and stores what its snapshot
writers print (``Data_out`` / ``Data_out_dust``, kernel.cu:232-826, printed
with ``%10.8lf``) as compressed .npz fixtures next to this script.

Needs the reference tree, named by the DS_REFERENCE_DIR environment variable
(there is no default); run it in a checkout that has one:  python tests/golden/make_golden.py
The fixtures are small and committed; tests only read them.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

TEMPLATE = """// Initial parameters
{X_min}\t\t// X_min
{X_max}\t\t\t// X_max
{Y_min}\t\t// Y_min
{Y_max}\t\t\t// Y_max
{Z_min}\t\t// Z_min
{Z_max}\t\t\t// Z_max
{typ}\t\t\t// Eq of State (0 - with e, 1 -  acoustic)
100000\t// Maximum of particle
{pol}\t\t\t// Particle on 1 length
{h}\t\t\t//\th
0.5\t\t\t// h_cell / h0
{tau}\t\t// tau
{t_end}\t\t\t// Time end
{t_out}\t\t// Time interval to output in files
{alpha}\t\t\t// alfa
{beta}\t\t\t// beta
{eps}\t\t// eps
"""

# name -> Init.txt values.  refA: particles sit on IDIC cell faces, so dust 1 and
# dust 2 split across faces and the reference's eps_2 guard (kernel.cu:2203)
# yields NaN at step 3 (the NaN onset is part of what is pinned).  refB / refC:
# no NaN for the stored steps; refC uses the acoustic EOS (Type_of_state 1).
CONFIGS = {
    "refA": dict(X_min=-1.2, X_max=1.2, Y_min=-0.8, Y_max=1.0, Z_min=-0.8, Z_max=1.0, typ=0, pol=10, h=0.2,
                 tau="5.0e-3", t_end=0.015, t_out=0.005, alpha=1.0, beta=2.0, eps=0.01),
    "refB": dict(X_min=-1.05, X_max=1.15, Y_min=-0.65, Y_max=0.85, Z_min=-0.72, Z_max=0.78, typ=0, pol=12,
                 h=0.19, tau="3.0e-3", t_end=0.03, t_out=0.015, alpha=1.0, beta=2.0, eps=0.01),
    "refC": dict(X_min=-1.05, X_max=1.15, Y_min=-0.65, Y_max=0.85, Z_min=-0.72, Z_max=0.78, typ=1, pol=10,
                 h=0.23, tau="4.0e-3", t_end=0.04, t_out=0.02, alpha=0.5, beta=1.0, eps=0.01),
}

GAS_COLS = ["x", "y", "z", "r", "mas", "rho", "p", "Vx", "Vy", "Vy2", "V", "e", "Ind", "Nn"]
DUST_COLS = ["x", "y", "z", "r", "mas", "rho", "t_stop", "Vx", "Vy", "Vy2", "V", "Ind", "Nn"]
GAS_KEEP = ["x", "y", "z", "rho", "p", "Vx", "Vy", "V", "e"]
DUST_KEEP = ["x", "y", "z", "rho", "t_stop", "Vx", "Vy", "V"]


def _read(path):
    with open(path) as f:
        lines = f.read().splitlines()
    t = float(lines[0].split("=")[1])
    rows = [[float(v) for v in l.split()] for l in lines[3:] if l.strip()]
    return t, np.array(rows, dtype=np.float64)


def build_reference() -> str:
    if not os.environ.get("DS_REFERENCE_DIR"):
        raise SystemExit("DS_REFERENCE_DIR is not set: point it at the reference tree (kernel.cu, IDIC.h, data.h)")
    r = subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True, capture_output=True, text=True)
    return r.stdout.strip().splitlines()[-1]


def run_config(exe: str, name: str, cfg: dict) -> dict:
    init = TEMPLATE.format(**cfg)
    out = {"init_txt": np.array(init)}
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "Data"))
        with open(os.path.join(d, "Init.txt"), "w") as f:
            f.write(init)
        subprocess.run([exe], cwd=d, check=True, stdout=subprocess.DEVNULL,
                       env=dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count() or 1)))
        files = sorted(f for f in os.listdir(os.path.join(d, "Data")) if f.startswith("G"))
        nsnap = len(files)
        t0, G0 = _read(os.path.join(d, "Data", "G0000000.dat"))
        ind = G0[:, GAS_COLS.index("Ind")].astype(np.int8)
        interior = ind == 0
        out["ind"] = ind
        out["x0"] = G0[:, 0]
        snaps = []
        for s in range(1, nsnap):
            t, G = _read(os.path.join(d, "Data", f"G{s:07d}.dat"))
            snaps.append(t)
            for c in GAS_KEEP:
                out[f"s{s}_gas_{c}"] = G[interior, GAS_COLS.index(c)]
            out[f"s{s}_gas_Nn"] = G[:, GAS_COLS.index("Nn")].astype(np.int32)
            for k in (1, 2):
                _, D = _read(os.path.join(d, "Data", f"D-{k}-{s:07d}.dat"))
                for c in DUST_KEEP:
                    out[f"s{s}_d{k}_{c}"] = D[interior, DUST_COLS.index(c)]
                out[f"s{s}_d{k}_Nn"] = D[:, DUST_COLS.index("Nn")].astype(np.int32)
        out["snap_times"] = np.array(snaps)
    return out


def main(argv):
    exe = build_reference()
    names = argv[1:] or list(CONFIGS)
    for name in names:
        data = run_config(exe, name, CONFIGS[name])
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: {len(data['snap_times'])} snapshots, {int((data['ind'] == 0).sum())} interior of "
              f"{len(data['ind'])}, {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main(sys.argv)
