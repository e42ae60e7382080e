"""Times the reference program's own FP64 GPU path against this library on
one P-E loop.  Measurement infrastructure only.

Both executables come from oracle/ref_gpu.sh: Pfmhzo.exe is the reference
program (HZO_Code_github: kernelCalc_antiferro + Depol_field with cuBLAS
PCG, FP64); Pfmhzo_gb is the same program -- the same main.cu, set-up,
input reading and output -- with Evolve / Depol_field on libcmsl_gb
(CMSL_PRECISION selects FP64 or FP32-refined).  One inputs tree is generated
(a columnar Voronoi grain map of the given size, one Landau set, one phase
fraction set: 40 % AFE, 60 % FE), each program runs one simulation in it,
and the "Kernel execution time" each Evolve prints (the P-E loop alone,
CUDA events) gives the cell-steps/s.  The loop's step count comes from the
Evolve schedule of the deck (the reference's own field staircase).

    python -m oracle.ref_gpu_time --nx 256 --ny 256 --nz 32 --grains 200
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_DIR = os.path.join(ROOT, "baseline", "_ref", "hzo")

# one Landau set (AFE alpha beta gamma g a0, FE alpha beta gamma g a0, DE alpha a0) and its reference phase
LANDAU = ("5.022532e+08 -9.065448e+10 2.189509e+12 5.453480e+08 1.0e+09 "
          "-2.98e+08 -8.520e+09 3.134e+11 -2.484e+08 1.0e+09 9.5e+09 2.372e+09 FE\n")


def deck(nx, ny, nz, Eap, delEap, num_steps, eps=(30.0, 30.0, 30.0)):
    return f"""device_flag = 0
nx = {nx}
ny = {ny}
nz = {nz}
del_h = 1.0
del_t = 0.01
delEap = {delEap:.6e}
Eap = {Eap:.6e}
num_steps = {num_steps}
out_flag = 0
dep_flag = 1
L_de = 1.0
kappa_de = 2.5e-09
kappa_fe = 5.066e-10
L_fe = 0.833
kappa_afe = 1.0e-09
L_afe = 0.2
dimx = 8
dimy = 4
dimz = 4
crystal_type = poly
PsNoise = 0.01
n_layers = 1
layer_counts = {nz}
G0 = 1.0
omg = 0.075
eps_fe = {eps[1]}
eps_afe = {eps[0]}
eps_de = {eps[2]}
z_bc_type = diri
do_pre_relax = 0
"""


def make_tree(root, nx, ny, nz, ng, seed, Eap, delEap, num_steps):
    sys.path.insert(0, ROOT)
    from cmsl_gb300 import formats as fm
    os.makedirs(os.path.join(root, "inputs", "struc1"), exist_ok=True)
    os.makedirs(os.path.join(root, "output"), exist_ok=True)
    with open(os.path.join(root, "inputs", "InputParams"), "w") as fh:
        fh.write(deck(nx, ny, nz, Eap, delEap, num_steps))
    with open(os.path.join(root, "landau.txt"), "w") as fh:
        fh.write(LANDAU)
    with open(os.path.join(root, "phase.txt"), "w") as fh:
        fh.write("40 60 0\n")
    om, cent, eul = fm.voronoi_columnar(nx, ny, nz, ng, seed)
    fm.write_grains(os.path.join(root, "inputs", "struc1"), "poly", os.path.join(root, "inputs", "gnumb_poly.txt"),
                    nx, ny, nz, om, cent, eul)
    # the loop length: the Evolve schedule of this deck
    d = fm.read_deck(os.path.join(root, "inputs", "InputParams"))
    v = [float(x) for x in LANDAU.split()[:12]]
    raw = [dict(alpha=v[0], beta=v[1], gamma1=v[2], g=v[3], a0=v[4], L=d["L_afe"], kappa=d["kappa_afe"],
                eps_r=d["eps_afe"]),
           dict(alpha=v[5], beta=v[6], gamma1=v[7], g=v[8], a0=v[9], L=d["L_fe"], kappa=d["kappa_fe"],
                eps_r=d["eps_fe"]),
           dict(alpha=v[10], beta=0.0, gamma1=0.0, g=0.0, a0=v[11], L=d["L_de"], kappa=d["kappa_de"],
                eps_r=d["eps_de"])]
    _, sc = fm.nondim(raw, 1, d["Eap"], d["delEap"])
    Ez, _, _, _ = fm.evolve_schedule(sc["maxEz"], sc["delEz"], d["num_steps"])
    return len(Ez)


def run(exe, root, env_extra, timeout):
    env = dict(os.environ, **env_extra)
    r = subprocess.run([exe, "0", os.path.join(root, "landau.txt"), os.path.join(root, "phase.txt"), "1"],
                       cwd=root, env=env, capture_output=True, text=True, timeout=timeout)
    m = re.findall(r"Kernel execution time: ([0-9.eE+-]+) s", r.stdout)
    if r.returncode != 0 or not m:
        raise RuntimeError("%s failed (rc %d): %s" % (os.path.basename(exe), r.returncode,
                                                      (r.stdout[-800:] + r.stderr[-800:]).strip()))
    return float(m[-1])


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--ny", type=int, default=256)
    ap.add_argument("--nz", type=int, default=32)
    ap.add_argument("--grains", type=int, default=200)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--Eap", type=float, default=3.0e8, help="loop amplitude, V/m")
    ap.add_argument("--delEap", type=float, default=3.0e7, help="field step of the staircase, V/m")
    ap.add_argument("--num-steps", type=int, default=2, help="time steps per field level")
    ap.add_argument("--timeout", type=float, default=1200.0)
    ap.add_argument("--only-reference", action="store_true", help="time Pfmhzo.exe alone")
    args = ap.parse_args(argv)
    print(json.dumps(measure(args)))


def build_reference(timeout: float = 600.0) -> bool:
    """Builds Pfmhzo.exe (and Pfmhzo_gb when the library is built) from the
    staged sources; False when they are not staged or the build fails."""
    if not os.path.exists(os.path.join(REF_DIR, "src", "evolve.cu")):
        return False
    r = subprocess.run(["sh", os.path.join(HERE, "ref_gpu.sh"), "build"], capture_output=True, text=True,
                       timeout=timeout)
    return r.returncode == 0 and os.path.exists(os.path.join(REF_DIR, "Pfmhzo.exe"))


def measure(args) -> dict:
    ref, gb = os.path.join(REF_DIR, "Pfmhzo.exe"), os.path.join(REF_DIR, "Pfmhzo_gb")
    runs = [("reference_fp64", ref, {})]
    if not getattr(args, "only_reference", False):
        runs += [("cmsl_fp64", gb, {"CMSL_PRECISION": "fp64"}), ("cmsl_fp32_refined", gb, {"CMSL_PRECISION": "fp32"})]
    for _, x, _ in runs:
        if not os.path.exists(x):
            raise SystemExit("%s missing: run oracle/ref_gpu.sh stage (where the reference is) and build" % x)
    N = args.nx * args.ny * args.nz
    out = {"grid": [args.nx, args.ny, args.nz], "cells": N, "grains": args.grains}
    for name, exe, env in runs:
        with tempfile.TemporaryDirectory() as root:
            steps = make_tree(root, args.nx, args.ny, args.nz, args.grains, args.seed, args.Eap, args.delEap,
                              args.num_steps)
            secs = run(exe, root, env, args.timeout)
        out[name] = {"seconds": secs, "steps": steps, "cell_steps_per_s": N * steps / secs}
    out["solve"] = ("the reference's PCG stop test (rz <= 1e-6 or rz/rz0 <= 1e-4, global.cu) for the FP64 runs; "
                    "the FP32-refined run refines to ||b - A phi|| <= 1e-8 ||b||")
    out["speedup_vs_reference_fp64"] = {k: out[k]["cell_steps_per_s"] / out["reference_fp64"]["cell_steps_per_s"]
                                        for k in ("cmsl_fp64", "cmsl_fp32_refined") if k in out}
    return out


if __name__ == "__main__":
    main()
