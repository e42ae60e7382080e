"""FP32_REFINED against FP64 over a whole P-E loop of a benchmark film.

Runs the film's loop twice on the GPU -- CMSL_FP64 (TDGL bit-identical to the
reference kernels, PCG to ||r|| <= tol ||b||) and CMSL_FP32_REFINED (refined
to the same residual target) -- from the same initial state, and reports the
relative errors of the remanent polarization and coercive field of the loop
(cmsl_gb300.pe), the max-abs / relative-L2 errors of the final P and phi, and
the cell-steps/s of both runs.

    python -m cmsl_gb300.precision --config 0
    python -m cmsl_gb300.precision --config 1 --steps-per-period 4000 --periods 1
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import pe
from . import workloads as wl


def run_loop(w, precision, tol=1e-8, inner_tol=1e-5, stream=None):
    import torch
    import cmsl_gb300 as cg
    kw = dict(pcg_crit=cg.CRIT_RELRES, tol_rel=tol, max_iter=20000)
    if precision == "fp32":
        kw.update(precision=cg.FP32_REFINED, refine_tol=tol, max_refine=6, inner_tol=inner_tol,
                  inner_max_iter=2000, warm_start=2)
    else:
        kw.update(precision=cg.FP64)
    s = w.sched
    with cg.Film(w.nx, w.ny, w.nz, w.omega, w.grain_mat, w.TR, w.mats, **w.film_kwargs(), **kw) as f:
        f.set_state(w.P_init)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f.run(s.Ez, s.rows)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        rows = f.rows(0, s.n_rows)
        P, phi = f.get_state()
        it, rf = f.iters(s.n_steps)
    return {"rows": rows, "P": P, "phi": phi, "secs": secs, "iters": float(np.mean(it)), "refine": float(np.mean(rf))}


def compare(w, tol=1e-8, inner_tol=1e-5) -> dict:
    r64 = run_loop(w, "fp64", tol)
    r32 = run_loop(w, "fp32", tol, inner_tol)
    E = w.sched.row_E
    m64 = pe.loop_metrics(E, r64["rows"][:, 0])
    m32 = pe.loop_metrics(E, r32["rows"][:, 0])
    cs = w.N * w.sched.n_steps
    Es, Ps = w.E0_ref / 1.0e8, w.P0_ref * 100.0
    return {
        "workload": w.name, "cells": w.N, "steps": w.sched.n_steps, "rows": w.sched.n_rows,
        "residual_target": tol,
        "fp64": {"Pr_uC_cm2": m64["Pr"] * Ps, "Ec_MV_cm": m64["Ec"] * Es, "cell_steps_per_s": cs / r64["secs"],
                 "pcg_iters_per_step": r64["iters"]},
        "fp32_refined": {"Pr_uC_cm2": m32["Pr"] * Ps, "Ec_MV_cm": m32["Ec"] * Es,
                         "cell_steps_per_s": cs / r32["secs"], "pcg_iters_per_step": r32["iters"],
                         "refine_passes_per_step": r32["refine"]},
        "speedup_fp32_over_fp64": r64["secs"] / r32["secs"],
        "rel_err": pe.relative_errors(m32, m64),
        "P_err": pe.field_errors(r32["P"], r64["P"]),
        "phi_err": pe.field_errors([r32["phi"]], [r64["phi"]]),
        "rows_max_abs_err": float(np.abs(r32["rows"][:, :10] - r64["rows"][:, :10]).max()),
    }


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--config", type=int, default=0, choices=[0, 1, 4])
    ap.add_argument("--steps-per-period", type=int, default=0, help="override the loop length")
    ap.add_argument("--periods", type=int, default=1)
    ap.add_argument("--tol", type=float, default=1e-8)
    args = ap.parse_args(argv)
    import torch
    torch.cuda.set_device(0)
    from . import build
    build.build()
    w = wl.config(args.config)
    if args.steps_per_period:
        w = wl.with_loop(w, args.steps_per_period, args.periods)
    print(json.dumps(compare(w, args.tol)))


if __name__ == "__main__":
    main()
