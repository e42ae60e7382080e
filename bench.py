#!/usr/bin/env python3
"""Benchmark: TDGL cell-steps/s including the depolarisation PCG.

A step is one time step of the P-E loop on the film of the second benchmark
configuration (256x256x32 cells, 200-grain columnar Voronoi from seed 1, 40 %
AFE grains, triangle field +-4 MV/cm at 4000 steps/period): the TDGL update,
the depolarisation solve to ||b - A phi|| <= 1e-8 ||b|| and the sweep-row
averages.  Inputs are synthetic (seeded generator; the reference ships no
grain maps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp32|fp64]
  python bench.py --impl reference ...   # the oracle (CPU FP64 port) on host cores

Under torchrun (N > 1) every rank advances its own film (replicas: the path
has no exchange step); value is all ranks' cell-steps over the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TDGL cell-steps/s incl. PCG, FP32-refined vs FP64 on GB300 at equal P-E error"
CONFIG_ID = 1

# Algorithmic bytes per cell (the compulsory DRAM traffic of the path, the
# roofline's numerator), with s = 4 (FP32) or 8 (FP64) bytes per stored value
# and the grain code 4 bytes; per-grain tables are cache-resident:
#   tdgl:  read 6 P, write 6 P, read phi, read the code, write div P  -> 14 s + 4
#   pcg:   one inner iteration: the SpMV reads p and the code and writes Ap;
#          the update reads x, r, Ap, p and writes x, r              -> 10 s + 4
#          (the direct inner solve is counted as one inner iteration)
#   ref:   one FP64-accurate refinement pass: read phi, div P, the code,
#          write r                                                     -> 28 (FP32 path)
ALG = {"fp32": {"tdgl": 14 * 4 + 4, "pcg": 10 * 4 + 4, "ref": 28},
       "fp64": {"tdgl": 14 * 8 + 4, "pcg": 10 * 8 + 4, "ref": 0}}
# The per-kernel algorithmic bytes of the roofline line (by kernel):
#   tdgl -> ALG tdgl; setup (first refinement pass; FP64: the RHS) and update
#   (update pass) -> ALG ref (FP64 rhs: read Pm, write b: 3 s + 4 + s);
#   spec (one direct solve) and pcg_iter / spmv+update -> ALG pcg;
#   tdgl_check (the TDGL step that also forms the previous step's deferred
#   check, one refinement pass's work) -> ALG tdgl + ALG ref.
# Bytes the kernels as designed move per launch (what they read and write,
# including the double-float potential and the warm start's older
# potentials), kept beside the algorithmic figure:
DESIGN_BYTES = {
    "fp32": {"tdgl": 6 * 4 * 2 + 8 + 4 + 2 * 8 + 8, "tdgl_check": 6 * 4 * 2 + 8 + 4 + 2 * 8 + 8 + 4 + 4 + 8,
             "setup": 8 + 12 + 4, "update": 8 + 4 + 4 + 4 + 8,
             "pcg_iter": 7 * 4 + 5 * 4, "spmv32": 4 * 4 + 2 * 4, "update32": 5 * 4 + 2 * 4, "spec": 40},
    "fp64": {"tdgl": 6 * 8 * 2 + 8 + 4, "setup": 24 + 8 + 4 + 8 + 8, "spmv": 8 * 3 + 4 + 16,
             "update": 5 * 8 + 2 * 8},
}
KERNELS = {"fp32": ["tdgl", "setup", "pcg_iter"], "fp64": ["tdgl", "setup", "spmv", "update"]}


def alg_bytes(mode: str, kernel: str) -> int:
    """Algorithmic bytes per cell of one launch of `kernel`."""
    a = ALG[mode]
    if kernel == "tdgl":
        return a["tdgl"]
    if kernel == "tdgl_check":
        return a["tdgl"] + a["ref"]
    if kernel in ("setup", "update") and mode == "fp32":
        return a["ref"]
    if mode == "fp64" and kernel == "setup":
        return 3 * 8 + 4 + 8
    if mode == "fp64" and kernel == "spmv":
        return 8 + 4 + 8                      # the SpMV part of one iteration
    if mode == "fp64" and kernel == "update":
        return a["pcg"] - (8 + 4 + 8)         # the update part
    return a["pcg"]                           # spec, pcg_iter, spmv32 + update32


def step_bytes(mode: str, n_iter: float, n_ref: float) -> float:
    """B_alg = B_tdgl + n_iter B_pcg + n_ref B_ref per cell-step."""
    a = ALG[mode]
    return a["tdgl"] + n_iter * a["pcg"] + n_ref * a["ref"]


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(workload: str):
    """Per-cell DRAM bytes per kernel of this workload from the committed ncu
    summary (profiles/traffic_per_cell.json), if measured."""
    p = os.path.join(ROOT, "profiles", "traffic_per_cell.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh).get(workload, {})
    return {}


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx.append(float(p[2]))
                except ValueError:
                    continue
                for n, v in zip(names, p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(ms: float, dist=None, device: str = "cpu") -> float:
    """The slowest rank's timed region (replicas run independently; the job
    is as fast as its slowest rank).  dist: torch.distributed when N > 1."""
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
    return float(t.item())


def replica_rate(cells_per_rank: int, steps: int, ms_max: float, world: int) -> float:
    """Whole-job cell-steps/s of `world` replicas of `cells_per_rank` cells
    each advancing `steps` steps within `ms_max` milliseconds (weak scaling)."""
    return world * cells_per_rank * steps / (ms_max * 1e-3)


def make_oracle_film(w, orc, crit_relres=True):
    import oracle
    f = oracle.Film(nx=w.nx, ny=w.ny, nz=w.nz, del_h=w.del_h, del_t=w.del_t, omega=w.omega,
                    grain_mat=w.grain_mat, TR=w.TR, mats=w.mats,
                    is_interface=orc.interface_flags(w.nx, w.ny, w.nz, w.omega, w.grain_mat),
                    dep_flag=1, eps_0_nd=w.eps_0_nd)
    if crit_relres:
        f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-8, 4000
    return f


def cpu_port_rate(w, steps: int, budget_s: float):
    """Times the oracle (FP64 CPU port, all host threads) on the film for up to
    `steps` steps or `budget_s` seconds; returns (cell-steps/s, steps, seconds)."""
    import oracle
    orc = oracle.load()
    f = make_oracle_film(w, orc)
    P = [p.copy() for p in w.P_init]
    phi = np.zeros(w.N)
    E = None
    done, t_total = 0, 0.0
    Ez = w.sched.Ez
    while done < steps:
        t0 = time.perf_counter()
        P, E, phi, _, _, rc = orc.run(f, P, phi, Ez[done:done + 1], np.array([0], np.int32), E=E)
        t_total += time.perf_counter() - t0
        done += 1
        if t_total > budget_s:
            break
    return w.N * done / t_total, done, t_total


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from cmsl_gb300 import workloads as wl
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    if args.config == 3:
        # the ensemble: one time step of each film in turn, within the budget
        ws = wl.ensemble(64, 100)
        cpu_port_rate(ws[0], 1, 30.0)
        tot_c, tot_s, done = 0, 0.0, 0
        for w in ws:
            if tot_s > 150.0 or done >= args.steps:
                break
            rate, n, secs = cpu_port_rate(w, 1, 30.0)
            tot_c += w.N * n
            tot_s += secs
            done += n
        rate = tot_c / tot_s
        line = {
            "impl": "reference", "metric": METRIC, "value": rate, "unit": "cell-steps/s", "n_gpus": args.gpus,
            "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / max(done, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "c3_ensemble64", "precision": "fp64", "pcg": "relres 1e-8",
                       "implementation": "oracle (CPU FP64 port of the reference kernels, OpenMP)"},
            "cpu_baseline": {"value": rate, "unit": "cell-steps/s", "cores": cores, "kind": "port",
                             "sample": "one time step of each of the first %d films" % done},
            "e2e": {"value": rate, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return 0
    w = wl.config(args.config)
    # each step is a bounded sample: the full film, one time step
    cpu_port_rate(w, max(1, min(args.warmup, 1)), 60.0)
    rate, done, secs = cpu_port_rate(w, args.steps, 150.0)
    gpu_ref = reference_gpu(w) if not args.no_ref_gpu else None
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "cell-steps/s", "n_gpus": args.gpus,
        "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(done, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "cells": w.N, "precision": "fp64", "pcg": "relres 1e-8",
                   "implementation": "oracle (CPU FP64 port of the reference kernels, OpenMP)"},
        "cpu_baseline": {"value": rate, "unit": "cell-steps/s", "cores": cores, "kind": "port",
                         "sample": "%d full time steps of %s (%d cells) from its initial state" %
                                   (done, w.name, w.N)},
        "e2e": {"value": rate, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_fp64_gpu": gpu_ref,
    }
    print(json.dumps(line))
    return 0


def reference_gpu(w):
    """The reference program's own FP64 GPU path (Pfmhzo.exe: its CUDA TDGL
    kernel and cuBLAS Jacobi-PCG) on a film of this workload's grid and grain
    count, built from the staged sources (oracle/ref_gpu.sh) and timed by the
    Evolve loop's own CUDA events; None when the sources are not staged."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
        from oracle import ref_gpu_time as rg
        if not rg.build_reference():
            return {"unavailable": "reference program sources not staged or its build failed"}
        amp = float(w.extra.get("Emax", 0.0)) * w.E0_ref          # V/m
        a = argparse.Namespace(nx=w.nx, ny=w.ny, nz=w.nz, grains=int(len(w.grain_mat)), seed=1,
                               Eap=amp, delEap=amp / 10.0, num_steps=4, timeout=600.0, only_reference=True)
        out = rg.measure(a)
        r = out["reference_fp64"]
        return {"value": r["cell_steps_per_s"], "unit": "cell-steps/s", "steps": r["steps"], "seconds": r["seconds"],
                "grid": out["grid"], "grains": out["grains"],
                "note": "Pfmhzo.exe (reference CUDA kernels + cuBLAS PCG, its own stop test rz <= 1e-6 or "
                        "rz/rz0 <= 1e-4), one staircase P-E loop of the reference deck on a columnar Voronoi map of "
                        "this grid, 40 % AFE, eps 30; Kernel execution time of its Evolve"}
    except Exception as exc:       # reported, never fatal to the CPU baseline
        return {"unavailable": "%s: %s" % (type(exc).__name__, str(exc)[:300])}


def film_kw(cg, fp64: bool, inner=None) -> dict:
    kw = dict(precision=cg.FP64 if fp64 else cg.FP32_REFINED, pcg_crit=cg.CRIT_RELRES, tol_rel=1e-8,
              max_iter=4000, refine_tol=1e-8, max_refine=6, inner_tol=1e-5, inner_max_iter=2000,
              warm_start=2)
    if inner is not None:
        kw["inner_solver"] = inner
    return kw


def timed_repeats(film, Ez, rows, W: int, K: int, R: int, stream, dist=None, clocks=None):
    """W untimed warm-up steps, then R timed regions of exactly K steps each
    (the P-E loop continues from region to region), each bracketed by a
    barrier and a device synchronisation and timed with CUDA events on the
    launch stream.  Returns the per-region milliseconds."""
    import torch
    sp = stream.cuda_stream
    out = []
    with torch.cuda.stream(stream):
        film.run(Ez[:W], rows[:W], stream=sp)
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        for r in range(R):
            e = Ez[W + r * K:W + (r + 1) * K]
            if dist:
                dist.barrier()
            torch.cuda.synchronize()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            film.run(e, rows[:K], stream=sp, sync=False)
            ev1.record(stream)
            ev1.synchronize()
            film.sync()
            torch.cuda.synchronize()
            out.append(ev0.elapsed_time(ev1))
    return out


def n_repeats(K: int, W: int, n_sched: int, est_ms_step: float, target_s: float = 1.5, r_min: int = 10) -> int:
    """Timed regions: at least r_min, enough for ~target_s of timed work (so
    the clock sampler sees the GPU under load), within the loop's schedule."""
    want = max(r_min, int(math.ceil(target_s * 1e3 / max(K * est_ms_step, 1e-6))))
    return max(1, min(want, (n_sched - W) // K))


def side_run(cg, w, fp64: bool, inner, K: int, stream, mats=None, name=""):
    """A short sample of another solver configuration of the same film (the
    PCG paths): cell-steps/s over K steps after 3 warm-up steps, the PCG
    iterations per step and the inner solve's kernel time."""
    import torch
    mm = w.mats if mats is None else mats
    f = cg.Film(w.nx, w.ny, w.nz, w.omega, w.grain_mat, w.TR, mm, **w.film_kwargs(), **film_kw(cg, fp64, inner))
    f.set_state(w.P_init)
    rows = np.arange(3 + K, dtype=np.int32)
    ms = timed_repeats(f, w.sched.Ez, rows, 3, K, 1, stream)
    it, rf = f.iters(K)
    kms = f.time_kernels(reps=5, stream=stream.cuda_stream)
    mode = "fp64" if fp64 else "fp32"
    n_iter, n_ref = float(np.mean(it)), float(np.mean(rf))
    rate = w.N * K / (ms[0] * 1e-3)
    out = {"value": rate, "unit": "cell-steps/s", "steps": K, "ms_per_step": ms[0] / K,
           "inner_solver": "direct" if f.inner_solver == cg.INNER_DIRECT else "pcg",
           "pcg_iters_per_step": n_iter, "refine_passes_per_step": n_ref,
           "eps_r": [float(v) for v in np.asarray(mm)[:, 7]],
           "frac_step": step_bytes(mode, n_iter, n_ref) * rate / 1e9 / measured_peaks()[0]}
    if not fp64 and f.inner_solver != cg.INNER_DIRECT:
        # kernel_ms[2]: one iteration of the persistent PCG over the film
        out["pcg_kernel"] = {"kernel": "k_pcg_cg2", "us_per_iter": kms[2] * 1e3,
                             "bytes_per_cell": ALG["fp32"]["pcg"],
                             "frac": ALG["fp32"]["pcg"] * w.N / (kms[2] * 1e-3) / 1e9 / measured_peaks()[0]}
    f.close()
    torch.cuda.synchronize()
    return out


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from cmsl_gb300 import build
    if rank == 0:
        build.build()
    if dist:
        dist.barrier()
    import cmsl_gb300 as cg
    from cmsl_gb300 import workloads as wl

    fp64 = args.precision == "fp64"
    mode = "fp64" if fp64 else "fp32"
    w = wl.config(args.config)
    film = cg.Film(w.nx, w.ny, w.nz, w.omega, w.grain_mat, w.TR, w.mats, **w.film_kwargs(), **film_kw(cg, fp64))
    if not args.no_autotune:
        film.autotune()
    tile_cfg = film.tile_config()
    film.set_state(w.P_init)
    K, W = args.steps, args.warmup
    n_sched = w.sched.n_steps
    rows = np.arange(max(W, K) + 1, dtype=np.int32)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    # a first timed region sizes the repeats
    probe = timed_repeats(film, w.sched.Ez, rows, W, K, 1, stream, dist)
    R = args.repeats or n_repeats(K, W + K, n_sched, probe[0] / K)
    film.set_state(w.P_init)
    clocks = Clocks(local)
    ms_all = timed_repeats(film, w.sched.Ez, rows, W, K, R, stream, dist, clocks)
    clk = clocks.stop()
    clk["repeats"] = R
    ms = statistics.median(ms_all)
    it, rf = film.iters(K)
    ms_max = max_over_ranks(ms, dist, "cuda")
    value = replica_rate(w.N, K, ms_max, world)

    # per-kernel device times (CUDA events on the launch stream)
    kms = film.time_kernels(reps=50, stream=sp)
    n_iter = float(np.mean(it))
    n_ref = float(np.mean(rf))
    direct = film.inner_solver == cg.INNER_DIRECT
    # direct solve: one full pass per step, the later ones (almost always)
    # update passes -- or, deferred (time_kernels reports no update pass), the
    # check formed inside the next TDGL step
    deferred = direct and kms[3] == 0.0
    names = (["tdgl_check", "setup", "spec"] if deferred else
             ["tdgl", "setup", "spec", "update"] if direct else KERNELS[mode])
    count = {"tdgl": 1.0, "tdgl_check": 1.0, "setup": 1.0 if direct else n_ref, "spmv": n_iter,
             "update": max(n_ref - 1.0, 0.0) if direct else n_iter, "pcg_iter": n_iter, "spec": n_iter}
    per_step = {k: kms[i] * count[k] for i, k in enumerate(names)}
    top = max(per_step, key=per_step.get)
    ki = names.index(top)
    peak, peak_kind = measured_peaks()
    b_alg = alg_bytes(mode, top)
    achieved = b_alg * w.N / (kms[ki] * 1e-3) / 1e9
    traffic = ncu_traffic(w.name).get(mode, {}).get(top)
    b_step = step_bytes(mode, n_iter, n_ref)
    roof = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "bytes_per_cell": b_alg, "design_bytes_per_cell": DESIGN_BYTES[mode].get(top),
            "traffic": (traffic * w.N) if traffic is not None else None,
            "kernel_ms": {k: float(kms[i]) for i, k in enumerate(names)},
            "kernel_frac": {k: alg_bytes(mode, k) * w.N / (kms[i] * 1e-3) / 1e9 / peak for i, k in enumerate(names)},
            "share": {k: per_step[k] / sum(per_step.values()) for k in per_step},
            "step_bytes_per_cell": b_step,
            "frac_step": b_step * value / world / 1e9 / peak,
            "step_model": "B_tdgl + n_iter B_pcg + n_ref B_ref = %d + %.2f x %d + %.2f x %d" % (
                ALG[mode]["tdgl"], n_iter, ALG[mode]["pcg"], n_ref, ALG[mode]["ref"])}
    if fp64:
        launches = int(K * 3 + 2 * it.sum())
    elif deferred:
        # TDGL (with the previous step's check), the passes but that check,
        # five per direct solve; after the step loop the last check's pass and
        # the kernel that opens it
        launches = int(K + (rf - 1).sum() + 5 * it.sum() + 2)
    elif direct:
        # TDGL, the refinement passes (the last one ends the step), five per direct solve
        launches = int(K + rf.sum() + 5 * it.sum())
    else:
        # TDGL, the refinement passes, one persistent PCG launch per pass but the last
        launches = int(2 * rf.sum())

    # end to end through the C ABI: host state in, K steps, host rows + state
    # out, the state arrays page-locked and allocated once (as a campaign
    # reuses them from loop to loop); the median of several calls
    P_in = [cg.pinned_empty(w.N) for _ in range(6)]
    for a, p in zip(P_in, w.P_init):
        a[:] = p
    st_out = ([cg.pinned_empty(w.N) for _ in range(6)], cg.pinned_empty(w.N))
    film.set_state(P_in)
    film.get_state(out=st_out)
    torch.cuda.synchronize()
    e2e_t = []
    for _ in range(args.e2e_repeats):
        t0 = time.perf_counter()
        film.set_state(P_in)
        film.run(w.sched.Ez[W:W + K], rows[:K])
        film.rows(0, K)
        film.get_state(out=st_out)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_t)
    esz = 8 if fp64 else 4
    h2d = 6 * w.N * esz + K * 12
    d2h = K * 88 + 6 * w.N * esz + w.N * 8
    e2e = {"value": w.N * K / e2e_s * world, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d // K,
           "d2h_bytes_per_step": d2h // K, "repeats": len(e2e_t),
           "note": "per call: host P upload, K steps with host field/row arrays, host rows, P and phi download "
                   "(state arrays page-locked, allocated once); median of the calls"}
    film.close()

    # the PCG paths (the metric's 'incl. PCG'): the same film with the inner
    # solve forced to the persistent Jacobi-PCG; the film with the reference
    # deck's three permittivities (which takes the PCG); the FP64 mode
    # (reference PCG) on both -- the FP32-over-FP64 speed-up at equal inner
    # algorithm next to the one the direct solve gives
    pcg = None
    if rank == 0 and world == 1 and not fp64 and not args.no_pcg:
        mats3 = np.array(w.mats, copy=True)
        mats3[:, 7] = [50.0, 30.0, 15.0]      # eps_afe, eps_fe, eps_de of src/inputs/InputParams
        Ks = max(5, min(K, 20))
        pcg = {"uni_eps_pcg": side_run(cg, w, False, cg.INNER_PCG, Ks, stream),
               "three_eps_pcg": side_run(cg, w, False, cg.INNER_PCG, Ks, stream, mats=mats3),
               "three_eps_preconditioned": side_run(cg, w, False, None, Ks, stream, mats=mats3),
               "fp64_uni_eps": side_run(cg, w, True, None, 3, stream),
               "fp64_three_eps": side_run(cg, w, True, None, 3, stream, mats=mats3)}
        pcg["three_eps_preconditioned"]["note"] = (
            "the direct solve with the middle of the film's permittivity range preconditions the double-float "
            "refinement with Chebyshev increments (the film's grains use eps 50 and 30)")
        pcg["speedup_fp32_over_fp64"] = {
            "direct_inner_solve": value / pcg["fp64_uni_eps"]["value"],
            "same_inner_pcg_uni_eps": pcg["uni_eps_pcg"]["value"] / pcg["fp64_uni_eps"]["value"],
            "same_inner_pcg_three_eps": pcg["three_eps_pcg"]["value"] / pcg["fp64_three_eps"]["value"],
            "three_eps_preconditioned": pcg["three_eps_preconditioned"]["value"] / pcg["fp64_three_eps"]["value"]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        rate, done, secs = cpu_port_rate(w, 3, 20.0)
        cpu = {"value": rate, "unit": "cell-steps/s", "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
               "sample": "%d time steps of %s on the oracle (FP64, %.1f s)" % (done, w.name, secs)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if fp64 else "f32", "data": "synthetic",
            "config": {"workload": w.name, "cells": w.N, "grid": [w.nx, w.ny, w.nz],
                       "precision": "fp64" if fp64 else "fp32-refined (fp64 phi, refine to 1e-8)",
                       "pcg": "||b-A phi|| <= 1e-8 ||b||", "parallelism": "replicas" if world > 1 else "single",
                       "tile": dict(tile_cfg, chosen_by="heuristic" if args.no_autotune
                                    else "autotuner (cmsl_film_autotune)"),
                       "timing": "%d timed regions of K steps, each bracketed by barrier + synchronize and timed "
                                 "with CUDA events on the launch stream; value from the median region" % R,
                       "l2": "no flush: per-step state %.0f MB > 129 MB L2" % (film_bytes(w, fp64) / 1e6)},
            "timed_regions_ms": {"median": ms, "min": min(ms_all), "max": max(ms_all), "n": len(ms_all)},
            "inner_solver": "direct (in-plane FFT + tridiagonal z, one solve per refinement pass)" if direct
            else ("pcg (Jacobi, reference algorithm)" if fp64 else "pcg (persistent single-reduction Jacobi-PCG)"),
            "pcg_iters_per_step": n_iter, "refine_passes_per_step": n_ref,
            "roofline": roof, "pcg_paths": pcg, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": launches * R,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def film_bytes(w, fp64: bool) -> int:
    """State a step reads and writes: two P sets, the potentials, the code."""
    s = 8 if fp64 else 4
    return w.N * (12 * s + 5 * 8 + 4)


def run_batch(args):
    """The batched ensemble: 64 films of uneven size advancing together
    (one graph per step over all films, per-film PCG masks), against the
    same films run one at a time through the single-film path."""
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    from cmsl_gb300 import build
    build.build()
    import cmsl_gb300 as cg
    from cmsl_gb300 import workloads as wl

    ws = wl.ensemble(64, 100)
    kw = dict(precision=cg.FP32_REFINED, pcg_crit=cg.CRIT_RELRES, tol_rel=1e-8, max_iter=4000, refine_tol=1e-8,
              max_refine=6, inner_tol=1e-5, inner_max_iter=2000, warm_start=2, dep_flag=1)
    descs = [dict(nx=w.nx, ny=w.ny, nz=w.nz, omega=w.omega, grain_mat=w.grain_mat, TR=w.TR, mats=w.mats,
                  del_h=w.del_h, del_t=w.del_t, eps_0_nd=w.eps_0_nd, **kw) for w in ws]
    cells = sum(w.N for w in ws)
    K, W = args.steps, args.warmup
    Ez = np.stack([w.sched.Ez[: W + K] for w in ws])
    rows = np.tile(np.arange(W + K, dtype=np.int32), (len(ws), 1))
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    b = cg.Batch(descs)
    if not args.no_autotune:
        b.autotune()
    b_tile = b.tile_config()
    for i, w in enumerate(ws):
        b.set_state(i, w.P_init)
    with torch.cuda.stream(stream):
        b.run(Ez[:, :W], rows[:, :W], stream=sp)
        torch.cuda.synchronize()
        clocks = Clocks(local)
        clocks.start()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        b.run(Ez[:, W:], rows[:, :K], stream=sp, sync=False)
        ev1.record(stream)
        ev1.synchronize()
        st = b.sync()
        clk = clocks.stop()
        ms = ev0.elapsed_time(ev1)
    its = np.stack([b.iters(i, K)[0] for i in range(len(ws))])
    rfs = np.stack([b.iters(i, K)[1] for i in range(len(ws))])
    value = cells * K / (ms * 1e-3)
    kms = b.time_kernels(reps=10, stream=sp)
    # inner solve: the direct spectral solve (ms[2] = one solve of every
    # film), or the persistent PCG (ms[2] = one iteration over every film)
    direct = b.inner_solver == cg.INNER_DIRECT
    deferred = direct and kms[3] == 0.0
    persistent = not direct and len(ws) <= 128 and os.environ.get("CMSL_PCG_TWO_KERNEL", "0") in ("", "0")
    names = (["tdgl_check", "setup", "spec"] if deferred else ["tdgl", "setup", "spec", "update"] if direct else
             ["tdgl", "setup", "pcg_iter"] if persistent else ["tdgl", "setup", "spmv32", "update32"])
    # the loops run while any film is active: per step, the most demanding film
    n_ref = float(np.mean(rfs.max(axis=0)))
    n_it = float(np.mean(its.max(axis=0)))
    count = {"tdgl": 1.0, "tdgl_check": 1.0, "setup": 1.0 if direct else n_ref, "update": max(n_ref - 1.0, 0.0),
             "spmv32": n_it,
             "update32": n_it, "pcg_iter": n_it, "spec": n_it}
    per_step = {k: kms[i] * count[k] for i, k in enumerate(names)}
    top = max(per_step, key=per_step.get)
    ki = names.index(top)
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes("fp32", top) * cells / (kms[ki] * 1e-3) / 1e9
    b_step = step_bytes("fp32", n_it, n_ref)
    roof = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "bytes_per_cell": alg_bytes("fp32", top),
            "design_bytes_per_cell": DESIGN_BYTES["fp32"].get(top), "step_bytes_per_cell": b_step,
            "frac_step": b_step * (cells * K / (ms * 1e-3)) / 1e9 / peak,
            "traffic": None, "kernel_ms": {k: float(kms[i]) for i, k in enumerate(names)},
            "share": {k: per_step[k] / sum(per_step.values()) for k in per_step}}

    # end to end through the C ABI: host states in, K steps, host rows and
    # states out, through page-locked arrays allocated once
    P_in, st_out = [], []
    for w in ws:
        P_in.append([cg.pinned_empty(w.N) for _ in range(6)])
        for a, p in zip(P_in[-1], w.P_init):
            a[:] = p
        st_out.append(([cg.pinned_empty(w.N) for _ in range(6)], cg.pinned_empty(w.N)))
    e2e_t = []
    for _ in range(max(1, args.e2e_repeats)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i, w in enumerate(ws):
            b.set_state(i, P_in[i])
        b.run(Ez[:, W:], rows[:, :K])
        for i in range(len(ws)):
            b.rows(i, 0, K)
            b.get_state(i, out=st_out[i])
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_t)
    b.close()

    # the same films one at a time (single-film path, persistent solver)
    seq_ms = 0.0
    with torch.cuda.stream(stream):
        for i, d in enumerate(descs):
            with cg.Film(**d) as f:
                if not args.no_autotune:
                    f.autotune()
                f.set_state(ws[i].P_init)
                f.run(Ez[i, :W], rows[i, :W], stream=sp)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                f.run(Ez[i, W:], rows[i, :K], stream=sp, sync=False)
                e1.record(stream)
                e1.synchronize()
                f.sync()
                seq_ms += e0.elapsed_time(e1)
    seq = cells * K / (seq_ms * 1e-3)

    cpu = None
    if not args.no_cpu:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        tot_c, tot_s, n = 0, 0.0, 0
        for w in ws[:8]:
            rate, done, secs = cpu_port_rate(w, 1, 5.0)
            tot_c += w.N * done
            tot_s += secs
            n += done
        cpu = {"value": tot_c / tot_s, "unit": "cell-steps/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
               "kind": "port", "sample": "one time step of each of the first 8 films on the oracle (FP64)"}
    h2d = sum(6 * w.N * 4 for w in ws) + K * 12 * len(ws)
    d2h = K * 88 * len(ws) + sum(6 * w.N * 4 + w.N * 8 for w in ws)
    line = {
        "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "c3_ensemble64", "films": len(ws), "cells": cells,
                   "precision": "fp32-refined (fp64 phi, refine to 1e-8)", "pcg": "||b-A phi|| <= 1e-8 ||b|| per film",
                   "parallelism": "single", "l2": "no flush: batch state > 129 MB L2",
                   "tile": dict(b_tile, chosen_by="heuristic" if args.no_autotune
                                else "autotuner (cmsl_batch_autotune)")},
        "sequential": {"value": seq, "unit": "cell-steps/s", "ms_per_step": seq_ms / K,
                       "speedup_batch_over_sequential": value / seq},
        "pcg_iters_per_step_max_film": n_it, "refine_passes_per_step_max_film": n_ref,
        "film_status_nonzero": int((st != 0).sum()),
        "roofline": roof, "cpu_baseline": cpu,
        "e2e": {"value": cells * K / e2e_s, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d // K,
                "d2h_bytes_per_step": d2h // K, "repeats": len(e2e_t), "note": "median of the calls"},
        "inner_solver": ("direct (in-plane FFT + tridiagonal z for every film, one launch set per refinement pass)"
                         if direct else "persistent PCG (one cooperative launch per refinement pass)" if persistent
                         else "two-kernel PCG"),
        "clocks": clk,
        "gpu_launches": (int(K + K * (n_ref - 1) + 5 * K * n_it + 2) if deferred else
                         int(K + K * n_ref + 5 * K * n_it) if direct else
                         int(K * 2 + 2 * K * n_ref) if persistent else int(K * 2 + K * n_ref + 2 * K * n_it)),
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="heuristic z chunk instead of the tile autotuner")
    ap.add_argument("--repeats", type=int, default=0, help="timed regions of K steps (0: enough for ~1.5 s, >= 10)")
    ap.add_argument("--e2e-repeats", type=int, default=5, help="end-to-end calls (the median is reported)")
    ap.add_argument("--no-pcg", action="store_true", help="skip the PCG-path samples")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="reference arm: skip the reference program's FP64 GPU path")
    ap.add_argument("--config", type=int, default=CONFIG_ID, choices=[0, 1, 2, 3, 4],
                    help="benchmark configuration (default 1; 3 = the 64-film batched ensemble)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.config == 3:
        return run_batch(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
