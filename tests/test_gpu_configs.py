"""GPU parity at the benchmark configurations' sizes, against the oracle.

The oracle (FP64 CPU restatement of the reference kernels, OpenMP on the host
cores) runs the same seeded films with the same schedule and the stop test
||b - A phi|| <= 1e-8 ||b||:

* configuration 0 (64x64x16, 20 grains, all FE, +-3 MV/cm, 2501 steps): the
  whole recorded loop.  FP64 mode: every sweep row and the final P and phi.
  FP32-refined: the remanent polarization of the loop within 1e-4 relative
  and the rows within 1e-5.  This loop never takes <P_z> through zero: the
  amplitude, 3 MV/cm, is below the film's intrinsic coercive field
  (a1 = -2e9, a11 = 1e10, a111 = 5e10: max of -df/dP on the unstable branch,
  4.44 MV/cm), so the coercive field of this loop is undefined.
* the same film at +-10 MV/cm on a 1000-step period, which switches (the
  grains' polar axes are tilted by up to acos 0.3 from z, so a grain sees
  E cos(theta), and the depolarisation field opposes the switch; at 6 MV/cm
  the loop still does not cross P = 0): Pr and Ec of the FP32-refined loop
  within 1e-4 of the oracle's.
* configurations 4 (128x128x16) and 1 (256x256x32): the first 20 steps from
  the configuration's initial state, both precisions.

FP64 tolerances: the TDGL step is bit-identical; the PCG's dot products are
summed in another order than the oracle's, which moves the potential by
rounding (~1e-14 relative per solve), and that difference is carried by the
dynamics from step to step.
"""
import math
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-8
FP64_REL = 1e-9          # FP64 mode vs the oracle: P, phi (of max |.|) and rows over a whole loop
FP32_P_REL = 2e-5        # FP32-refined P vs the FP64 oracle (of max |P|)
FP32_PHI_REL = 1e-4      # FP32-refined phi vs the FP64 oracle (of max |phi|)
FP32_ROWS_ABS = 1e-5     # FP32-refined sweep rows (non-dimensional averages)
LOOP_REL = 1e-4          # Pr / Ec of a loop, FP32-refined vs the FP64 oracle


@pytest.fixture(scope="module")
def cg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    from cmsl_gb300 import build
    build.build()
    import cmsl_gb300
    return cmsl_gb300


@pytest.fixture(scope="module")
def orc():
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    return oracle.load()


def _ofilm(w, orc):
    f = oracle.Film(nx=w.nx, ny=w.ny, nz=w.nz, del_h=w.del_h, del_t=w.del_t, omega=w.omega,
                    grain_mat=w.grain_mat, TR=w.TR, mats=w.mats,
                    is_interface=orc.interface_flags(w.nx, w.ny, w.nz, w.omega, w.grain_mat),
                    dep_flag=1, eps_0_nd=w.eps_0_nd)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, TOL, 20000
    return f


_cache = {}


def _oracle_run(orc, w, n_steps=None):
    key = (w.name, n_steps)
    if key not in _cache:
        f = _ofilm(w, orc)
        s = w.sched
        n = s.n_steps if n_steps is None else n_steps
        rows = s.rows[:n] if n_steps is None else np.arange(n, dtype=np.int32)
        P, _, phi, stats, iters, rc = orc.run(f, w.P_init, np.zeros(w.N), s.Ez[:n], rows)
        assert rc == 0
        _cache[key] = (P, phi, stats, iters)
    return _cache[key]


def _gpu_run(cg, w, precision, n_steps=None):
    s = w.sched
    n = s.n_steps if n_steps is None else n_steps
    rows = s.rows[:n] if n_steps is None else np.arange(n, dtype=np.int32)
    n_rows = s.n_rows if n_steps is None else n
    kw = dict(pcg_crit=cg.CRIT_RELRES, tol_rel=TOL, max_iter=20000)
    if precision == "fp32":
        kw.update(precision=cg.FP32_REFINED, refine_tol=TOL, max_refine=6, inner_tol=1e-5, inner_max_iter=2000,
                  warm_start=2)
    with cg.Film(w.nx, w.ny, w.nz, w.omega, w.grain_mat, w.TR, w.mats, **w.film_kwargs(), **kw) as g:
        g.set_state(w.P_init)
        g.run(s.Ez[:n], rows)
        P, phi = g.get_state()
        r = g.rows(0, n_rows)
        it, _ = g.iters(n)
    return P, phi, r, it


def _rel(got, want):
    g = np.concatenate([np.ravel(a) for a in got])
    w = np.concatenate([np.ravel(a) for a in want])
    return float(np.abs(g - w).max()) / max(float(np.abs(w).max()), 1e-300)


def _loop(w, rows):
    from cmsl_gb300 import pe
    return pe.loop_metrics(w.sched.row_E, rows[:, 0])


def test_c0_whole_loop_fp64(cg, orc):
    from cmsl_gb300 import workloads as wl
    w = wl.config(0)
    Pw, phiw, statw, itw = _oracle_run(orc, w)
    Pg, phig, rg, itg = _gpu_run(cg, w, "fp64")
    assert rg.shape == statw.shape
    assert _rel(Pg, Pw) <= FP64_REL
    assert _rel([phig], [phiw]) <= FP64_REL
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= FP64_REL * max(np.abs(statw[:, :10]).max(), 1.0)
    # iteration counts follow the oracle's (the same stop test on the same residuals)
    assert np.abs(itg.astype(int) - itw.astype(int)).max() <= 1


def test_c0_whole_loop_fp32_refined_pr(cg, orc):
    from cmsl_gb300 import workloads as wl
    w = wl.config(0)
    _, _, statw, _ = _oracle_run(orc, w)
    Pg, phig, rg, _ = _gpu_run(cg, w, "fp32")
    mw, mg = _loop(w, statw), _loop(w, rg)
    assert math.isfinite(mw["Pr"]) and abs(mg["Pr"] - mw["Pr"]) <= LOOP_REL * abs(mw["Pr"])
    # below the intrinsic coercive field: no P = 0 crossing in either run
    assert math.isnan(mw["Ec"]) and math.isnan(mg["Ec"])
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= FP32_ROWS_ABS


def test_c0_switching_loop_fp32_refined_pr_ec(cg, orc):
    from cmsl_gb300 import workloads as wl
    w = wl.hzo_film("c0_64x64x16_fe_10MVcm", 64, 64, 16, 20, 0, 0.0, E_amp_MVcm=10.0, steps_per_period=1000)
    _, _, statw, _ = _oracle_run(orc, w)
    _, _, rg, _ = _gpu_run(cg, w, "fp32")
    mw, mg = _loop(w, statw), _loop(w, rg)
    for k in ("Pr", "Ec"):
        assert math.isfinite(mw[k]), k
        assert abs(mg[k] - mw[k]) <= LOOP_REL * abs(mw[k]), (k, mg[k], mw[k])
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= FP32_ROWS_ABS


@pytest.mark.parametrize("cfg", [4, 1])
def test_config_segment_fp64(cg, orc, cfg):
    from cmsl_gb300 import workloads as wl
    w = wl.config(cfg)
    Pw, phiw, statw, itw = _oracle_run(orc, w, 20)
    Pg, phig, rg, itg = _gpu_run(cg, w, "fp64", 20)
    assert _rel(Pg, Pw) <= FP64_REL
    assert _rel([phig], [phiw]) <= FP64_REL
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= FP64_REL * max(np.abs(statw[:, :10]).max(), 1.0)
    assert np.abs(itg.astype(int) - itw.astype(int)).max() <= 1


@pytest.mark.parametrize("cfg", [4, 1])
def test_config_segment_fp32_refined(cg, orc, cfg):
    from cmsl_gb300 import workloads as wl
    w = wl.config(cfg)
    Pw, phiw, statw, _ = _oracle_run(orc, w, 20)
    Pg, phig, rg, _ = _gpu_run(cg, w, "fp32", 20)
    assert _rel(Pg, Pw) <= FP32_P_REL
    assert _rel([phig], [phiw]) <= FP32_PHI_REL
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= FP32_ROWS_ABS


@pytest.mark.parametrize("cfg", [4, 1])
def test_config_segment_deck_permittivities(cg, orc, cfg):
    """The configuration's film with the reference deck's permittivities
    (AFE 50, FE 30, DE 15, src/inputs/InputParams:34-36): the FP32-refined
    run takes the direct solve as the refinement's preconditioner (Chebyshev
    increments); 20 steps against the FP64 oracle with the same tolerances."""
    from cmsl_gb300 import workloads as wl
    w = wl.config(cfg)
    mats = np.array(w.mats, copy=True)
    mats[:, 7] = [50.0, 30.0, 15.0]
    f = oracle.Film(nx=w.nx, ny=w.ny, nz=w.nz, del_h=w.del_h, del_t=w.del_t, omega=w.omega,
                    grain_mat=w.grain_mat, TR=w.TR, mats=mats,
                    is_interface=orc.interface_flags(w.nx, w.ny, w.nz, w.omega, w.grain_mat),
                    dep_flag=1, eps_0_nd=w.eps_0_nd)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, TOL, 20000
    n = 20
    rows = np.arange(n, dtype=np.int32)
    Pw, _, phiw, statw, _, rc = orc.run(f, w.P_init, np.zeros(w.N), w.sched.Ez[:n], rows)
    assert rc == 0
    kw = dict(pcg_crit=cg.CRIT_RELRES, tol_rel=TOL, max_iter=20000, precision=cg.FP32_REFINED, refine_tol=TOL,
              max_refine=6, inner_tol=1e-5, inner_max_iter=2000, warm_start=2)
    with cg.Film(w.nx, w.ny, w.nz, w.omega, w.grain_mat, w.TR, mats, **w.film_kwargs(), **kw) as g:
        assert g.inner_solver == cg.INNER_DIRECT
        g.set_state(w.P_init)
        g.run(w.sched.Ez[:n], rows)
        Pg, phig = g.get_state()
        rg = g.rows(0, n)
    assert _rel(Pg, Pw) <= FP32_P_REL
    assert _rel([phig], [phiw]) <= FP32_PHI_REL
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= FP32_ROWS_ABS
