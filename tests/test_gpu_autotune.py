"""The tile-shape autotuner (cmsl_film_autotune / cmsl_batch_autotune): it
picks a z chunk among ceil(nz / n) for n = 1, 2, ... down to 4 planes (the
chunks of a column differ by one plane at most), leaves the state alone, and a tuned
film advances like an untuned one.  The items set the order of the PCG dot
products and row sums, so with the solve converged to 1e-12 the two runs
agree to 1e-9 of max |P| (FP64) / 1e-6 (FP32_REFINED), rows to 1e-9."""
import numpy as np
import pytest

import oracle
from tests.films import random_film


def chunk_candidates(nz):
    """The z chunks the autotuner tries for a thickest film of nz planes."""
    out, n = [], 1
    while n == 1 or -(-nz // n) >= 4:
        c = -(-nz // n)
        if c not in out:
            out.append(c)
        n += 1
    return out

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cmsl_gb300 import build
    build.build()
    import cmsl_gb300
    return cmsl_gb300


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_autotune_keeps_results(gpu, precision):
    f, P = random_film(40, 24, 20, seed=91, eps_0_nd=4.0, p_scale=0.2, layered=True)
    kw = dict(precision=gpu.FP64 if precision == "fp64" else gpu.FP32_REFINED)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    n = 12
    Ez = np.linspace(0.0, 0.3, n)
    rows = np.arange(n, dtype=np.int32)
    out = []
    for tune in (False, True):
        with gpu.Film.from_oracle_film(f, **kw) as g:
            g.set_state(P)
            if tune:
                zc = g.autotune()
                assert zc in chunk_candidates(20)
                Pt, _ = g.get_state()
                for a, b in zip(Pt, P):
                    assert np.array_equal(a, np.asarray(b, a.dtype)) or np.abs(a - b).max() <= 1e-7
            g.run(Ez, rows)
            out.append((g.get_state()[0], g.rows()))
    (P0, r0), (P1, r1) = out
    tol = 1e-9 if precision == "fp64" else 1e-6
    for a, b in zip(P0, P1):
        assert np.abs(a - b).max() <= tol * np.abs(b).max()
    assert np.abs(r0[:, :10] - r1[:, :10]).max() <= 1e-9 * max(np.abs(r1[:, :10]).max(), 1.0)


def test_batch_autotune(gpu):
    films = [random_film(*sh, seed=95 + i, eps_0_nd=3.0, p_scale=0.2)[0] for i, sh in
             enumerate([(32, 16, 6), (24, 20, 12)])]
    with gpu.Batch.from_oracle_films(films) as b:
        assert b.autotune() in chunk_candidates(12)


@pytest.mark.parametrize("inner", ["direct", "pcg"])
def test_autotune_before_any_state_on_tensor_copy_films(gpu, inner):
    """A film with full 32 x 8 tiles takes the tensor-copy (TMA) stencil
    passes; autotuning it straight after creation, before any set_state, runs
    those passes on the creation-time solver slots.  The run that follows
    matches the oracle (FP32-refined against FP64 solved to 1e-12)."""
    from cmsl_gb300 import workloads as wl
    w = wl.hzo_film("tma_64x32x10", 64, 32, 10, 7, 9, 0.4, E_amp_MVcm=4.0, steps_per_period=400)
    mats = np.array(w.mats, copy=True)
    if inner == "pcg":
        mats[:, 7] = [40.0, 30.0, 15.0]
    orc = oracle.load()
    f = oracle.Film(nx=w.nx, ny=w.ny, nz=w.nz, del_h=w.del_h, del_t=w.del_t, omega=w.omega,
                    grain_mat=w.grain_mat, TR=w.TR, mats=mats,
                    is_interface=orc.interface_flags(w.nx, w.ny, w.nz, w.omega, w.grain_mat),
                    dep_flag=1, eps_0_nd=w.eps_0_nd)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    n = 8
    Ez = w.sched.Ez[:n] * 40.0
    Pw, _, _, _, _, rc = orc.run(f, w.P_init, np.zeros(w.N), Ez)
    assert rc == 0
    with gpu.Film.from_oracle_film(f, precision=gpu.FP32_REFINED,
                                   inner_solver=gpu.INNER_DIRECT if inner == "direct" else gpu.INNER_PCG) as g:
        assert g.inner_solver == (gpu.INNER_DIRECT if inner == "direct" else gpu.INNER_PCG)
        assert g.autotune() in chunk_candidates(10)
        cfg = g.tile_config()
        assert cfg["x"] == 32 and cfg["y"] in (4, 8, 16) and cfg["z_chunk"] in chunk_candidates(10)
        g.set_state(w.P_init)
        g.run(Ez)
        Pg, _ = g.get_state()
    err = max(np.abs(a - b).max() / np.abs(b).max() for a, b in zip(Pg, Pw))
    assert err <= 2e-5
