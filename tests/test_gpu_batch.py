"""GPU parity of batches (cmsl_batch_*): films of uneven sizes, materials,
boundary conditions, tolerances and waveforms advancing together, each
checked against the oracle run of that film alone.

The tolerances are those of the single-film tests: FP64 P and rows to 1e-10
relative (dot-product summation order), FP32_REFINED against an FP64 oracle
solved to ||r|| <= 1e-12 ||b|| (P within 2e-5 of max |P|, phi 1e-4, rows 1e-5).
"""
import numpy as np
import pytest

import oracle
from tests.films import random_film

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


@pytest.fixture(scope="module")
def orc():
    return oracle.load()


def _films(fp32=False, neumann=True):
    """Four uneven films; the third has no depolarisation solve, the second
    has the Neumann z boundary unless neumann=False."""
    specs = [dict(shape=(16, 12, 6), seed=51, zbc=oracle.DIRICHLET, eps_0_nd=4.0),
             dict(shape=(33, 9, 5), seed=52, zbc=oracle.NEUMANN if neumann else oracle.DIRICHLET, eps_0_nd=3.0,
                  del_t=5e-4),
             dict(shape=(40, 17, 9), seed=53, zbc=oracle.DIRICHLET, dep_flag=0),
             dict(shape=(24, 20, 7), seed=54, zbc=oracle.DIRICHLET, eps_0_nd=5.0, fracs=(0.2, 0.6, 0.2))]
    out = []
    for s in specs:
        s = dict(s)
        shape = s.pop("shape")
        f, P = random_film(*shape, p_scale=0.2, layered=True, **s)
        if fp32:
            f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
        else:
            f.tol_abs, f.tol_rel = (1e-3, 1e-2) if s["seed"] % 2 else (1e-6, 1e-4)
        out.append((f, P))
    return out


def _schedule(n_films, n):
    """Per-film triangle-ish waveforms and row patterns (one film stores none)."""
    Ez = np.zeros((n_films, n))
    rows = np.full((n_films, n), -1, np.int32)
    for i in range(n_films):
        amp = 0.2 + 0.1 * i
        t = np.arange(n)
        Ez[i] = amp * (1.0 - np.abs(2.0 * t / (n - 1) - 1.0)) * (-1.0) ** i
        if i == 1:
            continue
        step = 1 + (i % 2)
        sel = t[::step]
        rows[i, sel] = np.arange(sel.size)
    return Ez, rows


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("graph", [True, False])
def test_batch_fp64_matches_oracle_per_film(gpu, orc, graph, monkeypatch):
    if not graph:
        monkeypatch.setenv("CMSL_NO_GRAPH", "1")
    films = _films()
    n = 16
    Ez, rows = _schedule(len(films), n)
    with gpu.Batch.from_oracle_films([f for f, _ in films]) as b:
        for i, (_, P) in enumerate(films):
            b.set_state(i, P)
        st = b.run(Ez, rows)
        assert (st == 0).all()
        for i, (f, P) in enumerate(films):
            Pw, _, phiw, statw, itw, rc = orc.run(f, P, np.zeros(f.N), Ez[i], rows[i])
            assert rc == 0
            Pg, phig = b.get_state(i)
            for a, w in zip(Pg, Pw):
                assert _rel(a, w) <= 1e-10, i
            if f.dep_flag:
                assert _rel(phig, phiw) <= 1e-9, i
            else:
                assert not phig.any()
            nr = int(rows[i].max()) + 1
            rg = b.rows(i, 0, nr) if nr > 0 else np.zeros((0, 11))
            assert np.abs(rg[:, :10] - statw[:, :10]).max(initial=0.0) <= 1e-10, i
            sel = rows[i] >= 0
            assert np.array_equal(rg[:, 10], np.flatnonzero(sel) + 1), i
            itg, rf = b.iters(i)
            assert np.abs(itg - itw).max() <= 1, i
            assert (rf == (1 if f.dep_flag else 0)).all(), i


@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("variant", ["persistent", "two_kernel", "neumann_mix"])
def test_batch_fp32_refined_vs_fp64_oracle(gpu, orc, graph, variant, monkeypatch):
    """Dirichlet films share one persistent PCG launch per refinement pass
    (each on its own block range with its own convergence); a batch holding a
    Neumann film, or CMSL_PCG_TWO_KERNEL=1, takes the masked two-kernel PCG."""
    if not graph:
        monkeypatch.setenv("CMSL_NO_GRAPH", "1")
    if variant == "two_kernel":
        monkeypatch.setenv("CMSL_PCG_TWO_KERNEL", "1")
    films = _films(fp32=True, neumann=variant == "neumann_mix")
    n = 20
    Ez, rows = _schedule(len(films), n)
    kw = dict(precision=gpu.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-4)
    with gpu.Batch.from_oracle_films([f for f, _ in films], **kw) as b:
        for i, (_, P) in enumerate(films):
            b.set_state(i, P)
        st = b.run(Ez, rows)
        assert (st == 0).all()
        for i, (f, P) in enumerate(films):
            Pw, _, phiw, statw, _, rc = orc.run(f, P, np.zeros(f.N), Ez[i], rows[i])
            assert rc == 0
            Pg, phig = b.get_state(i)
            for a, w in zip(Pg, Pw):
                assert np.abs(a - w).max() <= 2e-5 * np.abs(w).max(), i
            if f.dep_flag:
                assert _rel(phig, phiw) <= 1e-4, i
            nr = int(rows[i].max()) + 1
            if nr > 0:
                assert np.abs(b.rows(i, 0, nr)[:, :10] - statw[:, :10]).max() <= 1e-5, i
            it, rf = b.iters(i)
            if f.dep_flag:
                assert (rf >= 1).all() and (it >= 1).all(), i
            # the same film alone (persistent single-film solver)
            with gpu.Film.from_oracle_film(f, **kw) as g:
                g.set_state(P)
                g.run(Ez[i])
                Ps, _ = g.get_state()
            for a, w in zip(Pg, Ps):
                assert np.abs(a - w).max() <= 2e-5 * max(np.abs(w).max(), 1e-30), i


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp32_persistent"])
def test_batch_pcg_failure_marks_one_film(gpu, orc, precision):
    """A film whose state is not finite fails its solve (status 2, invalid
    initial residual) without stopping or changing the other films."""
    fp32 = precision != "fp64"
    films = _films(fp32=fp32, neumann=precision != "fp32_persistent")[:3]
    bad = 1
    n = 6
    Ez, rows = _schedule(len(films), n)
    kw = dict(precision=gpu.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-4) if fp32 else {}
    with gpu.Batch.from_oracle_films([f for f, _ in films], **kw) as b:
        for i, (_, P) in enumerate(films):
            if i == bad:
                P = [p.copy() for p in P]
                P[2][5] = np.nan
            b.set_state(i, P)
        st = b.run(Ez, rows)
        assert st[bad] == 2
        assert st[0] == 0 and st[2] == 0
        for i in (0, 2):
            f, P = films[i]
            Pw, *_ = orc.run(f, P, np.zeros(f.N), Ez[i], rows[i])
            Pg, _ = b.get_state(i)
            tol = 2e-5 if fp32 else 1e-10
            for a, w in zip(Pg, Pw):
                assert np.abs(a - w).max() <= tol * np.abs(w).max(), i


def test_batch_set_state_of_one_film(gpu, orc):
    """Re-seeding one film between runs restarts it and leaves the others'
    trajectories untouched."""
    films = _films()[:2]
    n = 8
    Ez, rows = _schedule(len(films), 2 * n)
    rng = np.random.default_rng(77)
    f1 = films[1][0]
    P1_new = [rng.uniform(-0.2, 0.2, f1.N) for _ in range(6)]
    with gpu.Batch.from_oracle_films([f for f, _ in films]) as b:
        for i, (_, P) in enumerate(films):
            b.set_state(i, P)
        assert (b.run(Ez[:, :n]) == 0).all()
        b.set_state(1, P1_new)
        assert (b.run(Ez[:, n:]) == 0).all()
        P0g, _ = b.get_state(0)
        P1g, _ = b.get_state(1)
    f0, P0 = films[0]
    Pw0, *_ = orc.run(f0, P0, np.zeros(f0.N), Ez[0])
    Pw1, *_ = orc.run(f1, P1_new, np.zeros(f1.N), Ez[1, n:])
    for a, w in zip(P0g, Pw0):
        assert _rel(a, w) <= 1e-10
    for a, w in zip(P1g, Pw1):
        assert _rel(a, w) <= 1e-10


def test_batch_time_kernels_and_bytes(gpu):
    films = _films(fp32=True)
    with gpu.Batch.from_oracle_films([f for f, _ in films], precision=gpu.FP32_REFINED) as b:
        for i, (_, P) in enumerate(films):
            b.set_state(i, P)
        ms = b.time_kernels(reps=3)
        # ms[3], the update pass, is 0 when the TDGL kernel forms its check
        assert (ms[:3] > 0).all() and (ms[3] >= 0) and np.isfinite(ms).all()
        cells = sum(f.N for f, _ in films)
        assert b.device_bytes() >= cells * 4 * 20
