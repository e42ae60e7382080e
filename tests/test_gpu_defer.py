"""Deferred checks of CMSL_FP32_REFINED: a step of a film with one
permittivity ends on its direct solve, and the next TDGL step forms the check
the update pass formed (r <- r - A dx, ||r|| <= refine_tol ||b||) while it
takes E from the warm start plus the pending correction.  A failed check
reopens the previous step, whose passes then end it again; a run's last
pending check runs as an update pass after its step loop.

Against the FP64 oracle (P within 2e-5 of max |P|, phi 1e-4, rows 1e-5, as
the other FP32-refined tests) and against the same film with the check in its
own update pass (CMSL_DEFER=0): the two schedules run the same refinement, so
their pass and solve counts per step are equal and their states agree to the
FP32 rounding of E."""
import numpy as np
import pytest

import oracle
from tests.films import MATS_DEFAULT, random_film

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


def _film(shape, seed, eps=30.0):
    mats = MATS_DEFAULT.copy()
    mats[:, 7] = eps
    f, P = random_film(*shape, seed=seed, eps_0_nd=4.0, mats=mats, p_scale=0.2, layered=True)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    return f, P


def _run(gpu, f, P, Ez, rows, monkeypatch, defer=True, graph=True, split=None, **kw):
    monkeypatch.setenv("CMSL_DEFER", "1" if defer else "0")
    monkeypatch.setenv("CMSL_NO_GRAPH", "0" if graph else "1")
    kw = {**dict(precision=gpu.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-5), **kw}
    with gpu.Film.from_oracle_film(f, **kw) as g:
        assert g.inner_solver == gpu.INNER_DIRECT
        g.set_state(P)
        if split:
            g.run(Ez[:split], rows[:split])
            g.run(Ez[split:], rows[split:])
        else:
            g.run(Ez, rows)
        Pg, phig = g.get_state()
        rg = g.rows()
        it, rf = g.iters()
        g.sync()
    return Pg, phig, rg, it, rf


def _close(a, b, tol):
    return max(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300) for x, y in zip(a, b)) <= tol


@pytest.mark.parametrize("shape,staging", [((64, 32, 13), "00"), ((64, 32, 13), "11"), ((48, 36, 9), None),
                                           ((96, 12, 7), None)])
def test_deferred_checks_match_oracle_and_update_pass(gpu, shape, staging, monkeypatch):
    """Full tiles with both stagings of the residual passes (the cp.async
    ring, tensor copies; CMSL_STAGING -- the TDGL kernel that forms the check
    has the ring) and partial tiles; the direct solve takes Dirichlet films."""
    if staging:
        monkeypatch.setenv("CMSL_STAGING", staging)
    f, P = _film(shape, seed=sum(shape))
    n = 24
    Ez = np.linspace(0.0, 0.35, n)
    rows = np.arange(n, dtype=np.int32)
    Pw, _, phiw, statw, _, rc = oracle.load().run(f, P, np.zeros(f.N), Ez, rows)
    assert rc == 0
    Pd, phid, rd, itd, rfd = _run(gpu, f, P, Ez, rows, monkeypatch, defer=True)
    Pu, phiu, ru, itu, rfu = _run(gpu, f, P, Ez, rows, monkeypatch, defer=False)
    for Pg, phig, rg in ((Pd, phid, rd), (Pu, phiu, ru)):
        assert _close(Pg, Pw, 2e-5)
        assert np.abs(phig - phiw).max() <= 1e-4 * np.abs(phiw).max()
        assert np.abs(rg[:, :10] - statw[:, :10]).max() <= 1e-5
    # the same refinement: passes and solves per step equal, states equal to
    # the FP32 rounding of E
    assert (rfd == rfu).all() and (itd == itu).all()
    assert (rfd >= 2).all()
    assert _close(Pd, Pu, 1e-6)
    assert np.abs(phid - phiu).max() <= 1e-6 * np.abs(phiu).max()
    # the run's last check ran after the step loop: phi meets the target in FP64
    orc = oracle.load()
    b = -orc.divergence(f, Pd[0], Pd[1], Pd[2])
    k = np.repeat(np.arange(f.nz), f.nx * f.ny)
    b[(k == 0) | (k == f.nz - 1)] = 0.0
    assert np.linalg.norm(b - orc.apply_A(f, phid)) <= 1.5e-8 * np.linalg.norm(b)


def test_failed_checks_reopen_their_steps(gpu, monkeypatch):
    """refine_tol 1e-11: one FP32 direct solve never meets it, so every
    deferred check fails, its step is reopened and ended by further passes,
    and the TDGL step runs again.  Same passes and solves per step as the
    update-pass schedule, and the oracle's states."""
    f, P = _film((48, 24, 11), seed=7)
    n = 12
    Ez = np.linspace(0.0, 0.3, n)
    rows = np.arange(n, dtype=np.int32)
    Pw, _, phiw, statw, _, rc = oracle.load().run(f, P, np.zeros(f.N), Ez, rows)
    assert rc == 0
    Pd, phid, rd, itd, rfd = _run(gpu, f, P, Ez, rows, monkeypatch, defer=True, refine_tol=1e-11)
    Pu, phiu, ru, itu, rfu = _run(gpu, f, P, Ez, rows, monkeypatch, defer=False, refine_tol=1e-11)
    assert (rfd == rfu).all() and (itd == itu).all()
    assert (rfd >= 3).all()                          # more than the first pass and one check
    assert _close(Pd, Pw, 2e-5) and _close(Pu, Pw, 2e-5)
    assert _close(Pd, Pu, 1e-6)
    assert np.abs(rd[:, :10] - statw[:, :10]).max() <= 1e-5


def test_deferred_checks_graph_and_plain_launches_agree(gpu, monkeypatch):
    """The step graph and the host-launched step (CMSL_NO_GRAPH=1) run the
    same kernels in the same order: bit-identical results, with the checks
    passing and (refine_tol 1e-11) failing."""
    f, P = _film((48, 24, 9), seed=11)
    n = 10
    Ez = np.linspace(0.0, 0.3, n)
    rows = np.arange(n, dtype=np.int32)
    for tol in (1e-8, 1e-11):
        a = _run(gpu, f, P, Ez, rows, monkeypatch, graph=True, refine_tol=tol)
        b = _run(gpu, f, P, Ez, rows, monkeypatch, graph=False, refine_tol=tol)
        for x, y in zip(a[0], b[0]):
            assert np.array_equal(x, y)
        assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
        assert np.array_equal(a[3], b[3]) and np.array_equal(a[4], b[4])


def test_deferred_checks_across_runs(gpu, monkeypatch):
    """Two runs of 8 and 12 steps against one of 20: the first run's last
    check runs after its step loop, and the second run starts from a
    resolved potential."""
    f, P = _film((64, 32, 13), seed=3)
    n = 20
    Ez = np.linspace(0.0, 0.3, n)
    rows = np.arange(n, dtype=np.int32)
    P1, phi1, r1, it1, rf1 = _run(gpu, f, P, Ez, rows, monkeypatch)
    P2, phi2, r2, it2, rf2 = _run(gpu, f, P, Ez, rows, monkeypatch, split=8)
    assert _close(P2, P1, 1e-6)
    assert np.abs(phi2 - phi1).max() <= 1e-6 * np.abs(phi1).max()
    # the second run's rows (a larger row range reallocates the row buffer)
    assert np.abs(r2[8:20, :10] - r1[8:20, :10]).max() <= 1e-6
    assert (rf2 >= 2).all()


def test_batch_with_deferred_and_ordinary_films(gpu, monkeypatch):
    """A batch of a one-permittivity film (deferred checks) and a
    three-permittivity one (preconditioned refinement, every pass in its
    step) against each film alone."""
    fa, Pa = _film((48, 24, 9), seed=21)
    mats = MATS_DEFAULT.copy()
    mats[:, 7] = [50.0, 30.0, 15.0]
    fb, Pb = random_film(48, 24, 9, seed=22, eps_0_nd=4.0, mats=mats, p_scale=0.2, layered=True)
    fb.crit, fb.tol_rel, fb.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    n = 10
    Ez = np.linspace(0.0, 0.3, n)
    rows = np.arange(n, dtype=np.int32)
    monkeypatch.setenv("CMSL_DEFER", "1")
    kw = dict(precision=gpu.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-5)
    alone = []
    for f, P in ((fa, Pa), (fb, Pb)):
        with gpu.Film.from_oracle_film(f, **kw) as g:
            g.set_state(P)
            g.run(Ez, rows)
            alone.append((g.get_state()[0], g.iters()[1]))
    with gpu.Batch.from_oracle_films([fa, fb], **kw) as b:
        b.set_state(0, Pa)
        b.set_state(1, Pb)
        b.run(np.stack([Ez, Ez]), np.stack([rows, rows]))
        for i in range(2):
            Pg, _ = b.get_state(i)
            _, rf = b.iters(i)
            assert _close(Pg, alone[i][0], 1e-6)
            assert (rf == alone[i][1]).all()


def test_batch_where_some_checks_fail(gpu, monkeypatch):
    """Two one-permittivity films in a batch, one with refine_tol 1e-11 (every
    deferred check fails and reopens the step) and one with 1e-8 (its checks
    pass; it stays pending through the reopened step and is checked again
    when the step repeats): each film as it runs alone."""
    fa, Pa = _film((48, 24, 9), seed=31)
    fb, Pb = _film((64, 32, 7), seed=32)
    n = 10
    Ez = np.linspace(0.0, 0.3, n)
    rows = np.arange(n, dtype=np.int32)
    monkeypatch.setenv("CMSL_DEFER", "1")
    base = dict(precision=gpu.FP32_REFINED, inner_tol=1e-5)
    tols = (1e-11, 1e-8)
    alone = []
    for (f, P), tol in zip(((fa, Pa), (fb, Pb)), tols):
        with gpu.Film.from_oracle_film(f, refine_tol=tol, **base) as g:
            g.set_state(P)
            g.run(Ez, rows)
            alone.append((g.get_state(), g.iters()[1], g.rows()))
    from cmsl_gb300.film import _oracle_kw
    with gpu.Batch([{**_oracle_kw(f), **base, "refine_tol": tol} for f, tol in zip((fa, fb), tols)]) as b:
        b.set_state(0, Pa)
        b.set_state(1, Pb)
        b.run(np.stack([Ez, Ez]), np.stack([rows, rows]))
        for i in range(2):
            (Pg, phig) = b.get_state(i)
            _, rf = b.iters(i)
            (Pw, phiw), rfw, rw = alone[i]
            assert _close(Pg, Pw, 1e-6)
            assert np.abs(phig - phiw).max() <= 1e-6 * np.abs(phiw).max()
            assert (rf == rfw).all()
            assert np.abs(b.rows(i)[:, :10] - rw[:, :10]).max() <= 1e-6
        # every step of the first film reopened; the second settles to its two passes after the cold start
        assert (b.iters(0)[1] >= 3).all() and b.iters(1)[1][-1] == 2


@pytest.mark.parametrize("tol", [1e-8, 1e-11])
def test_rows_totalled_by_the_residual_pass(gpu, tol, monkeypatch):
    """A film whose residual pass has more blocks than one wave (256 x 128 x
    24 in 4-plane chunks: 768 items of 32 x 8 columns) has its sweep rows
    totalled by block 0 of each step's first residual pass, the TDGL step's
    last block forming only the check's r.r.  Its rows match the oracle's
    and the update-pass schedule's (rows formed in the TDGL step), with the
    checks passing and (refine_tol 1e-11) failing, the reopened steps' rows
    formed again when they repeat."""
    monkeypatch.setenv("CMSL_ZCHUNK", "4")
    f, P = _film((256, 128, 24), seed=41)
    n = 8
    Ez = np.linspace(0.0, 0.3, n)
    rows = np.arange(n, dtype=np.int32)
    Pw, _, phiw, statw, _, rc = oracle.load().run(f, P, np.zeros(f.N), Ez, rows)
    assert rc == 0
    Pd, phid, rd, itd, rfd = _run(gpu, f, P, Ez, rows, monkeypatch, defer=True, refine_tol=tol)
    Pu, phiu, ru, itu, rfu = _run(gpu, f, P, Ez, rows, monkeypatch, defer=False, refine_tol=tol)
    assert (rfd == rfu).all()
    if tol < 1e-10:
        assert (rfd >= 3).all()
    for rg in (rd, ru):
        assert np.abs(rg[:, :10] - statw[:, :10]).max() <= 1e-5
    assert np.abs(rd[:, :11] - ru[:, :11]).max() <= 1e-6
    assert np.array_equal(rd[:, 10], np.arange(1, n + 1))       # the step count column
    assert _close(Pd, Pw, 2e-5) and _close(Pd, Pu, 1e-6)
