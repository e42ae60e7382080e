"""The direct (spectral) inner solve of CMSL_FP32_REFINED: films whose
materials share one permittivity, Dirichlet z boundary, 2^a 3^b sides; the
refinement passes after it (full double-float residuals, or FP32 updates
r <- r - A dx once the residual is small).
Against the FP64 oracle solved to ||r|| <= 1e-12 ||b|| with the tolerances
of the other FP32_REFINED tests (P within 2e-5 of max |P|, phi 1e-4, rows
1e-5), and against the same film with the PCG inner solve."""
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


def _uniform(shape, seed, eps=30.0):
    mats = MATS_DEFAULT.copy()
    mats[:, 7] = eps
    f, P = random_film(*shape, seed=seed, eps_0_nd=4.0, mats=mats, p_scale=0.2, layered=True)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    return f, P


@pytest.mark.parametrize("layout", ["columns", "rows", "clusters"])
@pytest.mark.parametrize("shape", [(32, 24, 8), (48, 36, 10), (64, 16, 5), (96, 12, 7), (8, 9, 3), (27, 32, 12),
                                   (64, 64, 10), (128, 32, 9), (32, 256, 6), (256, 64, 7)])
def test_direct_solve_run_vs_oracle(gpu, shape, layout, monkeypatch):
    """The three forms of the solve: rows (five passes), columns (x
    transforms, one block per mirror pair of columns for y, z and y, x
    transforms; CMSL_SPEC_COLS=1) and clusters (the x and y transforms of a
    packed plane in one block cluster, the z solve column by column;
    CMSL_SPEC_CL=1 where every side is a power of two, a multiple of 8 and at
    least 32 -- other films take the rows here)."""
    monkeypatch.setenv("CMSL_SPEC_CL", "1" if layout == "clusters" else "0")
    monkeypatch.setenv("CMSL_SPEC_COLS", "1" if layout == "columns" else "0")
    f, P = _uniform(shape, seed=sum(shape))
    n = 16
    Ez = np.linspace(0.0, 0.35, n)
    rows = np.arange(n, dtype=np.int32)
    Pw, _, phiw, statw, _, rc = oracle.load().run(f, P, np.zeros(f.N), Ez, rows)
    assert rc == 0
    kw = dict(precision=gpu.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-5)
    with gpu.Film.from_oracle_film(f, **kw) as g:
        assert g.inner_solver == gpu.INNER_DIRECT
        g.set_state(P)
        g.run(Ez, rows)
        Pg, phig = g.get_state()
        rg = g.rows()
        it, rf = g.iters()
    for a, b in zip(Pg, Pw):
        assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max()
    assert np.abs(phig - phiw).max() <= 1e-4 * np.abs(phiw).max()
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= 1e-5
    # one direct solve per refinement pass, a few passes per step
    assert (rf >= 2).all() and (rf <= 4).all() and (it == rf - 1).all()
    # the last step ended on an update pass (r <- r - A dx) or a full one:
    # either way the potential meets the refinement target in FP64
    orc = oracle.load()
    b = -orc.divergence(f, Pg[0], Pg[1], Pg[2])
    k = np.repeat(np.arange(f.nz), f.nx * f.ny)
    b[(k == 0) | (k == f.nz - 1)] = 0.0
    assert np.linalg.norm(b - orc.apply_A(f, phig)) <= 1.5e-8 * np.linalg.norm(b)
    with gpu.Film.from_oracle_film(f, inner_solver=gpu.INNER_PCG, **kw) as g:
        assert g.inner_solver == gpu.INNER_PCG
        g.set_state(P)
        g.run(Ez, rows)
        Pp, _ = g.get_state()
    for a, b in zip(Pg, Pp):
        assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max()


def test_direct_solve_reaches_refine_tolerance(gpu):
    """One refined depolarisation solve: ||b - A phi|| <= 1e-8 ||b|| in FP64."""
    f, P = _uniform((48, 24, 12), seed=3)
    orc = oracle.load()
    with gpu.Film.from_oracle_film(f, precision=gpu.FP32_REFINED, refine_tol=1e-8) as g:
        assert g.inner_solver == gpu.INNER_DIRECT
        g.set_state(P)
        res = g.depol()
        Pg, phi = g.get_state()
    assert res["status"] == 0 and res["refine"] <= 4
    b = -orc.divergence(f, Pg[0], Pg[1], Pg[2])
    k = np.repeat(np.arange(f.nz), f.nx * f.ny)
    b[(k == 0) | (k == f.nz - 1)] = 0.0
    r = b - orc.apply_A(f, phi)
    assert np.linalg.norm(r) <= 1.2e-8 * np.linalg.norm(b)


def test_direct_solve_selection(gpu):
    kw = dict(precision=gpu.FP32_REFINED)
    f, P = _uniform((30, 24, 6), seed=4)             # 30 = 2 * 3 * 5: not 2^a 3^b
    with gpu.Film.from_oracle_film(f, **kw) as g:
        assert g.inner_solver == gpu.INNER_PCG
    with pytest.raises(gpu.CmslError):
        gpu.Film.from_oracle_film(f, inner_solver=gpu.INNER_DIRECT, **kw)
    f2, _ = random_film(32, 24, 6, seed=5)          # three permittivities, 40 / 30 / 15
    with gpu.Film.from_oracle_film(f2, **kw) as g:   # ratio 2.7: the solve preconditions the refinement
        assert g.inner_solver == gpu.INNER_DIRECT
    mats = MATS_DEFAULT.copy()
    mats[:, 7] = [300.0, 30.0, 15.0]                 # ratio 20: AUTO takes the PCG, DIRECT may be asked for
    f4, _ = random_film(32, 24, 6, seed=5, mats=mats)
    with gpu.Film.from_oracle_film(f4, **kw) as g:
        assert g.inner_solver == gpu.INNER_PCG
    with gpu.Film.from_oracle_film(f4, inner_solver=gpu.INNER_DIRECT, **kw) as g:
        assert g.inner_solver == gpu.INNER_DIRECT
    f3, _ = _uniform((32, 24, 6), seed=6)
    with gpu.Film.from_oracle_film(f3) as g:          # FP64: the reference's PCG
        assert g.inner_solver == gpu.INNER_PCG


def test_direct_solve_batch(gpu):
    """A batch of uneven one-eps films (one without depolarisation) takes the
    direct solve; every film against its oracle run and its solo run."""
    shapes = [(32, 24, 8), (48, 36, 6), (64, 16, 5), (24, 27, 7)]
    films = []
    for i, sh in enumerate(shapes):
        f, P = _uniform(sh, seed=40 + i, eps=20.0 + 5 * i)
        if i == 2:
            f.dep_flag = 0
        films.append((f, P))
    n = 12
    Ez = np.stack([np.linspace(0.0, 0.2 + 0.05 * i, n) for i in range(len(films))])
    rows = np.tile(np.arange(n, dtype=np.int32), (len(films), 1))
    kw = dict(precision=gpu.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-5)
    orc = oracle.load()
    with gpu.Batch.from_oracle_films([f for f, _ in films], **kw) as b:
        assert b.inner_solver == gpu.INNER_DIRECT
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
                assert np.abs(phig - phiw).max() <= 1e-4 * np.abs(phiw).max(), i
            assert np.abs(b.rows(i)[:, :10] - statw[:, :10]).max() <= 1e-5, i
            it, rf = b.iters(i)
            if f.dep_flag:
                assert (rf >= 2).all() and (it == rf - 1).all(), i
            with gpu.Film.from_oracle_film(f, **kw) as g:
                g.set_state(P)
                g.run(Ez[i])
                Ps, _ = g.get_state()
            for a, w in zip(Pg, Ps):
                assert np.abs(a - w).max() <= 2e-5 * max(np.abs(w).max(), 1e-30), i


@pytest.mark.parametrize("eps", [(40.0, 30.0, 15.0), (40.0, 30.0, 30.0), (100.0, 30.0, 15.0)])
@pytest.mark.parametrize("shape", [(32, 24, 8), (48, 36, 10), (27, 32, 12)])
def test_preconditioned_refinement_several_eps(gpu, shape, eps):
    """Several permittivities with the direct solve: the solve with one
    reference eps (the middle of the film's range) preconditions the
    double-float refinement, whose residual pass applies the true operator
    (harmonic face eps), with Chebyshev increments.  Against the FP64 oracle
    solved to 1e-12 with the tolerances of the other FP32-refined tests; the
    potential meets the refinement target in FP64; the passes per step stay
    within what the fixed-step contraction (kappa - 1) / (kappa + 1) would
    need from a cold start."""
    mats = MATS_DEFAULT.copy()
    mats[:, 7] = eps
    f, P = random_film(*shape, seed=sum(shape) + int(eps[0]), eps_0_nd=4.0, mats=mats, p_scale=0.2, layered=True)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    n = 10
    Ez = np.linspace(0.0, 0.35, n)
    rows = np.arange(n, dtype=np.int32)
    orc = oracle.load()
    Pw, _, phiw, statw, _, rc = orc.run(f, P, np.zeros(f.N), Ez, rows)
    assert rc == 0
    kw = dict(precision=gpu.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-5, max_refine=6,
              inner_solver=gpu.INNER_DIRECT)
    with gpu.Film.from_oracle_film(f, **kw) as g:
        assert g.inner_solver == gpu.INNER_DIRECT
        g.set_state(P)
        g.run(Ez, rows)
        Pg, phig = g.get_state()
        rg = g.rows()
        it, rf = g.iters()
    for a, b in zip(Pg, Pw):
        assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max()
    assert np.abs(phig - phiw).max() <= 1e-4 * np.abs(phiw).max()
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= 1e-5
    used = sorted(set(float(mats[m, 7]) for m in np.unique(f.grain_mat)))
    kappa = used[-1] / used[0]
    rho = (kappa - 1.0) / (kappa + 1.0)
    bound = 3 + (int(np.ceil(np.log(1e-8) / np.log(rho))) if rho > 0 else 0)
    assert (rf >= 2).all() and (rf <= bound).all(), (rf, bound)
    b = -orc.divergence(f, Pg[0], Pg[1], Pg[2])
    k = np.repeat(np.arange(f.nz), f.nx * f.ny)
    b[(k == 0) | (k == f.nz - 1)] = 0.0
    assert np.linalg.norm(b - orc.apply_A(f, phig)) <= 1.5e-8 * np.linalg.norm(b)
