"""The adjoint of the TDGL step and the depolarisation solve
(cmsl_film_loop_gradient, cmsl_gb300.adjoint) against central finite
differences of the same forward model, FP64 films with tightly converged
solves.  Tolerance: |adjoint - FD| <= 1e-3 |FD| + 1e-6 max |FD| per
parameter."""
import dataclasses

import numpy as np
import pytest

import oracle
from tests.films import random_film

pytestmark = pytest.mark.gpu

COLS = (0, 1, 2, 3, 5)   # alpha, beta, gamma, g, kappa in the 8-column material rows


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cmsl_gb300 import build
    build.build()
    import cmsl_gb300
    return cmsl_gb300


def _problem(dep=1, n=40, seed=61):
    f, P = random_film(20, 16, 6, seed=seed, fracs=(0.4, 0.4, 0.2), eps_0_nd=4.0, p_scale=0.3, layered=True,
                       dep_flag=dep)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-13, 20000
    t = np.arange(n)
    Ez = 0.4 * np.sin(2.0 * np.pi * t / n)
    rows = t.astype(np.int32)
    return f, P, Ez, rows


def _loop(gpu, f, P, Ez, rows, mats):
    f2 = dataclasses.replace(f, mats=np.asarray(mats, np.float64))
    with gpu.Film.from_oracle_film(f2) as g:
        g.set_state(P)
        g.run(Ez, rows)
        return g.rows(0, rows.size)[:, 0].copy()


def _loss(gpu, f, P, Ez, rows, mats, target):
    d = _loop(gpu, f, P, Ez, rows, mats) - target
    return float(np.mean(d * d))


def _grad(gpu, f, P, Ez, rows, target, K):
    with gpu.Film.from_oracle_film(f) as g:
        g.set_state(P)
        return g.loop_gradient(Ez, rows, target, checkpoint_every=K)


@pytest.mark.parametrize("dep", [1, 0])
def test_adjoint_matches_finite_differences(gpu, dep):
    f, P, Ez, rows = _problem(dep=dep)
    mats0 = np.array(f.mats, np.float64)
    pert = mats0.copy()
    pert[:, [0, 1, 2, 5]] *= 1.03
    target = _loop(gpu, f, P, Ez, rows, pert)
    L, g = _grad(gpu, f, P, Ez, rows, target, K=16)
    assert L == pytest.approx(_loss(gpu, f, P, Ez, rows, mats0, target), rel=1e-12, abs=0.0)
    fd = np.zeros((3, 5))
    for m in range(3):
        for p, col in enumerate(COLS):
            h = 1e-5 * max(abs(mats0[m, col]), 1.0)
            mp, mm = mats0.copy(), mats0.copy()
            mp[m, col] += h
            mm[m, col] -= h
            fd[m, p] = (_loss(gpu, f, P, Ez, rows, mp, target) - _loss(gpu, f, P, Ez, rows, mm, target)) / (2 * h)
    scale = np.abs(fd).max()
    assert scale > 0
    assert (np.abs(g - fd) <= 1e-3 * np.abs(fd) + 1e-6 * scale).all(), (g, fd)


def test_checkpoint_interval_does_not_change_the_gradient(gpu):
    f, P, Ez, rows = _problem()
    target = np.zeros(rows.size)
    L1, g1 = _grad(gpu, f, P, Ez, rows, target, K=3)
    L2, g2 = _grad(gpu, f, P, Ez, rows, target, K=rows.size)
    assert L1 == L2
    assert np.allclose(g1, g2, rtol=1e-12, atol=0.0)


def test_rejects_unsupported_films(gpu):
    f, P, Ez, rows = _problem()
    with gpu.Film.from_oracle_film(f, precision=gpu.FP32_REFINED) as g:
        g.set_state(P)
        with pytest.raises(gpu.CmslError):
            g.loop_gradient(Ez, rows, np.zeros(rows.size))
    f.zbc = oracle.NEUMANN
    with gpu.Film.from_oracle_film(f) as g:
        g.set_state(P)
        with pytest.raises(gpu.CmslError):
            g.loop_gradient(Ez, rows, np.zeros(rows.size))


def test_autograd_function_landau_coefficients(gpu):
    """torch.autograd over the SI coefficients (a1, a11, a111, G, J) of a
    small loop against central differences (relative step 1e-4)."""
    import torch
    from cmsl_gb300 import adjoint as adj
    from cmsl_gb300 import workloads as wl
    w = wl.hzo_film("fit_24x24x6", 24, 24, 6, 8, 5, 0.4, E_amp_MVcm=4.0, steps_per_period=160)
    fit = adj.LoopFit(w, adj.THETA_NOMINAL.copy(), checkpoint_every=50, tol=1e-12)
    fit.target = fit.loop(adj.THETA_NOMINAL * np.array([1.1, 0.9, 1.05, 1.15, 0.85]))
    theta = torch.tensor(adj.THETA_NOMINAL, dtype=torch.float64, requires_grad=True)
    loss = adj.landau_loop_loss(theta, fit)
    loss.backward()
    g = theta.grad.numpy()
    assert float(loss.detach()) == pytest.approx(fit.loss(adj.THETA_NOMINAL), rel=1e-12)
    fd = np.zeros(5)
    for i in range(5):
        h = 1e-4 * abs(adj.THETA_NOMINAL[i])
        tp, tm = adj.THETA_NOMINAL.copy(), adj.THETA_NOMINAL.copy()
        tp[i] += h
        tm[i] -= h
        fd[i] = (fit.loss(tp) - fit.loss(tm)) / (2 * h)
    assert (np.abs(g - fd) <= 1e-3 * np.abs(fd) + 1e-6 * np.abs(fd).max()).all(), (g, fd)


def test_adjoint_matches_oracle_finite_differences(gpu):
    """An FP64 reference gradient independent of this library: central
    differences of the loss computed entirely by the oracle (the CPU FP64
    restatement of the reference kernels and Depol_field PCG, solved to
    1e-13), against the adjoint on the GPU.  Same tolerance as the GPU
    finite differences above."""
    f, P, Ez, rows = _problem(n=30, seed=62)
    orc = oracle.load()
    mats0 = np.array(f.mats, np.float64)

    def oloss(mats, target):
        f2 = dataclasses.replace(f, mats=np.asarray(mats, np.float64))
        _, _, _, st, _, rc = orc.run(f2, P, np.zeros(f.N), Ez, rows)
        assert rc == 0
        d = st[:, 0] - target
        return float(np.mean(d * d))

    pert = mats0.copy()
    pert[:, [0, 1, 2, 5]] *= 1.03
    f2 = dataclasses.replace(f, mats=pert)
    _, _, _, st, _, rc = orc.run(f2, P, np.zeros(f.N), Ez, rows)
    assert rc == 0
    target = st[:, 0].copy()
    L, g = _grad(gpu, f, P, Ez, rows, target, K=10)
    assert L == pytest.approx(oloss(mats0, target), rel=1e-9, abs=0.0)
    fd = np.zeros((3, 5))
    for m in range(3):
        for p, col in enumerate(COLS):
            h = 1e-5 * max(abs(mats0[m, col]), 1.0)
            mp, mm = mats0.copy(), mats0.copy()
            mp[m, col] += h
            mm[m, col] -= h
            fd[m, p] = (oloss(mp, target) - oloss(mm, target)) / (2 * h)
    scale = np.abs(fd).max()
    assert scale > 0
    assert (np.abs(g - fd) <= 1e-3 * np.abs(fd) + 1e-6 * scale).all(), (g, fd)
