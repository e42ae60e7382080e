"""GPU parity: libcmsl_gb (through its C ABI) against the oracle.

FP64 mode: the TDGL step, operator, Jacobi diagonal and E field are compared
bit for bit (the kernels use explicitly rounded FP64 operations in the
reference's order); PCG-dependent quantities agree to dot-product summation
order (relative 1e-10 after tens of steps).
FP32_REFINED mode: compared with an FP64 oracle run whose PCG is converged
far below the refinement target; tolerances are stated per test.
"""
import os

import numpy as np
import pytest

import oracle
from tests.films import random_film

pytestmark = pytest.mark.gpu

SIZES = [(4, 4, 3), (5, 7, 4), (16, 12, 6), (33, 9, 5), (40, 17, 9), (64, 16, 8)]


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


def _film(cg, f, **kw):
    return cg.Film.from_oracle_film(f, **kw)


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("shape", SIZES)
@pytest.mark.parametrize("zbc", [oracle.DIRICHLET, oracle.NEUMANN])
def test_tdgl_step_bitwise(gpu, orc, shape, zbc):
    f, P = random_film(*shape, seed=sum(shape), zbc=zbc, layered=True)
    phi = np.random.default_rng(3).normal(size=f.N) * 0.2
    E = orc.efield(f, phi)
    want, _ = orc.tdgl_step(f, P, 0.173, E)
    with _film(gpu, f) as g:
        g.set_state(P, phi)
        g.tdgl_step(0.173)
        got, phi_out = g.get_state()
    assert _same(got, want)
    assert np.array_equal(phi_out, phi)


@pytest.mark.parametrize("shape", SIZES)
def test_tdgl_step_no_depolarisation(gpu, orc, shape):
    f, P = random_film(*shape, seed=2 + sum(shape), dep_flag=0)
    want, _ = orc.tdgl_step(f, P, -0.31)
    with _film(gpu, f) as g:
        g.set_state(P)
        g.tdgl_step(-0.31)
        got, _ = g.get_state()
    assert _same(got, want)


@pytest.mark.parametrize("shape", SIZES)
@pytest.mark.parametrize("zbc", [oracle.DIRICHLET, oracle.NEUMANN])
def test_operator_diag_efield_bitwise(gpu, orc, shape, zbc):
    f, P = random_film(*shape, seed=7, zbc=zbc)
    x = np.random.default_rng(5).normal(size=f.N)
    with _film(gpu, f) as g:
        assert np.array_equal(g.apply_operator(x), orc.apply_A(f, x))
        assert np.array_equal(g.diag_inv(), orc.diag_inv(f))
        g.set_state(P, x)
        assert _same(g.efield(), orc.efield(f, x))


@pytest.mark.parametrize("shape", [(16, 12, 6), (33, 9, 5), (40, 17, 9)])
@pytest.mark.parametrize("zbc", [oracle.DIRICHLET, oracle.NEUMANN])
def test_depol_solve_fp64(gpu, orc, shape, zbc):
    f, P = random_film(*shape, seed=11, zbc=zbc, eps_0_nd=3.0)
    f.tol_abs, f.tol_rel = 1e-10, 1e-8
    phi0 = np.zeros(f.N)
    phi_w, E_w, _, info = orc.depol_field(f, P[:3], phi0)
    with _film(gpu, f) as g:
        g.set_state(P, phi0)
        res = g.depol()
        _, phi = g.get_state()
    assert res["status"] == 0 and info["status"] == 0
    assert abs(res["iters"] - info["iters"]) <= 1
    assert np.abs(phi - phi_w).max() <= 1e-10 * np.abs(phi_w).max()


@pytest.mark.parametrize("shape", [(16, 12, 6), (33, 9, 5)])
@pytest.mark.parametrize("graph", [True, False])
def test_run_fp64_matches_oracle(gpu, orc, shape, graph, monkeypatch):
    """Twenty full steps (TDGL + depolarisation) with a staircase field and a
    sweep row per step: P, phi and rows to 1e-10 relative."""
    if not graph:
        monkeypatch.setenv("CMSL_NO_GRAPH", "1")
    f, P = random_film(*shape, seed=21, eps_0_nd=4.0, p_scale=0.2)
    f.tol_abs, f.tol_rel = 1e-3, 1e-2           # the reference's defaults
    n = 20
    Ez = np.linspace(0.0, 0.5, n)
    rows = np.arange(n, dtype=np.int32)
    Pw, Ew, phiw, statw, itw, rc = orc.run(f, P, np.zeros(f.N), Ez, rows)
    assert rc == 0
    with _film(gpu, f) as g:
        g.set_state(P)
        g.run(Ez, rows)
        Pg, phig = g.get_state()
        rg = g.rows()
        itg, _ = g.iters()
    for a, b in zip(Pg, Pw):
        assert np.abs(a - b).max() <= 1e-10 * max(1e-30, np.abs(b).max())
    assert np.abs(phig - phiw).max() <= 1e-9 * np.abs(phiw).max()
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= 1e-10
    assert np.array_equal(rg[:, 10], np.arange(1, n + 1))
    assert np.abs(itg - itw).max() <= 1


def test_rows_material_fractions(gpu, orc):
    f, P = random_film(24, 20, 6, seed=4, fracs=(0.3, 0.5, 0.2))
    with _film(gpu, f) as g:
        g.set_state(P)
        g.run(np.array([0.1]), np.array([0], np.int32))
        r = g.rows()[0]
        Pg, _ = g.get_state()
    Pn, loc = orc.tdgl_step(f, P, 0.1)
    st = orc.sweep_stats(f, Pn[2], Pn[5], loc[2], loc[5])
    assert np.allclose(r[:10], st[:10], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("shape", [(16, 12, 6), (40, 17, 9)])
def test_run_fp32_refined_vs_fp64_oracle(gpu, orc, shape):
    """FP32 fields + FP64-refined potential against the FP64 oracle solved to
    ||r|| <= 1e-12 ||b||: fields within 2e-5 of max |P| after 30 steps,
    potential within 1e-4 relative, rows within 1e-5."""
    f, P = random_film(*shape, seed=31, eps_0_nd=4.0, p_scale=0.2)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    n = 30
    Ez = np.linspace(0.0, -0.4, n)
    rows = np.arange(n, dtype=np.int32)
    Pw, _, phiw, statw, _, rc = orc.run(f, P, np.zeros(f.N), Ez, rows)
    assert rc == 0
    import cmsl_gb300 as cg
    with _film(gpu, f, precision=cg.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-4) as g:
        g.set_state(P)
        g.run(Ez, rows)
        Pg, phig = g.get_state()
        rg = g.rows()
        it, rf = g.iters()
    for a, b in zip(Pg, Pw):
        assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max()
    assert np.abs(phig - phiw).max() <= 1e-4 * np.abs(phiw).max()
    assert np.abs(rg[:, :10] - statw[:, :10]).max() <= 1e-5
    assert (rf >= 1).all() and (it >= 1).all()


def test_fp32_refined_reaches_refine_tolerance(gpu, orc):
    """After one refined solve ||b - A phi|| / ||b|| <= 1e-8 (checked in FP64 by the oracle)."""
    f, P = random_film(40, 17, 9, seed=41, eps_0_nd=4.0)
    import cmsl_gb300 as cg
    with _film(gpu, f, precision=cg.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-4) as g:
        g.set_state(P)
        res = g.depol()
        Pg, phi = g.get_state()
    assert res["status"] == 0
    div = orc.divergence(f, Pg[0], Pg[1], Pg[2])
    b = -div
    k = np.repeat(np.arange(f.nz), f.nx * f.ny)
    b[(k == 0) | (k == f.nz - 1)] = 0.0
    r = b - orc.apply_A(f, phi)
    assert np.linalg.norm(r) <= 1.2e-8 * np.linalg.norm(b)


def test_fp32_refined_uniform_eps(gpu, orc):
    """Every material with the same eps_r selects the constant-coefficient
    operator specialisation of the persistent solver."""
    from tests.films import MATS_DEFAULT
    mats = MATS_DEFAULT.copy()
    mats[:, 7] = 30.0
    f, P = random_film(40, 17, 9, seed=43, eps_0_nd=4.0, mats=mats, p_scale=0.2)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    n = 12
    Ez = np.linspace(0.0, 0.3, n)
    Pw, _, phiw, _, _, rc = orc.run(f, P, np.zeros(f.N), Ez)
    assert rc == 0
    import cmsl_gb300 as cg
    with _film(gpu, f, precision=cg.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-5) as g:
        g.set_state(P)
        g.run(Ez)
        Pg, phig = g.get_state()
    for a, b in zip(Pg, Pw):
        assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max()
    assert np.abs(phig - phiw).max() <= 1e-4 * np.abs(phiw).max()


@pytest.mark.parametrize("two_kernel", [False, True])
def test_fp32_refined_neumann(gpu, orc, two_kernel, monkeypatch):
    """Neumann film (one pinned cell, ill-conditioned operator) in
    FP32_REFINED mode with the persistent single-reduction inner solver and
    with the two-kernel one: no PCG failure, fields within 2e-5 of max |P|
    and potential within 1e-4 of the FP64 oracle after 20 steps."""
    if two_kernel:
        monkeypatch.setenv("CMSL_PCG_TWO_KERNEL", "1")
    f, P = random_film(33, 9, 5, seed=52, zbc=oracle.NEUMANN, eps_0_nd=3.0, del_t=5e-4, p_scale=0.2,
                       layered=True)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    n = 20
    Ez = 0.3 * np.sin(np.linspace(0.0, 3.0, n))
    Pw, _, phiw, _, _, rc = orc.run(f, P, np.zeros(f.N), Ez)
    assert rc == 0
    import cmsl_gb300 as cg
    with _film(gpu, f, precision=cg.FP32_REFINED, refine_tol=1e-8, inner_tol=1e-4) as g:
        g.set_state(P)
        g.run(Ez)
        Pg, phig = g.get_state()
        it, rf = g.iters()
    for a, b in zip(Pg, Pw):
        assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max()
    assert np.abs(phig - phiw).max() <= 1e-4 * np.abs(phiw).max()
    assert (rf >= 1).all()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_checkpoint_restart_continues_the_run(gpu, orc, precision, tmp_path):
    """A film written to the reference's checkpoint file and restarted in a
    new film continues the same trajectory: P after 10 more steps within
    1e-9 (FP64) / 2e-5 (FP32_REFINED) of the uninterrupted run; the file's E
    is the field of the written potential."""
    import cmsl_gb300 as cg
    from cmsl_gb300 import formats as fm
    f, P = random_film(24, 20, 7, seed=71, eps_0_nd=4.0, p_scale=0.2, layered=True)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    kw = {} if precision == "fp64" else dict(precision=cg.FP32_REFINED, refine_tol=1e-10, inner_tol=1e-5)
    Ez = np.linspace(0.0, 0.3, 20)
    ck = tmp_path / "ck.bin"
    with _film(gpu, f, **kw) as a:
        a.set_state(P)
        a.run(Ez[:10])
        a.write_checkpoint(ck, peloop=1, count=10, Ez_ext=Ez[9], incEz=Ez[1] - Ez[0])
        _, phi_a = a.get_state()
        a.run(Ez[10:])
        Pa, _ = a.get_state()
    Pf, Ef, pe, cnt, ez, inc = fm.read_checkpoint(str(ck), f.nx, f.ny, f.nz)
    assert (pe, cnt, ez) == (1, 10, Ez[9])
    assert all(np.array_equal(x, y) for x, y in zip(Ef, orc.efield(f, phi_a)))
    with _film(gpu, f, **kw) as b:
        info = b.read_checkpoint(ck)
        assert info["count"] == 10
        b.run(Ez[10:])
        Pb, _ = b.get_state()
    tol = 1e-9 if precision == "fp64" else 2e-5
    for x, y in zip(Pb, Pa):
        assert np.abs(x - y).max() <= tol * np.abs(y).max()
