"""The allocation-free depolarisation solve against the film API.

cmsl_depol_solve_noalloc serves callers that cannot allocate device memory
themselves (the buffers here come from the caller, torch in this test).  Two
calls in a row -- the second warm-started from the first's potential, with a
new polarisation -- must give the potential cmsl_film_depol gives for the
same inputs, within the FP64 PCG tolerance of the other parity tests
(1e-10 of max |phi|).  This file is collected last so that a run that stops
at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests.films import random_film

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cmsl_gb300 import build
    build.build()
    import cmsl_gb300
    from cmsl_gb300 import _lib
    return torch, cmsl_gb300, _lib


def _noalloc(torch, _lib, f, Pm, phi_dev, tol_abs, tol_rel):
    dev = torch.device("cuda", 0)
    mat = torch.as_tensor(np.asarray(f.grain_mat)[np.asarray(f.omega)].astype(np.int32), device=dev)
    P = [torch.as_tensor(np.ascontiguousarray(p, np.float64), device=dev) for p in Pm]
    eps = (C.c_double * 3)(*[float(e) for e in np.asarray(f.mats)[:, 7]])
    it = np.zeros(1, np.int32)
    st = np.zeros(1, np.int32)
    torch.cuda.synchronize()
    rc = _lib.lib().cmsl_depol_solve_noalloc(
        f.nx, f.ny, f.nz, f.del_h, int(f.zbc), f.eps_0_nd, C.c_void_p(mat.data_ptr()), eps,
        C.c_void_p(P[0].data_ptr()), C.c_void_p(P[1].data_ptr()), C.c_void_p(P[2].data_ptr()),
        C.c_void_p(phi_dev.data_ptr()), tol_abs, tol_rel, 4000, int(f.crit), None,
        it.ctypes.data_as(C.POINTER(C.c_int32)), st.ctypes.data_as(C.POINTER(C.c_int32)))
    _lib.check(rc)
    torch.cuda.synchronize()
    return int(it[0]), int(st[0])


# (40, 17, 9): two x tiles (one partial) and partial y tiles; (20, 5, 4): one
# partial tile; (64, 64, 32): the scratch array full (131072 cells).
@pytest.mark.parametrize("shape", [(40, 17, 9), (20, 5, 4), (64, 64, 32)])
@pytest.mark.parametrize("zbc", [oracle.DIRICHLET, oracle.NEUMANN])
def test_noalloc_matches_film_depol_twice(setup, zbc, shape):
    torch, cg, _lib = setup
    f, P1 = random_film(*shape, seed=51, zbc=zbc, eps_0_nd=3.0)
    f.tol_abs, f.tol_rel = 1e-10, 1e-8
    _, P2 = random_film(*shape, seed=52, zbc=zbc, eps_0_nd=3.0)
    phi0 = np.zeros(f.N)
    # existing entry point: two solves in a row, the second warm-started
    with cg.Film.from_oracle_film(f) as g:
        g.set_state(P1, phi0)
        r1 = g.depol()
        _, want1 = g.get_state()
        g.set_state(P2, want1)
        r2 = g.depol()
        _, want2 = g.get_state()
    phi = torch.zeros(f.N, dtype=torch.float64, device="cuda")
    it1, st1 = _noalloc(torch, _lib, f, P1[:3], phi, f.tol_abs, f.tol_rel)
    got1 = phi.cpu().numpy().copy()
    it2, st2 = _noalloc(torch, _lib, f, P2[:3], phi, f.tol_abs, f.tol_rel)
    got2 = phi.cpu().numpy()
    assert st1 == 0 and st2 == 0 and r1["status"] == 0 and r2["status"] == 0
    assert it1 == r1["iters"] and it2 == r2["iters"]
    assert np.abs(got1 - want1).max() <= 1e-10 * np.abs(want1).max()
    assert np.abs(got2 - want2).max() <= 1e-10 * np.abs(want2).max()


def test_noalloc_rejects_oversize_grid(setup):
    torch, cg, _lib = setup
    eps = (C.c_double * 3)(30.0, 30.0, 30.0)
    it = np.zeros(1, np.int32)
    st = np.zeros(1, np.int32)
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    rc = _lib.lib().cmsl_depol_solve_noalloc(
        128, 128, 16, 0.5, 0, 1.0, p, eps, p, p, p, p, 1e-3, 1e-2, 10, 0, None,
        it.ctypes.data_as(C.POINTER(C.c_int32)), st.ctypes.data_as(C.POINTER(C.c_int32)))
    assert rc == 1
    assert b"131072" in _lib.lib().cmsl_last_error()


@pytest.mark.parametrize("zbc", [oracle.DIRICHLET, oracle.NEUMANN])
def test_noalloc_matches_oracle(setup, zbc):
    """One solve against the oracle's restatement of Depol_field
    (depol_varEPS.cu:332-595) directly: same potential to the PCG's
    dot-product summation order, iteration count within one."""
    torch, cg, _lib = setup
    f, P = random_film(40, 17, 9, seed=53, zbc=zbc, eps_0_nd=3.0)
    f.tol_abs, f.tol_rel = 1e-10, 1e-8
    phi0 = np.random.default_rng(4).normal(size=f.N) * 0.01
    want, _, _, info = oracle.load().depol_field(f, P[:3], phi0)
    phi = torch.as_tensor(phi0.copy(), device="cuda")
    it, st = _noalloc(torch, _lib, f, P[:3], phi, f.tol_abs, f.tol_rel)
    got = phi.cpu().numpy()
    assert st == 0 and info["status"] == 0
    assert abs(it - info["iters"]) <= 1
    assert np.abs(got - want).max() <= 1e-10 * np.abs(want).max()


def test_noalloc_rejects_bad_material(setup):
    """A material id outside 0..2 is reported as an argument error (the
    solve's material check is read on the caller's stream)."""
    torch, cg, _lib = setup
    f, P = random_film(20, 5, 4, seed=54)
    f.grain_mat = np.asarray(f.grain_mat).copy()
    f.grain_mat[int(np.asarray(f.omega)[0])] = 3      # the grain of cell 0
    phi = torch.zeros(f.N, dtype=torch.float64, device="cuda")
    with pytest.raises(cg.CmslError) as e:
        _noalloc(torch, _lib, f, P[:3], phi, 1e-10, 1e-8)
    assert e.value.status == 1 and "material" in str(e.value)
