"""Checks against the committed outputs of the reference's own kernels
(tests/golden/ref_kernels.npz, made by tests/golden/make_golden.py from the
reference sources compiled for the host).  The oracle must reproduce them bit
for bit; the GPU (FP64 mode, through the C ABI) likewise for the TDGL step,
operator, Jacobi diagonal and E field, and to PCG summation order for the
depolarisation solve.  Unlike tests/test_oracle_pin.py these run where the
reference sources are absent."""
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "ref_kernels.npz"))
CASES = range(int(G["n_cases"][0]))


def film(c):
    p = "c%d_" % c
    nx, ny, nz, zbc, dep = (int(v) for v in G[p + "dims"])
    h, dt, eps0, _ = G[p + "scal"]
    return oracle.Film(nx=nx, ny=ny, nz=nz, del_h=float(h), del_t=float(dt), omega=G[p + "omega"],
                       grain_mat=G[p + "grain_mat"], TR=G[p + "TR"], mats=G[p + "mats"], is_interface=G[p + "iface"],
                       dep_flag=dep, zbc=zbc, eps_0_nd=float(eps0), tol_abs=1e-10, tol_rel=1e-8)


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("c", CASES)
def test_oracle_reproduces_reference_outputs(c):
    o = oracle.load()
    f = film(c)
    p = "c%d_" % c
    Ez = float(G[p + "scal"][3])
    Pn, _ = o.tdgl_step(f, list(G[p + "P"]), Ez, list(G[p + "E"]))
    assert same(Pn, G[p + "Pn"])
    assert np.array_equal(o.divergence(f, *G[p + "P"][:3]), G[p + "div"])
    assert np.array_equal(o.apply_A(f, G[p + "x"]), G[p + "Ax"])
    assert np.array_equal(o.diag_inv(f), G[p + "dinv"])
    assert same(o.efield(f, G[p + "phi"]), G[p + "E"])
    phi, E, _, info = o.depol_field(f, list(G[p + "P"][:3]), np.zeros(f.N))
    assert abs(info["iters"] - int(G[p + "depol_iters"][0])) <= 1
    assert np.abs(phi - G[p + "depol_phi"]).max() <= 1e-10 * np.abs(G[p + "depol_phi"]).max()


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES)
def test_gpu_reproduces_reference_outputs(c):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cmsl_gb300 import build
    build.build()
    import cmsl_gb300 as cg
    f = film(c)
    p = "c%d_" % c
    Ez = float(G[p + "scal"][3])
    with cg.Film.from_oracle_film(f) as g:
        g.set_state(list(G[p + "P"]), G[p + "phi"])
        assert same(g.efield(), G[p + "E"])
        g.tdgl_step(Ez)
        Pn, _ = g.get_state()
        assert same(Pn, G[p + "Pn"])
        assert np.array_equal(g.apply_operator(G[p + "x"]), G[p + "Ax"])
        assert np.array_equal(g.diag_inv(), G[p + "dinv"])
        g.set_state(list(G[p + "P"]), np.zeros(f.N))
        if f.dep_flag:
            res = g.depol()
            _, phi = g.get_state()
            assert abs(res["iters"] - int(G[p + "depol_iters"][0])) <= 1
            assert np.abs(phi - G[p + "depol_phi"]).max() <= 1e-10 * np.abs(G[p + "depol_phi"]).max()
