"""The two stagings of the FP32 stencil passes on films with full 32 x 8
tiles -- the cp.async ring (0) and tensor copies (1) -- in every combination
for the TDGL and the residual passes, each fixed through CMSL_STAGING at film
creation, advance a film like the FP64 oracle solved to 1e-12 (max |P| error
<= 2e-5 of max |P|, as the other FP32-refined parity tests).  Both residual
kernels are covered: one permittivity (direct inner solve) and three
(persistent PCG), Dirichlet and Neumann z boundaries.  The checks after a
step's direct solve stay in their own update pass here (CMSL_DEFER=0), so
that the tensor-copy TDGL kernel runs; tests/test_gpu_defer.py covers the
TDGL kernel that forms them."""
import numpy as np
import pytest

import oracle

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


def _oracle_film(orc, w, mats, zbc):
    f = oracle.Film(nx=w.nx, ny=w.ny, nz=w.nz, del_h=w.del_h, del_t=w.del_t, omega=w.omega,
                    grain_mat=w.grain_mat, TR=w.TR, mats=mats,
                    is_interface=orc.interface_flags(w.nx, w.ny, w.nz, w.omega, w.grain_mat),
                    dep_flag=1, zbc=zbc, eps_0_nd=w.eps_0_nd)
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    return f


@pytest.mark.parametrize("staging", ["00", "11", "01", "10"])
@pytest.mark.parametrize("eps", ["one", "three"])
@pytest.mark.parametrize("zbc", [oracle.DIRICHLET, oracle.NEUMANN])
def test_staging_matches_oracle(gpu, orc, staging, eps, zbc, monkeypatch):
    from cmsl_gb300 import workloads as wl
    w = wl.hzo_film("stg_64x32x13", 64, 32, 13, 9, 21, 0.4, E_amp_MVcm=4.0, steps_per_period=400)
    mats = np.array(w.mats, copy=True)
    if eps == "three":
        mats[:, 7] = [40.0, 30.0, 15.0]
    f = _oracle_film(orc, w, mats, zbc)
    n = 6
    Ez = w.sched.Ez[:n] * 40.0
    rng = np.random.default_rng(5)
    P0 = [p + rng.normal(scale=0.05, size=w.N) for p in w.P_init]
    Pw, _, _, _, _, rc = orc.run(f, P0, np.zeros(w.N), Ez)
    assert rc == 0
    monkeypatch.setenv("CMSL_STAGING", staging)
    monkeypatch.setenv("CMSL_DEFER", "0")       # the tensor-copy TDGL (deferred checks run on the ring)
    with gpu.Film.from_oracle_film(f, precision=gpu.FP32_REFINED) as g:
        cfg = g.tile_config()
        names = ("cp.async ring", "tensor copies")
        assert cfg["tdgl_staging"] == names[int(staging[0])]
        assert cfg["residual_staging"] == names[int(staging[1])]
        g.set_state(P0)
        g.run(Ez)
        Pg, _ = g.get_state()
        g.sync()
    err = max(np.abs(a - b).max() / np.abs(b).max() for a, b in zip(Pg, Pw))
    assert err <= 2e-5


@pytest.mark.parametrize("tile_y", [4, 8, 16])
@pytest.mark.parametrize("eps", ["one", "three"])
@pytest.mark.parametrize("shape", [(64, 32, 13), (40, 20, 9)])
def test_tile_height_matches_oracle(gpu, orc, tile_y, eps, shape, monkeypatch):
    """The FP32 stencil passes with tiles of 32 x 4, 32 x 8 and 32 x 16
    columns (CMSL_TILE_Y; the autotuner's choices), on a film of full tiles
    and one with partial tiles in x and y, against the FP64 oracle (same
    tolerance as above)."""
    from cmsl_gb300 import workloads as wl
    w = wl.hzo_film("tile_%dx%dx%d" % shape, *shape, 9, 23, 0.4, E_amp_MVcm=4.0, steps_per_period=400)
    mats = np.array(w.mats, copy=True)
    if eps == "three":
        mats[:, 7] = [50.0, 30.0, 15.0]
    f = _oracle_film(orc, w, mats, oracle.DIRICHLET)
    n = 6
    Ez = w.sched.Ez[:n] * 40.0
    rng = np.random.default_rng(6)
    P0 = [p + rng.normal(scale=0.05, size=w.N) for p in w.P_init]
    Pw, _, _, _, _, rc = orc.run(f, P0, np.zeros(w.N), Ez)
    assert rc == 0
    monkeypatch.setenv("CMSL_TILE_Y", str(tile_y))
    with gpu.Film.from_oracle_film(f, precision=gpu.FP32_REFINED) as g:
        cfg = g.tile_config()
        assert cfg["x"] == 32 and cfg["y"] == tile_y
        g.set_state(P0)
        g.run(Ez)
        Pg, _ = g.get_state()
    err = max(np.abs(a - b).max() / np.abs(b).max() for a, b in zip(Pg, Pw))
    assert err <= 2e-5
