"""State transfers through the C ABI: where the device reads the host's page
tables (Grace-Blackwell), set_state/get_state convert on the GPU reading and
writing the caller's arrays in place; CMSL_HOST_COPY=1 forces the host-side
conversion.  Both paths round-trip the state (FP64 bit for bit; FP32_REFINED:
P rounded to float, phi to the double-float pair) and give identical runs."""
import numpy as np
import pytest

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


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("with_phi", [True, False])
def test_state_round_trip_and_run(gpu, precision, with_phi, monkeypatch):
    """With a potential and without one (zero start): the GPU conversion
    (one launch for the whole FP32 state each way) and the host-side one give
    the same state and identical runs."""
    f, P = random_film(36, 20, 10, seed=101, eps_0_nd=3.0, p_scale=0.2)
    phi = np.random.default_rng(5).normal(0.0, 0.3, f.N) if with_phi else None
    kw = dict(precision=gpu.FP64 if precision == "fp64" else gpu.FP32_REFINED)
    Ez = np.linspace(0.0, 0.2, 6)
    out = []
    for host_copy in ("0", "1"):
        monkeypatch.setenv("CMSL_HOST_COPY", host_copy)
        with gpu.Film.from_oracle_film(f, **kw) as g:
            g.set_state(P, phi)
            Pg, phig = g.get_state()
            for a, b in zip(Pg, P):
                want = b if precision == "fp64" else np.asarray(b, np.float32).astype(np.float64)
                assert np.array_equal(a, want)
            if phi is None:
                assert not phig.any()
            elif precision == "fp64":
                assert np.array_equal(phig, phi)
            else:
                assert np.abs(phig - phi).max() <= 1e-14 * np.abs(phi).max()
            g.run(Ez)
            out.append(g.get_state())
    for a, b in zip(out[0][0], out[1][0]):
        assert np.array_equal(a, b)
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_page_locked_outputs(gpu, precision):
    """get_state into page-locked arrays (written by the GPU) gives the same
    values as into fresh pageable arrays, for a film and for a batch."""
    f, P = random_film(36, 20, 10, seed=103, eps_0_nd=3.0, p_scale=0.2)
    kw = dict(precision=gpu.FP64 if precision == "fp64" else gpu.FP32_REFINED)
    Ez = np.linspace(0.0, 0.2, 6)
    P_in = [gpu.pinned_empty(f.N) for _ in range(6)]
    for a, p in zip(P_in, P):
        a[:] = p
    out = ([gpu.pinned_empty(f.N) for _ in range(6)], gpu.pinned_empty(f.N))
    with gpu.Film.from_oracle_film(f, **kw) as g:
        g.set_state(P_in)
        g.run(Ez)
        Pa, pha = g.get_state()
        Pb, phb = g.get_state(out=out)
        assert Pb[0] is out[0][0] and phb is out[1]
        for a, b in zip(Pa, Pb):
            assert np.array_equal(a, b)
        assert np.array_equal(pha, phb)
    f2, P2 = random_film(24, 24, 8, seed=104, eps_0_nd=3.0, p_scale=0.2)
    with gpu.Batch.from_oracle_films([f, f2], **kw) as b:
        b.set_state(0, P)
        b.set_state(1, P2)
        b.run(np.stack([Ez, Ez]))
        for i, n in enumerate((f.N, f2.N)):
            o = ([gpu.pinned_empty(n) for _ in range(6)], gpu.pinned_empty(n))
            Pa, pha = b.get_state(i)
            Pb, phb = b.get_state(i, out=o)
            for a, c in zip(Pa, Pb):
                assert np.array_equal(a, c)
            assert np.array_equal(pha, phb)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_page_locked_inputs(gpu, precision):
    """set_state from page-locked P and phi gives the state and the run
    that pageable inputs give, and page-locked outputs read it back
    identically."""
    f, P = random_film(36, 20, 10, seed=107, eps_0_nd=3.0, p_scale=0.2)
    phi = np.random.default_rng(7).normal(0.0, 0.3, f.N)
    kw = dict(precision=gpu.FP64 if precision == "fp64" else gpu.FP32_REFINED)
    Ez = np.linspace(0.0, 0.2, 6)
    P_in = [gpu.pinned_empty(f.N) for _ in range(6)]
    for a, p in zip(P_in, P):
        a[:] = p
    phi_in = gpu.pinned_empty(f.N)
    phi_in[:] = phi
    res = []
    for Pu, phu in ((P, phi), (P_in, phi_in)):
        with gpu.Film.from_oracle_film(f, **kw) as g:
            g.set_state(Pu, phu)
            s0 = g.get_state()
            g.run(Ez)
            out = ([gpu.pinned_empty(f.N) for _ in range(6)], gpu.pinned_empty(f.N))
            s1 = g.get_state(out=out)
            res.append((s0, [np.array(a) for a in s1[0]], np.array(s1[1])))
    for a, b in zip(res[0][0][0], res[1][0][0]):
        assert np.array_equal(a, b)
    assert np.array_equal(res[0][0][1], res[1][0][1])
    for a, b in zip(res[0][1], res[1][1]):
        assert np.array_equal(a, b)
    assert np.array_equal(res[0][2], res[1][2])


def test_bad_out_arrays(gpu):
    f, P = random_film(12, 12, 4, seed=105, eps_0_nd=3.0, p_scale=0.2)
    with gpu.Film.from_oracle_film(f) as g:
        with pytest.raises(ValueError):
            g.get_state(out=([np.zeros(f.N)] * 5, np.zeros(f.N)))
        with pytest.raises(ValueError):
            g.get_state(out=([np.zeros(f.N)] * 6, np.zeros(f.N - 1)))
        with pytest.raises(ValueError):
            g.get_state(out=([np.zeros(f.N, np.float32)] * 6, np.zeros(f.N)))
