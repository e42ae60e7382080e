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
def test_state_round_trip_and_run(gpu, precision, monkeypatch):
    f, P = random_film(36, 20, 10, seed=101, eps_0_nd=3.0, p_scale=0.2)
    phi = np.random.default_rng(5).normal(0.0, 0.3, f.N)
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
            if precision == "fp64":
                assert np.array_equal(phig, phi)
            else:
                assert np.abs(phig - phi).max() <= 1e-14 * np.abs(phi).max()
            g.run(Ez)
            out.append(g.get_state())
    for a, b in zip(out[0][0], out[1][0]):
        assert np.array_equal(a, b)
    assert np.array_equal(out[0][1], out[1][1])
