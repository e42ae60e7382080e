"""FP32_REFINED against FP64 over a whole (short) P-E loop: remanent
polarization and coercive field of the loop within 1e-4 relative, the
sweep rows within 1e-5 (cmsl_gb300.precision, cmsl_gb300.pe)."""
import math

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cmsl_gb300 import build
    build.build()


def test_short_loop_pr_ec(gpu):
    from cmsl_gb300 import precision
    from cmsl_gb300 import workloads as wl
    w = wl.hzo_film("loop_48x48x12_afe40", 48, 48, 12, 12, 9, 0.4, E_amp_MVcm=4.0, steps_per_period=600)
    r = precision.compare(w, tol=1e-8)
    assert r["rel_err"]["Pr"] <= 1e-4
    if math.isfinite(r["rel_err"]["Ec"]):
        assert r["rel_err"]["Ec"] <= 1e-4
    assert r["rows_max_abs_err"] <= 1e-5
