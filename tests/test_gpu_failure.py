"""Failure detection of the persistent PCG's grid barrier, without a GPU fault.

The cooperative FP32 PCG synchronises its blocks with a software grid barrier
whose waits are bounded.  The failure is made on the host: at film creation
CMSL_PCG_HOLD_BLOCK names a block that never arrives at a barrier (a flag
that nothing sets) and CMSL_PCG_SPIN_LIMIT shortens every wait to a few
microseconds.  Every block's wait then runs out, the kernel returns, the
film's sync reports CMSL_ERR_CUDA, and the context stays usable: a film
created afterwards without the injection runs and matches the oracle.
"""
import os

import numpy as np
import pytest

import oracle
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


def _env(**kw):
    old = {k: os.environ.get(k) for k in kw}
    for k, v in kw.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = v
    return old


def test_pcg_barrier_timeout_is_reported_and_context_survives(gpu):
    cg = gpu
    # three permittivities (40 / 30 / 15), the inner solve forced to the persistent PCG
    f, P = random_film(64, 32, 8, seed=71, eps_0_nd=3.0, p_scale=0.2)
    Ez = np.full(3, 0.1)
    kw = dict(precision=cg.FP32_REFINED, refine_tol=1e-8, max_refine=4, inner_tol=1e-5, inner_solver=cg.INNER_PCG)
    old = _env(CMSL_PCG_HOLD_BLOCK="1", CMSL_PCG_SPIN_LIMIT="2000")
    try:
        g = cg.Film.from_oracle_film(f, **kw)
    finally:
        _env(**old)
    try:
        assert g.inner_solver == cg.INNER_PCG
        g.set_state(P)
        with pytest.raises(cg.CmslError) as e:
            g.run(Ez)
        assert e.value.status == 2 and "barrier timed out" in str(e.value)
    finally:
        g.close()
    # the context is intact: the same film without the injection matches the oracle
    f.crit, f.tol_rel, f.max_iter = oracle.CRIT_RELRES, 1e-12, 20000
    Pw, _, _, _, _, rc = oracle.load().run(f, P, np.zeros(f.N), Ez)
    assert rc == 0
    with cg.Film.from_oracle_film(f, **kw) as h:
        h.set_state(P)
        h.run(Ez)
        Pg, _ = h.get_state()
    err = max(np.abs(a - b).max() / np.abs(b).max() for a, b in zip(Pg, Pw))
    assert err <= 2e-5
