"""cmsl_gb300 -- GB300 (sm_103a) implementation of the HZO TDGL + Jacobi-PCG
phase-field hot path of jhb6617-arch/cmsl.

The compute runs in libcmsl_gb.so (hand-written CUDA, C ABI in
include/cmsl.h).  This package is its Python face: ``Film`` (one film on the
GPU), ``Batch`` (many films advancing together), the reference's input
formats and set-up (``formats``), the P-E loop schedule of ``Evolve``
(``schedule``) and the synthetic workloads the benchmarks use
(``workloads``).
"""
from ._lib import (  # noqa: F401
    FP64, FP32_REFINED, DIRICHLET, NEUMANN, CRIT_REF, CRIT_RELRES, INNER_AUTO, INNER_PCG, INNER_DIRECT,
    CmslError, LIB_PATH,
)
from .film import Batch, Film, pinned_empty  # noqa: F401
