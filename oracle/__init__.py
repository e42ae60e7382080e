"""The oracle: CPU FP64 restatement of the HZO TDGL + Jacobi-PCG hot path.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg as the checker; the product package
``cmsl_gb300`` never imports it.

``oracle.liboracle.so`` is the restatement (``oracle/cmsl_oracle.c``), built by
``oracle/Makefile``.  ``oracle/_ref/libcmsl_ref.so`` is the reference's own
kernels compiled for the host by ``oracle/build_ref.sh``; it exists only where
the reference sources are available and is used to pin the restatement.
``oracle/ref_gpu.sh`` and ``oracle/ref_gpu_time.py`` build and time the
reference program's own FP64 GPU path for comparison; nothing of the library
links or runs them.
"""
from .oracle import (  # noqa: F401
    Film, OracleLib, RefLib, load, load_ref, build, build_ref, MAT_AFE, MAT_FE, MAT_DE,
    DIRICHLET, NEUMANN, CRIT_REF, CRIT_RELRES, reference_root, stage_ref_gpu,
)
