"""Generates tests/golden/ref_kernels.npz: outputs of the reference's own
kernels (HZO_Code_github/src/kernels_evol.cu, depol_varEPS.cu, compiled for the
host by oracle/build_ref.sh) on small seeded films.  Run where the reference
sources are available:

    python tests/golden/make_golden.py

The fixture lets machines without the reference check results against the
reference's outputs (tests/test_golden.py).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from tests.films import random_film  # noqa: E402

CASES = [
    # (nx, ny, nz, seed, zbc, dep, layered)
    (8, 8, 4, 1, 0, 1, True),
    (13, 9, 5, 2, 0, 1, True),
    (34, 6, 4, 3, 0, 1, False),     # two x tiles, a partial one
    (10, 8, 6, 4, 1, 1, True),      # Neumann z
    (9, 7, 5, 5, 0, 0, True),       # no depolarisation
]


def main():
    ref = oracle.load_ref()
    if ref is None:
        raise SystemExit("reference sources not available")
    out = {}
    for c, (nx, ny, nz, seed, zbc, dep, layered) in enumerate(CASES):
        f, P = random_film(nx, ny, nz, seed=100 + seed, zbc=zbc, dep_flag=dep, layered=layered, eps_0_nd=3.0)
        rng = np.random.default_rng(200 + seed)
        phi = rng.normal(size=f.N) * 0.2
        E = ref.efield(f, phi)
        Ez = float(rng.uniform(-0.5, 0.5))
        Pn, loc = ref.tdgl_step(f, P, Ez, E)
        x = rng.normal(size=f.N)
        pfx = "c%d_" % c
        out[pfx + "dims"] = np.array([nx, ny, nz, zbc, dep], np.int32)
        out[pfx + "scal"] = np.array([f.del_h, f.del_t, f.eps_0_nd, Ez])
        out[pfx + "omega"] = np.asarray(f.omega, np.int32)
        out[pfx + "grain_mat"] = np.asarray(f.grain_mat, np.int32)
        out[pfx + "TR"] = np.asarray(f.TR)
        out[pfx + "mats"] = np.asarray(f.mats)
        out[pfx + "iface"] = np.asarray(f.is_interface, np.int32)
        out[pfx + "P"] = np.stack(P)
        out[pfx + "phi"] = phi
        out[pfx + "x"] = x
        out[pfx + "E"] = np.stack(E)
        out[pfx + "Pn"] = np.stack(Pn)
        out[pfx + "div"] = ref.divergence(f, *P[:3])
        out[pfx + "Ax"] = ref.apply_A(f, x)
        out[pfx + "dinv"] = ref.diag_inv(f)
        phi_s, E_s, it = ref.depol_field(f, P[:3], np.zeros(f.N), tol_abs=1e-10, tol_rel=1e-8)
        out[pfx + "depol_phi"] = phi_s
        out[pfx + "depol_E"] = np.stack(E_s)
        out[pfx + "depol_iters"] = np.array([it], np.int32)
    out["n_cases"] = np.array([len(CASES)], np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_kernels.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_kernels.npz"))


if __name__ == "__main__":
    main()
