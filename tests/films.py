"""Seeded small films for the parity tests (numpy only, no GPU).

``random_film`` builds a columnar periodic-Voronoi grain map, random grain
materials and orientations, and per-material non-dimensional parameters in
the ranges the reference's decks produce, plus a random initial state.
"""
from __future__ import annotations

import numpy as np

import oracle

# Non-dimensional per-material rows (AFE, FE, DE): alpha, beta, gamma, g, a0, kappa, L, eps_r.
# Values follow the reference's non-dimensionalisation of its SingleL_input deck
# (main.cu:232-256) with the kinetic and gradient terms of the configuration in use.
MATS_DEFAULT = np.array([
    [0.62, -1.05, 1.30, 0.68, 0.50, 12.5, 1.5, 40.0],   # AFE
    [-1.00, -0.75, 1.10, -0.80, 0.50, 12.5, 6.0, 30.0],  # FE
    [3.10, 0.00, 0.00, 0.00, 0.80, 31.0, 6.0, 15.0],     # DE
])


def voronoi_columnar(nx, ny, nz, n_grains, rng):
    """Periodic in-plane Voronoi map, columnar through z; grain ids 0..n-1."""
    sx = rng.uniform(0, nx, n_grains)
    sy = rng.uniform(0, ny, n_grains)
    ii, jj = np.meshgrid(np.arange(nx) + 0.5, np.arange(ny) + 0.5, indexing="xy")
    dx = np.abs(ii[..., None] - sx)
    dy = np.abs(jj[..., None] - sy)
    dx = np.minimum(dx, nx - dx)
    dy = np.minimum(dy, ny - dy)
    g2 = np.argmin(dx * dx + dy * dy, axis=-1).astype(np.int32)  # [ny, nx]
    return np.ascontiguousarray(np.broadcast_to(g2, (nz, ny, nx)).reshape(-1))


def euler_tr(n, rng):
    phi = rng.uniform(0, 2 * np.pi, n)
    cth = rng.uniform(0.3, 1.0, n) * rng.choice([-1.0, 1.0], n)
    theta = np.arccos(cth)
    psi = rng.uniform(0, 2 * np.pi, n)
    return oracle.load().tr_from_euler(phi, theta, psi)


def random_film(nx, ny, nz, seed=0, n_grains=None, fracs=(0.4, 0.5, 0.1), dep_flag=1,
                zbc=oracle.DIRICHLET, mats=None, del_h=0.5, del_t=1e-3, eps_0_nd=2.0,
                layered=False, p_scale=0.3):
    rng = np.random.default_rng(seed)
    if n_grains is None:
        n_grains = max(2, (nx * ny) // 24)
    omega = voronoi_columnar(nx, ny, nz, n_grains, rng)
    if layered and nz >= 4:
        # a second grain set in the upper half: exercises z interfaces
        top = voronoi_columnar(nx, ny, nz, n_grains, rng) + n_grains
        kk = np.repeat(np.arange(nz), nx * ny)
        omega = np.where(kk >= nz // 2, top, omega).astype(np.int32)
        n_grains *= 2
    gm = rng.choice([0, 1, 2], size=n_grains, p=np.asarray(fracs) / np.sum(fracs)).astype(np.int32)
    tr = euler_tr(n_grains, rng)
    flags = oracle.load().interface_flags(nx, ny, nz, omega, gm)
    f = oracle.Film(nx=nx, ny=ny, nz=nz, del_h=del_h, del_t=del_t, omega=omega, grain_mat=gm, TR=tr,
                    mats=MATS_DEFAULT.copy() if mats is None else np.asarray(mats, np.float64),
                    is_interface=flags, dep_flag=dep_flag, zbc=zbc, eps_0_nd=eps_0_nd)
    N = nx * ny * nz
    P = [rng.uniform(-p_scale, p_scale, N) for _ in range(6)]
    return f, P
