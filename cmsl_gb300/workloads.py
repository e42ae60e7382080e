"""Seeded synthetic films with the shapes of the benchmark configurations.

No grain maps ship with the reference (HZO_Code_github has no gdata_*.bin),
so every film is generated: a columnar periodic Voronoi map from in-plane
seed points, grain orientations with |cos(theta)| uniform in [0.3, 1] and
phi, psi uniform in [0, 2 pi), and a seeded choice of AFE grains.

Landau coefficients are given in SI (f = a1 P^2 + a11 P^4 + a111 P^6) and
mapped to the reference's convention f = (alpha+g)/4 P^2 + beta/32 P^4 +
gamma/192 P^6 (PyhtonScriptsToFindLandauCoeffs/fe_range_1.py:68-83):
alpha = 4 a1 - g, beta = 32 a11, gamma = 192 a111, with g = J (the antipolar
coupling) for AFE grains and 0 for FE grains.  The reference's own
non-dimensionalisation against the FE phase follows (main.cu:200-256,
global.cu:30-31).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import schedule as sch

T0 = 3.0e-9          # global.cu:30
L0 = 1.0e-9          # global.cu:31
EPS0 = 8.854e-12     # main.cu:344


def compute_p0(alpha, beta, g, gamma1, transition_type=0):
    """main.cu:200-213."""
    if transition_type == 2:
        return 2.0 * math.sqrt((g - alpha) / beta)
    disc = beta * beta - 4.0 * gamma1 * (alpha - g)
    if -1e-14 < disc < 0.0:
        disc = 0.0
    if disc < 0.0:
        return 1.0
    num = 2.0 * abs(beta) + 2.0 * math.sqrt(disc)
    if gamma1 == 0.0:
        return 1.0
    return math.sqrt(num / gamma1)


def make_phase_refs(raw: dict):
    """main.cu:215-230 -> (alpha_ref, P0_ref)."""
    alpha_ref = abs(raw["alpha"])
    if raw["beta"] == 0.0 and raw["gamma1"] == 0.0 and raw["g"] == 0.0:
        p0 = 1.0
    else:
        p0 = compute_p0(raw["alpha"], raw["beta"], raw["g"], raw["gamma1"], raw.get("transition_type", 0))
        if not math.isfinite(p0) or p0 <= 0.0:
            p0 = 1.0
    return alpha_ref, p0


def make_nd(raw: dict, alpha_ref: float, P0_ref: float):
    """main.cu:232-256 -> [alpha, beta, gamma, g, a0, kappa, L, eps_r]."""
    a = raw["alpha"] / alpha_ref
    if not (raw["beta"] == 0.0 and raw["gamma1"] == 0.0 and raw["g"] == 0.0):
        b = (raw["beta"] * P0_ref * P0_ref) / (8.0 * alpha_ref)
        c = (raw["gamma1"] * pow(P0_ref, 4.0)) / (48.0 * alpha_ref)
        g = raw["g"] / alpha_ref
    else:
        b = c = g = 0.0
    a0 = (4.0 * raw["a0"]) / alpha_ref
    L = 0.25 * raw["L"] * alpha_ref * T0
    kap = raw["kappa"] / (alpha_ref * L0 * L0)
    return np.array([a, b, c, g, a0, kap, L, raw["eps_r"]], np.float64)


def voronoi_columnar(nx: int, ny: int, nz: int, n_grains: int, rng) -> np.ndarray:
    """Periodic in-plane Voronoi map (nearest seed under the minimum-image
    distance), repeated through z.  Returns omega in C order."""
    sx = rng.uniform(0.0, nx, n_grains)
    sy = rng.uniform(0.0, ny, n_grains)
    xs = np.arange(nx) + 0.5
    g2 = np.empty((ny, nx), np.int32)
    step = max(1, 4_000_000 // max(1, nx * n_grains))
    for j0 in range(0, ny, step):
        j1 = min(ny, j0 + step)
        ys = (np.arange(j0, j1) + 0.5)[:, None, None]
        dx = np.abs(xs[None, :, None] - sx[None, None, :])
        dx = np.minimum(dx, nx - dx)
        dy = np.abs(ys - sy[None, None, :])
        dy = np.minimum(dy, ny - dy)
        g2[j0:j1] = np.argmin(dx * dx + dy * dy, axis=-1)
    return np.ascontiguousarray(np.broadcast_to(g2, (nz, ny, nx)).reshape(-1))


def orientations(n: int, rng):
    """Euler angles (phi, theta, psi) with |cos theta| ~ U[0.3, 1]."""
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    cth = rng.uniform(0.3, 1.0, n) * rng.choice([-1.0, 1.0], n)
    psi = rng.uniform(0.0, 2.0 * np.pi, n)
    return phi, np.arccos(cth), psi


def tr_from_euler(phi, theta, psi) -> np.ndarray:
    """Bunge ZXZ lab->crystal rotation per grain, row major (grain_io.cu:103-126)."""
    sph, cph = np.sin(phi), np.cos(phi)
    sth, cth = np.sin(theta), np.cos(theta)
    sps, cps = np.sin(psi), np.cos(psi)
    T = np.empty((phi.size, 9))
    T[:, 0] = cph * cps - (cth * sph) * sps
    T[:, 1] = sph * cps + (cth * cph) * sps
    T[:, 2] = sth * sps
    T[:, 3] = -cph * sps - (cth * sph) * cps
    T[:, 4] = -sph * sps + (cth * cph) * cps
    T[:, 5] = sth * cps
    T[:, 6] = sth * sph
    T[:, 7] = -(sth * cph)
    T[:, 8] = cth
    return T.reshape(-1)


@dataclass
class Workload:
    name: str
    nx: int
    ny: int
    nz: int
    omega: np.ndarray
    grain_mat: np.ndarray
    TR: np.ndarray
    mats: np.ndarray          # [3, 8] non-dimensional (AFE, FE, DE)
    del_h: float
    del_t: float
    eps_0_nd: float
    E0_ref: float
    P0_ref: float
    P_init: list
    sched: sch.Schedule
    extra: dict = field(default_factory=dict)

    @property
    def N(self) -> int:
        return self.nx * self.ny * self.nz

    def film_kwargs(self) -> dict:
        return dict(del_h=self.del_h, del_t=self.del_t, eps_0_nd=self.eps_0_nd, dep_flag=1)


def hzo_film(name, nx, ny, nz, n_grains, seed, afe_frac, *, a1=-2.0e9, a11=1.0e10, a111=5.0e10,
             G=1.0e-10, J=3.0e9, eps_b=30.0, L=1.0, dt=1.0e-3, dx=0.5, a0=1.0e9,
             init="pz", E_amp_MVcm=3.0, steps_per_period=2000, n_periods=1, fixed_steps=None):
    rng = np.random.default_rng(seed)
    omega = voronoi_columnar(nx, ny, nz, n_grains, rng)
    phi, theta, psi = orientations(n_grains, rng)
    TR = tr_from_euler(phi, theta, psi)
    n_afe = int(round(afe_frac * n_grains))
    gm = np.full(n_grains, 1, np.int32)
    if n_afe:
        gm[rng.permutation(n_grains)[:n_afe]] = 0
    fe_raw = dict(alpha=4.0 * a1, beta=32.0 * a11, gamma1=192.0 * a111, g=0.0, a0=a0, L=L, kappa=G,
                  eps_r=eps_b)
    afe_raw = dict(alpha=4.0 * a1 - J, beta=32.0 * a11, gamma1=192.0 * a111, g=J, a0=a0, L=L, kappa=G,
                   eps_r=eps_b)
    de_raw = dict(alpha=abs(4.0 * a1), beta=0.0, gamma1=0.0, g=0.0, a0=a0, L=L, kappa=G, eps_r=eps_b)
    alpha_ref, P0_ref = make_phase_refs(fe_raw)          # reference phase: FE
    mats = np.stack([make_nd(afe_raw, alpha_ref, P0_ref), make_nd(fe_raw, alpha_ref, P0_ref),
                     make_nd(de_raw, alpha_ref, P0_ref)])
    E0_ref = (0.25 * alpha_ref * P0_ref * P0_ref) / P0_ref   # main.cu:273-274
    eps_0_nd = 4.0 / (EPS0 * abs(fe_raw["alpha"]))          # main.cu:343-344
    N = nx * ny * nz
    P = [np.zeros(N) for _ in range(6)]
    mat_cell = gm[omega]
    if init == "pz":
        u = rng.uniform(-0.01, 0.01, N) / P0_ref
        P[2] = np.where(mat_cell == 1, u, 0.0)
        for q in (3, 4, 5):                               # AFE start of init_conf.cu:48-56
            P[q] = np.where(mat_cell == 0, 1.0, 0.0)
    else:
        for q in range(6):
            P[q] = rng.uniform(-0.1, 0.1, N)
    Emax = E_amp_MVcm * 1.0e8 / E0_ref                       # V/m -> non-dimensional
    if fixed_steps:
        sched = sch.constant_schedule(Emax, fixed_steps, row_every=10)
    else:
        sched = sch.triangle_schedule(Emax, steps_per_period, n_periods)
    return Workload(name, nx, ny, nz, omega, gm, TR, mats, dx, dt, eps_0_nd, E0_ref, P0_ref, P, sched,
                    extra={"Emax": Emax})


def with_loop(w: Workload, steps_per_period: int, n_periods: int = 1) -> Workload:
    """The same film on a triangle loop of another length (same amplitude)."""
    return Workload(w.name + "_loop%dx%d" % (steps_per_period, n_periods), w.nx, w.ny, w.nz, w.omega, w.grain_mat,
                    w.TR, w.mats, w.del_h, w.del_t, w.eps_0_nd, w.E0_ref, w.P0_ref, w.P_init,
                    sch.triangle_schedule(w.extra["Emax"], steps_per_period, n_periods), dict(w.extra))


def config(i: int) -> Workload:
    """The five benchmark configurations (single films; config 3 is one of
    its 64 films, see ensemble())."""
    if i == 0:
        return hzo_film("c0_64x64x16_fe", 64, 64, 16, 20, 0, 0.0, E_amp_MVcm=3.0, steps_per_period=2000)
    if i == 1:
        return hzo_film("c1_256x256x32_afe40", 256, 256, 32, 200, 1, 0.4, E_amp_MVcm=4.0,
                        steps_per_period=4000, n_periods=2)
    if i == 2:
        return hzo_film("c2_512x512x64_afe25", 512, 512, 64, 2000, 2, 0.25, init="random",
                        E_amp_MVcm=2.0, fixed_steps=500)
    if i == 4:
        return hzo_film("c4_128x128x16_afe30", 128, 128, 16, 50, 3, 0.3, E_amp_MVcm=4.0,
                        steps_per_period=4000)
    raise ValueError("config %d is not a single film" % i)


def ensemble(n: int = 64, seed0: int = 100):
    """Config 3: n films of uneven size, seeds seed0..seed0+n-1."""
    films = []
    for f in range(n):
        r = np.random.default_rng(seed0 + f)
        side = int(r.choice([64, 96, 128, 192, 256]))
        nz = int(r.choice([8, 16, 32]))
        ng = int(r.integers(10, 401))
        afe = float(r.uniform(0.0, 0.6))
        amp = float(r.uniform(2.0, 5.0))
        films.append(hzo_film("c3_film%02d" % f, side, side, nz, ng, seed0 + f, afe, E_amp_MVcm=amp,
                              steps_per_period=2000))
    return films
