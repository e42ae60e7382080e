"""Landau-coefficient fitting on P-E loops: the misfit of a simulated loop
against a target loop, its gradient by the hand-written adjoint of the TDGL
step and the depolarisation solve (``cmsl_film_loop_gradient``), and a
``torch.autograd.Function`` over it.

The coefficients theta = (a1, a11, a111, G, J) are the SI Landau expansion
f = a1 P^2 + a11 P^4 + a111 P^6, the gradient coefficient and the antipolar
coupling, mapped to the reference's per-material parameters as
``workloads.hzo_film`` does (PyhtonScriptsToFindLandauCoeffs/fe_range_1.py:
68-83; FE: alpha = 4 a1, beta = 32 a11, gamma = 192 a111, g = 0; AFE: alpha =
4 a1 - J, g = J; DE: alpha = |4 a1|; kappa = G) and made non-dimensional
with the scales of the nominal coefficients (main.cu:200-256), which stay
fixed while theta moves: the loss compares loops in the same units.

    python -m cmsl_gb300.adjoint --config 4 [--steps-per-period N] [--rel-h 1e-4,1e-6] [--params a1,G]
"""
from __future__ import annotations

import argparse
import json
import time
from dataclasses import dataclass, field

import numpy as np

from . import workloads as wl

THETA_NAMES = ("a1", "a11", "a111", "G", "J")
THETA_NOMINAL = np.array([-2.0e9, 1.0e10, 5.0e10, 1.0e-10, 3.0e9])


@dataclass
class LoopFit:
    """One film, one field schedule, one target loop."""
    work: wl.Workload
    theta0: np.ndarray                       # nominal coefficients (fix the scales)
    target: np.ndarray = None                # [n_rows] target <Pm_z> per row
    a0: float = 1.0e9
    L: float = 1.0
    eps_b: float = 30.0
    tol: float = 1e-11
    checkpoint_every: int = 200
    alpha_ref: float = field(init=False)
    P0_ref: float = field(init=False)

    def __post_init__(self):
        fe = self._raw(self.theta0)[1]
        self.alpha_ref, self.P0_ref = wl.make_phase_refs(fe)

    def _raw(self, theta):
        a1, a11, a111, G, J = (float(x) for x in theta)
        com = dict(a0=self.a0, L=self.L, kappa=G, eps_r=self.eps_b)
        afe = dict(alpha=4.0 * a1 - J, beta=32.0 * a11, gamma1=192.0 * a111, g=J, **com)
        fe = dict(alpha=4.0 * a1, beta=32.0 * a11, gamma1=192.0 * a111, g=0.0, **com)
        de = dict(alpha=abs(4.0 * a1), beta=0.0, gamma1=0.0, g=0.0, **com)
        return afe, fe, de

    def mats(self, theta) -> np.ndarray:
        """[3, 8] non-dimensional parameters (AFE, FE, DE) at theta."""
        return np.stack([wl.make_nd(r, self.alpha_ref, self.P0_ref) for r in self._raw(theta)])

    def dmats(self, theta) -> np.ndarray:
        """[3, 5, 5]: d (alpha, beta, gamma, g, kappa)_material / d theta."""
        ar, p0 = self.alpha_ref, self.P0_ref
        J = np.zeros((3, 5, 5))
        kap = 1.0 / (ar * wl.L0 * wl.L0)
        for m in (0, 1):                     # AFE, FE: the Landau polynomial
            J[m, 0, 0] = 4.0 / ar
            J[m, 1, 1] = 32.0 * p0 * p0 / (8.0 * ar)
            J[m, 2, 2] = 192.0 * p0 ** 4 / (48.0 * ar)
            J[m, 4, 3] = kap
        J[0, 0, 4] = -1.0 / ar               # AFE alpha = 4 a1 - J
        J[0, 3, 4] = 1.0 / ar                # AFE g = J
        J[2, 0, 0] = 4.0 * np.sign(theta[0]) / ar
        J[2, 4, 3] = kap
        return J

    def film(self, theta):
        import cmsl_gb300 as cg
        w = self.work
        return cg.Film(w.nx, w.ny, w.nz, w.omega, w.grain_mat, w.TR, self.mats(theta), **w.film_kwargs(),
                       precision=cg.FP64, pcg_crit=cg.CRIT_RELRES, tol_rel=self.tol, max_iter=20000)

    def loop(self, theta) -> np.ndarray:
        """<Pm_z> of every row of the loop at theta (forward only)."""
        s = self.work.sched
        with self.film(theta) as f:
            f.set_state(self.work.P_init)
            f.run(s.Ez, s.rows)
            return f.rows(0, s.n_rows)[:, 0].copy()

    def loss(self, theta) -> float:
        d = self.loop(theta) - self.target
        return float(np.mean(d * d))

    def loss_and_grad(self, theta):
        """(loss, d loss / d theta [5]) by the adjoint."""
        s = self.work.sched
        with self.film(theta) as f:
            f.set_state(self.work.P_init)
            L, g = f.loop_gradient(s.Ez, s.rows, self.target, self.checkpoint_every)
        return L, np.einsum("mp,mpt->t", g, self.dmats(theta))

    def workspace_bytes(self) -> int:
        """Device memory the adjoint allocates for one call."""
        w, s = self.work, self.work.sched
        K = min(self.checkpoint_every, s.n_steps)
        nseg = -(-s.n_steps // K)
        n = w.N
        return 8 * n * (7 * nseg + 6 * K + 14)


def _autograd_function():
    import torch

    class LandauLoopLoss(torch.autograd.Function):
        """loss(theta) of a LoopFit; backward through the adjoint."""

        @staticmethod
        def forward(ctx, theta, fit):
            L, g = fit.loss_and_grad(theta.detach().cpu().numpy().astype(np.float64))
            ctx.save_for_backward(torch.as_tensor(g, dtype=theta.dtype, device=theta.device))
            return theta.new_tensor(L)

        @staticmethod
        def backward(ctx, gout):
            (g,) = ctx.saved_tensors
            return gout * g, None

    return LandauLoopLoss


_FN = None


def landau_loop_loss(theta, fit: LoopFit):
    """torch scalar loss of the loop at theta (a float64 tensor of 5 values);
    ``.backward()`` gives d loss / d theta by the adjoint."""
    global _FN
    if _FN is None:
        _FN = _autograd_function()
    return _FN.apply(theta, fit)


def config4_fit(seed: int = 3, steps_per_period: int = 0, checkpoint_every: int = 200, tol: float = 1e-11):
    """The coefficient-fitting problem of benchmark configuration 4: the
    128x128x16, 50-grain, 30 % AFE film on a +-4 MV/cm loop; the target loop is
    the model's own at theta perturbed by seeded factors in [0.8, 1.2]."""
    w = wl.config(4)
    if steps_per_period:
        w = wl.with_loop(w, steps_per_period, 1)
    fit = LoopFit(w, THETA_NOMINAL.copy(), checkpoint_every=checkpoint_every, tol=tol)
    factors = np.random.default_rng(seed).uniform(0.8, 1.2, 5)
    fit.target = fit.loop(THETA_NOMINAL * factors)
    return fit, factors


def gradient_check(fit: LoopFit, theta, rel_h=(1e-4,), params=THETA_NAMES):
    """Adjoint gradient against central differences (step rel_h |theta_i|, for
    each rel_h and each named parameter); times the forward and the adjoint."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L = fit.loss(theta)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    La, g = fit.loss_and_grad(theta)
    torch.cuda.synchronize()
    t_adj = time.perf_counter() - t0
    fd = {}
    for name in params:
        i = THETA_NAMES.index(name)
        for rh in rel_h:
            h = rh * abs(theta[i])
            tp, tm = theta.copy(), theta.copy()
            tp[i] += h
            tm[i] -= h
            v = (fit.loss(tp) - fit.loss(tm)) / (2.0 * h)
            fd["%s@%g" % (name, rh)] = {"fd": v, "adjoint": float(g[i]),
                                        "rel_diff": abs(g[i] - v) / abs(v) if v != 0.0 else float("nan")}
    return {"loss": L, "loss_adjoint_pass": La, "grad_adjoint": dict(zip(THETA_NAMES, g.tolist())), "fd": fd,
            "forward_s": t_fwd, "adjoint_s": t_adj, "adjoint_over_forward": t_adj / t_fwd}


def main(argv=None):
    ap = argparse.ArgumentParser(description="adjoint gradient of the P-E loop misfit (configuration 4)")
    ap.add_argument("--config", type=int, default=4, choices=[4])
    ap.add_argument("--steps-per-period", type=int, default=0, help="override the loop length")
    ap.add_argument("--checkpoint-every", type=int, default=200)
    ap.add_argument("--tol", type=float, default=1e-11)
    ap.add_argument("--rel-h", default="1e-4", help="comma-separated relative FD steps")
    ap.add_argument("--params", default=",".join(THETA_NAMES), help="comma-separated parameters to difference")
    args = ap.parse_args(argv)
    import torch
    torch.cuda.set_device(0)
    from . import build
    build.build()
    fit, factors = config4_fit(steps_per_period=args.steps_per_period, checkpoint_every=args.checkpoint_every,
                               tol=args.tol)
    r = gradient_check(fit, THETA_NOMINAL.copy(), rel_h=[float(x) for x in args.rel_h.split(",")],
                       params=[p for p in args.params.split(",") if p])
    with fit.film(THETA_NOMINAL) as f:
        film_bytes = f.device_bytes()
    r.update({"workload": fit.work.name, "cells": fit.work.N, "steps": fit.work.sched.n_steps,
              "rows": fit.work.sched.n_rows, "checkpoint_every": fit.checkpoint_every,
              "theta_names": list(THETA_NAMES), "target_factors": factors.tolist(),
              "film_device_bytes": film_bytes, "adjoint_workspace_bytes": fit.workspace_bytes()})
    print(json.dumps(r))


if __name__ == "__main__":
    main()
