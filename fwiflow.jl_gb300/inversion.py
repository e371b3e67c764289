"""Elastic FWI for Vp on the GB300 operator, with a pluggable gradient
preconditioner (none, the diagonal pseudo-Hessian from the source
illumination, or the learned CNN of precond.py).

Parameterisation as in the reference's examples: Vs = Vp / sqrt(3), density
from Gardner (rho = 310 Vp^0.25), lambda / mu in MPa from the velocities
(src/Utils.jl:221-227). Only the cells of the inversion mask change: the
interior of the padded grid without its top 10 rows (src/FWI.jl:47-49);
elsewhere the model stays at the starting model, as compute_misfit's masking
does (src/FWI.jl:171-177). Vp is kept in [vmin, vmax].

Optimisers (the reference hands the TF gradient to L-BFGS-B; here the loop is
explicit so the preconditioner can enter):
  `descent`  preconditioned steepest descent with a three-point line search;
             a preconditioned step that does not lower the misfit falls back
             to the plain gradient step (which thereby judges it).
  `lbfgs`    limited-memory BFGS (two-loop recursion) on the plain gradient,
             or preconditioned: the initial inverse Hessian of each
             iteration is the scaled diagonal gain of a preconditioner
             (pseudo-Hessian or learned) at the current model.
Each records, per iteration, the misfit, the relative model error
|Vp - Vp_true| / |Vp_true| over the mask and the wall time (GPU work
synchronised), so `time_to_error` can read the time to a target error.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Callable, List, Optional

import numpy as np

from .utils import velocity_to_moduli


def inversion_mask(nz_pad: int, nx_pad: int, nz: int, nx: int, nPml: int, top_rows: int = 10) -> np.ndarray:
    m = np.zeros((nz_pad, nx_pad))
    m[nPml + top_rows: nPml + nz, nPml: nPml + nx] = 1.0
    return m


def moduli_of_vp(vp):
    """(lambda, mu [MPa], rho) for Vs = Vp / sqrt(3) and Gardner density."""
    rho = 310.0 * vp ** 0.25
    lam, mu = velocity_to_moduli(vp, vp / np.sqrt(3.0), rho)
    return lam, mu, rho


def chain_to_vp(vp, g_lambda, g_mu, g_den):
    """dJ/dVp from dJ/dlambda, dJ/dmu (per MPa) and dJ/drho: lambda = mu =
    rho Vp^2 / 3e6, rho = 310 Vp^0.25."""
    rho = 310.0 * vp ** 0.25
    drho = 77.5 * vp ** -0.75
    dmod = (drho * vp * vp + 2.0 * rho * vp) / 3e6
    return (g_lambda + g_mu) * dmod + g_den * drho


@dataclass
class History:
    misfit: List[float] = field(default_factory=list)
    model_error: List[float] = field(default_factory=list)
    wall: List[float] = field(default_factory=list)
    evals: List[int] = field(default_factory=list)
    fallback: List[bool] = field(default_factory=list)

    def time_to_error(self, target: float) -> Optional[float]:
        for e, t in zip(self.model_error, self.wall):
            if e <= target:
                return t
        return None

    def as_dict(self) -> dict:
        return {"misfit": self.misfit, "model_error": self.model_error, "wall_s": self.wall, "evals": self.evals,
                "fallback": self.fallback}


class VpProblem:
    """Misfit and Vp gradient of one survey, observed data resident on the
    device (staged once), on an FwiContext."""

    def __init__(self, ctx, stf, shot_ids, obs, vp_start, vp_true, mask, vmin=1400.0, vmax=5000.0):
        self.ctx, self.mask = ctx, mask
        self.vp0 = np.asarray(vp_start, dtype=np.float64)
        self.vp_true = np.asarray(vp_true, dtype=np.float64)
        self.vmin, self.vmax = vmin, vmax
        self.n_shots = len(shot_ids)
        ctx.stage_shots(stf, shot_ids, obs=obs)
        self.evals = 0

    def full(self, vp):
        return np.clip(self.vp0 * (1 - self.mask) + vp * self.mask, self.vmin, self.vmax)

    def model_error(self, vp) -> float:
        m = self.mask > 0
        v = self.full(vp)
        return float(np.linalg.norm(v[m] - self.vp_true[m]) / np.linalg.norm(self.vp_true[m]))

    def misfit(self, vp) -> float:
        self.ctx.set_model(*moduli_of_vp(self.full(vp)))
        self.ctx.run(0)
        self.evals += 1
        return self.ctx.fetch(misfit=True)[0]

    def misfit_grad(self, vp, illumination: bool = False):
        """(misfit, dJ/dVp masked, (g_lambda, g_mu, g_den), illumination or None)."""
        v = self.full(vp)
        self.ctx.set_illumination(illumination)
        self.ctx.set_model(*moduli_of_vp(v))
        self.ctx.run(1)
        J, gl, gm, gd, _ = self.ctx.fetch(misfit=True, grads=True, n_shots=self.n_shots)
        illum = self.ctx.illumination() if illumination else None
        self.ctx.set_illumination(False)
        self.evals += 1
        return J, chain_to_vp(v, gl, gm, gd) * self.mask, (gl, gm, gd), illum


def _line_search(problem: VpProblem, vp, J, d, step: float):
    """Search along -d scaled so that the largest change is `step` m/s:
    tries a, then 2a if a lowers the misfit (else a/2, a/4, ... five times),
    and the minimum of the parabola through the best point and its
    neighbours. Returns (vp, J, largest change in m/s) or None when no point
    lowers the misfit."""
    dmax = float(np.max(np.abs(d)))
    if dmax == 0.0:
        return None
    a = step / dmax
    pts = [(0.0, J)]
    Ja = problem.misfit(vp - a * d)
    pts.append((a, Ja))
    if Ja < J:
        J2 = problem.misfit(vp - 2 * a * d)
        pts.append((2 * a, J2))
    else:
        k = 0.5
        for _ in range(5):
            Jk = problem.misfit(vp - k * a * d)
            pts.append((k * a, Jk))
            if Jk < J:
                break
            k *= 0.5
    pts.sort()
    best = min(pts, key=lambda p: p[1])
    i = pts.index(best)
    if 0 < i < len(pts) - 1:  # parabola through the best point and its neighbours
        (x0, y0), (x1, y1), (x2, y2) = pts[i - 1], pts[i], pts[i + 1]
        den = (x0 - x1) * (x0 - x2) * (x1 - x2)
        A = (x2 * (y1 - y0) + x1 * (y0 - y2) + x0 * (y2 - y1)) / den
        B = (x2 * x2 * (y0 - y1) + x1 * x1 * (y2 - y0) + x0 * x0 * (y1 - y2)) / den
        if A > 0:
            xm = -B / (2 * A)
            if x0 < xm < x2 and abs(xm - x1) > 1e-3 * x1:
                Jm = problem.misfit(vp - xm * d)
                if Jm < best[1]:
                    best = (xm, Jm)
    if best[1] >= J:
        return None
    return vp - best[0] * d, best[1], best[0] * dmax


def descent(problem: VpProblem, iters: int, precondition: Optional[Callable] = None, step_max: float = 60.0,
            target_error: Optional[float] = None) -> History:
    """Preconditioned steepest descent. precondition(vp, g_vp, grads,
    illum, mask) -> direction (None: the plain gradient); it gets the
    illumination, which is then accumulated during the gradient runs."""
    h = History()
    vp = problem.vp0.copy()
    t0 = time.perf_counter()
    J = None
    h.model_error.append(problem.model_error(vp))
    h.wall.append(0.0)
    h.evals.append(0)
    h.fallback.append(False)
    step = step_max  # trial largest change (m/s); follows the last accepted one
    for _ in range(iters):
        J, g, grads, illum = problem.misfit_grad(vp, illumination=precondition is not None)
        if not h.misfit:
            h.misfit.append(J)
        used_fallback = False
        res = None
        if precondition is not None:
            d = precondition(problem.full(vp), g, grads, illum, problem.mask) * problem.mask
            if np.sum(d * g) > 0:  # a descent direction
                res = _line_search(problem, vp, J, d, step)
        if res is None:
            used_fallback = precondition is not None
            res = _line_search(problem, vp, J, g, step)
        if res is None:
            break
        vp, J, change = res
        step = min(step_max, 1.5 * change)
        vp = np.clip(vp, problem.vmin, problem.vmax)
        h.misfit.append(J)
        h.model_error.append(problem.model_error(vp))
        h.wall.append(time.perf_counter() - t0)
        h.evals.append(problem.evals)
        h.fallback.append(used_fallback)
        if target_error is not None and h.model_error[-1] <= target_error:
            break
    h.final_vp = problem.full(vp)
    return h


def lbfgs(problem: VpProblem, iters: int, memory: int = 5, step_max: float = 60.0,
          target_error: Optional[float] = None, gain: Optional[Callable] = None) -> History:
    """L-BFGS (two-loop recursion, memory pairs) with the same line search;
    the first step (and any step after a failed search) is a steepest-descent
    step. gain(vp, g_vp, grads, illum, mask) -> diagonal gain G (None: the
    plain method) makes it preconditioned: the initial inverse Hessian of each
    iteration is gamma G at the current model, gamma = s.y / y.(G y) from the
    newest pair (the steepest-descent steps use G g); the illumination is then
    accumulated during the gradient runs."""
    h = History()
    vp = problem.vp0.copy()
    t0 = time.perf_counter()
    h.model_error.append(problem.model_error(vp))
    h.wall.append(0.0)
    h.evals.append(0)
    h.fallback.append(False)
    S, Y = [], []
    step = step_max
    want_illum = gain is not None

    def diag(v, g_, grads, illum):
        return np.ones_like(g_) if gain is None else gain(problem.full(v), g_, grads, illum, problem.mask)

    J, g, grads, illum = problem.misfit_grad(vp, illumination=want_illum)
    G = diag(vp, g, grads, illum)
    h.misfit.append(J)
    for _ in range(iters):
        q = g.copy()
        alphas = []
        for s, y in reversed(list(zip(S, Y))):
            a = np.sum(s * q) / np.sum(y * s)
            alphas.append(a)
            q -= a * y
        if S:
            q = G * q * (np.sum(S[-1] * Y[-1]) / np.sum(Y[-1] * G * Y[-1]))
        else:
            q = G * q
        for (s, y), a in zip(zip(S, Y), reversed(alphas)):
            b = np.sum(y * q) / np.sum(y * s)
            q += (a - b) * s
        d = q * problem.mask
        res = _line_search(problem, vp, J, d, step) if np.sum(d * g) > 0 else None
        fell_back = False
        if res is None:
            S.clear()
            Y.clear()
            fell_back = True
            res = _line_search(problem, vp, J, g, step)
            if res is None:
                break
        vp_new, _, change = res
        step = min(step_max, 1.5 * change)
        vp_new = np.clip(vp_new, problem.vmin, problem.vmax)
        J_new, g_new, grads, illum = problem.misfit_grad(vp_new, illumination=want_illum)
        G = diag(vp_new, g_new, grads, illum)
        s, y = vp_new - vp, g_new - g
        if np.sum(s * y) > 1e-12 * np.linalg.norm(s) * np.linalg.norm(y):
            S.append(s)
            Y.append(y)
            if len(S) > memory:
                S.pop(0)
                Y.pop(0)
        vp, J, g = vp_new, J_new, g_new
        h.misfit.append(J)
        h.model_error.append(problem.model_error(vp))
        h.wall.append(time.perf_counter() - t0)
        h.evals.append(problem.evals)
        h.fallback.append(fell_back)
        if target_error is not None and h.model_error[-1] <= target_error:
            break
    h.final_vp = problem.full(vp)
    return h


def pseudo_hessian_preconditioner(eps: Optional[float] = None) -> Callable:
    """d = g_vp / (H + eps max_mask H): the exact diagonal preconditioner the
    network stands in for."""
    from .precond import EPS, illumination_gain

    def apply(vp, g_vp, grads, illum, mask):
        return g_vp * illumination_gain(illum, mask, EPS if eps is None else eps)

    return apply


def pseudo_hessian_gain(eps: Optional[float] = None) -> Callable:
    """The diagonal pseudo-Hessian preconditioner as a gain on the Vp
    gradient (for L-BFGS's initial inverse Hessian)."""
    from .precond import EPS, illumination_gain

    def gain(vp, g_vp, grads, illum, mask):
        return illumination_gain(illum, mask, EPS if eps is None else eps)

    return gain


def learned_gain(net) -> Callable:
    """The network's predicted gain on the Vp gradient: exp of the mean of its
    three log-gain channels."""

    def gain(vp, g_vp, grads, illum, mask):
        from .precond import features

        out = net.predict(features(*grads, illum, mask))
        return np.exp(np.clip(out.mean(axis=0), -30.0, 5.0))

    return gain


def learned_preconditioner(net) -> Callable:
    """d = dVp of the network's preconditioned lambda / mu / rho gradients."""

    def apply(vp, g_vp, grads, illum, mask):
        pl, pm, pd = net.precondition(*grads, illum, mask)
        return chain_to_vp(vp, pl, pm, pd)

    return apply
