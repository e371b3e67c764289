"""Finite-difference checks of the operator gradient (the role of the
reference's gradient test, FwiOp/gradtest.jl:122-171).

`probe_directions` draws smooth random model perturbations masked to the
interior (at least `margin` cells from the CPML, as gradtest.jl:122-126 masks
the PML); `directional_check` compares the central difference
(J(m + h v) - J(m - h v)) / 2h with the adjoint-state directional derivative
<g, v> for each probe; `taylor_errors` returns |J(m + h v) - J(m) - h <g, v>|
over decreasing h (second order when the gradient is the derivative of J).

The reference's gradient is the adjoint-state gradient of its own
discretisation choices (staggered-time imaging, boundary-saving
reconstruction), not the exact derivative of its discrete misfit: on a
coarsely sampled model the two differ by several percent, and that gap is a
property of the method that this package reproduces, not an error of the
port.

    python fwiflow.jl_gb300/gradcheck.py [--workload dipping_grf] [--probes 32] [--nsteps N]

prints one JSON line with the per-parameter statistics of a GPU run.
"""
from __future__ import annotations

from typing import Callable, Dict, List, Sequence

import numpy as np


def smooth(a: np.ndarray, sigma: float) -> np.ndarray:
    """Separable Gaussian smoothing (reflecting edges), numpy only."""
    if sigma <= 0:
        return a
    r = int(np.ceil(3 * sigma))
    k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma) ** 2)
    k /= k.sum()
    out = a
    for ax in (0, 1):
        pad = [(0, 0), (0, 0)]
        pad[ax] = (r, r)
        p = np.pad(out, pad, mode="reflect")
        out = np.apply_along_axis(lambda v: np.convolve(v, k, mode="valid"), ax, p)
    return out


def interior_mask(nz_pad: int, nx_pad: int, nPml: int, nPad: int, margin: int = 5) -> np.ndarray:
    m = np.zeros((nz_pad, nx_pad))
    m[nPml + margin: nz_pad - nPml - nPad - margin, nPml + margin: nx_pad - nPml - margin] = 1.0
    return m


def probe_directions(shape, n: int, mask: np.ndarray, seed: int = 0, sigma: float = 2.0) -> List[np.ndarray]:
    """n smooth unit-norm directions, zero outside `mask`."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        v = smooth(rng.standard_normal(shape), sigma) * mask
        out.append(v / np.linalg.norm(v))
    return out


def directional_check(misfit: Callable[[Dict[str, np.ndarray]], float], model: Dict[str, np.ndarray],
                      grads: Dict[str, np.ndarray], probes: Sequence[tuple], h_rel: float = 1e-3) -> List[dict]:
    """For each (name, v) in probes: central difference of `misfit` along v in
    parameter `name` (step h = h_rel * |m_name| / |v|) and the adjoint
    directional derivative <grads[name], v>."""
    out = []
    for name, v in probes:
        m = model[name]
        h = h_rel * np.linalg.norm(m) / np.linalg.norm(v)
        plus = dict(model)
        minus = dict(model)
        plus[name] = m + h * v
        minus[name] = m - h * v
        fd = (misfit(plus) - misfit(minus)) / (2.0 * h)
        ad = float(np.sum(grads[name] * v))
        out.append({"param": name, "fd": float(fd), "adjoint": ad,
                    "rel_err": float(abs(fd - ad) / max(abs(fd), 1e-300))})
    return out


def taylor_errors(misfit: Callable[[Dict[str, np.ndarray]], float], model: Dict[str, np.ndarray],
                  grads: Dict[str, np.ndarray], name: str, v: np.ndarray, hs: Sequence[float]) -> List[tuple]:
    """(h, |J(m+hv) - J(m)|, |J(m+hv) - J(m) - h <g, v>|) for each h."""
    J0 = misfit(model)
    gv = float(np.sum(grads[name] * v))
    out = []
    for h in hs:
        p = dict(model)
        p[name] = model[name] + h * v
        Jh = misfit(p)
        out.append((float(h), abs(Jh - J0), abs(Jh - J0 - h * gv)))
    return out


def main(argv=None) -> None:
    import argparse
    import json
    import os
    import sys
    import tempfile

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as ge

    fw = ge.load_package()
    from fwiflow_gb300 import synthetic

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="dipping_grf", choices=["dipping_grf", "small_layered"])
    ap.add_argument("--probes", type=int, default=32)
    ap.add_argument("--nsteps", type=int, default=None)
    ap.add_argument("--h-rel", type=float, default=1e-3)
    args = ap.parse_args(argv)
    kw = {"nSteps": args.nsteps} if args.nsteps else {}
    w = synthetic.dipping_grf(**kw) if args.workload == "dipping_grf" else synthetic.small_layered(**kw)
    para = w.write_files(tempfile.mkdtemp())
    ids = list(range(len(w.shots)))
    ctx = fw.FwiContext(para, 0)
    obs = ctx.obs(*w.moduli(w.vp_obs), w.stf, ids, write_files=False)
    lam, mu, rho = w.moduli()
    model = {"lambda": lam, "mu": mu, "den": rho}
    J, gl, gm, gd, _ = ctx.misfit_grad(lam, mu, rho, w.stf, ids, obs=obs)
    grads = {"lambda": gl, "mu": gm, "den": gd}
    mask = interior_mask(w.nz_pad, w.nx_pad, w.nPml, w.nPad)
    dirs = probe_directions(lam.shape, args.probes, mask, seed=2)
    names = ["lambda", "mu", "den"]
    probes = [(names[k % 3], v) for k, v in enumerate(dirs)]

    def misfit(m):
        return ctx.misfit(m["lambda"], m["mu"], m["den"], w.stf, ids, obs=obs)

    res = directional_check(misfit, model, grads, probes, args.h_rel)
    summ = {}
    for n in names:
        e = np.array([r["rel_err"] for r in res if r["param"] == n])
        s = [np.sign(r["fd"]) == np.sign(r["adjoint"]) for r in res if r["param"] == n]
        summ[n] = {"probes": int(e.size), "median_rel_err": float(np.median(e)), "max_rel_err": float(e.max()),
                   "sign_agree": int(sum(s))}
    fd = np.array([r["fd"] for r in res])
    ad = np.array([r["adjoint"] for r in res])
    line = {"check": "central FD vs adjoint directional derivative", "workload": w.name, "cells": w.cells,
            "nSteps": w.nSteps, "probes": args.probes, "h_rel": args.h_rel, "misfit": J, "per_param": summ,
            "cosine_fd_adjoint": float(fd @ ad / (np.linalg.norm(fd) * np.linalg.norm(ad)))}
    print(json.dumps(line))
    ctx.close()


if __name__ == "__main__":
    main()
