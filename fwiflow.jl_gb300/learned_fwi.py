"""Learned-preconditioner FWI experiment: time to a target relative model
error, learned vs plain, on one GPU.

1. Training set: for each training model of the layered + random-field family
   (synthetic.layered_grf, seeds train_seed..), the operator computes the
   observed data of the true model and, at the starting model, the lambda /
   mu / rho gradients with the source illumination; each gives one (features,
   pseudo-Hessian target, mask) sample (precond.py).
2. The CNN trains on those samples with the library's own kernels (Adam).
3. Held-out models (seeds eval_seed..): inversions from the starting model
   with plain steepest descent, learned-preconditioned descent (falling back
   to the plain step when its step does not lower the misfit), the exact
   pseudo-Hessian descent, plain L-BFGS and L-BFGS whose initial inverse
   Hessian is the learned (lbfgs_learned) or the pseudo-Hessian
   (lbfgs_pseudo_hessian) gain; each records misfit, model error and wall
   time per iteration.

4. Extended runs (--long-models M --long-iters N): on the first M held-out
   models, plain L-BFGS and learned L-BFGS continue to N iterations; each
   records its lowest relative model error, the time to reach it, and the
   time to the target error if it gets there.

    python fwiflow.jl_gb300/learned_fwi.py [--train-models 64] [--eval-models 4] [--iters 20]
                                           [--long-models 0] [--long-iters 100] [--out FILE]

prints one JSON line (per method: the median over the held-out models of the
time to the target error and of the final error; the learned methods also
with the training cost -- data generation plus training -- spread over the
held-out inversions, and added in full).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np


def main(argv=None) -> None:
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as ge

    fw = ge.load_package()
    from fwiflow_gb300 import inversion, precond, synthetic

    ap = argparse.ArgumentParser()
    ap.add_argument("--train-models", type=int, default=64)
    ap.add_argument("--eval-models", type=int, default=4)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--target-error", type=float, default=0.01)
    ap.add_argument("--nz", type=int, default=256)
    ap.add_argument("--nx", type=int, default=768)
    ap.add_argument("--shots", type=int, default=16)
    ap.add_argument("--nsteps", type=int, default=2000)
    ap.add_argument("--smooth", type=float, default=4.0, help="starting model: true model smoothed (cells)")
    ap.add_argument("--train-seed", type=int, default=1000)
    ap.add_argument("--eval-seed", type=int, default=2000)
    ap.add_argument("--methods", default="plain,learned,pseudo_hessian,lbfgs")
    ap.add_argument("--long-models", type=int, default=0, help="held-out models of the extended runs")
    ap.add_argument("--long-iters", type=int, default=100, help="iterations of the extended runs")
    ap.add_argument("--out", default=None, help="write the full histories (JSON) here")
    args = ap.parse_args(argv)

    def log(*a):
        print(*a, file=sys.stderr, flush=True)

    def model(seed):
        return synthetic.layered_grf(seed, nz=args.nz, nx=args.nx, n_shots=args.shots, nSteps=args.nsteps,
                                     smooth_cells=args.smooth)

    w0 = model(args.train_seed)
    para = w0.write_files(tempfile.mkdtemp())  # geometry shared by the whole family
    ctx = fw.FwiContext(para, 0)
    ids = list(range(len(w0.shots)))
    mask = inversion.inversion_mask(w0.nz_pad, w0.nx_pad, w0.nz, w0.nx, w0.nPml)

    def problem_of(w):
        obs = ctx.obs(*inversion.moduli_of_vp(w.vp_obs), w.stf, ids, write_files=False)
        return inversion.VpProblem(ctx, w.stf, ids, obs, w.vp, w.vp_obs, mask)

    def sample_of(prob):
        _, g, grads, illum = prob.misfit_grad(prob.vp0, illumination=True)
        return (precond.features(*grads, illum, mask), precond.pseudo_hessian_target(*grads, illum, mask), mask)

    t0 = time.perf_counter()
    train = [sample_of(problem_of(model(args.train_seed + k))) for k in range(args.train_models)]
    t_data = time.perf_counter() - t0
    log(f"training set: {len(train)} samples in {t_data:.1f} s")
    evals = [model(args.eval_seed + k) for k in range(args.eval_models)]
    val = [sample_of(problem_of(w)) for w in evals]

    net = precond.CnnPreconditioner(w0.nz_pad, w0.nx_pad, seed=0)
    t0 = time.perf_counter()
    loss0 = net.evaluate(val)
    hist = net.train(train, args.epochs, lr=args.lr)
    t_train = time.perf_counter() - t0
    val_loss = net.evaluate(val)
    log(f"trained {args.epochs} epochs in {t_train:.1f} s: train loss {hist[0]:.4g} -> {hist[-1]:.4g}, "
        f"held-out loss {loss0:.4g} -> {val_loss:.4g}")

    methods = args.methods.split(",")
    if "plain" in methods:  # plain first: its final error is the reference level
        methods = ["plain"] + [m for m in methods if m != "plain"]
    results = {m: [] for m in methods}
    for w in evals:
        ref_err = None
        for m in methods:
            prob = problem_of(w)
            if m == "plain":
                h = inversion.descent(prob, args.iters)
            elif m == "learned":
                h = inversion.descent(prob, args.iters, inversion.learned_preconditioner(net))
            elif m == "pseudo_hessian":
                h = inversion.descent(prob, args.iters, inversion.pseudo_hessian_preconditioner())
            elif m == "lbfgs":
                h = inversion.lbfgs(prob, args.iters)
            elif m == "lbfgs_learned":
                h = inversion.lbfgs(prob, args.iters, gain=inversion.learned_gain(net))
            elif m == "lbfgs_pseudo_hessian":
                h = inversion.lbfgs(prob, args.iters, gain=inversion.pseudo_hessian_gain())
            else:
                raise ValueError(m)
            d = h.as_dict()
            d["time_to_target_s"] = h.time_to_error(args.target_error)
            if m == "plain":
                ref_err = h.model_error[-1]
            d["plain_final_error"] = ref_err
            d["time_to_plain_final_s"] = h.time_to_error(ref_err) if ref_err is not None else None
            d["seed"] = w.extra["seed"]
            results[m].append(d)
            log(f"model {w.extra['seed']} {m:15s} error {h.model_error[0]:.5f} -> {h.model_error[-1]:.5f} "
                f"in {len(h.model_error) - 1} it, {h.wall[-1]:.1f} s, time to {args.target_error:g}: "
                f"{d['time_to_target_s']}, to plain's final error: {d['time_to_plain_final_s']}")

    def med(v):
        v = [x for x in v if x is not None]
        return float(np.median(v)) if v else None

    # Extended runs: does either L-BFGS reach the target, and how low does it go?
    long_runs = {"lbfgs": [], "lbfgs_learned": []}
    for w in evals[:args.long_models]:
        for m in long_runs:
            prob = problem_of(w)
            gain = inversion.learned_gain(net) if m == "lbfgs_learned" else None
            h = inversion.lbfgs(prob, args.long_iters, gain=gain)
            k = int(np.argmin(h.model_error))
            long_runs[m].append({"seed": w.extra["seed"], "iters": len(h.model_error) - 1,
                                 "start_error": h.model_error[0], "lowest_error": h.model_error[k],
                                 "iteration_of_lowest": k, "time_to_lowest_s": h.wall[k],
                                 "time_to_target_s": h.time_to_error(args.target_error),
                                 "final_misfit_ratio": h.misfit[-1] / h.misfit[0], "wall_s": h.wall[-1],
                                 "history": h.as_dict()})
            log(f"extended model {w.extra['seed']} {m:15s} lowest error {h.model_error[k]:.5f} at it {k} "
                f"({h.wall[k]:.1f} s); time to {args.target_error:g}: {h.time_to_error(args.target_error)}")

    train_cost = t_data + t_train
    n_inv = max(1, len(evals))
    summary = {}
    for m, rs in results.items():
        tt = [r["time_to_target_s"] for r in rs]
        tp = [r["time_to_plain_final_s"] for r in rs]
        summary[m] = {"reached": sum(t is not None for t in tt), "models": len(rs),
                      "median_time_to_target_s": med(tt),
                      "median_time_to_plain_final_error_s": med(tp),
                      "median_final_misfit_ratio": med([r["misfit"][-1] / r["misfit"][0] for r in rs]),
                      "median_final_error": med([r["model_error"][-1] for r in rs]),
                      "median_start_error": med([r["model_error"][0] for r in rs]),
                      "median_wall_s": med([r["wall_s"][-1] for r in rs])}
        if "learned" in m:  # the network's cost: amortised over the held-out inversions, and in full
            summary[m]["median_time_to_plain_final_error_with_amortised_training_s"] = med(
                [None if t is None else t + train_cost / n_inv for t in tp])
            summary[m]["median_time_to_plain_final_error_with_full_training_s"] = med(
                [None if t is None else t + train_cost for t in tp])
    extended = {}
    for m, rs in long_runs.items():
        if rs:
            extended[m] = {"models": len(rs), "iters": args.long_iters,
                           "reached_target": sum(r["time_to_target_s"] is not None for r in rs),
                           "median_lowest_error": med([r["lowest_error"] for r in rs]),
                           "median_time_to_lowest_s": med([r["time_to_lowest_s"] for r in rs]),
                           "median_start_error": med([r["start_error"] for r in rs]),
                           "per_model": [{k: v for k, v in r.items() if k != "history"} for r in rs]}
    line = {"experiment": "time to relative model error, learned vs plain preconditioner",
            "target_error": args.target_error, "grid": [w0.nz_pad, w0.nx_pad], "nSteps": args.nsteps,
            "shots": args.shots, "train_models": args.train_models, "eval_models": args.eval_models,
            "iters": args.iters, "training_data_s": t_data, "training_s": t_train, "train_loss": hist,
            "heldout_loss": [loss0, val_loss], "methods": summary, "extended_runs": extended}
    print(json.dumps(line))
    if args.out:
        with open(args.out, "w") as f:
            json.dump({"summary": line, "histories": results,
                   "extended_histories": {m: [r["history"] for r in rs] for m, rs in long_runs.items()}}, f)
    ctx.close()


if __name__ == "__main__":
    main()
