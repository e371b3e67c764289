"""Benchmark of the GB300 elastic FWI operator: batched forward + adjoint
throughput (Gpts/s = grid cells x time steps x shots per second of one
misfit + gradient evaluation) against the HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload batched_uneven|dipping_grf|small_layered|faulted_grf] [--shots S]
                    [--nsteps T] [--tile-widths a,b,c,d] [--tile-rows a,b,c,d] [--e2e-steps E]
                    [--no-compare-single] [--no-cpu-baseline] [--cpu-sample-steps T]

Default workload: 64 shots of the 512x1536-interior dipping-layer model, each
with its own aperture window (400-1536 columns), record length (1500-4000
steps) and Ricker frequency (8-12 Hz), all in one misfit + gradient call.
One step = one misfit + gradient call (forward sweep with boundary saving,
residual, reverse / adjoint sweeps with imaging) over the workload's shots.
`value`: model, shots and observed data resident in HBM, CUDA events on the
library's stream around fwigb_run. `e2e`: the public C-ABI call
fwigb_misfit_grad_obs with pinned host buffers (model in, gradients out),
min(K, E) calls. `roofline`: per-sweep times of one call measured inside the
call (an event pair around each sweep step, all shot packs of the step).
`one_shot_per_launch`: the same call with every shot in a group of its own
(unless --no-compare-single).
`--impl reference` times the reference algorithm's CPU implementation (the
oracle restatement, all host threads) on a bounded number of time steps of
the same workload. `cpu_baseline` (N = 1 only): the same oracle on the
first steps of the same workload. With N > 1 (torchrun) the multi-shot
workloads grow to N times their shots and each rank runs its cost-balanced
share (weak scaling); the single-shot workloads run one replica per rank.
Shots with their own aperture window and record length count their own
cells and steps.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

# Algorithmic bytes per grid cell and time step of each sweep (FP32 arrays read
# or written once): forward stress 11 floats, forward velocity 9, backward B 24,
# backward C 22; forward + adjoint = 264 B per cell-step.
SWEEP_NAMES = ["fwd_stress", "fwd_velocity", "bwd_B", "bwd_C"]
SWEEP_KERNELS = ["k_fwd_stress", "k_fwd_velocity", "k_bwd_B", "k_bwd_C"]
SWEEP_BYTES = [44, 36, 96, 88]
FWD_ADJ_BYTES = 264


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(name, nsteps=None, shots=None):
    ge.load_package()
    from fwiflow_gb300 import synthetic

    if name == "small_layered":
        return synthetic.small_layered(**({"nSteps": nsteps} if nsteps else {}))
    if name == "faulted_grf":
        return synthetic.faulted_grf(shot_subset=shots or 16, **({"nSteps": nsteps} if nsteps else {}))
    if name == "batched_uneven":
        kw = {"n_shots": shots or 64}
        if nsteps:  # scale the record lengths down (profiler captures)
            kw["steps"] = (max(2, nsteps * 3 // 8), nsteps)
        return synthetic.batched_uneven(**kw)
    return synthetic.dipping_grf(**({"nSteps": nsteps} if nsteps else {}))


def shot_sizes(w, ids=None):
    """(cells, steps) of every shot (or of the shots `ids`): its sub-grid
    (aperture window + 2 nPml columns) and its record length."""
    out = []
    for s in (w.shots if ids is None else [w.shots[k] for k in ids]):
        nx = s["win_x1"] - s["win_x0"] + 1 + 2 * w.nPml if "win_x0" in s else w.nx_pad
        out.append((w.nz_pad * nx, int(s.get("nSteps", w.nSteps))))
    return out


def sweep_cell_steps(w, ids=None):
    """Cell-steps each sweep kind processes in one misfit + gradient call
    (over the shots `ids`, default all): forward stress / velocity and
    backward B run nSteps-1 times per shot, backward C nSteps times."""
    sz = shot_sizes(w, ids)
    fwd = sum(c * (n - 1) for c, n in sz)
    return [fwd, fwd, fwd, sum(c * n for c, n in sz)]


def describe(w):
    sz = shot_sizes(w)
    if w.name == "batched_uneven":
        return (f"{w.name}: {w.nz}x{w.nx} interior + {w.nPml} CPML (nPad {w.nPad}); {len(w.shots)} shots, aperture "
                f"windows {min(c for c, _ in sz) // w.nz_pad - 2 * w.nPml}..{max(c for c, _ in sz) // w.nz_pad - 2 * w.nPml}"
                f" columns, record lengths {min(n for _, n in sz)}..{max(n for _, n in sz)} steps, Ricker 8-12 Hz, "
                f"dx {w.dx} m, dt {w.dt * 1e3:g} ms, FP32; one misfit+gradient per step")
    shots = f"{len(w.shots)} of the survey's 128 shots" if w.name == "faulted_grf" else f"{len(w.shots)} shot(s)"
    return (f"{w.name}: {w.nz}x{w.nx} interior + {w.nPml} CPML (nPad {w.nPad}) = {w.nz_pad}x{w.nx_pad} cells, "
            f"{w.nSteps} steps, {shots}, dx {w.dx} m, dt {w.dt * 1e3:g} ms, FP32; "
            f"one misfit+gradient per step")


def store_gib(w):
    """Boundary store streamed per call: 5 fields x the 5-layer ring of every
    shot's sub-grid x its record length."""
    tot = 0
    for c, n in shot_sizes(w):
        nx = c // w.nz_pad
        ring = 10 * (nx - 2 * w.nPml + 4) + 10 * (w.nz_pad - 2 * w.nPml - w.nPad - 6)
        tot += n * 5 * 4 * ring
    return tot / 2 ** 30


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 8:
                    continue
                try:
                    sm.append(float(parts[0]))
                    smax.append(float(parts[1]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[4:8]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_oracle_case(w, n_steps_sample):
    """The CPU sample of the workload: its first n_steps_sample time steps
    (and, for windowed shots, its first shot), with the observed data of the
    sample computed once by the oracle. Returns (workload, para, obs)."""
    orc = ge.load_oracle()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    from dataclasses import replace

    shots = [dict(s, nSteps=min(int(s.get("nSteps", n_steps_sample)), n_steps_sample)) for s in w.shots]
    if any("win_x0" in s for s in w.shots):
        shots = shots[:1]  # one windowed shot bounds the sample
    ws = replace(w, nSteps=n_steps_sample, stf=np.ascontiguousarray(w.stf[:len(shots), :n_steps_sample]),
                 shots=shots)
    tmp = tempfile.mkdtemp()
    para = ws.write_files(tmp)
    ids = list(range(len(ws.shots)))
    obs = orc.cufd(2, *ws.moduli(ws.vp_obs), ws.stf, ids, para, nthreads=cpu_threads(), write_files=False,
                   want_gathers=True)["gathers"]
    return ws, para, obs


def run_cpu_oracle(case, reps=1):
    """Times the oracle (reference algorithm on all host cores) on a sample
    from cpu_oracle_case: misfit + gradient. Returns (Gpts/s, seconds, threads)."""
    ws, para, obs = case
    orc = ge.load_oracle()
    ids = list(range(len(ws.shots)))
    nthreads = cpu_threads()
    lam, mu, rho = ws.moduli()
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        orc.cufd(1, lam, mu, rho, ws.stf, ids, para, nthreads=nthreads, obs=obs)
        orc.cufd(0, lam, mu, rho, ws.stf, ids, para, nthreads=nthreads, obs=obs)
        times.append(time.perf_counter() - t0)
    pts = sum(c * n for c, n in shot_sizes(ws))
    return pts / min(times) / 1e9, times, nthreads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched_uneven",
                    choices=["batched_uneven", "dipping_grf", "small_layered", "faulted_grf"])
    ap.add_argument("--shots", type=int, default=None, help="shots of the batched_uneven workload (default 64) / of the faulted_grf survey (default 16 of 128)")
    ap.add_argument("--no-compare-single", action="store_true",
                    help="skip the timing of one step with one shot per launch on the same workload")
    ap.add_argument("--e2e-steps", type=int, default=3, help="end-to-end calls timed (at most --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-steps", type=int, default=3000)
    ap.add_argument("--nsteps", type=int, default=None,
                    help="override the workload's time steps (small cases for profiler captures)")
    ap.add_argument("--tile-widths", default=None,
                    help="fix the four sweeps' tile widths, e.g. 4,8,4,4 (default: autotuned)")
    ap.add_argument("--tile-rows", default=None,
                    help="fix the four sweeps' depths per thread, e.g. 2,2,1,1 (default: autotuned)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    # With N > 1 ranks the multi-shot workloads grow to N times their shots
    # (the first shots are those of the one-rank workload) and every rank
    # takes its cost-balanced share (weak scaling, no exchange in the timed
    # region); a lone-shot workload runs as N replicas.
    sharded = world > 1 and args.workload in ("batched_uneven", "faulted_grf")
    default_shots = {"batched_uneven": 64, "faulted_grf": 16}.get(args.workload)
    w = workload(args.workload, args.nsteps, (args.shots or default_shots) * world if sharded else args.shots)
    metric, unit = "fwd+adj Gpts/s vs HBM roofline", "Gpts/s"
    all_ids = list(range(len(w.shots)))
    if sharded:
        from fwiflow_gb300.shots import shard_shots, shot_costs

        costs = shot_costs(shot_sizes(w))
        ids = shard_shots(all_ids, world, costs)[rank]
    else:
        costs, ids = None, all_ids
    cell_steps = sum(c * n for c, n in shot_sizes(w))  # whole job (all ranks' shots when sharded)
    cfg = {"workload": describe(w), "cells": w.cells, "nSteps": w.nSteps, "shots": len(w.shots),
           "cell_steps_per_call": cell_steps,
           "parallelism": (f"shots sharded over {world} ranks" if sharded else f"replicas x{world}") if world > 1
           else "single GPU",
           "l2": "flushed between timed steps (256 MiB write); each step also streams a "
                 f"{store_gib(w):.2f} GiB boundary store"}

    if args.impl == "reference":
        if rank != 0:
            return
        n_sample = max(20, min(args.cpu_sample_steps, w.nSteps) // 2)
        case = cpu_oracle_case(w, n_sample)
        vals = []
        for _ in range(args.warmup):
            run_cpu_oracle(case)
        t_all = []
        for _ in range(args.steps):
            g, t, threads = run_cpu_oracle(case)
            vals.append(g)
            t_all += t
        value = statistics.median(vals)
        sample = (f"first {n_sample} of {w.nSteps} time steps of the same grid and shots, misfit + gradient "
                  f"(oracle restatement of the reference cufd path, OpenMP)")
        line = {"impl": "reference", "metric": metric, "value": value, "unit": unit, "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(t_all),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": cfg,
                "cpu_baseline": {"value": value, "unit": unit, "cores": threads, "kind": "port", "sample": sample},
                "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch

    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    fw = ge.load_package()
    ge._build_lib()
    tmp = tempfile.mkdtemp()
    para = w.write_files(tmp)
    ctx = fw.FwiContext(para, local_rank)
    if args.tile_widths:
        ctx.set_tile_config([int(v) for v in args.tile_widths.split(",")])
    if args.tile_rows:
        ctx.set_tile_rows([int(v) for v in args.tile_rows.split(",")])
    obs = ctx.obs(*w.moduli(w.vp_obs), w.stf, ids, write_files=False)
    lam, mu, rho = w.moduli()
    ctx.set_model(lam, mu, rho)
    ctx.stage_shots(w.stf, ids, obs=obs)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local_rank))
    flush = torch.empty(64 * 2 ** 20, dtype=torch.float32, device="cuda")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        ctx.run(1)
    ctx.synchronize()
    clocks = ClockSampler(local_rank)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stops = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    # The NVTX range marks the timed steps for profilers (ncu --nvtx
    # --nvtx-include "timed_steps/" captures only their launches).
    torch.cuda.nvtx.range_push("timed_steps")
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            ctx.run(1)
            stops[k].record(stream)
    torch.cuda.nvtx.range_pop()
    ctx.synchronize()
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches_per_step = ctx.last_launch_count()
    cfg["tile_widths"] = dict(zip(SWEEP_NAMES, ctx.tile_config()))
    cfg["tile_rows_per_thread"] = dict(zip(SWEEP_NAMES, ctx.tile_rows()))
    cfg["tile_registers"] = dict(zip(SWEEP_NAMES, ctx.tile_registers()))
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, stops)]
    dev_s = sum(step_ms) / 1e3
    if world > 1:
        t = torch.tensor([dev_s, wall], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_s, wall = float(t[0]), float(t[1])
    pts_step = sum(c * n for c, n in shot_sizes(w, ids))  # this rank's cell-steps per call
    job_pts = cell_steps if sharded else world * pts_step
    value = job_pts * args.steps / dev_s / 1e9

    # Per-sweep timing for the roofline, measured inside one call: an event
    # pair around every sweep step (all shot packs of the step; the pair costs
    # a few microseconds per step and stops the next sweep's launch from
    # overlapping this one's tail). A sweep's algorithmic bytes over the call
    # are its bytes per cell times the cell-steps its launches processed.
    ctx.set_kernel_timing(True)
    ctx.run(1)
    tot_ms, cnt = ctx.kernel_times()
    ctx.set_kernel_timing(False)
    ctx.run(1)
    # Supplementary: a CUDA graph of 50 back-to-back sweep steps over the
    # whole group (no event pair between them).
    us_graph = np.array([ctx.sweep_time(k, 50) for k in range(4)])
    cs = sweep_cell_steps(w, ids)
    k_dom = int(np.argmax(tot_ms))
    peak, peak_kind = peaks()
    kbytes_call = [SWEEP_BYTES[k] * cs[k] for k in range(4)]
    achieved = kbytes_call[k_dom] / (tot_ms[k_dom] * 1e-3) / 1e9
    per_kernel = {SWEEP_NAMES[k]: {"launches": int(cnt[k]), "avg_us": 1e3 * tot_ms[k] / max(cnt[k], 1),
                                   "share": float(tot_ms[k] / tot_ms.sum()),
                                   "algorithmic_GBps": kbytes_call[k] / (tot_ms[k] * 1e-3) / 1e9,
                                   "graph_avg_us_all_shots": float(us_graph[k])}
                  for k in range(4)}
    bytes_launch = kbytes_call[k_dom] / max(cnt[k_dom], 1)  # per sweep step, averaged over the call
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if os.path.exists(tfile):
        # "<kernel> <DRAM bytes of one sweep step> <cells it covered>"; scaled
        # to this call's average active cells per sweep step.
        for line in open(tfile):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == SWEEP_KERNELS[k_dom] and not line.startswith("#"):
                traffic = float(parts[1]) * (cs[k_dom] / max(cnt[k_dom], 1)) / float(parts[2])
    step_gbps = FWD_ADJ_BYTES * pts_step / (dev_s / args.steps) / 1e9

    # End to end through the public C ABI with pinned host buffers.
    def pinned(a, dtype):
        t = torch.empty(a.shape, dtype=dtype, pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()

    lam_h, mu_h, rho_h = (pinned(a, torch.float64) for a in (lam, mu, rho))
    stf_h = pinned(w.stf, torch.float64)
    obs_blk = np.zeros((len(ids), ctx.nrec_max, w.nSteps), dtype=np.float32)
    for i, o in enumerate(obs):
        obs_blk[i, :o.shape[0], :o.shape[1]] = o
    obs_h = pinned(obs_blk, torch.float32)
    out = {k: pinned(np.zeros((w.nz_pad, w.nx_pad)), torch.float64) for k in ("gl", "gm", "gd")}
    gs_h = pinned(np.zeros((len(ids), w.nSteps)), torch.float64)
    mis = np.zeros(1)
    lib = ctx._lib
    from fwiflow_gb300 import _lib

    ids_a = np.asarray(ids, dtype=np.int32)

    def rank_call(l, m, d, stf, mine):
        assert list(mine) == list(ids)
        _lib.check(lib.fwigb_misfit_grad_obs(ctx._h, _lib.dptr(lam_h), _lib.dptr(mu_h), _lib.dptr(rho_h),
                                             _lib.dptr(stf_h), stf_h.shape[0], _lib.iptr(ids_a), len(ids),
                                             _lib.fptr(obs_h), _lib.dptr(mis), _lib.dptr(out["gl"]),
                                             _lib.dptr(out["gm"]), _lib.dptr(out["gd"]), _lib.dptr(gs_h)), ctx._h)
        return float(mis[0]), out["gl"], out["gm"], out["gd"], gs_h

    def e2e_call():
        if sharded:  # a data-parallel step: this rank's shots, then one all-reduce of misfit and gradients
            from fwiflow_gb300.shots import sharded_misfit_grad

            sharded_misfit_grad(rank_call, lam_h, mu_h, rho_h, stf_h, all_ids, rank=rank, world=world, costs=costs,
                                device=torch.device("cuda", local_rank))
        else:
            rank_call(lam_h, mu_h, rho_h, stf_h, ids)

    e2e_call()
    n_e2e = max(1, min(args.steps, args.e2e_steps))
    barrier()
    t1 = time.perf_counter()
    for _ in range(n_e2e):
        e2e_call()
    barrier()
    e2e_s = time.perf_counter() - t1
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t[0])
    e2e_val = job_pts * n_e2e / e2e_s / 1e9
    h2d = 3 * w.cells * 8 + stf_h.nbytes + obs_h.nbytes
    d2h = 3 * w.cells * 8 + len(ids) * w.nSteps * 8 + 8

    single = None
    if not args.no_compare_single:
        # The same call with one shot per launch (groups of one shot).
        ctx.set_model(lam, mu, rho)
        ctx.stage_shots(w.stf, ids, obs=obs)
        ctx.set_batching(max_shots=1)
        ctx.run(1)
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            ctx.run(1)
            e1.record(stream)
        ctx.synchronize()
        torch.cuda.synchronize()
        s_single = e0.elapsed_time(e1) / 1e3
        ctx.set_batching(max_shots=0)
        single = {"value": pts_step / s_single / 1e9, "unit": unit, "ms_per_step": 1e3 * s_single,
                  "groups": ctx.last_group_count(),
                  "batched_over_single": (pts_step * args.steps / dev_s) / (pts_step / s_single),
                  "note": "same call, every shot in a group of its own (one shot per launch)"}

    if rank != 0:
        return
    line = {
        "metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dev_s / args.steps, "wall_ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": cfg,
        "roofline": {"bound": "hbm", "kernel": SWEEP_KERNELS[k_dom], "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                     if peak_kind == "measured" else "fallback 6.8 TB/s",
                     "traffic": traffic, "algorithmic_bytes_per_launch": bytes_launch,
                     "launch_unit": "one sweep step: the launches of all shot packs of the group at one time step",
                     "launch_timing": "CUDA events around every sweep step of one misfit + gradient call",
                     "step_algorithmic_GBps": step_gbps, "step_frac": step_gbps / peak,
                     "sweeps_ms_per_call": float(tot_ms.sum()), "kernels": per_kernel},
        "e2e": {"value": e2e_val, "unit": unit, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "calls_timed": n_e2e},
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": clk,
    }
    if single:
        line["one_shot_per_launch"] = single
    if not args.no_cpu_baseline and world == 1:  # the host-core baseline is taken at N = 1 only
        g, t, threads = run_cpu_oracle(cpu_oracle_case(w, min(args.cpu_sample_steps, w.nSteps)))
        line["cpu_baseline"] = {"value": g, "unit": unit, "cores": threads, "kind": "port",
                                "sample": f"first {min(args.cpu_sample_steps, w.nSteps)} of {w.nSteps} time steps, "
                                          f"same grid and shots, misfit + gradient, {t[0]:.1f} s"}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
