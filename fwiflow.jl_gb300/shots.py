"""Shot sharding across ranks (one GPU per rank).

Shots are independent (libCUFD.cu:157 loops over them with no exchange), so
a data-parallel FWI step gives every rank its own subset of the shot list
and sums the results once per gradient: misfit and the three model gradients
are added over ranks; the source-time-function gradient rows of different
ranks are disjoint and are gathered into the caller's shot order. This is the
reference's own multi-GPU recipe (one `fwi_op` per `gpu_id` on a slice of
the shots, summed by the optimiser; docs/src/tutorials/fwi_lowlevel.md:139-151)
done inside one call.

The exchange runs through torch.distributed on host float64 tensors (gloo)
or on the current CUDA device (nccl); with a world size of 1 it is skipped.
"""
from __future__ import annotations

from typing import Callable, List, Optional, Sequence

import numpy as np


def shot_costs(shot_sizes: Sequence[tuple]) -> List[float]:
    """Work of each shot: sub-grid cells x record length."""
    return [float(c) * float(n) for c, n in shot_sizes]


def shard_shots(shot_ids: Sequence[int], world: int, costs: Optional[Sequence[float]] = None) -> List[List[int]]:
    """Splits shot_ids over `world` ranks, balancing the summed cost (longest
    processing time first: shots by decreasing cost, each to the least loaded
    rank; ties by rank). Equal costs give a round robin. Every shot lands on
    exactly one rank; within a rank the caller's order is kept."""
    ids = [int(s) for s in shot_ids]
    if world < 1:
        raise ValueError("world must be >= 1")
    if costs is None:
        costs = [1.0] * len(ids)
    if len(costs) != len(ids):
        raise ValueError("one cost per shot")
    order = sorted(range(len(ids)), key=lambda k: (-float(costs[k]), k))
    load = [0.0] * world
    owner = [0] * len(ids)
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += float(costs[k])
    return [[ids[k] for k in range(len(ids)) if owner[k] == r] for r in range(world)]


def _allreduce_sum(arrays, group=None, device=None):
    """Sums float64 numpy arrays over the ranks in place (one flat buffer)."""
    import torch
    import torch.distributed as dist

    flat = np.concatenate([np.asarray(a, dtype=np.float64).ravel() for a in arrays])
    t = torch.from_numpy(flat)
    if device is not None:
        t = t.to(device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out = t.cpu().numpy()
    pos = 0
    res = []
    for a in arrays:
        n = np.asarray(a).size
        res.append(out[pos:pos + n].reshape(np.asarray(a).shape))
        pos += n
    return res


def sharded_misfit_grad(evaluate: Callable, lam, mu, den, stf, shot_ids: Sequence[int], *, rank: int, world: int,
                        costs: Optional[Sequence[float]] = None, group=None, device=None):
    """One data-parallel misfit + gradient over `shot_ids`.

    `evaluate(lam, mu, den, stf, ids)` runs this rank's shots and returns
    (misfit, g_lambda, g_mu, g_den, g_stf[len(ids)][nSteps]) -- e.g.
    `FwiContext.misfit_grad` (with obs bound) of this rank's GPU. Returns the
    same tuple over all shots, identical on every rank, with g_stf rows in
    the order of `shot_ids`."""
    ids = [int(s) for s in shot_ids]
    shards = shard_shots(ids, world, costs)
    mine = shards[rank]
    nz, nx = np.asarray(lam).shape
    nt = np.atleast_2d(stf).shape[1]
    if mine:
        J, gl, gm, gd, gs = evaluate(lam, mu, den, stf, mine)
    else:
        J, gl, gm, gd, gs = 0.0, np.zeros((nz, nx)), np.zeros((nz, nx)), np.zeros((nz, nx)), np.zeros((0, nt))
    g_stf = np.zeros((len(ids), nt))
    pos = {s: k for k, s in enumerate(ids)}
    for row, s in zip(np.asarray(gs), mine):
        g_stf[pos[s]] = row
    if world == 1:
        return float(J), np.asarray(gl), np.asarray(gm), np.asarray(gd), g_stf
    Jt, gl, gm, gd, g_stf = _allreduce_sum([np.array([J]), gl, gm, gd, g_stf], group=group, device=device)
    return float(Jt[0]), gl, gm, gd, g_stf
