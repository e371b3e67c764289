"""Shot sharding over ranks (fwiflow_gb300.shots): the assignment, and a
world-size-2 gloo run on CPU whose per-rank evaluation is the oracle on the
rank's shots. The summed result must equal one oracle call over all shots:
misfit and gradients to 1e-6 relative (the reference, and so the oracle,
accumulates both over the shots of a call in FP32, so splitting the shots
moves them by FP32 rounding), g_stf rows exactly (they are disjoint)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import ROOT, rel


def test_shard_covers_every_shot_once(fw):
    from fwiflow_gb300.shots import shard_shots

    ids = [5, 1, 7, 3, 2, 9, 0]
    costs = [3.0, 1.0, 4.0, 1.0, 5.0, 9.0, 2.0]
    for world in (1, 2, 3, 7, 9):
        sh = shard_shots(ids, world, costs)
        assert len(sh) == world
        flat = sorted(s for r in sh for s in r)
        assert flat == sorted(ids)
        for r in sh:  # caller's order kept within a rank
            assert r == [s for s in ids if s in r]
    # Longest processing time first balances 9 / (5 + 4) / ...
    sh = shard_shots(ids, 2, costs)
    loads = [sum(c for s, c in zip(ids, costs) if s in r) for r in sh]
    assert abs(loads[0] - loads[1]) <= max(costs)
    assert shard_shots([0, 1, 2, 3], 2) == [[0, 2], [1, 3]]  # equal costs: round robin
    with pytest.raises(ValueError):
        shard_shots([0, 1], 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, para, out_dir):
    import sys

    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import __graft_entry__ as ge

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ge.load_package()
    orc = ge.load_oracle()
    from fwiflow_gb300 import synthetic
    from fwiflow_gb300.shots import sharded_misfit_grad

    w = synthetic.tiny(nz=24, nx=40, nPml=8, nSteps=120, n_shots=5, seed=7)
    lam, mu, rho = w.moduli()

    def evaluate(lam, mu, den, stf, ids):
        r1 = orc.cufd(1, lam, mu, den, stf, ids, para)
        J = orc.cufd(0, lam, mu, den, stf, ids, para)["misfit"]
        # The reference fills g_stf rows by local shot order (libCUFD.cu:455).
        return J, r1["g_lambda"], r1["g_mu"], r1["g_den"], r1["g_stf"][:len(ids)]

    ids = [4, 0, 3, 1, 2]
    costs = [1.0, 2.0, 3.0, 4.0, 5.0]
    res = sharded_misfit_grad(evaluate, lam, mu, rho, w.stf, ids, rank=rank, world=world, costs=costs)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), J=res[0], gl=res[1], gm=res[2], gd=res[3], gs=res[4])
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_sum_matches_one_call(fw, orc, tmp_path):
    from fwiflow_gb300 import synthetic

    w = synthetic.tiny(nz=24, nx=40, nPml=8, nSteps=120, n_shots=5, seed=7)
    para = w.write_files(str(tmp_path))
    lo, mo, ro = w.moduli(w.vp_obs)
    orc.cufd(2, lo, mo, ro, w.stf, list(range(5)), para)
    mp.start_processes(_rank_main, args=(2, _free_port(), para, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    r = [np.load(os.path.join(tmp_path, f"rank{k}.npz")) for k in range(2)]
    for k in ("J", "gl", "gm", "gd", "gs"):
        assert np.array_equal(r[0][k], r[1][k]), k  # every rank holds the same result
    ids = [4, 0, 3, 1, 2]
    lam, mu, rho = w.moduli()
    one = orc.cufd(1, lam, mu, rho, w.stf, ids, para)
    J = orc.cufd(0, lam, mu, rho, w.stf, ids, para)["misfit"]
    assert abs(float(r[0]["J"]) - J) <= 1e-6 * abs(J)
    for k, name in (("gl", "g_lambda"), ("gm", "g_mu"), ("gd", "g_den")):
        assert rel(r[0][k], one[name]) < 1e-6, k
    assert np.array_equal(r[0]["gs"], one["g_stf"][:len(ids)])
