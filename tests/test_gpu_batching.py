"""Batched shots on the sm_103a path: shots with their own aperture window and
record length, run as concurrent groups (each sweep launch covers a pack of
up to 16 shots of the group, whose slots and tensor maps travel as the
kernel parameter; a one-group call replays from a CUDA graph).

A windowed shot is defined as the reference run alone on the shot's sub-model
(padded columns win_x0 .. win_x1 + 2 nPml) for its own record length, its
gradient added into the full grid at the window's offset; the oracle runs it
exactly that way. Tolerances as in the other parity tests: gathers and misfit
1e-4 relative L2, gradients 1e-3 (FP32).
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

TOL_DATA = 1e-4
TOL_GRAD = 1e-3


def uneven_tiny(n_shots, seed, nz=40, nx=96, nPml=10, nSteps=260, min_width=24):
    """A `tiny` model whose shots each get a seed-drawn aperture window (at
    least min_width interior columns, receivers on every window column at
    depth 2), record length (nSteps/2 .. nSteps) and Ricker frequency."""
    from fwiflow_gb300 import synthetic
    from fwiflow_gb300.utils import sourceGene

    w = synthetic.tiny(nz=nz, nx=nx, nPml=nPml, nSteps=nSteps, n_shots=n_shots, seed=seed)
    rng = np.random.default_rng(seed + 100)
    rows = []
    for s in w.shots:
        wd = int(rng.integers(min_width, nx + 1))
        xs = s["x_src"]
        w0 = int(np.clip(xs - wd // 2, 0, nx - wd))
        s["win_x0"], s["win_x1"] = w0, w0 + wd - 1
        s["x_rec"] = list(range(w0, w0 + wd))
        s["z_rec"] = [2] * wd
        s["nSteps"] = int(rng.integers(nSteps // 2, nSteps + 1))
        rows.append(sourceGene(float(rng.uniform(8.0, 12.0)), nSteps, w.dt))
    w.shots[0]["nSteps"] = nSteps  # one shot spans the full record
    w.stf = np.concatenate(rows, axis=0)
    return w


def _observe(orc, w, para, ids):
    lo, mo, ro = w.moduli(w.vp_obs)
    return orc.cufd(2, lo, mo, ro, w.stf, ids, para, write_files=True, want_gathers=True)["gathers"]


def test_windows_and_record_lengths_match_oracle(gpu_lib, fw, orc, tmp_path):
    w = uneven_tiny(n_shots=5, seed=11)
    para = w.write_files(str(tmp_path))
    ids = list(range(len(w.shots)))
    ref = _observe(orc, w, para, ids)
    ctx = fw.FwiContext(para, 0)
    for sid, s in zip(ids, w.shots):
        nrec, nt, x_off, nxs = ctx.shot_info(sid)
        assert (nrec, nt, x_off, nxs) == (len(s["x_rec"]), s["nSteps"], s["win_x0"],
                                          s["win_x1"] - s["win_x0"] + 1 + 2 * w.nPml)
    got = ctx.obs(*w.moduli(w.vp_obs), w.stf, ids, write_files=False)
    for a, b, s in zip(got, ref, w.shots):
        assert a.shape == (len(s["x_rec"]), s["nSteps"])
        assert rel(a, b) < TOL_DATA
    lam, mu, rho = w.moduli()
    r1 = orc.cufd(1, lam, mu, rho, w.stf, ids, para)
    J0 = orc.cufd(0, lam, mu, rho, w.stf, ids, para)["misfit"]
    J, gl, gm, gd, gs = ctx.misfit_grad(lam, mu, rho, w.stf, ids)
    assert abs(J - J0) <= TOL_DATA * abs(J0)
    for k, a in (("g_lambda", gl), ("g_mu", gm), ("g_den", gd), ("g_stf", gs)):
        assert rel(a, r1[k]) < TOL_GRAD, (k, rel(a, r1[k]))
    # Outside every shot's sub-grid the gradient is exactly zero.
    covered = np.zeros(w.nx_pad, dtype=bool)
    for s in w.shots:
        covered[s["win_x0"]: s["win_x1"] + 1 + 2 * w.nPml] = True
    assert not np.any(gl[:, ~covered])
    ctx.close()


def test_group_size_changes_no_bit(gpu_lib, fw, orc, tmp_path):
    """20 shots as one group (two parameter packs), as groups of 7 and as
    groups of 2: misfit, gradients and gathers are bit-identical (per-shot
    gradients are reduced in the same fixed order), and match the oracle.
    One shot at a time runs the lone-shot instantiation of the sweeps, which
    the compiler may contract differently (fused multiply-adds): equal to
    rounding (1e-6)."""
    w = uneven_tiny(n_shots=20, seed=12, nx=80, nSteps=200)
    para = w.write_files(str(tmp_path))
    ids = list(range(len(w.shots)))
    _observe(orc, w, para, ids)
    lam, mu, rho = w.moduli()
    ctx = fw.FwiContext(para, 0)
    results, gathers = [], []
    for cap, n_groups in ((0, 1), (7, 3), (2, 10), (1, 20)):
        ctx.set_batching(max_shots=cap)
        results.append(ctx.misfit_grad(lam, mu, rho, w.stf, ids))
        assert ctx.last_group_count() == n_groups
        gathers.append(ctx.obs(*w.moduli(w.vp_obs), w.stf, ids, write_files=False))
    for r in results[1:3]:
        assert r[0] == results[0][0]
        for x, y in zip(r[1:], results[0][1:]):
            assert np.array_equal(x, y)
    for g in gathers[1:3]:
        for x, y in zip(g, gathers[0]):
            assert np.array_equal(x, y)
    lone = results[3]
    assert abs(lone[0] - results[0][0]) <= 1e-6 * abs(results[0][0])
    for x, y in zip(lone[1:], results[0][1:]):
        assert rel(x, y) < 1e-6
    for x, y in zip(gathers[3], gathers[0]):
        assert rel(x, y) < 1e-6
    r1 = orc.cufd(1, lam, mu, rho, w.stf, ids, para)
    J0 = orc.cufd(0, lam, mu, rho, w.stf, ids, para)["misfit"]
    assert abs(results[0][0] - J0) <= TOL_DATA * abs(J0)
    for k, a in zip(("g_lambda", "g_mu", "g_den", "g_stf"), results[0][1:]):
        assert rel(a, r1[k]) < TOL_GRAD, (k, rel(a, r1[k]))
    ctx.close()


def test_memory_budget_splits_groups(gpu_lib, fw, tmp_path):
    """A device-memory budget for at least two (and fewer than six) shots'
    state splits six shots into several groups with the same results (to
    rounding: a group left with one shot runs the lone-shot sweeps)."""
    w = uneven_tiny(n_shots=6, seed=13, nSteps=160)
    para = w.write_files(str(tmp_path))
    ids = list(range(len(w.shots)))
    ctx = fw.FwiContext(para, 0)
    g_obs = ctx.obs(*w.moduli(w.vp_obs), w.stf, ids, write_files=False)
    lam, mu, rho = w.moduli()
    a = ctx.misfit_grad(lam, mu, rho, w.stf, ids, obs=g_obs)
    assert ctx.last_group_count() == 1
    # Per-shot state of the widest window: 18 fields + 3 gradients on its
    # sub-grid, plus its boundary store over its record.
    ldz = -(-(w.nz_pad) // 32) * 32
    nxs = max(ctx.shot_info(s)[3] for s in ids)
    per_fields = (18 + 3) * ldz * nxs * 4
    ctx.set_batching(max_shots=0, mem_budget_bytes=2 * per_fields + 2 * 20 * (w.nz_pad + nxs) * 5 * 4 * w.nSteps)
    b = ctx.misfit_grad(lam, mu, rho, w.stf, ids, obs=g_obs)
    assert ctx.last_group_count() > 1
    assert abs(a[0] - b[0]) <= 1e-6 * abs(a[0])
    for x, y in zip(a[1:], b[1:]):
        assert rel(x, y) < 1e-6
    ctx.close()


def test_illumination_matches_oracle(gpu_lib, fw, orc, tmp_path):
    """Source illumination sum_t (vz^2 + vx^2) over all shots, windowed and
    uneven ones included, against the oracle (1e-4 relative L2); it is
    accumulated in any run (here a misfit-only one) and only when enabled."""
    w = uneven_tiny(n_shots=4, seed=14, nSteps=200)
    para = w.write_files(str(tmp_path))
    ids = list(range(len(w.shots)))
    _observe(orc, w, para, ids)
    lam, mu, rho = w.moduli()
    ref = orc.cufd(0, lam, mu, rho, w.stf, ids, para, want_illum=True)["illum"]
    ctx = fw.FwiContext(para, 0)
    ctx.set_illumination(True)
    J = ctx.misfit(lam, mu, rho, w.stf, ids)
    assert rel(ctx.illumination(), ref) < TOL_DATA
    ctx.set_batching(max_shots=1)
    ctx.misfit_grad(lam, mu, rho, w.stf, ids)
    assert rel(ctx.illumination(), ref) < TOL_DATA
    ctx.set_illumination(False)
    assert ctx.misfit(lam, mu, rho, w.stf, ids) == pytest.approx(J, rel=1e-6)
    with pytest.raises(fw.FwiError):
        ctx.illumination()
    ctx.close()


def test_batched_graph_replay_is_identical(gpu_lib, fw, orc, tmp_path):
    """A batched group (its shots' slots and tensor maps in the parameter pack
    of each sweep launch) replays its whole call from a CUDA graph: same bits as eager launches, across a model change
    (replay) and a different shot set (re-recorded); and the replayed call
    matches the oracle."""
    w = uneven_tiny(n_shots=6, seed=17)
    para = w.write_files(str(tmp_path))
    ids = list(range(len(w.shots)))
    ref = _observe(orc, w, para, ids)
    ctx = fw.FwiContext(para, 0)
    lam, mu, rho = w.moduli()
    eager, graph = [], []
    for enable, out in ((False, eager), (True, graph)):
        ctx.set_graphs(enable)
        for scale in (1.0, 1.01, 1.0):
            out.append(ctx.misfit_grad(lam * scale, mu, rho, w.stf, ids, obs=ref))
        out.append(ctx.misfit_grad(lam, mu, rho, w.stf, ids[:4], obs=ref[:4]))
        assert ctx.last_group_count() == 1
    for a, b in zip(eager, graph):
        assert a[0] == b[0]
        for x, y in zip(a[1:], b[1:]):
            assert np.array_equal(x, y)
    assert graph[0][0] == graph[2][0] and graph[0][0] != graph[1][0]
    J_ref = orc.cufd(0, lam, mu, rho, w.stf, ids, para, obs=ref)["misfit"]
    o = orc.cufd(1, lam, mu, rho, w.stf, ids, para, obs=ref)
    assert abs(graph[2][0] - J_ref) <= TOL_DATA * abs(J_ref)
    for k, a in (("g_lambda", graph[2][1]), ("g_mu", graph[2][2]), ("g_den", graph[2][3])):
        assert rel(a, o[k]) < TOL_GRAD, k
    ctx.close()
