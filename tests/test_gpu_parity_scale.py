"""Parity with the oracle at the sizes the benchmark runs.

* The 512x1536-interior dipping model in full (608x1600 cells, 3000 steps,
  1 shot, 1536 receivers): gathers, misfit and gradients; and, on the same
  model, central finite differences against adjoint directional derivatives
  on the GPU and on the oracle, probe by probe.
* Four of the benchmark's 64 batched shots with their own aperture windows,
  record lengths (the longest of the 64 among them) and Ricker frequencies,
  run as one group.
* The full-scale geometry (1024x3072 interior, 40 CPML cells, nPad 16:
  1120x3152 cells, dx 5 m, dt 0.5 ms, 3072 receivers) on one shot with a
  600-step record.
Tolerances as in the other parity tests: gathers and misfit 1e-4 relative L2,
gradients 1e-3 (FP32). The source-wavelet gradient is the adjoint field at one
cell after thousands of FP32 steps, a much less averaged quantity than the
model gradients: its bar is max(1e-3, 4 x the case's FP32 floor), the floor
being how far the oracle built with FP32 arithmetic only lies from the
reference-precision oracle on the same case (5.6e-3 on the dipping model,
against ~1e-6 for the model gradients), computed live as in the golden tests.
The oracle runs on all host cores (tens of seconds per case).
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

TOL_DATA = 1e-4
TOL_GRAD = 1e-3


def _parity(fw, orc, w, para, ids, check_stf=True):
    lo, mo, ro = w.moduli(w.vp_obs)
    ref_obs = orc.cufd(2, lo, mo, ro, w.stf, ids, para, write_files=False, want_gathers=True)["gathers"]
    ctx = fw.FwiContext(para, 0)
    g = ctx.obs(lo, mo, ro, w.stf, ids, write_files=False)
    for k, (a, b) in enumerate(zip(g, ref_obs)):
        assert a.shape == b.shape
        assert rel(a, b) < TOL_DATA, ("gathers", k, rel(a, b))
    lam, mu, rho = w.moduli()
    o = orc.cufd(1, lam, mu, rho, w.stf, ids, para, obs=ref_obs)
    o["misfit"] = orc.cufd(0, lam, mu, rho, w.stf, ids, para, obs=ref_obs)["misfit"]  # (calc_id 1 returns none)
    J, gl, gm, gd, gs = ctx.misfit_grad(lam, mu, rho, w.stf, ids, obs=ref_obs)
    assert abs(J - o["misfit"]) <= TOL_DATA * abs(o["misfit"]), (J, o["misfit"])
    for k, a in (("g_lambda", gl), ("g_mu", gm), ("g_den", gd)):
        assert rel(a, o[k]) < TOL_GRAD, (k, rel(a, o[k]))
    if check_stf:  # (ids are 0 .. n-1 here: the oracle's row of shot i is row i)
        o32 = orc.cufd(1, lam, mu, rho, w.stf, ids, para, obs=ref_obs, precision="fp32")
        for i in range(len(ids)):
            tol = max(TOL_GRAD, 4.0 * rel(o32["g_stf"][i], o["g_stf"][i]))
            assert rel(gs[i], o["g_stf"][i]) < tol, ("g_stf", i, rel(gs[i], o["g_stf"][i]), tol)
    return ctx, ref_obs, o, (J, gl, gm, gd)


@pytest.fixture(scope="module")
def dipping(tmp_path_factory, fw, orc):
    from fwiflow_gb300 import synthetic

    w = synthetic.dipping_grf()
    para = w.write_files(str(tmp_path_factory.mktemp("dipping")))
    ctx, obs, o, gpu = _parity(fw, orc, w, para, [0])
    yield w, para, ctx, obs, o, gpu
    ctx.close()


def test_full_dipping_model_matches_oracle(gpu_lib, dipping):
    w, _, _, _, _, _ = dipping
    assert (w.nz_pad, w.nx_pad, w.nSteps, len(w.shots[0]["x_rec"])) == (608, 1600, 3000, 1536)


def test_full_dipping_model_fd_gap_is_the_oracles(gpu_lib, fw, orc, dipping):
    """The adjoint-state gradient of the reference's scheme is not the exact
    derivative of its discrete misfit; on this model the central difference
    and <g, v> differ by several percent. Per probe (one per parameter), the
    GPU's finite difference and adjoint directional derivative each match the
    oracle's, so the gap between them is the oracle's gap."""
    from fwiflow_gb300 import gradcheck

    w, para, ctx, obs, o, (J, gl, gm, gd) = dipping
    lam, mu, rho = w.moduli()
    model = {"lambda": lam, "mu": mu, "den": rho}
    mask = gradcheck.interior_mask(w.nz_pad, w.nx_pad, w.nPml, w.nPad)
    dirs = gradcheck.probe_directions(lam.shape, 3, mask, seed=2)
    probes = [(("lambda", "mu", "den")[k], v) for k, v in enumerate(dirs)]
    h_rel = 1e-2  # large enough that FP32 rounding of J stays far below J(m+hv) - J(m-hv)

    def gpu_misfit(m):
        return ctx.misfit(m["lambda"], m["mu"], m["den"], w.stf, [0], obs=obs)

    def orc_misfit(m):
        return orc.cufd(0, m["lambda"], m["mu"], m["den"], w.stf, [0], para, obs=obs)["misfit"]

    g = gradcheck.directional_check(gpu_misfit, model, {"lambda": gl, "mu": gm, "den": gd}, probes, h_rel)
    r = gradcheck.directional_check(orc_misfit, model,
                                    {"lambda": o["g_lambda"], "mu": o["g_mu"], "den": o["g_den"]}, probes, h_rel)
    for a, b in zip(g, r):
        assert abs(a["fd"] - b["fd"]) <= 2e-3 * abs(b["fd"]), (a, b)
        assert abs(a["adjoint"] - b["adjoint"]) <= 1e-3 * abs(b["adjoint"]), (a, b)
        assert abs(a["rel_err"] - b["rel_err"]) <= 2e-3 * max(1.0, b["rel_err"]), (a, b)


def test_batched_shot_subset_matches_oracle(gpu_lib, fw, orc, tmp_path):
    """Four of the 64 benchmark shots: the longest record, the widest and the
    narrowest aperture window, and shot 0, run together as one group."""
    from dataclasses import replace

    from fwiflow_gb300 import synthetic

    w64 = synthetic.batched_uneven()
    steps = [s["nSteps"] for s in w64.shots]
    widths = [s["win_x1"] - s["win_x0"] for s in w64.shots]
    pick = []
    for k in (int(np.argmax(steps)), int(np.argmax(widths)), int(np.argmin(widths)), 0):
        if k not in pick:
            pick.append(k)
    w = replace(w64, shots=[w64.shots[k] for k in pick], stf=np.ascontiguousarray(w64.stf[pick]))
    assert max(s["nSteps"] for s in w.shots) == w64.nSteps == max(steps)
    para = w.write_files(str(tmp_path))
    ids = list(range(len(pick)))
    ctx, _, _, _ = _parity(fw, orc, w, para, ids)
    assert ctx.last_group_count() == 1
    ctx.close()


def test_full_scale_geometry_one_shot_matches_oracle(gpu_lib, fw, orc, tmp_path):
    """nPml 40 and nPad 16 move the CPML, ring and fast-tile boundaries
    relative to the 32-cell cases."""
    from fwiflow_gb300 import synthetic

    w = synthetic.faulted_grf(nSteps=600, shot_subset=1)
    assert (w.nz_pad, w.nx_pad, w.nPml, w.nPad) == (1120, 3152, 40, 16)
    para = w.write_files(str(tmp_path))
    ctx, _, _, _ = _parity(fw, orc, w, para, [0])
    ctx.close()
