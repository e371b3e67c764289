"""The drop-in surface, called the way the reference's callers call it.

* fwigb_cufd with calc_id 0 / 1 / 2 and exactly the arguments of the TF op's
  forward / backward / obscalc (deps/CustomOps/FWI/FwiOp.h:14-34): misfit is
  null for calc_id 1, gradients are null for 0 and 2, stf has one row per
  survey shot, shot_ids are a non-contiguous, unordered subset; observed data
  go through Data/Shot<id>.bin as in the reference (libCUFD.cu:189-200,
  514-521).
* The Python mirror of src/Core.jl:20-53 (fwi_op, fwi_op_grad, fwi_obs_op) and
  of src/FWI.jl:109-189 (compute_observation, compute_misfit).
Checked against the oracle on the same inputs: gathers and misfit 1e-4
relative L2, gradients 1e-3 (FP32).
"""
import ctypes

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

TOL_DATA = 1e-4
TOL_GRAD = 1e-3


def survey4(tmp_path, seed=21):
    """A tiny model with 4 survey shots, each with its own Ricker frequency."""
    from fwiflow_gb300 import synthetic
    from fwiflow_gb300.utils import sourceGene

    w = synthetic.tiny(nz=36, nx=72, nPml=10, nSteps=220, n_shots=4, seed=seed)
    w.stf = np.concatenate([sourceGene(f, w.nSteps, w.dt) for f in (8.0, 9.0, 10.5, 12.0)], axis=0)
    para = w.write_files(str(tmp_path))
    return w, para


def _cufd(lib, calc_id, w, para, ids, misfit=None, grads=None, stf=None):
    from fwiflow_gb300 import _lib

    lam, mu, rho = (np.ascontiguousarray(a) for a in w.moduli(w.vp_obs if calc_id == 2 else w.vp))
    stf = np.ascontiguousarray(w.stf if stf is None else stf)
    ids_a = np.ascontiguousarray(ids, dtype=np.int32)
    g = grads or (None, None, None, None)
    rc = lib.fwigb_cufd(_lib.dptr(misfit), *(_lib.dptr(a) for a in g), _lib.dptr(lam), _lib.dptr(mu),
                        _lib.dptr(rho), _lib.dptr(stf), calc_id, 0, len(ids), _lib.iptr(ids_a), para.encode())
    _lib.check(rc)


def test_cufd_as_the_tf_op_calls_it(gpu_lib, fw, orc, tmp_path):
    w, para = survey4(tmp_path)
    ids = [3, 1]
    # obscalc: calc_id 2, misfit pointer passed and ignored, Shot<id>.bin written.
    dummy = np.zeros(1)
    _cufd(gpu_lib, 2, w, para, ids, misfit=dummy)
    ref = orc.cufd(2, *w.moduli(w.vp_obs), w.stf, ids, para, write_files=False, want_gathers=True)["gathers"]
    for sid, r in zip(ids, ref):
        got = np.fromfile(tmp_path / "Data" / f"Shot{sid}.bin", dtype=np.float32)
        assert got.size == r.size
        assert rel(got, r.ravel()) < TOL_DATA, sid
    assert not (tmp_path / "Data" / "Shot0.bin").exists()  # only the call's shots are written
    # forward: calc_id 0, misfit only; observed data from the files just written.
    J = np.zeros(1)
    _cufd(gpu_lib, 0, w, para, ids, misfit=J)
    J_ref = orc.cufd(0, *w.moduli(w.vp), w.stf, ids, para)["misfit"]
    assert abs(J[0] - J_ref) <= TOL_DATA * abs(J_ref)
    o = orc.cufd(1, *w.moduli(w.vp), w.stf, ids, para)
    # backward: calc_id 1, misfit null; grad_stf has one row per survey shot,
    # of which the first len(ids) are written (local shot order).
    gl, gm, gd = (np.zeros((w.nz_pad, w.nx_pad)) for _ in range(3))
    gs = np.full(w.stf.shape, 7.0)
    _cufd(gpu_lib, 1, w, para, ids, grads=(gl, gm, gd, gs))
    for k, a in (("g_lambda", gl), ("g_mu", gm), ("g_den", gd)):
        assert rel(a, o[k]) < TOL_GRAD, (k, rel(a, o[k]))
    assert rel(gs[:len(ids)], o["g_stf"][:len(ids)]) < TOL_GRAD
    assert np.all(gs[len(ids):] == 7.0)
    # The same subset in the other order permutes g_stf rows and nothing else.
    gl2, gm2, gd2 = (np.zeros_like(gl) for _ in range(3))
    gs2 = np.zeros(w.stf.shape)
    _cufd(gpu_lib, 1, w, para, ids[::-1], grads=(gl2, gm2, gd2, gs2))
    assert rel(gl2, gl) < 1e-6 and rel(gd2, gd) < 1e-6
    assert rel(gs2[0], gs[1]) < 1e-6 and rel(gs2[1], gs[0]) < 1e-6


def test_cufd_reports_errors_instead_of_exiting(gpu_lib, fw, tmp_path):
    from fwiflow_gb300 import _lib

    w, para = survey4(tmp_path)
    J = np.zeros(1)
    with pytest.raises(_lib.FwiError) as e:
        _cufd(gpu_lib, 0, w, para, [9], misfit=J)  # no shot 9 in the survey
    assert e.value.status == 1
    with pytest.raises(_lib.FwiError) as e:
        _cufd(gpu_lib, 0, w, str(tmp_path / "missing.json"), [0], misfit=J)
    assert e.value.status == 2


def test_python_operator_surface(gpu_lib, fw, orc, tmp_path):
    """fwi_obs_op / fwi_op / fwi_op_grad (src/Core.jl:20-53)."""
    w, para = survey4(tmp_path, seed=22)
    ids = np.array([2, 0], dtype=np.int32)
    assert fw.fwi_obs_op(*w.moduli(w.vp_obs), w.stf, 0, ids, para) == 0.0
    ref = orc.cufd(2, *w.moduli(w.vp_obs), w.stf, ids, para, write_files=False, want_gathers=True)["gathers"]
    for sid, r in zip(ids, ref):
        got = np.fromfile(tmp_path / "Data" / f"Shot{sid}.bin", dtype=np.float32)
        assert rel(got, r.ravel()) < TOL_DATA
    lam, mu, rho = w.moduli(w.vp)
    o = orc.cufd(1, lam, mu, rho, w.stf, ids, para)
    J_ref = orc.cufd(0, lam, mu, rho, w.stf, ids, para)["misfit"]
    J = fw.fwi_op(lam, mu, rho, w.stf, 0, ids, para)
    assert abs(J - J_ref) <= TOL_DATA * abs(J_ref)
    gl, gm, gd, gs = fw.fwi_op_grad(lam, mu, rho, w.stf, 0, ids, para)
    assert gs.shape == w.stf.shape
    for k, a in (("g_lambda", gl), ("g_mu", gm), ("g_den", gd)):
        assert rel(a, o[k]) < TOL_GRAD, k
    assert rel(gs[:2], o["g_stf"][:2]) < TOL_GRAD and np.all(gs[2:] == 0.0)
    # The autograd wrapper scales the operator's gradients by the cotangent.
    import torch

    ctx = fw.FwiContext(para, 0)
    t = [torch.tensor(a, requires_grad=True) for a in (lam, mu, rho, w.stf)]
    y = fw.FwiOpFunction.apply(*t, ctx, ids)
    (3.0 * y).backward()
    # (a second context may pick other tile shapes: equal to rounding)
    assert abs(float(y) - J) <= 1e-6 * abs(J)
    assert rel(t[0].grad.numpy(), 3.0 * gl) < 1e-6 and rel(t[2].grad.numpy(), 3.0 * gd) < 1e-6
    ctx.close()


def test_fwi_geometry_wrappers(gpu_lib, fw, orc, tmp_path):
    """compute_observation / compute_misfit of src/FWI.jl:109-189: interior-
    sized velocities are padded, shot ids are 1-based, gathers come back as
    [shot][nSteps][nrec], and the masked gradient w.r.t. cp, cs, rho is the
    chain rule of velocity_to_moduli applied to the operator's gradient."""
    from fwiflow_gb300.utils import padding, sourceGene, velocity_to_moduli

    nz, nx = 40, 64
    zz, xx = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    cp_true = 2000.0 + 800.0 * zz / nz
    # (a strong anomaly, so the misfit is not a small difference of large values)
    cp0 = cp_true + 400.0 * np.exp(-((zz - 22) ** 2 + (xx - 30) ** 2) / 72.0)
    cs_true, cs0 = cp_true / np.sqrt(3.0), cp0 / np.sqrt(3.0)
    rho = 2200.0 * np.ones((nz, nx))
    fwi = fw.FWI(nz, nx, 20.0, 20.0, 240, 0.002, ind_src_z=[2, 2, 2], ind_src_x=[10, 32, 53],
                 ind_rec_z=[2] * nx, ind_rec_x=list(range(nx)), f0=10.0, nPml=10, workspace=str(tmp_path))
    stf = sourceGene(10.0, 240, 0.002)
    d = fw.compute_observation(fwi, cp_true, cs_true, rho, stf, shot_ids=[3, 1])
    assert d.shape == (2, 240, nx)
    lam_t, mu_t = velocity_to_moduli(*(padding(a, fwi.nPml, fwi.nPad) for a in (cp_true, cs_true, rho)))
    rho_p = padding(rho, fwi.nPml, fwi.nPad)
    stf3 = np.repeat(stf.reshape(1, -1), 3, axis=0)
    ref = orc.cufd(2, lam_t, mu_t, rho_p, stf3, [2, 0], fwi.para_path, write_files=False,
                   want_gathers=True)["gathers"]
    assert rel(d[0], ref[0].T) < TOL_DATA and rel(d[1], ref[1].T) < TOL_DATA
    # Observed data for every shot, then the masked misfit and gradient.
    fw.compute_observation(fwi, cp_true, cs_true, rho, stf)
    J, g_cp, g_cs, g_rho, _ = fw.compute_misfit(fwi, cp0, cs0, rho, stf, is_masked=True, with_grad=True)
    cp_p, cs_p = padding(cp0, fwi.nPml, fwi.nPad), padding(cs0, fwi.nPml, fwi.nPad)
    lam, mu = velocity_to_moduli(cp_p, cs_p, rho_p)
    o = orc.cufd(1, lam, mu, rho_p, stf3, [0, 1, 2], fwi.para_path)
    J_ref = orc.cufd(0, lam, mu, rho_p, stf3, [0, 1, 2], fwi.para_path)["misfit"]
    assert abs(J - J_ref) <= TOL_DATA * abs(J_ref)
    assert abs(fw.compute_misfit(fwi, cp0, cs0, rho, stf, is_masked=True) - J) <= 1e-9 * abs(J)
    exp_cp = o["g_lambda"] * 2 * cp_p * rho_p / 1e6
    exp_cs = (o["g_lambda"] * (-4 * cs_p) + o["g_mu"] * 2 * cs_p) * rho_p / 1e6
    exp_rho = o["g_den"] + o["g_lambda"] * (cp_p ** 2 - 2 * cs_p ** 2) / 1e6 + o["g_mu"] * cs_p ** 2 / 1e6
    assert rel(g_cp, exp_cp) < TOL_GRAD and rel(g_cs, exp_cs) < TOL_GRAD and rel(g_rho, exp_rho) < TOL_GRAD
    # Unmasked form: outside the mask the reference model is used and the
    # gradient is zero.
    J2, g2, _, _, _ = fw.compute_misfit(fwi, cp0, cs0, rho, stf, cp_ref=cp_true, cs_ref=cs_true, rho_ref=rho,
                                        with_grad=True)
    mask = fwi.mask()
    assert np.all(g2[mask == 0] == 0.0) and J2 < J
