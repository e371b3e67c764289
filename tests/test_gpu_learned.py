"""The learned preconditioner end to end on the GPU: training samples from
the operator (gradients + source illumination), training with the library's
CNN kernels, and what the trained network gains over the method without it
on a held-out model of the same family:

* its update points where the diagonal pseudo-Hessian preconditioner points
  (cosine > 0.9 over the mask) and, what preconditioning is for, balances
  deep against shallow updates like it: the ratio of update norms over the
  lower and upper halves of the mask is within a factor 1.5 of the exact
  preconditioner's, and at least twice as close (in log) as the plain
  gradient's;
* four descent iterations with it lower the misfit more than four plain
  gradient iterations (each with the same line search; the plain step is the
  learned step's fallback).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cos(a, b):
    return float(np.sum(a * b) / (np.linalg.norm(a) * np.linalg.norm(b)))


def test_learned_preconditioner_gains_over_plain(gpu_lib, fw, tmp_path):
    from fwiflow_gb300 import inversion, precond, synthetic

    kw = dict(nz=96, nx=256, n_shots=6, nSteps=900, smooth_cells=4.0)
    w0 = synthetic.layered_grf(10, **kw)
    para = w0.write_files(str(tmp_path))
    ctx = fw.FwiContext(para, 0)
    ids = list(range(len(w0.shots)))
    mask = inversion.inversion_mask(w0.nz_pad, w0.nx_pad, w0.nz, w0.nx, w0.nPml)

    def problem(w):
        obs = ctx.obs(*inversion.moduli_of_vp(w.vp_obs), w.stf, ids, write_files=False)
        return inversion.VpProblem(ctx, w.stf, ids, obs, w.vp, w.vp_obs, mask)

    samples = []
    for seed in range(10, 16):
        p = problem(synthetic.layered_grf(seed, **kw))
        _, g, grads, illum = p.misfit_grad(p.vp0, illumination=True)
        samples.append((precond.features(*grads, illum, mask), precond.pseudo_hessian_target(*grads, illum, mask),
                        mask))
    net = precond.CnnPreconditioner(w0.nz_pad, w0.nx_pad, seed=0)
    hist = net.train(samples, epochs=40, lr=2e-3)
    assert hist[-1] < 0.2 * hist[0]

    held = synthetic.layered_grf(99, **kw)
    p = problem(held)
    _, g, grads, illum = p.misfit_grad(p.vp0, illumination=True)
    exact = inversion.pseudo_hessian_preconditioner()(p.full(p.vp0), g, grads, illum, mask) * mask
    learned = inversion.learned_preconditioner(net)(p.full(p.vp0), g, grads, illum, mask) * mask
    c_learned, c_plain = _cos(learned, exact), _cos(g, exact)
    assert c_learned > 0.9, (c_learned, c_plain)
    rows = np.nonzero(mask.any(axis=1))[0]
    mid = (rows[0] + rows[-1] + 1) // 2

    def balance(d):
        return np.linalg.norm(d[mid:]) / np.linalg.norm(d[:mid])

    e_learned = abs(np.log(balance(learned) / balance(exact)))
    e_plain = abs(np.log(balance(g) / balance(exact)))
    assert e_learned < np.log(1.5), (e_learned, e_plain)
    assert e_learned < 0.5 * e_plain, (e_learned, e_plain)

    h_plain = inversion.descent(problem(held), 4)
    h_learned = inversion.descent(problem(held), 4, inversion.learned_preconditioner(net))
    assert h_learned.misfit[-1] < h_plain.misfit[-1], (h_learned.misfit, h_plain.misfit)
    ctx.close()
