"""The gradient against central finite differences of the misfit, on the GPU
and on the oracle (the reference's algorithm in double-promoted FP32).

The reference's adjoint-state gradient is not the exact derivative of its
discrete misfit (staggered-time imaging, boundary-saving reconstruction); on
this coarse model the central difference and <g, v> differ by 5-25 %. The GPU
must reproduce that gap, not close it: per probe its finite difference and
its adjoint directional derivative each match the oracle's (2e-3 and 1e-3
relative), every sign agrees, and the gap stays below 35 %."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_directional_derivatives_match_oracle(gpu_lib, fw, orc, tmp_path):
    from fwiflow_gb300 import gradcheck, synthetic

    w = synthetic.tiny(nz=40, nx=60, nPml=12, nSteps=300, n_shots=2, seed=0)
    para = w.write_files(str(tmp_path))
    ids = [0, 1]
    lo, mo, ro = w.moduli(w.vp_obs)
    orc.cufd(2, lo, mo, ro, w.stf, ids, para)
    lam, mu, rho = w.moduli()
    model = {"lambda": lam, "mu": mu, "den": rho}
    ctx = fw.FwiContext(para, 0)
    _, gl, gm, gd, _ = ctx.misfit_grad(lam, mu, rho, w.stf, ids)
    r1 = orc.cufd(1, lam, mu, rho, w.stf, ids, para)
    mask = gradcheck.interior_mask(w.nz_pad, w.nx_pad, w.nPml, w.nPad)
    dirs = gradcheck.probe_directions(lam.shape, 6, mask, seed=5)
    probes = [(("lambda", "mu", "den")[k % 3], v) for k, v in enumerate(dirs)]

    def gpu_misfit(m):
        return ctx.misfit(m["lambda"], m["mu"], m["den"], w.stf, ids)

    def orc_misfit(m):
        return orc.cufd(0, m["lambda"], m["mu"], m["den"], w.stf, ids, para)["misfit"]

    g = gradcheck.directional_check(gpu_misfit, model, {"lambda": gl, "mu": gm, "den": gd}, probes)
    o = gradcheck.directional_check(orc_misfit, model,
                                    {"lambda": r1["g_lambda"], "mu": r1["g_mu"], "den": r1["g_den"]}, probes)
    for a, b in zip(g, o):
        assert abs(a["fd"] - b["fd"]) <= 2e-3 * abs(b["fd"]), (a, b)
        assert abs(a["adjoint"] - b["adjoint"]) <= 1e-3 * abs(b["adjoint"]), (a, b)
        assert np.sign(a["fd"]) == np.sign(a["adjoint"])
        assert a["rel_err"] < 0.35
    ctx.close()
