"""The optimisers of fwiflow_gb300.inversion on a CPU stand-in for VpProblem:
an ill-conditioned separable quadratic misfit (no GPU). L-BFGS whose initial
inverse Hessian is the exact diagonal gain reaches a lower misfit in the same
iterations than plain L-BFGS, and plain L-BFGS than steepest descent."""
import numpy as np


class QuadraticProblem:
    """J(v) = 0.5 sum_c h_c (v_c - t_c)^2 over a 'mask'; the same interface
    as inversion.VpProblem (misfit, misfit_grad, full, model_error)."""

    def __init__(self, n=400, seed=0):
        rng = np.random.default_rng(seed)
        self.h = np.exp(rng.uniform(np.log(1e-3), 0.0, n))  # curvature spread over 3 decades
        self.t = 2000.0 + 100.0 * rng.standard_normal(n)
        self.vp0 = self.t + 50.0 * rng.standard_normal(n)
        self.vp_true = self.t
        self.mask = np.ones(n)
        self.vmin, self.vmax = 0.0, 1e9
        self.evals = 0

    def full(self, v):
        return np.asarray(v, dtype=np.float64)

    def model_error(self, v):
        return float(np.linalg.norm(v - self.t) / np.linalg.norm(self.t))

    def misfit(self, v):
        self.evals += 1
        return float(0.5 * np.sum(self.h * (v - self.t) ** 2))

    def misfit_grad(self, v, illumination=False):
        self.evals += 1
        g = self.h * (v - self.t)
        return float(0.5 * np.sum(self.h * (v - self.t) ** 2)), g, (g, g, g), (self.h if illumination else None)


def test_preconditioned_lbfgs_converges_faster(fw):
    from fwiflow_gb300 import inversion

    iters = 12
    sd = inversion.descent(QuadraticProblem(), iters, step_max=200.0)
    plain = inversion.lbfgs(QuadraticProblem(), iters, step_max=200.0)
    exact = inversion.lbfgs(QuadraticProblem(), iters, step_max=200.0,
                            gain=lambda v, g, grads, illum, mask: 1.0 / illum)
    assert plain.misfit[-1] < sd.misfit[-1], (plain.misfit[-1], sd.misfit[-1])
    assert exact.misfit[-1] < 1e-3 * plain.misfit[-1], (exact.misfit[-1], plain.misfit[-1])
    assert exact.model_error[-1] < plain.model_error[-1]
