"""The allocation-free misfit entry point against the regular one.

fwigb_misfit_gathers_noalloc exists for callers that cannot call cudaMalloc,
such as an operator running inside a framework that owns the GPU's memory pool
(TensorFlow, as for FwiFlow's own op, or an XLA / JAX runtime) or a service with
a fixed device-memory budget. It keeps its scratch in a static device array,
so this test calls it twice in a row (the second call sees the first call's
leftovers in that array) and compares both results with the allocating path
(fwigb_misfit_grad with a scratch directory, which writes the tapered synthetic
and the adjoint source it injects): the misfit, the adjoint source d_res and
the tapered synthetic d_syn. The device buffers below are the test's own.
"""
import ctypes
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_MISFIT = 1e-6  # both sum the same tapered residuals in double
TOL_TRACES = 1e-6  # relative L2 of d_res / d_syn: the same float products (taper weights may differ by an ulp)


@pytest.fixture
def noalloc(gpu_lib):
    fn = gpu_lib.fwigb_misfit_gathers_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                   ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    fn.restype = ctypes.c_int
    gpu_lib.fwigb_noalloc_last_error.restype = ctypes.c_char_p
    return fn, gpu_lib.fwigb_noalloc_last_error


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_noalloc_misfit_matches_allocating_entry_point(noalloc, fw, tmp_path):
    import torch
    from fwiflow_gb300 import synthetic

    w = synthetic.tiny(nz=40, nx=64, nPml=10, nSteps=240, n_shots=1, seed=11)
    para = w.write_files(str(tmp_path))
    scratch = tmp_path / "scratch"
    scratch.mkdir()
    p = json.load(open(para))
    p["scratch_dir_name"] = str(scratch)
    with open(para, "w") as f:
        f.write(json.dumps(p, separators=(",", ":")))
    ctx = fw.FwiContext(para, 0)
    obs = ctx.obs(*w.moduli(w.vp_obs), w.stf, [0], write_files=True)[0]
    syn = ctx.obs(*w.moduli(w.vp), w.stf, [0], write_files=False)[0]
    expected = ctx.misfit(*w.moduli(w.vp), w.stf, [0])  # allocating path, reads Data/Shot0.bin
    J_grad = ctx.misfit_grad(*w.moduli(w.vp), w.stf, [0])[0]  # writes the scratch files
    ctx.close()
    assert abs(J_grad - expected) <= TOL_MISFIT * abs(expected)
    nrec, nt = obs.shape
    res_ref = np.fromfile(scratch / "Residual_Shot0.bin", dtype=np.float32).reshape(nrec, nt)
    syn_ref = np.fromfile(scratch / "Syn_Shot0.bin", dtype=np.float32).reshape(nrec, nt)

    fn, last_error = noalloc
    d_obs = torch.from_numpy(np.ascontiguousarray(obs)).cuda()
    results = []
    for _ in range(2):
        d_syn = torch.from_numpy(np.ascontiguousarray(syn)).cuda()
        d_res = torch.full((nrec, nt), float("nan"), device="cuda")
        torch.cuda.synchronize()
        out = ctypes.c_double(-1.0)
        rc = fn(d_obs.data_ptr(), d_syn.data_ptr(), d_res.data_ptr(), nrec, nt, w.dt, ctypes.byref(out), None)
        assert rc == 0, last_error()
        results.append(out.value)
        res = d_res.cpu().numpy()
        assert np.isfinite(res).all()
        assert float(np.abs(res[:, 0]).max()) == 0.0  # sample 0 carries no residual
        assert _rel(res, res_ref) < TOL_TRACES, _rel(res, res_ref)
        assert _rel(d_syn.cpu().numpy(), syn_ref) < TOL_TRACES
    for v in results:
        assert abs(v - expected) <= TOL_MISFIT * abs(expected), (v, expected)
    assert results[0] == results[1]


def test_noalloc_rejects_sizes_beyond_its_scratch(noalloc):
    fn, last_error = noalloc
    dummy = 1  # never dereferenced: the size checks come before any device work
    out = ctypes.c_double(0.0)
    rc = fn(dummy, dummy, dummy, 65537, 100, 0.001, ctypes.byref(out), None)
    assert rc == 1 and b"65536" in last_error()
    rc = fn(dummy, dummy, dummy, 10, 100, 1e-45, ctypes.byref(out), None)  # 100 * dt * 0.005 underflows to 0
    assert rc == 1 and b"taper" in last_error()
