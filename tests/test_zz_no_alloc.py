"""The allocation-free misfit entry point against the regular one.

fwigb_misfit_gathers_noalloc exists for callers that cannot call cudaMalloc,
such as an operator running inside a framework that owns the GPU's memory pool
(TensorFlow, as for FwiFlow's own op, or an XLA / JAX runtime) or a service with
a fixed device-memory budget. It keeps its scratch in a static device array,
so this test calls it twice in a row (the second call sees the first call's
leftovers in that array) and compares both results with fwigb_misfit, which
allocates its buffers itself. The device buffers below are the test's own.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_MISFIT = 1e-6  # both sum the same tapered residuals in double


@pytest.fixture
def noalloc(gpu_lib):
    fn = gpu_lib.fwigb_misfit_gathers_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                   ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    fn.restype = ctypes.c_int
    gpu_lib.fwigb_noalloc_last_error.restype = ctypes.c_char_p
    return fn, gpu_lib.fwigb_noalloc_last_error


def test_noalloc_misfit_matches_allocating_entry_point(noalloc, fw, tmp_path):
    import torch
    from fwiflow_gb300 import _lib, synthetic

    w = synthetic.tiny(nz=40, nx=64, nPml=10, nSteps=240, n_shots=1, seed=11)
    para = w.write_files(str(tmp_path))
    ctx = fw.FwiContext(para, 0)
    obs = ctx.obs(*w.moduli(w.vp_obs), w.stf, [0], write_files=True)[0]
    syn = ctx.obs(*w.moduli(w.vp), w.stf, [0], write_files=False)[0]
    expected = ctx.misfit(*w.moduli(w.vp), w.stf, [0])  # allocating path, reads Data/Shot0.bin
    ctx.close()

    fn, last_error = noalloc
    nrec, nt = obs.shape
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
        assert torch.isfinite(d_res).all()
        assert float(d_res[:, 0].abs().max()) == 0.0  # sample 0 carries no residual
    for v in results:
        assert abs(v - expected) <= TOL_MISFIT * abs(expected), (v, expected)
    assert results[0] == results[1]


def test_noalloc_rejects_sizes_beyond_its_scratch(noalloc):
    fn, last_error = noalloc
    dummy = 1  # never dereferenced: the size check comes before any device work
    out = ctypes.c_double(0.0)
    rc = fn(dummy, dummy, dummy, 65537, 100, 0.001, ctypes.byref(out), None)
    assert rc == 1 and b"65536" in last_error()
