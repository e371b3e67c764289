"""Failure paths of the library, exercised without faulting the GPU.

The reference exits the process on these conditions (utilities.h:25-33,
utilities.cu:239); this library returns a status and keeps the context
usable:
* a bounded device wait that runs out (FWIGB_ERR_TIMEOUT), made to run out
  by the test hook fwigb_test_inject_wait_timeout: the first forward sweep of
  a run waits, after its staged tiles have landed, for a barrier phase that
  nothing completes, so no copy is in flight when it gives up;
* a model that breaks the Courant bound (FWIGB_ERR_COURANT);
* group state that cannot fit the device-memory budget, and a grid whose
  buffers cannot be allocated at all (FWIGB_ERR_OOM).
After each failure the same context (or a new one) computes the correct
result: bit-identical to the result before the failure.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(tmp_path, n_shots):
    from fwiflow_gb300 import synthetic

    w = synthetic.tiny(nz=40, nx=60, nPml=10, nSteps=180, n_shots=n_shots, seed=31)
    para = w.write_files(str(tmp_path))
    return w, para


@pytest.mark.parametrize("n_shots", [1, 2])  # a lone shot replays a CUDA graph; two run eagerly
def test_wait_timeout_is_reported_and_the_context_recovers(n_shots, gpu_lib, fw, tmp_path):
    from fwiflow_gb300 import _lib

    w, para = _case(tmp_path, n_shots)
    ids = list(range(n_shots))
    ctx = fw.FwiContext(para, 0)
    obs = ctx.obs(*w.moduli(w.vp_obs), w.stf, ids, write_files=True)
    J0, gl0, gm0, gd0, gs0 = ctx.misfit_grad(*w.moduli(), w.stf, ids)
    ctx.test_inject_wait_timeout(True)
    for call in (lambda: ctx.misfit_grad(*w.moduli(), w.stf, ids), lambda: ctx.misfit(*w.moduli(), w.stf, ids),
                 lambda: ctx.obs(*w.moduli(), w.stf, ids, write_files=False)):
        with pytest.raises(_lib.FwiError) as e:
            call()
        assert e.value.status == 7 and "bounded wait" in str(e.value)
    ctx.test_inject_wait_timeout(False)
    J1, gl1, gm1, gd1, gs1 = ctx.misfit_grad(*w.moduli(), w.stf, ids)
    assert J1 == J0
    for a, b in ((gl1, gl0), (gm1, gm0), (gd1, gd0), (gs1, gs0)):
        assert np.array_equal(a, b)
    g = ctx.obs(*w.moduli(w.vp_obs), w.stf, ids, write_files=False)
    assert all(np.array_equal(a, b) for a, b in zip(g, obs))
    ctx.close()


def test_courant_violation_is_reported(gpu_lib, fw, tmp_path):
    from fwiflow_gb300 import _lib

    w, para = _case(tmp_path, 1)
    ctx = fw.FwiContext(para, 0)
    ctx.obs(*w.moduli(w.vp_obs), w.stf, [0], write_files=True)
    J0 = ctx.misfit(*w.moduli(), w.stf, [0])
    fast = 3.0 * w.vp  # Courant number ~1.3 at dx 20 m, dt 2 ms
    with pytest.raises(_lib.FwiError) as e:
        ctx.misfit(*w.moduli(fast), w.stf, [0])
    assert e.value.status == 3 and "Courant" in str(e.value)
    with pytest.raises(_lib.FwiError) as e:  # the rejected model is not kept
        ctx.run(0)
    assert e.value.status == 1 and "no model" in str(e.value)
    assert ctx.misfit(*w.moduli(), w.stf, [0]) == J0
    ctx.close()


def test_memory_budget_too_small_is_reported(gpu_lib, fw, tmp_path):
    from fwiflow_gb300 import _lib

    w, para = _case(tmp_path, 2)
    ctx = fw.FwiContext(para, 0)
    ctx.obs(*w.moduli(w.vp_obs), w.stf, [0, 1], write_files=True)
    J0, gl0, *_ = ctx.misfit_grad(*w.moduli(), w.stf, [0, 1])
    ctx.set_batching(0, 1024)  # 1 KiB: not even one shot's wavefields
    with pytest.raises(_lib.FwiError) as e:
        ctx.misfit_grad(*w.moduli(), w.stf, [0, 1])
    assert e.value.status == 5 and "do not fit" in str(e.value)
    ctx.set_batching(1, 0)  # one shot per group fits
    J1, gl1, *_ = ctx.misfit_grad(*w.moduli(), w.stf, [0, 1])
    assert ctx.last_group_count() == 2
    assert abs(J1 - J0) <= 1e-5 * abs(J0) and np.linalg.norm(gl1 - gl0) <= 1e-5 * np.linalg.norm(gl0)
    ctx.close()


def test_unallocatable_grid_is_reported(gpu_lib, fw, tmp_path):
    """A 200000 x 200000 grid needs ~1.4 TB of media arrays: the context
    cannot be created, and the failure is a status, not an exit."""
    from fwiflow_gb300 import _lib
    from fwiflow_gb300.utils import paraGen, surveyGen

    para, survey = str(tmp_path / "para.json"), str(tmp_path / "survey.json")
    paraGen(200000, 200000, 10.0, 10.0, 100, 0.001, 10.0, 32, 32, para, survey, str(tmp_path / "Data"))
    surveyGen([2], [100], [2], [100], survey)
    with pytest.raises(_lib.FwiError) as e:
        fw.FwiContext(para, 0)
    assert e.value.status == 5
    # The device is still usable.
    w, para2 = _case(tmp_path / "ok", 1)
    ctx = fw.FwiContext(para2, 0)
    g = ctx.obs(*w.moduli(w.vp_obs), w.stf, [0], write_files=False)
    assert np.isfinite(g[0]).all() and np.abs(g[0]).max() > 0
    ctx.close()
