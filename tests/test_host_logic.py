"""Host-side logic that needs no GPU: file formats, Ricker source, moduli,
padding, and the C ABI library's exported symbols and argument checks."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def test_default_nPad_quirk(fw):
    # src/FWI.jl:12: nPad = 32 - mod(nz + 2 nPml, 32) -> 32 when already aligned.
    assert fw.default_nPad(100, 32) == 28
    assert fw.default_nPad(512, 32) == 32
    assert fw.default_nPad(1024, 40) == 16


def test_paragen_surveygen_roundtrip(fw, tmp_path):
    para = str(tmp_path / "p.json")
    survey = str(tmp_path / "s.json")
    fw.paraGen(192, 264, 20.0, 20.0, 1000, 0.002, 8.0, 32, 28, para, survey, str(tmp_path / "Data"),
               scratch_dir_name=str(tmp_path / "scr"))
    with open(para) as f:
        lines = f.read().split("\n")
    assert len(lines) == 1  # the reference reads only the first line
    p = json.loads(lines[0])
    assert list(p)[:9] == ["nz", "nx", "dz", "dx", "nSteps", "dt", "f0", "nPoints_pml", "nPad"]
    assert isinstance(p["dt"], float) and isinstance(p["nz"], int)
    assert os.path.isdir(tmp_path / "Data") and os.path.isdir(tmp_path / "scr")
    fw.surveyGen([2, 2], [50, 150], [2] * 5, [0, 1, 2, 3, 4], survey)
    s = json.loads(open(survey).read())
    assert s["nShots"] == 2 and s["shot1"]["x_src"] == 150 and s["shot0"]["nrec"] == 5


def test_sourcegene_is_integrated_ricker(fw):
    f, n, dt = 8.0, 500, 0.002
    src = fw.sourceGene(f, n, dt)
    assert src.shape == (1, n)
    t = dt * np.arange(n) - 1.2 / f
    e = np.pi ** 2 * f ** 2
    ricker = (1 - 2 * e * t ** 2) * np.exp(-e * t ** 2)
    np.testing.assert_allclose(src[0], np.cumsum(ricker) * dt, rtol=1e-12, atol=1e-15)


def test_velocity_to_moduli(fw):
    lam, mu = fw.velocity_to_moduli(np.array([3000.0]), np.array([3000.0 / np.sqrt(3)]), np.array([2000.0]))
    assert np.allclose(mu, 3000.0 ** 2 / 3 * 2000 / 1e6)
    assert np.allclose(lam, mu)  # Vs = Vp / sqrt(3) gives lambda == mu


def test_symmetric_padding_matches_tf_semantics(fw):
    a = np.arange(6.0).reshape(2, 3)
    p = fw.padding(a, 2, 1)
    # tf.pad SYMMETRIC repeats the edge: [1,0 | 0,1,2 | 2,1]
    assert p.shape == (2 + 2 + 3, 3 + 4)
    np.testing.assert_array_equal(p[2, :], [1, 0, 0, 1, 2, 2, 1])
    np.testing.assert_array_equal(p[:, 2], [3, 0, 0, 3, 3, 0, 0])


def test_mask(fw):
    g = fw.FWIGeometry(nz=20, nx=30, dz=10.0, dx=10.0, nSteps=10, dt=0.001, nPml=5)
    m = g.mask()
    assert m.shape == (g.nz_pad, g.nx_pad)
    assert m[:5].sum() == 0 and m[5:15].sum() == 0  # PML rows and the top 10 interior rows
    assert m[15, 5] == 1 and m[15, 4] == 0


def _header_functions():
    hdr = open(os.path.join(ROOT, "include", "fwiflow_gb300.h")).read()
    return sorted(set(re.findall(r"\b(fwigb_[a-z_]+)\s*\(", hdr)))


def test_library_exports_every_header_symbol(fw):
    """The sm_103a library is cross-compiled here; load it and check that every
    function declared in include/fwiflow_gb300.h is exported (no compute)."""
    import __graft_entry__ as ge

    path = ge._build_lib()
    lib = ctypes.CDLL(path)
    names = _header_functions()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_every_header_function_has_a_python_signature(fw):
    """The ctypes table covers the whole C ABI (argument and result types of
    every function in include/fwiflow_gb300.h)."""
    from fwiflow_gb300 import _lib

    missing = [n for n in _header_functions() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_create_reports_parameter_errors_without_gpu(fw, tmp_path):
    """Parameter problems are reported as FWIGB_ERR_PARAM before any CUDA call
    (the reference asserts or exits, Parameter.cpp:35-116)."""
    import __graft_entry__ as ge

    ge._build_lib()
    from fwiflow_gb300 import _lib

    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.fwigb_create(str(tmp_path / "nope.json").encode(), 0, ctypes.byref(h))
    assert rc == 2 and b"cannot open" in lib.fwigb_last_global_error()
    bad = tmp_path / "bad.json"
    bad.write_text('{"nz": 100, "nx": 100}')
    rc = lib.fwigb_create(str(bad).encode(), 0, ctypes.byref(h))
    assert rc == 2 and b"dz" in lib.fwigb_last_global_error()
    bad.write_text('{"nz": 100, "nx":')
    rc = lib.fwigb_create(str(bad).encode(), 0, ctypes.byref(h))
    assert rc == 2
    # Survey missing a shot field.
    para = str(tmp_path / "p.json")
    survey = str(tmp_path / "s.json")
    fw.paraGen(96, 84, 20.0, 20.0, 100, 0.002, 8.0, 12, 32, para, survey, str(tmp_path / "Data"))
    with open(survey, "w") as f:
        f.write('{"nShots": 1, "shot0": {"z_src": 2, "x_src": 10, "nrec": 3, "z_rec": [2, 2]}}')
    rc = lib.fwigb_create(para.encode(), 0, ctypes.byref(h))
    assert rc == 2 and b"x_rec" in lib.fwigb_last_global_error()


def test_no_cpu_fallback_when_library_missing(fw, tmp_path, monkeypatch):
    from fwiflow_gb300 import _lib

    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load(str(tmp_path / "missing.so"))


def test_benchmark_workloads_are_stable(fw):
    """The synthetic workloads the benchmark times satisfy the CFL bound of
    the scheme (max Vp dt / dx * sqrt(2) (9/8 + 1/24) < 1) and have the sizes
    their descriptions state."""
    import numpy as np

    from fwiflow_gb300 import synthetic

    courant = np.sqrt(2.0) * (9.0 / 8.0 + 1.0 / 24.0)
    for w, shape in ((synthetic.dipping_grf(nSteps=10), (608, 1600)),
                     (synthetic.batched_uneven(n_shots=4, steps=(5, 10)), (608, 1600)),
                     (synthetic.faulted_grf(nSteps=10, shot_subset=2), (1120, 3152))):
        assert (w.nz_pad, w.nx_pad) == shape
        assert max(w.vp.max(), w.vp_obs.max()) * w.dt / w.dx * courant < 1.0
    f = synthetic.faulted_grf(nSteps=10, n_shots=128, shot_subset=None)
    assert len(f.shots) == 128 and all(len(s["x_rec"]) == 3072 for s in f.shots[:2])


def test_reference_arm_prints_the_contract_line(fw):
    """bench.py --impl reference (the oracle on the host cores) prints one JSON
    line with the reference arm's keys, on a small workload."""
    import subprocess
    import sys

    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "small_layered", "--steps", "1", "--warmup", "0", "--cpu-sample-steps", "60"],
                         capture_output=True, text=True, timeout=300, check=True).stdout
    line = json.loads(out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "Gpts/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "Gpts/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    for k in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
              "dtype", "data", "config"):
        assert k in line, k
