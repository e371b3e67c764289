import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as ge  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a library")


@pytest.fixture(scope="session")
def fw():
    return ge.load_package()


@pytest.fixture(scope="session")
def orc():
    import subprocess

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return ge.load_oracle()


@pytest.fixture(scope="session")
def gpu_lib(fw):
    """Builds (if needed) and loads the CUDA library; GPU tests only."""
    ge._build_lib()
    from fwiflow_gb300 import _lib

    return _lib.load()


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(str(d["meta"]))
    return d, meta


def golden_workload(name, tmp_path):
    """Rebuild a golden case's workload and write its files into tmp_path."""
    from fwiflow_gb300 import synthetic

    d, meta = load_golden(name)
    if meta["builder"] == "tiny":
        w = synthetic.tiny(**meta["kwargs"])
    else:
        w = getattr(synthetic, meta["builder"])()
    if "window_seed" in meta:
        rng = np.random.default_rng(meta["window_seed"])
        for s in w.shots:
            n = len(s["x_rec"])
            T = w.nSteps * w.dt
            s["win_start"] = list(rng.uniform(0.0, 0.2 * T, n))
            s["win_end"] = list(rng.uniform(0.6 * T, 1.1 * T, n))
            s["weights"] = list(rng.uniform(0.5, 1.5, n))
    para = w.write_files(str(tmp_path))
    if "window_seed" in meta or "filter" in meta or meta.get("src_update"):
        p = json.load(open(para))
        if "window_seed" in meta:
            p["if_win"] = True
        if "filter" in meta:
            p["filter"] = meta["filter"]
        if meta.get("src_update"):
            p["if_src_update"] = True
        with open(para, "w") as f:
            f.write(json.dumps(p, separators=(",", ":")))
    if meta["builder"] == "tiny":
        moduli = lambda v: synthetic.tiny_moduli(w, v)  # noqa: E731
    else:
        moduli = w.moduli
    return d, w, para, moduli


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
