"""Generate the golden fixtures of tests/golden/ from the reference itself.

The reference FWI core (FwiFlow.jl deps/CustomOps/FWI/Src) is compiled for the
host CPU by oracle/Makefile.refhost (its CUDA kernels run under the emulation
shim in oracle/refhost/) and driven through its own `cufd` entry point with
parameter / survey / Data files written by the package's paraGen / surveyGen.
Run from the repository root, where the reference sources are available:

    make -C oracle -f Makefile.refhost REF=/path/to/FwiFlow.jl
    python tests/golden/make_golden.py [case ...]     (default: every case)

Cases (all seeded, see fwiflow.jl_gb300/synthetic.py):
  tiny_elastic   32x48 interior, nPml 10, 200 steps, 2 shots: gathers, misfit, gradients
  tiny_acoustic  same geometry with Vs = 0 and constant density (the mu == 0 path)
  tiny_window    1 shot with per-trace windows and weights (if_win, utilities.cu:653-705)
  tiny_filter    2 shots with the band-pass "filter" of the parameter file (bp_filter1d,
                 utilities.cu:872-923, applied at libCUFD.cu:273-277 and 301-304)
  tiny_scratch   the tiny_filter case with a "scratch_dir_name": the scratch outputs of its
                 gradient call (libCUFD.cu:493-511) per shot
  tiny_srcupd    2 shots with "if_src_update": the per-frequency source-wavelet update of the
                 residual path (source_update / source_update_adj, utilities.cu:927-1080, applied
                 at libCUFD.cu:279-299); with its scratch outputs (updated wavelet included)
  tiny_srcupd_filter  the same with the band-pass filter on as well
  small_layered  the 100x200, 1000-step, 2-shot workload: misfit, norms and a strided
                 subsample of gathers and gradients
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

fw = ge.load_package()
orc = ge.load_oracle()
from fwiflow_gb300 import synthetic  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
STRIDE = 16


def run_case(w, with_window=False, para_extra=None):
    tmp = tempfile.mkdtemp()
    if with_window:
        rng = np.random.default_rng(7)
        for s in w.shots:
            n = len(s["x_rec"])
            T = w.nSteps * w.dt
            s["win_start"] = list(rng.uniform(0.0, 0.2 * T, n))
            s["win_end"] = list(rng.uniform(0.6 * T, 1.1 * T, n))
            s["weights"] = list(rng.uniform(0.5, 1.5, n))
        para = w.write_files(tmp)
        p = json.load(open(para))
        p["if_win"] = True
        with open(para, "w") as f:
            f.write(json.dumps(p, separators=(",", ":")))
    else:
        para = w.write_files(tmp)
    if para_extra:
        p = json.load(open(para))
        p.update(para_extra)
        with open(para, "w") as f:
            f.write(json.dumps(p, separators=(",", ":")))
    moduli = (lambda v: synthetic.tiny_moduli(w, v)) if w.name == "tiny" else w.moduli
    lo, mo, ro = moduli(w.vp_obs)
    lam, mu, rho = moduli(w.vp)
    ids = list(range(len(w.shots)))
    r2 = orc.refhost_cufd(2, lo, mo, ro, w.stf, ids, para)
    r0 = orc.refhost_cufd(0, lam, mu, rho, w.stf, ids, para)
    r1 = orc.refhost_cufd(1, lam, mu, rho, w.stf, ids, para)
    return para, r2, r0, r1


def save_full(name, w, r2, r0, r1, extra=None, **meta):
    np.savez_compressed(
        os.path.join(OUT, f"{name}.npz"),
        **(extra or {}),
        gathers=np.stack(r2["gathers"]).astype(np.float32),
        misfit=np.float64(r0["misfit"]),
        g_lambda=r1["g_lambda"].astype(np.float32),
        g_mu=r1["g_mu"].astype(np.float32),
        g_den=r1["g_den"].astype(np.float32),
        g_stf=r1["g_stf"].astype(np.float32),
        meta=json.dumps(meta),
    )


FILTER = [3.0, 6.0, 14.0, 24.0]  # band-pass corners [Hz] of the tiny_filter case


def main():
    if not orc.refhost_available():
        raise SystemExit("oracle/_ref/librefhost_fwi.so missing: build it with oracle/Makefile.refhost")
    cases = set(sys.argv[1:]) or {"tiny_elastic", "tiny_acoustic", "tiny_window", "tiny_filter", "tiny_scratch",
                                  "tiny_srcupd", "tiny_srcupd_filter",
                                  "small_layered"}
    if "tiny_scratch" in cases:
        kw = dict(nz=32, nx=48, nPml=10, nSteps=200, n_shots=2, seed=3)
        w = synthetic.tiny(**kw)
        scratch = tempfile.mkdtemp()
        run_case(w, para_extra={"filter": FILTER, "scratch_dir_name": scratch})
        out = {}
        for sid in range(len(w.shots)):
            for name in ("Residual_Shot", "Syn_Shot", "CondObs_Shot", "src_updated"):
                out[f"{name}{sid}"] = np.fromfile(os.path.join(scratch, f"{name}{sid}.bin"), dtype=np.float32)
        np.savez_compressed(os.path.join(OUT, "tiny_scratch.npz"), **out,
                            meta=json.dumps({"builder": "tiny", "filter": FILTER, "kwargs": kw}))
    for name in ("tiny_srcupd", "tiny_srcupd_filter"):
        if name not in cases:
            continue
        kw = dict(nz=32, nx=48, nPml=10, nSteps=200, n_shots=2, seed=4)
        w = synthetic.tiny(**kw)
        scratch = tempfile.mkdtemp()
        extra_para = {"if_src_update": True, "scratch_dir_name": scratch}
        meta = {"builder": "tiny", "src_update": True, "kwargs": kw}
        if name.endswith("_filter"):
            extra_para["filter"] = meta["filter"] = FILTER
        _, r2, r0, r1 = run_case(w, para_extra=extra_para)
        extra = {}
        for sid in range(len(w.shots)):
            for f in ("Residual_Shot", "Syn_Shot", "CondObs_Shot", "src_updated"):
                extra[f"{f}{sid}"] = np.fromfile(os.path.join(scratch, f"{f}{sid}.bin"), dtype=np.float32)
        save_full(name, w, r2, r0, r1, extra=extra, **meta)
    if "tiny_filter" in cases:
        kw = dict(nz=32, nx=48, nPml=10, nSteps=200, n_shots=2, seed=3)
        w = synthetic.tiny(**kw)
        _, r2, r0, r1 = run_case(w, para_extra={"filter": FILTER})
        save_full("tiny_filter", w, r2, r0, r1, builder="tiny", filter=FILTER, kwargs=kw)
    if not cases & {"tiny_elastic", "tiny_acoustic", "tiny_window", "small_layered"}:
        print("golden fixtures written to", OUT)
        return
    w = synthetic.tiny(nz=32, nx=48, nPml=10, nSteps=200, n_shots=2, seed=0)
    _, r2, r0, r1 = run_case(w)
    save_full("tiny_elastic", w, r2, r0, r1, builder="tiny", kwargs=dict(nz=32, nx=48, nPml=10, nSteps=200,
                                                                            n_shots=2, seed=0))
    w = synthetic.tiny(nz=32, nx=48, nPml=10, nSteps=200, n_shots=2, seed=1, cs_zero=True)
    _, r2, r0, r1 = run_case(w)
    save_full("tiny_acoustic", w, r2, r0, r1, builder="tiny", kwargs=dict(nz=32, nx=48, nPml=10, nSteps=200,
                                                                             n_shots=2, seed=1, cs_zero=True))
    w = synthetic.tiny(nz=32, nx=48, nPml=10, nSteps=200, n_shots=1, seed=2)
    _, r2, r0, r1 = run_case(w, with_window=True)
    save_full("tiny_window", w, r2, r0, r1, builder="tiny", window_seed=7,
              kwargs=dict(nz=32, nx=48, nPml=10, nSteps=200, n_shots=1, seed=2))
    w = synthetic.small_layered()
    _, r2, r0, r1 = run_case(w)
    g = np.stack(r2["gathers"]).astype(np.float32)
    np.savez_compressed(
        os.path.join(OUT, "small_layered.npz"),
        stride=np.int64(STRIDE),
        misfit=np.float64(r0["misfit"]),
        gathers_sub=g.reshape(-1)[::STRIDE],
        gathers_norm=np.float64(np.linalg.norm(g.astype(np.float64))),
        g_lambda_sub=r1["g_lambda"].reshape(-1)[::STRIDE].astype(np.float32),
        g_mu_sub=r1["g_mu"].reshape(-1)[::STRIDE].astype(np.float32),
        g_den_sub=r1["g_den"].reshape(-1)[::STRIDE].astype(np.float32),
        g_norms=np.array([np.linalg.norm(r1[k]) for k in ("g_lambda", "g_mu", "g_den", "g_stf")]),
        g_stf=r1["g_stf"].astype(np.float32),
        meta=json.dumps({"builder": "small_layered"}),
    )
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
