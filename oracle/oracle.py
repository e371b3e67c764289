"""Python driver of the CPU oracle and of the host build of the reference.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py (CPU baseline / reference arm). The product package never imports it.

* `cufd(...)` runs oracle/fwi_oracle.cpp (oracle/_build/liboracle_fwi.so), after
  restating the reference's parameter and survey parsing (Parameter.cpp:16-178,
  Src_Rec.cu:19-245) and its file I/O of observed data (libCUFD.cu:189-192,
  514-521).
* Shots of this package's survey extension (per-shot record length "nSteps"
  and aperture window "win_x0" .. "win_x1" of interior columns) are defined
  as the reference run alone on the shot's sub-model (padded columns win_x0 ..
  win_x1 + 2 nPml) for its own record length; `cufd` runs each such shot that
  way and adds its gradient into the full grid at its column offset.
* `refhost_cufd(...)` runs the reference's own sources compiled for the host
  (oracle/_ref/librefhost_fwi.so, built by oracle/Makefile.refhost); it exists
  only where the reference sources were available at build time.
"""
from __future__ import annotations

import ctypes
import json
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "liboracle_fwi.so")
# Same algorithm built with FP32 arithmetic only (-DORACLE_FP32): its distance
# from the reference is the rounding floor of FP32 for a given case.
ORACLE_FP32_LIB = os.path.join(HERE, "_build", "liboracle_fwi_fp32.so")
REFHOST_LIB = os.path.join(HERE, "_ref", "librefhost_fwi.so")


class _Para(ctypes.Structure):
    _fields_ = [("nz", ctypes.c_int), ("nx", ctypes.c_int), ("nSteps", ctypes.c_int), ("nPml", ctypes.c_int),
                ("nPad", ctypes.c_int), ("dz", ctypes.c_float), ("dx", ctypes.c_float), ("dt", ctypes.c_float),
                ("f0", ctypes.c_float), ("if_win", ctypes.c_int), ("if_filter", ctypes.c_int),
                ("filter", ctypes.c_float * 4), ("if_src_update", ctypes.c_int)]


class _Shot(ctypes.Structure):
    _fields_ = [("z_src", ctypes.c_int), ("x_src", ctypes.c_int), ("nrec", ctypes.c_int),
                ("z_rec", ctypes.POINTER(ctypes.c_int)), ("x_rec", ctypes.POINTER(ctypes.c_int)),
                ("win_start", ctypes.POINTER(ctypes.c_float)), ("win_end", ctypes.POINTER(ctypes.c_float)),
                ("weights", ctypes.POINTER(ctypes.c_float))]


_oracles = {}
_refhost = None


def _load_oracle(precision: str = "reference"):
    if precision not in _oracles:
        path = ORACLE_LIB if precision == "reference" else ORACLE_FP32_LIB
        if not os.path.exists(path):
            raise RuntimeError(f"oracle library not built: {path} (run make -C oracle)")
        lib = ctypes.CDLL(path)
        lib.oracle_cufd.restype = ctypes.c_int
        lib.oracle_cufd_full.restype = ctypes.c_int
        _oracles[precision] = lib
    return _oracles[precision]


def refhost_available() -> bool:
    return os.path.exists(REFHOST_LIB)


def _load_refhost():
    global _refhost
    if _refhost is None:
        lib = ctypes.CDLL(REFHOST_LIB)
        lib.refhost_cufd.restype = ctypes.c_int
        _refhost = lib
    return _refhost


def read_first_line_json(path: str) -> dict:
    """The reference parses only the first line of its JSON files (Parameter.cpp:28)."""
    with open(path) as f:
        return json.loads(f.readline())


def load_para(path: str) -> dict:
    """Parameter.cpp:16-178: required keys and optional switches."""
    j = read_first_line_json(path)
    for k in ("nz", "nx", "dz", "dx", "nSteps", "nPoints_pml", "nPad", "dt", "f0", "survey_fname", "data_dir_name"):
        if k not in j:
            raise KeyError(f"parameter file lacks {k}")
    return {
        "nz": int(j["nz"]), "nx": int(j["nx"]), "dz": float(j["dz"]), "dx": float(j["dx"]),
        "nSteps": int(j["nSteps"]), "nPml": int(j["nPoints_pml"]), "nPad": int(j["nPad"]),
        "dt": float(j["dt"]), "f0": float(j["f0"]), "survey_fname": j["survey_fname"],
        "data_dir_name": j["data_dir_name"], "scratch_dir_name": j.get("scratch_dir_name"),
        "if_win": bool(j.get("if_win", False)), "filter": j.get("filter"),
        "if_src_update": bool(j.get("if_src_update", False)),
    }


def load_shots(survey_fname: str, shot_ids: Sequence[int], if_win: bool) -> list:
    """Src_Rec.cu:80-200: per shot source / receiver indices (0-based interior)."""
    s = read_first_line_json(survey_fname)
    out = []
    for sid in shot_ids:
        d = s[f"shot{int(sid)}"]
        shot = {"z_src": int(d["z_src"]), "x_src": int(d["x_src"]), "nrec": int(d["nrec"]),
                "z_rec": np.asarray(d["z_rec"], dtype=np.int32)[: int(d["nrec"])],
                "x_rec": np.asarray(d["x_rec"], dtype=np.int32)[: int(d["nrec"])]}
        if "nSteps" in d:
            shot["nSteps"] = int(d["nSteps"])
        if "win_x0" in d:
            shot["win_x0"], shot["win_x1"] = int(d["win_x0"]), int(d["win_x1"])
        if if_win:
            shot["win_start"] = np.asarray(d["win_start"], dtype=np.float32)
            shot["win_end"] = np.asarray(d["win_end"], dtype=np.float32)
            shot["weights"] = np.asarray(d["weights"], dtype=np.float32)
        out.append(shot)
    return out


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _run_group(p: dict, shots: list, ids: Sequence[int], nz: int, nx: int, nt: int, lam, mu, den, stf, calc_id: int,
               obs, nthreads: int, precision: str, illum: Optional[np.ndarray] = None):
    """One oracle_cufd call over shots sharing one grid and record length."""
    fl = p.get("filter")
    para = _Para(nz, nx, nt, p["nPml"], p["nPad"], p["dz"], p["dx"], p["dt"], p["f0"], int(p["if_win"]),
                 int(fl is not None), (ctypes.c_float * 4)(*(fl if fl is not None else [0.0] * 4)),
                 int(p.get("if_src_update", False)))
    keep = []
    carr = (_Shot * len(shots))()
    for i, s in enumerate(shots):
        carr[i].z_src, carr[i].x_src, carr[i].nrec = s["z_src"], s["x_src"], s["nrec"]
        zr = np.ascontiguousarray(s["z_rec"], dtype=np.int32)
        xr = np.ascontiguousarray(s["x_rec"], dtype=np.int32)
        keep += [zr, xr]
        carr[i].z_rec, carr[i].x_rec = _iptr(zr), _iptr(xr)
        if p["if_win"]:
            ws, we, wt = (np.ascontiguousarray(s[k], dtype=np.float32) for k in ("win_start", "win_end", "weights"))
            keep += [ws, we, wt]
            carr[i].win_start, carr[i].win_end, carr[i].weights = _fptr(ws), _fptr(we), _fptr(wt)
    n = len(shots)
    obs_ptrs = (ctypes.POINTER(ctypes.c_float) * max(n, 1))()
    if calc_id in (0, 1):
        obs = [np.ascontiguousarray(o, dtype=np.float32).reshape(-1) for o in obs]
        for i, o in enumerate(obs):
            if o.size != shots[i]["nrec"] * nt:
                raise ValueError("observed data of wrong size")
            obs_ptrs[i] = _fptr(o)
    syn = [np.zeros(s["nrec"] * nt, dtype=np.float32) for s in shots]
    syn_ptrs = (ctypes.POINTER(ctypes.c_float) * max(n, 1))()
    for i, a in enumerate(syn):
        syn_ptrs[i] = _fptr(a)
    res = [np.zeros(s["nrec"] * nt, dtype=np.float32) for s in shots]
    res_ptrs = (ctypes.POINTER(ctypes.c_float) * max(n, 1))()
    for i, a in enumerate(res):
        res_ptrs[i] = _fptr(a)
    src = [np.zeros(nt, dtype=np.float32) for _ in shots]
    src_ptrs = (ctypes.POINTER(ctypes.c_float) * max(n, 1))()
    for i, a in enumerate(src):
        src_ptrs[i] = _fptr(a)
    misfit = ctypes.c_double(0.0)
    g_lam = np.zeros((nz, nx))
    g_mu = np.zeros((nz, nx))
    g_den = np.zeros((nz, nx))
    g_stf = np.zeros_like(stf)
    cids = np.asarray(ids, dtype=np.int32)
    lib = _load_oracle(precision)
    args = (ctypes.byref(para), carr, n, _iptr(cids), _dptr(lam), _dptr(mu), _dptr(den), _dptr(stf), int(calc_id),
            obs_ptrs, syn_ptrs, res_ptrs, ctypes.byref(misfit), _dptr(g_lam), _dptr(g_mu), _dptr(g_den), _dptr(g_stf),
            int(nthreads))
    rc = lib.oracle_cufd_full(*args, None if illum is None else _dptr(illum), src_ptrs)
    if rc != 0:
        raise RuntimeError(f"oracle_cufd failed with status {rc}")
    return (misfit.value, g_lam, g_mu, g_den, g_stf, [a.reshape(s["nrec"], nt) for a, s in zip(syn, shots)],
            (src, [a.reshape(s["nrec"], nt) for a, s in zip(res, shots)]))


def cufd(calc_id: int, lam, mu, den, stf, shot_ids, para_fname: str, *, nthreads: int = 0,
         obs: Optional[Sequence[np.ndarray]] = None, write_files: bool = True, want_gathers: bool = False,
         precision: str = "reference", want_illum: bool = False) -> dict:
    """Oracle run of one `cufd` call (libCUFD.cu:34-580).

    lam, mu [MPa] and den are row-major float64 [nz][nx]; stf is
    [nShotsTotal][nSteps]. shot_ids are 0-based. For calc_id 0/1 observed data
    are read from `data_dir_name/Shot<id>.bin` unless `obs` is given; for
    calc_id 2 the gathers are written there when `write_files`.
    Returns misfit, g_lambda, g_mu, g_den, g_stf and (optionally) gathers
    (shot k's gather is [nrec][its record length]; for calc_id 0/1 the
    processed synthetic, with "wavelets": each shot's source wavelet as the
    residual path leaves it, updated under if_src_update, and "residuals":
    the adjoint sources).
    precision "fp32" runs the FP32-only build (no double promotions).
    want_illum adds "illum": the source illumination (sum over shots and
    forward steps of vz^2 + vx^2 after each velocity update), [nz][nx].
    """
    p = load_para(para_fname)
    shot_ids = [int(v) for v in np.asarray(shot_ids).ravel()]
    shots = load_shots(p["survey_fname"], shot_ids, p["if_win"])
    nz, nx, nt = p["nz"], p["nx"], p["nSteps"]
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    den = np.ascontiguousarray(den, dtype=np.float64)
    stf = np.ascontiguousarray(np.atleast_2d(stf), dtype=np.float64)
    if lam.shape != (nz, nx) or mu.shape != (nz, nx) or den.shape != (nz, nx):
        raise ValueError(f"model shape must be {(nz, nx)}")
    if calc_id in (0, 1) and obs is None:
        obs = [np.fromfile(os.path.join(p["data_dir_name"], f"Shot{sid}.bin"), dtype=np.float32,
                           count=s["nrec"] * s.get("nSteps", nt)) for sid, s in zip(shot_ids, shots)]
    extended = any("nSteps" in s or "win_x0" in s for s in shots)
    illum = np.zeros((nz, nx)) if want_illum else None
    if not extended:
        misfit, g_lam, g_mu, g_den, g_stf, gathers, (wavelets, residuals) = _run_group(p, shots, shot_ids, nz, nx, nt, lam, mu,
                                                                          den, stf, calc_id, obs, nthreads,
                                                                          precision, illum)
    else:
        # Each shot alone on its sub-model, for its own record length.
        misfit = 0.0
        g_lam, g_mu, g_den = np.zeros((nz, nx)), np.zeros((nz, nx)), np.zeros((nz, nx))
        g_stf = np.zeros_like(stf)
        gathers, wavelets, residuals = [], [], []
        nPml = p["nPml"]
        for k, (sid, s) in enumerate(zip(shot_ids, shots)):
            ntk = s.get("nSteps", nt)
            x0 = s.get("win_x0", 0)
            x1 = s.get("win_x1", nx - 2 * nPml - 1)
            cols = slice(x0, x1 + 1 + 2 * nPml)
            sub = dict(s)
            sub["x_src"] = s["x_src"] - x0
            sub["x_rec"] = np.asarray(s["x_rec"], dtype=np.int32) - x0
            nxk = x1 - x0 + 1 + 2 * nPml
            stf_k = np.ascontiguousarray(stf[sid:sid + 1, :ntk])
            ob = None if obs is None else [obs[k]]
            il = None if illum is None else np.zeros((nz, nxk))
            m, gl, gm, gd, gs, gth, (wv, rs) = _run_group(p, [sub], [0], nz, nxk, ntk, np.ascontiguousarray(lam[:, cols]),
                                               np.ascontiguousarray(mu[:, cols]), np.ascontiguousarray(den[:, cols]),
                                               stf_k, calc_id, ob, nthreads, precision, il)
            if il is not None:
                illum[:, cols] += il
            misfit += m
            g_lam[:, cols] += gl
            g_mu[:, cols] += gm
            g_den[:, cols] += gd
            g_stf[sid, :ntk] += gs[0]
            gathers += gth
            wavelets += wv
            residuals += rs
    out = {"misfit": misfit, "g_lambda": g_lam, "g_mu": g_mu, "g_den": g_den, "g_stf": g_stf}
    if illum is not None:
        out["illum"] = illum
    if calc_id == 2 and write_files:
        for sid, a in zip(shot_ids, gathers):
            a.astype(np.float32).tofile(os.path.join(p["data_dir_name"], f"Shot{sid}.bin"))
    if want_gathers:
        out["gathers"] = gathers
        if calc_id in (0, 1):
            out["wavelets"] = wavelets
            out["residuals"] = residuals
    return out


def refhost_cufd(calc_id: int, lam, mu, den, stf, shot_ids, para_fname: str) -> dict:
    """The reference driver itself (host build). Gathers of calc_id 2 are
    written by it to data_dir_name and read back here."""
    p = load_para(para_fname)
    shot_ids = [int(v) for v in np.asarray(shot_ids).ravel()]
    nz, nx, nt = p["nz"], p["nx"], p["nSteps"]
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    den = np.ascontiguousarray(den, dtype=np.float64)
    stf = np.ascontiguousarray(np.atleast_2d(stf), dtype=np.float64)
    misfit = ctypes.c_double(0.0)
    g_lam = np.zeros((nz, nx))
    g_mu = np.zeros((nz, nx))
    g_den = np.zeros((nz, nx))
    g_stf = np.zeros_like(stf)
    ids = np.asarray(shot_ids, dtype=np.int32)
    _load_refhost().refhost_cufd(ctypes.byref(misfit), _dptr(g_lam), _dptr(g_mu), _dptr(g_den), _dptr(g_stf),
                                 _dptr(lam), _dptr(mu), _dptr(den), _dptr(stf), int(calc_id), len(shot_ids),
                                 _iptr(ids), para_fname.encode())
    out = {"misfit": misfit.value, "g_lambda": g_lam, "g_mu": g_mu, "g_den": g_den, "g_stf": g_stf}
    if calc_id == 2:
        shots = load_shots(p["survey_fname"], shot_ids, False)
        out["gathers"] = [np.fromfile(os.path.join(p["data_dir_name"], f"Shot{sid}.bin"), dtype=np.float32,
                                      count=s["nrec"] * nt).reshape(s["nrec"], nt)
                          for sid, s in zip(shot_ids, shots)]
    return out
