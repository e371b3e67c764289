"""Host-side helpers of the FwiFlow FWI surface: parameter / survey files,
Ricker source, velocity-to-moduli and model padding.

Python restatement of FwiFlow.jl `src/Utils.jl` and the geometry part of
`src/FWI.jl`, so that files written here are read unchanged by the reference
operator and by this package's C-ABI (and vice versa).
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

__all__ = [
    "paraGen",
    "surveyGen",
    "surveyGen_shots",
    "sourceGene",
    "velocity_to_moduli",
    "padding",
    "default_nPad",
    "FWIGeometry",
]


def default_nPad(nz: int, nPml: int) -> int:
    """z padding that makes nz + 2 nPml + nPad a multiple of 32.

    Same rule as `nPad = 32 - mod(nz + 2 nPml, 32)` (src/FWI.jl:12), which
    yields 32, not 0, when the sum is already a multiple of 32.
    """
    return 32 - ((nz + 2 * nPml) % 32)


def paraGen(nz: int, nx: int, dz: float, dx: float, nSteps: int, dt: float, f0: float, nPml: int, nPad: int,
            para_fname: str, survey_fname: str, data_dir_name: str, *, if_win: bool = False,
            filter_para: Optional[Sequence[float]] = None, if_src_update: bool = False,
            scratch_dir_name: str = "", extra: Optional[dict] = None) -> None:
    """Write the one-line JSON parameter file (src/Utils.jl:21-63).

    `nz`, `nx` are the padded grid sizes. Keys and their order follow the
    reference; `extra` adds optional keys this package understands (ignored by
    the reference parser).
    """
    para: dict = {}
    para["nz"] = int(nz)
    para["nx"] = int(nx)
    para["dz"] = float(dz)
    para["dx"] = float(dx)
    para["nSteps"] = int(nSteps)
    para["dt"] = float(dt)
    para["f0"] = float(f0)
    para["nPoints_pml"] = int(nPml)
    para["nPad"] = int(nPad)
    if if_win:
        para["if_win"] = True
    if filter_para is not None:
        para["filter"] = [float(v) for v in filter_para]
    if if_src_update:
        para["if_src_update"] = True
    para["survey_fname"] = survey_fname
    para["data_dir_name"] = data_dir_name
    os.makedirs(data_dir_name, exist_ok=True)
    if scratch_dir_name:
        para["scratch_dir_name"] = scratch_dir_name
        os.makedirs(scratch_dir_name, exist_ok=True)
    if extra:
        para.update(extra)
    with open(para_fname, "w") as f:
        f.write(json.dumps(para, separators=(",", ":")))


def surveyGen(z_src, x_src, z_rec, x_rec, survey_fname: str, Windows=None, Weights=None) -> None:
    """Write the one-line JSON survey file, all shots sharing one receiver
    spread (src/Utils.jl:80-109). Indices are 0-based interior cells."""
    z_src = [int(v) for v in z_src]
    x_src = [int(v) for v in x_src]
    z_rec = [int(v) for v in z_rec]
    x_rec = [int(v) for v in x_rec]
    shots = []
    for i in range(len(x_src)):
        shot = {"z_src": z_src[i], "x_src": x_src[i], "nrec": len(x_rec), "z_rec": z_rec, "x_rec": x_rec}
        if Windows is not None:
            shot["win_start"] = [float(v) for v in Windows[f"shot{i}"]["start"]]
            shot["win_end"] = [float(v) for v in Windows[f"shot{i}"]["end"]]
        if Weights is not None:
            shot["weights"] = [float(v) for v in Weights[f"shot{i}"]["weights"]]
        shots.append(shot)
    surveyGen_shots(shots, survey_fname)


def surveyGen_shots(shots: Sequence[dict], survey_fname: str) -> None:
    """Write a survey file with per-shot receiver spreads.

    Each entry holds z_src, x_src, z_rec, x_rec (0-based interior indices) and
    optionally win_start, win_end, weights. The file format is the reference's
    (`{"nShots": n, "shot0": {...}, ...}`, read by Src_Rec.cu:19-245). Two
    optional keys of this package, which the reference's parser ignores, are
    passed through: "nSteps" (the shot's record length, at most the parameter
    file's) and "win_x0" / "win_x1" (the shot's aperture window of interior
    columns).
    """
    survey: dict = {"nShots": len(shots)}
    for i, s in enumerate(shots):
        d = {"z_src": int(s["z_src"]), "x_src": int(s["x_src"]), "nrec": len(s["x_rec"]),
             "z_rec": [int(v) for v in s["z_rec"]], "x_rec": [int(v) for v in s["x_rec"]]}
        for k in ("win_start", "win_end", "weights"):
            if k in s:
                d[k] = [float(v) for v in s[k]]
        for k in ("nSteps", "win_x0", "win_x1"):
            if k in s:
                d[k] = int(s[k])
        survey[f"shot{i}"] = d
    with open(survey_fname, "w") as f:
        f.write(json.dumps(survey, separators=(",", ":")))


def sourceGene(f: float, nStep: int, delta_t: float) -> np.ndarray:
    """Integrated Ricker wavelet times dt, shape (1, nStep) (src/Utils.jl:116-132)."""
    e = np.pi * np.pi * f * f
    t_delay = 1.2 / f
    t = delta_t * np.arange(nStep, dtype=np.float64) - t_delay
    src = (1.0 - 2.0 * e * t ** 2) * np.exp(-e * t ** 2)
    src = np.cumsum(src)
    return (src * delta_t).reshape(1, nStep)


def velocity_to_moduli(cp, cs, den):
    """lambda, mu in MPa from cp, cs [m/s] and density (src/Utils.jl:221-227)."""
    cp = np.asarray(cp, dtype=np.float64)
    cs = np.asarray(cs, dtype=np.float64)
    den = np.asarray(den, dtype=np.float64)
    lam = (cp * cp - 2.0 * cs * cs) * den / 1e6
    mu = cs * cs * den / 1e6
    return lam, mu


def padding(a, nPml: int, nPad: int) -> np.ndarray:
    """Symmetric padding by nPml on top/left/right and nPml + nPad at the
    bottom, as tf.pad(..., "SYMMETRIC") in src/FWI.jl:193-205."""
    return np.pad(np.asarray(a, dtype=np.float64), ((nPml, nPml + nPad), (nPml, nPml)), mode="symmetric")


@dataclass
class FWIGeometry:
    """The `FWI` struct of src/FWI.jl:3-25 without the TensorFlow members."""

    nz: int
    nx: int
    dz: float
    dx: float
    nSteps: int
    dt: float
    f0: float = 4.5
    nPml: int = 32
    nPad: Optional[int] = None
    ind_src_z: Sequence[int] = field(default_factory=list)
    ind_src_x: Sequence[int] = field(default_factory=list)
    ind_rec_z: Sequence[int] = field(default_factory=list)
    ind_rec_x: Sequence[int] = field(default_factory=list)

    def __post_init__(self) -> None:
        if self.nPad is None:
            self.nPad = default_nPad(self.nz, self.nPml)

    @property
    def nz_pad(self) -> int:
        return self.nz + 2 * self.nPml + self.nPad

    @property
    def nx_pad(self) -> int:
        return self.nx + 2 * self.nPml

    def mask(self) -> np.ndarray:
        """1 on the interior except its top 10 rows (src/FWI.jl:47-49)."""
        m = np.zeros((self.nz_pad, self.nx_pad))
        m[self.nPml:self.nPml + self.nz, self.nPml:self.nPml + self.nx] = 1.0
        m[self.nPml:self.nPml + 10, :] = 0.0
        return m
