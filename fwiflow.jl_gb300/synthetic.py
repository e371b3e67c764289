"""Seeded synthetic survey workloads (no public data is used).

Each builder returns a `Workload`: the padded geometry, a model pair (the
model to evaluate and the model the observed data come from) as Vp / Vs /
density on the padded grid, the per-shot source / receiver layout and the
source time functions. Vs = Vp / sqrt(3), density = 310 Vp^0.25 (Gardner),
sources are the integrated Ricker of `sourceGene` (src/Utils.jl:116-132).

  small_layered     4 flat layers + Gaussian anomaly, 100x200 interior, 1000 steps, 2 shots
  dipping_grf       8 dipping layers x (1 + 3% Gaussian random field), 512x1536, 3000 steps, 1 shot
  batched_uneven    the dipping_grf family, 64 shots with their own aperture window,
                    record length and Ricker frequency
  tiny              a few-second case for smoke tests and parity tests
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .utils import default_nPad, padding, paraGen, sourceGene, surveyGen_shots, velocity_to_moduli


@dataclass
class Workload:
    name: str
    nz: int  # interior
    nx: int
    nPml: int
    nPad: int
    dz: float
    dx: float
    dt: float
    nSteps: int
    f0: float
    vp: np.ndarray        # padded [nz_pad][nx_pad], model to evaluate
    vp_obs: np.ndarray    # padded, model of the observed data
    shots: List[dict]     # z_src, x_src, z_rec, x_rec (0-based interior indices)
    stf: np.ndarray       # [n_shots][nSteps]
    extra: dict = field(default_factory=dict)

    @property
    def nz_pad(self) -> int:
        return self.nz + 2 * self.nPml + self.nPad

    @property
    def nx_pad(self) -> int:
        return self.nx + 2 * self.nPml

    @property
    def cells(self) -> int:
        return self.nz_pad * self.nx_pad

    def moduli(self, vp: Optional[np.ndarray] = None):
        vp = self.vp if vp is None else vp
        vs = vp / np.sqrt(3.0)
        rho = 310.0 * vp ** 0.25
        lam, mu = velocity_to_moduli(vp, vs, rho)
        return lam, mu, rho

    def write_files(self, workdir: str, para_name: str = "para.json", survey_name: str = "survey.json") -> str:
        """Writes the parameter and survey files (and the Data directory)."""
        os.makedirs(workdir, exist_ok=True)
        para = os.path.join(workdir, para_name)
        survey = os.path.join(workdir, survey_name)
        paraGen(self.nz_pad, self.nx_pad, self.dz, self.dx, self.nSteps, self.dt, self.f0, self.nPml, self.nPad, para,
                survey, os.path.join(workdir, "Data"))
        surveyGen_shots(self.shots, survey)
        return para


def gaussian_random_field(shape, corr_cells: float, rng: np.random.Generator) -> np.ndarray:
    """Zero-mean, unit-variance field: white noise smoothed by a Gaussian whose
    standard deviation is corr_cells / sqrt(2) (spectral multiplication)."""
    noise = rng.standard_normal(shape)
    kz = np.fft.fftfreq(shape[0])[:, None]
    kx = np.fft.fftfreq(shape[1])[None, :]
    sig = corr_cells / np.sqrt(2.0)
    filt = np.exp(-2.0 * (np.pi * sig) ** 2 * (kz ** 2 + kx ** 2))
    f = np.real(np.fft.ifft2(np.fft.fft2(noise) * filt))
    f -= f.mean()
    return f / (f.std() + 1e-30)


def _layers(nz: int, nx: int, vmin: float, vmax: float, n: int, dip_deg: float = 0.0) -> np.ndarray:
    zz, xx = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(nx, dtype=np.float64), indexing="ij")
    depth = zz - np.tan(np.deg2rad(dip_deg)) * (xx - nx / 2)
    k = np.clip(np.floor(depth / (nz / n)), 0, n - 1)
    return vmin + (vmax - vmin) * k / (n - 1)


def small_layered(nSteps: int = 1000) -> Workload:
    """4 flat layers Vp 1500..3500 (25 cells each) + Gaussian anomaly (sigma 8
    cells, +200 m/s evaluated, -200 m/s observed) at (50, 100); 2 shots at
    x = 50, 150, depth 2; 200 receivers at depth 2; dx 20 m, dt 2 ms, f0 8 Hz."""
    nz, nx, nPml = 100, 200, 32
    nPad = default_nPad(nz, nPml)
    base = _layers(nz, nx, 1500.0, 3500.0, 4)
    zz, xx = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    g = np.exp(-((zz - 50.0) ** 2 + (xx - 100.0) ** 2) / (2 * 8.0 ** 2))
    vp = padding(base + 200.0 * g, nPml, nPad)
    vp_obs = padding(base - 200.0 * g, nPml, nPad)
    shots = [{"z_src": 2, "x_src": xs, "z_rec": [2] * nx, "x_rec": list(range(nx))} for xs in (50, 150)]
    stf = np.repeat(sourceGene(8.0, nSteps, 0.002), 2, axis=0)
    return Workload("small_layered", nz, nx, nPml, nPad, 20.0, 20.0, 0.002, nSteps, 8.0, vp, vp_obs, shots, stf)


def dipping_grf(seed: int = 2, nz: int = 512, nx: int = 1536, nSteps: int = 3000, n_shots: int = 1) -> Workload:
    """8 dipping (5 deg) layers Vp 1500..4500 times (1 + 0.03 GRF(corr 20)), seeded;
    observed data from the unperturbed layers; dx 10 m, dt 1 ms, f0 10 Hz;
    shots evenly spread at depth 2 (one shot: x = nx/2); receivers on every
    column at depth 2."""
    rng = np.random.default_rng(seed)
    nPml = 32
    nPad = default_nPad(nz, nPml)
    base = _layers(nz, nx, 1500.0, 4500.0, 8, dip_deg=5.0)
    pert = gaussian_random_field((nz, nx), 20.0, rng)
    vp = padding(base * (1.0 + 0.03 * pert), nPml, nPad)
    vp_obs = padding(base, nPml, nPad)
    xs = [nx // 2] if n_shots == 1 else list(np.linspace(16, nx - 17, n_shots).astype(int))
    shots = [{"z_src": 2, "x_src": int(x), "z_rec": [2] * nx, "x_rec": list(range(nx))} for x in xs]
    stf = np.repeat(sourceGene(10.0, nSteps, 0.001), len(shots), axis=0)
    return Workload("dipping_grf", nz, nx, nPml, nPad, 10.0, 10.0, 0.001, nSteps, 10.0, vp, vp_obs, shots, stf)


def faulted_grf(seed: int = 5, nz: int = 1024, nx: int = 3072, nSteps: int = 6000, n_shots: int = 128,
                shot_subset: Optional[int] = None) -> Workload:
    """The full-scale model: 8 layers Vp 1500..4500 m/s cut by 3 normal faults
    (60 degree fault planes at seeded positions, hanging wall thrown down by
    10-40 cells), times (1 + 0.03 GRF(corr 20)); dx 5 m, dt 0.5 ms, f0 15 Hz,
    nPml 40; n_shots sources evenly spread at depth 2, receivers on every
    column at depth 2. The observed data come from the model, the starting
    model is the model smoothed by 20 cells. shot_subset keeps the first that
    many shots of the evenly spread set (a slice of the survey for timing)."""
    from .gradcheck import smooth

    rng = np.random.default_rng(seed)
    nPml = 40
    nPad = default_nPad(nz, nPml)
    zz, xx = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(nx, dtype=np.float64), indexing="ij")
    shift = np.zeros((nz, nx))
    for _ in range(3):
        xf = rng.uniform(0.15, 0.85) * nx
        throw = rng.uniform(10.0, 40.0)
        # hanging wall: right of the plane x = xf + (z / tan 60)
        shift += np.where(xx > xf + zz / np.tan(np.deg2rad(60.0)), throw, 0.0)
    depth = zz - shift
    k = np.clip(np.floor(depth / (nz / 8)), 0, 7)
    base = 1500.0 + (4500.0 - 1500.0) * k / 7
    true = base * (1.0 + 0.03 * gaussian_random_field((nz, nx), 20.0, rng))
    vp0 = smooth(true, 20.0)
    xs = np.linspace(16, nx - 17, n_shots).astype(int)
    if shot_subset is not None:
        xs = xs[:shot_subset]
    shots = [{"z_src": 2, "x_src": int(x), "z_rec": [2] * nx, "x_rec": list(range(nx))} for x in xs]
    stf = np.repeat(sourceGene(15.0, nSteps, 0.0005), len(shots), axis=0)
    return Workload("faulted_grf", nz, nx, nPml, nPad, 5.0, 5.0, 0.0005, nSteps, 15.0, padding(vp0, nPml, nPad),
                    padding(true, nPml, nPad), shots, stf)


def batched_uneven(seed: int = 3, nz: int = 512, nx: int = 1536, n_shots: int = 64, width=(400, 1536),
                   steps=(1500, 4000), f0=(8.0, 12.0), nSteps: Optional[int] = None) -> Workload:
    """The dipping_grf model family with n_shots shots, each with its own
    aperture window (width drawn uniformly in `width` interior columns,
    centred on the source where the model allows), record length (uniform in
    `steps`; the parameter file's nSteps is the largest) and Ricker frequency
    (uniform in `f0`). Sources at depth 2 at seed-drawn columns; receivers on
    every column of the window at depth 2."""
    rng = np.random.default_rng(seed)
    nPml = 32
    nPad = default_nPad(nz, nPml)
    base = _layers(nz, nx, 1500.0, 4500.0, 8, dip_deg=5.0)
    pert = gaussian_random_field((nz, nx), 20.0, rng)
    vp = padding(base * (1.0 + 0.03 * pert), nPml, nPad)
    vp_obs = padding(base, nPml, nPad)
    shots = []
    nts, f0s = [], []
    for _ in range(n_shots):
        w = int(rng.integers(width[0], min(width[1], nx) + 1))
        xs = int(rng.integers(4, nx - 4))
        w0 = int(np.clip(xs - w // 2, 0, nx - w))
        nt = int(rng.integers(steps[0], steps[1] + 1))
        nts.append(nt)
        f0s.append(float(rng.uniform(f0[0], f0[1])))
        shots.append({"z_src": 2, "x_src": xs, "z_rec": [2] * w, "x_rec": list(range(w0, w0 + w)), "nSteps": nt,
                      "win_x0": w0, "win_x1": w0 + w - 1})
    nt_max = max(nts) if nSteps is None else nSteps
    stf = np.concatenate([sourceGene(f, nt_max, 0.001) for f in f0s], axis=0)
    w = Workload("batched_uneven", nz, nx, nPml, nPad, 10.0, 10.0, 0.001, nt_max, 10.0, vp, vp_obs, shots, stf)
    w.extra["f0"] = f0s
    return w


def layered_grf(seed: int, nz: int = 256, nx: int = 768, n_shots: int = 16, nSteps: int = 2000,
                dx: float = 10.0, dt: float = 0.001, f0: float = 10.0, smooth_cells: float = 10.0,
                start: str = "smooth") -> Workload:
    """One model of the learned-preconditioner family: 5-9 layers (Vp from
    1500 m/s at the top to 3500-4500 m/s at the bottom, random interface
    depths and a common dip of up to 5 degrees) times (1 + 3 % GRF, corr. 20
    cells), seeded. `vp_obs` is the true model and `vp` the starting model of
    an inversion: the true model smoothed by a Gaussian of `smooth_cells`
    (start "smooth"), or the layers without the random field smoothed by it
    (start "background"). n_shots sources evenly spread at depth 2, receivers
    on every column at depth 2; Ricker f0."""
    rng = np.random.default_rng(seed)
    nPml = 32
    nPad = default_nPad(nz, nPml)
    nl = int(rng.integers(5, 10))
    vbot = float(rng.uniform(3500.0, 4500.0))
    cuts = np.sort(rng.uniform(0.08, 0.95, nl - 1)) * nz
    vels = np.sort(rng.uniform(1500.0, vbot, nl))
    vels[0] = 1500.0
    dip = np.tan(np.deg2rad(rng.uniform(-5.0, 5.0)))
    zz, xx = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    depth = zz - dip * (xx - nx / 2)
    layer = np.searchsorted(cuts, depth)
    base = vels[np.clip(layer, 0, nl - 1)]
    true = base * (1.0 + 0.03 * gaussian_random_field((nz, nx), 20.0, rng))
    from .gradcheck import smooth

    if start == "smooth":
        vp0 = smooth(true, smooth_cells)
    elif start == "background":
        vp0 = smooth(base, smooth_cells)
    else:
        raise ValueError(start)
    xs = np.linspace(16, nx - 17, n_shots).astype(int)
    shots = [{"z_src": 2, "x_src": int(x), "z_rec": [2] * nx, "x_rec": list(range(nx))} for x in xs]
    stf = np.repeat(sourceGene(f0, nSteps, dt), n_shots, axis=0)
    w = Workload("layered_grf", nz, nx, nPml, nPad, dx, dx, dt, nSteps, f0, padding(vp0, nPml, nPad),
                 padding(true, nPml, nPad), shots, stf)
    w.extra["seed"] = seed
    return w


def tiny(nz: int = 40, nx: int = 60, nPml: int = 12, nSteps: int = 300, n_shots: int = 2, seed: int = 0,
         cs_zero: bool = False) -> Workload:
    """Small smooth model with a Gaussian anomaly for parity tests (seconds on a CPU)."""
    rng = np.random.default_rng(seed)
    nPad = default_nPad(nz, nPml)
    zz, xx = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    base = 1800.0 + 1200.0 * zz / nz
    g = np.exp(-((zz - nz / 2) ** 2 + (xx - nx / 2) ** 2) / (2 * (min(nz, nx) / 8) ** 2))
    pert = 0.02 * gaussian_random_field((nz, nx), 4.0, rng)
    vp = padding(base * (1 + pert) + 150.0 * g, nPml, nPad)
    vp_obs = padding(base, nPml, nPad)
    xs = np.linspace(8, nx - 9, n_shots).astype(int)
    shots = [{"z_src": 2, "x_src": int(x), "z_rec": [2] * nx, "x_rec": list(range(nx))} for x in xs]
    stf = np.repeat(sourceGene(10.0, nSteps, 0.002), n_shots, axis=0)
    w = Workload("tiny", nz, nx, nPml, nPad, 20.0, 20.0, 0.002, nSteps, 10.0, vp, vp_obs, shots, stf)
    if cs_zero:
        w.extra["cs_zero"] = True
    return w


def tiny_moduli(w: Workload, vp: np.ndarray):
    """Moduli of a `tiny` workload, with Vs = 0 (acoustic) when requested."""
    if w.extra.get("cs_zero"):
        rho = 2500.0 * np.ones_like(vp)
        lam, mu = velocity_to_moduli(vp, np.zeros_like(vp), rho)
        return lam, mu, rho
    return w.moduli(vp)
