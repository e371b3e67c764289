"""The FwiFlow FWI operator surface on top of the GB300 C ABI.

Mirrors, with the same argument meaning and units:
  fwi_op / fwi_obs_op                 src/Core.jl:20-53 (TF ops FwiOp / FwiOpGrad / FwiObsOp)
  FWI, compute_observation,           src/FWI.jl:3-189
  compute_misfit
`fwi_op` returns the misfit; its gradient (lambda, mu, den, stf) comes from
`fwi_op_grad` or from the autograd wrapper `FwiOpFunction`, which, unlike the
reference's FwiOpGrad (FwiOp.cpp:207-222), scales the gradients by the
incoming cotangent.
"""
from __future__ import annotations

import os
import tempfile
from typing import Optional, Sequence

import numpy as np

from . import _lib
from .utils import FWIGeometry, padding, paraGen, surveyGen, velocity_to_moduli

__all__ = ["FwiContext", "fwi_op", "fwi_op_grad", "fwi_obs_op", "FWI", "compute_observation", "compute_misfit",
           "FwiOpFunction"]


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


class FwiContext:
    """One parameter file on one GPU (a `fwigb_ctx`): geometry parsed once,
    device buffers kept across calls."""

    def __init__(self, para_fname: str, gpu_id: int = 0):
        lib = _lib.load()
        h = _lib._V()
        _lib.check(lib.fwigb_create(para_fname.encode(), int(gpu_id), _lib.ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.para_fname = para_fname
        nz, nx, nt, nsh, nrm = (_lib.ctypes.c_int() for _ in range(5))
        _lib.check(lib.fwigb_geometry(h, *(_lib.ctypes.byref(v) for v in (nz, nx, nt, nsh, nrm))), h)
        self.nz, self.nx, self.nSteps = nz.value, nx.value, nt.value
        self.n_survey_shots, self.nrec_max = nsh.value, nrm.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fwigb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- helpers
    def nrec(self, shot_id: int) -> int:
        v = _lib.ctypes.c_int()
        _lib.check(self._lib.fwigb_shot_nrec(self._h, int(shot_id), _lib.ctypes.byref(v)), self._h)
        return v.value

    def shot_info(self, shot_id: int):
        """(nrec, nSteps, x_off, nx) of a survey shot: receivers, record length
        and the padded columns of its sub-grid."""
        vals = [_lib.ctypes.c_int() for _ in range(4)]
        _lib.check(self._lib.fwigb_shot_info(self._h, int(shot_id), *(_lib.ctypes.byref(x) for x in vals)), self._h)
        return tuple(x.value for x in vals)

    def _model(self, lam, mu, den):
        lam, mu, den = _f64(lam), _f64(mu), _f64(den)
        for a in (lam, mu, den):
            if a.shape != (self.nz, self.nx):
                raise ValueError(f"model arrays must be {(self.nz, self.nx)}, got {a.shape}")
        return lam, mu, den

    def _stf_ids(self, stf, shot_ids):
        stf = _f64(np.atleast_2d(stf))
        if stf.shape[1] != self.nSteps:
            raise ValueError(f"stf rows must have nSteps={self.nSteps} samples")
        ids = np.ascontiguousarray(np.asarray(shot_ids, dtype=np.int32).ravel())
        return stf, ids

    def _obs_block(self, obs, ids):
        blk = np.zeros((len(ids), self.nrec_max, self.nSteps), dtype=np.float32)
        for i, (o, sid) in enumerate(zip(obs, ids)):
            o = np.asarray(o, dtype=np.float32)
            nrec, nt = self.shot_info(sid)[:2]
            blk[i, :nrec, :nt] = o.reshape(nrec, nt)
        return blk

    # -- operator calls
    def misfit(self, lam, mu, den, stf, shot_ids, obs: Optional[Sequence[np.ndarray]] = None) -> float:
        """FwiOp (cufd calc_id 0)."""
        lam, mu, den = self._model(lam, mu, den)
        stf, ids = self._stf_ids(stf, shot_ids)
        out = np.zeros(1)
        if obs is None:
            _lib.check(self._lib.fwigb_misfit(self._h, _lib.dptr(lam), _lib.dptr(mu), _lib.dptr(den), _lib.dptr(stf),
                                              stf.shape[0], _lib.iptr(ids), len(ids), _lib.dptr(out)), self._h)
        else:
            blk = self._obs_block(obs, ids)
            _lib.check(self._lib.fwigb_misfit_grad_obs(
                self._h, _lib.dptr(lam), _lib.dptr(mu), _lib.dptr(den), _lib.dptr(stf), stf.shape[0], _lib.iptr(ids),
                len(ids), _lib.fptr(blk), _lib.dptr(out), None, None, None, None), self._h)
        return float(out[0])

    def misfit_grad(self, lam, mu, den, stf, shot_ids, obs: Optional[Sequence[np.ndarray]] = None):
        """FwiOpGrad (cufd calc_id 1) plus the misfit of the same forward pass.
        Returns (misfit, g_lambda, g_mu, g_den, g_stf[n_shots][nSteps])."""
        lam, mu, den = self._model(lam, mu, den)
        stf, ids = self._stf_ids(stf, shot_ids)
        out = np.zeros(1)
        gl, gm, gd = (np.zeros((self.nz, self.nx)) for _ in range(3))
        gs = np.zeros((len(ids), self.nSteps))
        if obs is None:
            _lib.check(self._lib.fwigb_misfit_grad(
                self._h, _lib.dptr(lam), _lib.dptr(mu), _lib.dptr(den), _lib.dptr(stf), stf.shape[0], _lib.iptr(ids),
                len(ids), _lib.dptr(out), _lib.dptr(gl), _lib.dptr(gm), _lib.dptr(gd), _lib.dptr(gs)), self._h)
        else:
            blk = self._obs_block(obs, ids)
            _lib.check(self._lib.fwigb_misfit_grad_obs(
                self._h, _lib.dptr(lam), _lib.dptr(mu), _lib.dptr(den), _lib.dptr(stf), stf.shape[0], _lib.iptr(ids),
                len(ids), _lib.fptr(blk), _lib.dptr(out), _lib.dptr(gl), _lib.dptr(gm), _lib.dptr(gd),
                _lib.dptr(gs)), self._h)
        return float(out[0]), gl, gm, gd, gs

    def obs(self, lam, mu, den, stf, shot_ids, write_files: bool = True):
        """FwiObsOp (cufd calc_id 2). Returns a list of [nrec][nSteps] gathers."""
        lam, mu, den = self._model(lam, mu, den)
        stf, ids = self._stf_ids(stf, shot_ids)
        blk = np.zeros((len(ids), self.nrec_max, self.nSteps), dtype=np.float32)
        _lib.check(self._lib.fwigb_obs(self._h, _lib.dptr(lam), _lib.dptr(mu), _lib.dptr(den), _lib.dptr(stf),
                                       stf.shape[0], _lib.iptr(ids), len(ids), _lib.fptr(blk), int(write_files)),
                   self._h)
        out = []
        for i, s in enumerate(ids):
            nrec, nt = self.shot_info(s)[:2]
            out.append(blk[i, :nrec, :nt])
        return out

    # -- staged interface (model / shots resident on the device)
    def set_model(self, lam, mu, den) -> None:
        lam, mu, den = self._model(lam, mu, den)
        _lib.check(self._lib.fwigb_set_model(self._h, _lib.dptr(lam), _lib.dptr(mu), _lib.dptr(den)), self._h)

    def stage_shots(self, stf, shot_ids, obs: Optional[Sequence[np.ndarray]] = None, with_obs: bool = True) -> None:
        stf, ids = self._stf_ids(stf, shot_ids)
        blk = self._obs_block(obs, ids) if obs is not None else None
        self._staged_keep = (stf, ids, blk)
        _lib.check(self._lib.fwigb_stage_shots(self._h, _lib.dptr(stf), stf.shape[0], _lib.iptr(ids), len(ids),
                                               int(with_obs), _lib.fptr(blk)), self._h)

    def run(self, calc_id: int) -> None:
        _lib.check(self._lib.fwigb_run(self._h, int(calc_id)), self._h)

    def fetch(self, misfit=True, grads=False, n_shots: int = 0):
        out = np.zeros(1)
        gl = gm = gd = gs = None
        if grads:
            gl, gm, gd = (np.zeros((self.nz, self.nx)) for _ in range(3))
            gs = np.zeros((n_shots, self.nSteps))
        _lib.check(self._lib.fwigb_fetch(self._h, _lib.dptr(out) if misfit else None, _lib.dptr(gl), _lib.dptr(gm),
                                         _lib.dptr(gd), _lib.dptr(gs), None), self._h)
        return float(out[0]), gl, gm, gd, gs

    def synchronize(self) -> None:
        _lib.check(self._lib.fwigb_synchronize(self._h), self._h)

    @property
    def stream(self) -> int:
        return int(self._lib.fwigb_stream(self._h) or 0)

    def last_launch_count(self) -> int:
        return int(self._lib.fwigb_last_launch_count(self._h))

    def set_batching(self, max_shots: int = 0, mem_budget_bytes: int = 0) -> None:
        """Cap the shots per concurrent group (0: none) and the group state's
        device memory (0: 90% of free memory)."""
        _lib.check(self._lib.fwigb_set_batching(self._h, int(max_shots), int(mem_budget_bytes)), self._h)

    def last_group_count(self) -> int:
        return int(self._lib.fwigb_last_group_count(self._h))

    def test_inject_wait_timeout(self, enable: bool) -> None:
        """Failure-path test hook: while enabled, every run's first forward
        sweep lets its bounded wait run out and the call raises FwiError with
        status ERR_TIMEOUT; the context stays usable."""
        _lib.check(self._lib.fwigb_test_inject_wait_timeout(self._h, int(enable)), self._h)

    def set_illumination(self, enable: bool = True) -> None:
        """Accumulate the source illumination sum_t (vz^2 + vx^2) in the
        following runs (all their shots)."""
        _lib.check(self._lib.fwigb_set_illumination(self._h, int(enable)), self._h)

    def illumination(self) -> np.ndarray:
        """The last run's illumination, [nz][nx] float64."""
        out = np.zeros((self.nz, self.nx))
        _lib.check(self._lib.fwigb_fetch_illumination(self._h, _lib.dptr(out)), self._h)
        return out

    def tile_config(self):
        """Tile widths of (forward stress, forward velocity, backward B, backward C)."""
        t = np.zeros(4, dtype=np.int32)
        _lib.check(self._lib.fwigb_tile_config(self._h, _lib.iptr(t)), self._h)
        return [int(v) for v in t]

    def tile_rows(self):
        """Depths per thread of (forward stress, forward velocity, backward B, backward C)."""
        t = np.zeros(4, dtype=np.int32)
        _lib.check(self._lib.fwigb_tile_rows(self._h, _lib.iptr(t)), self._h)
        return [int(v) for v in t]

    def tile_registers(self):
        """Registers per thread of the four sweeps' tiles (the backward one-row
        tiles run at 32 or 40, picked by the autotuner)."""
        t = np.zeros(4, dtype=np.int32)
        _lib.check(self._lib.fwigb_tile_registers(self._h, _lib.iptr(t)), self._h)
        return [int(v) for v in t]

    def set_tile_registers(self, regs) -> None:
        """Fix the backward sweeps' one-row register budget (entries 2, 3: 32 or 40)."""
        t = np.ascontiguousarray(regs, dtype=np.int32)
        _lib.check(self._lib.fwigb_set_tile_registers(self._h, _lib.iptr(t)), self._h)

    def set_tile_config(self, widths=None) -> None:
        """Fix the four tile widths (4, 8 or 16); None re-enables the autotuner."""
        t = None if widths is None else np.ascontiguousarray(widths, dtype=np.int32)
        _lib.check(self._lib.fwigb_set_tile_config(self._h, _lib.iptr(t)), self._h)

    def set_tile_rows(self, rows) -> None:
        """Fix the depths per thread (1 or 2) of the four sweeps."""
        t = np.ascontiguousarray(rows, dtype=np.int32)
        _lib.check(self._lib.fwigb_set_tile_rows(self._h, _lib.iptr(t)), self._h)

    def set_graphs(self, enable: bool) -> None:
        """Replay a single-group call's launch sequence (a lone shot or a
        batched group) from a CUDA graph (default on)."""
        _lib.check(self._lib.fwigb_set_graphs(self._h, int(enable)), self._h)

    def sweep_time(self, kind: int, reps: int = 50) -> float:
        """Microseconds per launch of sweep `kind` (0 F1, 1 F2, 2 B, 3 C) on
        the last run's group, from a CUDA graph of back-to-back launches."""
        out = np.zeros(1)
        _lib.check(self._lib.fwigb_sweep_time(self._h, int(kind), int(reps), _lib.dptr(out)), self._h)
        return float(out[0])

    def set_kernel_timing(self, enable: bool) -> None:
        _lib.check(self._lib.fwigb_set_kernel_timing(self._h, int(enable)), self._h)

    def kernel_times(self):
        """(total_ms[4], launches[4]) of the last run, by kernel kind
        (forward stress, forward velocity, backward B, backward C)."""
        ms = np.zeros(4)
        n = (_lib.ctypes.c_longlong * 4)()
        _lib.check(self._lib.fwigb_kernel_times(self._h, _lib.dptr(ms), n), self._h)
        return ms, np.array(list(n), dtype=np.int64)


_contexts: dict = {}


def _ctx(para_fname: str, gpu_id: int) -> FwiContext:
    key = (os.path.abspath(para_fname), int(gpu_id))
    c = _contexts.get(key)
    if c is None:
        c = FwiContext(para_fname, gpu_id)
        _contexts[key] = c
    return c


def fwi_op(lam, mu, den, stf, gpu_id: int, shot_ids, para_fname: str) -> float:
    """Misfit of the FWI operator (src/Core.jl:20-31, cufd calc_id 0).
    shot_ids are 0-based; lam, mu in MPa."""
    return _ctx(para_fname, gpu_id).misfit(lam, mu, den, stf, shot_ids)


def fwi_op_grad(lam, mu, den, stf, gpu_id: int, shot_ids, para_fname: str):
    """Gradients of fwi_op w.r.t. (lam, mu, den, stf) as FwiOpGrad returns
    them (FwiOp.cpp:130-223); g_stf has the shape of stf with the first
    len(shot_ids) rows filled."""
    stf2 = np.atleast_2d(np.asarray(stf, dtype=np.float64))
    _, gl, gm, gd, gs = _ctx(para_fname, gpu_id).misfit_grad(lam, mu, den, stf2, shot_ids)
    g_stf = np.zeros_like(stf2)
    g_stf[:gs.shape[0]] = gs
    return gl, gm, gd, g_stf


def fwi_obs_op(lam, mu, den, stf, gpu_id: int, shot_ids, para_fname: str) -> float:
    """Forward modelling (src/Core.jl:42-53, cufd calc_id 2): writes
    data_dir_name/Shot<id>.bin for every shot and returns 0.0 like FwiObsOp."""
    _ctx(para_fname, gpu_id).obs(lam, mu, den, stf, shot_ids, write_files=True)
    return 0.0


class FWI(FWIGeometry):
    """`FWI` of src/FWI.jl:3-60: geometry, mask, and a workspace holding the
    parameter file, the survey file and the Data directory."""

    def __init__(self, nz, nx, dz, dx, nSteps, dt, *, ind_src_z, ind_src_x, ind_rec_z, ind_rec_x, f0=4.5, nPml=32,
                 nPad=None, workspace: Optional[str] = None, para_fname="para_file.json",
                 survey_fname="survey_file.json", data_dir_name="Data"):
        super().__init__(nz=nz, nx=nx, dz=float(dz), dx=float(dx), nSteps=nSteps, dt=float(dt), f0=float(f0),
                         nPml=nPml, nPad=nPad, ind_src_z=list(ind_src_z), ind_src_x=list(ind_src_x),
                         ind_rec_z=list(ind_rec_z), ind_rec_x=list(ind_rec_x))
        assert len(self.ind_rec_x) == len(self.ind_rec_z)
        assert len(self.ind_src_x) == len(self.ind_src_z)
        self.WORKSPACE = workspace or tempfile.mkdtemp()
        self.para_path = os.path.join(self.WORKSPACE, para_fname)
        self.survey_path = os.path.join(self.WORKSPACE, survey_fname)
        self.data_dir = os.path.join(self.WORKSPACE, data_dir_name)
        paraGen(self.nz_pad, self.nx_pad, dz, dx, nSteps, dt, self.f0, self.nPml, self.nPad, self.para_path,
                self.survey_path, self.data_dir)
        surveyGen(self.ind_src_z, self.ind_src_x, self.ind_rec_z, self.ind_rec_x, self.survey_path)

    def try_pad(self, a) -> np.ndarray:
        a = np.asarray(a, dtype=np.float64)
        if a.shape == (self.nz_pad, self.nx_pad):
            return a
        if a.shape != (self.nz, self.nx):
            raise ValueError("model must be interior-sized or padded-sized (no resampling here)")
        return padding(a, self.nPml, self.nPad)


def _shot_ids0(fwi: FWI, shot_ids) -> np.ndarray:
    if shot_ids is None:
        shot_ids = np.arange(1, len(fwi.ind_src_x) + 1)
    return np.asarray(shot_ids, dtype=np.int64) - 1


def _stf_rows(fwi: FWI, stf) -> np.ndarray:
    stf = np.asarray(stf, dtype=np.float64)
    if stf.ndim == 1 or stf.shape[0] == 1:
        stf = np.repeat(stf.reshape(1, -1), len(fwi.ind_src_z), axis=0)
    return stf


def compute_observation(fwi: FWI, cp, cs, rho, stf, shot_ids=None, gpu_id: int = 0) -> np.ndarray:
    """Gathers data[shot, nSteps, nrec] (src/FWI.jl:109-135); shot_ids 1-based."""
    cp, cs, rho = fwi.try_pad(cp), fwi.try_pad(cs), fwi.try_pad(rho)
    lam, mu = velocity_to_moduli(cp, cs, rho)
    ids = _shot_ids0(fwi, shot_ids)
    g = _ctx(fwi.para_path, gpu_id).obs(lam, mu, rho, _stf_rows(fwi, stf), ids, write_files=True)
    return np.stack([a.T for a in g]).astype(np.float64)


def compute_misfit(fwi: FWI, cp, cs, rho, stf, shot_ids=None, gpu_id: int = 0, is_masked: bool = False, cp_ref=None,
                   cs_ref=None, rho_ref=None, with_grad: bool = False):
    """Misfit (and optionally gradients w.r.t. cp, cs, rho through the chain
    rule of velocity_to_moduli and the mask) of src/FWI.jl:156-189."""
    cp, cs, rho = fwi.try_pad(cp), fwi.try_pad(cs), fwi.try_pad(rho)
    mask = fwi.mask()
    if not is_masked:
        if cp_ref is None:
            raise ValueError("compute_misfit with is_masked=False needs cp_ref, cs_ref, rho_ref")
        cp_ref, cs_ref, rho_ref = fwi.try_pad(cp_ref), fwi.try_pad(cs_ref), fwi.try_pad(rho_ref)
        cp_m = cp * mask + cp_ref * (1 - mask)
        cs_m = cs * mask + cs_ref * (1 - mask)
        rho_m = rho * mask + rho_ref * (1 - mask)
    else:
        cp_m, cs_m, rho_m = cp, cs, rho
    lam, mu = velocity_to_moduli(cp_m, cs_m, rho_m)
    ids = _shot_ids0(fwi, shot_ids)
    ctx = _ctx(fwi.para_path, gpu_id)
    stf = _stf_rows(fwi, stf)
    if not with_grad:
        return ctx.misfit(lam, mu, rho_m, stf, ids)
    J, gl, gm, gd, gs = ctx.misfit_grad(lam, mu, rho_m, stf, ids)
    # lam = (cp^2 - 2 cs^2) rho / 1e6, mu = cs^2 rho / 1e6
    g_cp = gl * 2 * cp_m * rho_m / 1e6
    g_cs = (gl * (-4 * cs_m) + gm * 2 * cs_m) * rho_m / 1e6
    g_rho = gd + gl * (cp_m ** 2 - 2 * cs_m ** 2) / 1e6 + gm * cs_m ** 2 / 1e6
    if not is_masked:
        g_cp, g_cs, g_rho = g_cp * mask, g_cs * mask, g_rho * mask
    return J, g_cp, g_cs, g_rho, gs


try:  # optional autograd wrapper (the Python counterpart of a ChainRules rrule)
    import torch

    class FwiOpFunction(torch.autograd.Function):
        """misfit = FwiOpFunction.apply(lam, mu, den, stf, ctx_obj, shot_ids);
        backward multiplies the operator's gradients by the incoming cotangent."""

        @staticmethod
        def forward(fctx, lam, mu, den, stf, op: FwiContext, shot_ids):
            J, gl, gm, gd, gs = op.misfit_grad(lam.detach().cpu().numpy(), mu.detach().cpu().numpy(),
                                               den.detach().cpu().numpy(), stf.detach().cpu().numpy(), shot_ids)
            g_stf = np.zeros(tuple(stf.shape))
            g_stf.reshape(-1, op.nSteps)[:gs.shape[0]] = gs
            fctx.save_for_backward(*(torch.from_numpy(a) for a in (gl, gm, gd, g_stf)))
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(fctx, dy):
            gl, gm, gd, gs = fctx.saved_tensors
            return gl * dy, gm * dy, gd * dy, gs * dy, None, None
except ImportError:  # pragma: no cover
    FwiOpFunction = None
