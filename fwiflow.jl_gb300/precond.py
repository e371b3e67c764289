"""Learned gradient preconditioner: a 6-layer 3x3 CNN (32 channels, GELU)
that maps the raw lambda / mu / rho gradients and the source illumination of
an FWI iteration to a preconditioned update. It stands in for the diagonal
pseudo-Hessian preconditioner g / (H_diag + eps), with H_diag the source
illumination sum_t (vz^2 + vx^2), and is trained on (gradient,
illumination) pairs generated by the operator itself.

Output head: the network's 3 output channels are log-gains, one per
parameter, and the preconditioned update is g_c * exp(out_c). The training
target is the log of the pseudo-Hessian gain eps / (H_n + eps) (H_n the
illumination over its maximum in the mask), so the loss weighs the relative
gain error of a dark deep cell like that of a bright shallow one; regressing
g * gain directly lets the bright cells dominate.

Every arithmetic step of the network runs in the library's own sm_103a
kernels (csrc/cnn.cu: BF16 tensor-core convolutions with FP32 accumulation,
weight gradients, masked MSE, Adam); torch tensors only hold the device
memory, and the torch current stream is the one the kernels run on. The
convolutions with 32 outputs -- the first five layers and every data
gradient -- have two kernels: a persistent warp-specialised tcgen05 kernel
(TMA-fed input ring, tensor-memory accumulators; use_tc=True) and a
warp-level mma.sync kernel (the default). Measured on GB300 (32 -> 32
channels, benchmark_convs) the mma.sync kernel is the faster at every image
size tried (188 / 203 / 222 against 138 / 182 / 212 TFLOP/s on 352 x 832 /
608 x 1600 / 1120 x 3152 pixels): both are bound by the input loads and the
GELU epilogue, not the tensor pipe. The 3-output head and the weight
gradients always run on mma.sync.

Image layout of the kernels: pixel p = x * Hz + z (z fastest), channels
innermost; a model-shaped array (nz, nx) maps to it by transposition.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np

from . import _lib

N_IN, N_OUT, WIDTH, DEPTH = 5, 3, 32, 6
EPI_GELU, EPI_LINEAR_F32, EPI_DGELU = 0, 1, 2


def _torch():
    import torch

    return torch


def _rms(a, m):
    s = float(np.sqrt(np.mean(np.square(a[m])))) if m.any() else 0.0
    return s if s > 0 else 1.0


def gradient_scales(g_lambda, g_mu, g_den, mask) -> np.ndarray:
    """RMS of each raw gradient inside the mask: the per-channel unit of the
    network's inputs and outputs."""
    m = mask > 0
    return np.array([_rms(g, m) for g in (g_lambda, g_mu, g_den)])


EPS = 1e-3  # damping of the pseudo-Hessian, relative to its maximum inside the mask


def normalized_illumination(illum, mask) -> np.ndarray:
    """Illumination over its maximum inside the mask, clipped to [0, 1] (the
    cells next to the sources, outside the mask, are far brighter)."""
    m = mask > 0
    imax = float(illum[m].max()) if m.any() and illum[m].max() > 0 else 1.0
    return np.clip(illum / imax, 0.0, 1.0)


def features(g_lambda, g_mu, g_den, illum, mask) -> np.ndarray:
    """The 5 input channels, each (nz, nx): the three gradients in units of
    their RMS inside the mask, the normalised illumination, and its log10
    (floored at 1e-6) mapped to [0, 1]."""
    sc = gradient_scales(g_lambda, g_mu, g_den, mask)
    e = normalized_illumination(illum, mask)
    return np.stack([g_lambda / sc[0], g_mu / sc[1], g_den / sc[2], e, (np.log10(np.maximum(e, 1e-6)) + 6.0) / 6.0])


def illumination_gain(illum, mask, eps: float = EPS) -> np.ndarray:
    """The diagonal pseudo-Hessian preconditioner as a gain, in units of its
    value at the brightest masked cell: eps_n / (H_n + eps_n) with H_n the
    normalised illumination (so the gain is at most 1)."""
    return eps / (normalized_illumination(illum, mask) + eps)


def pseudo_hessian_target(g_lambda, g_mu, g_den, illum, mask, eps: float = EPS) -> np.ndarray:
    """Training target (3, nz, nx): the log of the pseudo-Hessian gain for
    each parameter (the update is then g_c * exp(target_c) = g_c / (H_diag +
    eps max H_diag) up to a constant), zero outside the mask."""
    lg = np.log(illumination_gain(illum, mask, eps)) * mask
    return np.stack([lg, lg, lg])


class CnnPreconditioner:
    """The network and its training state on one GPU, for images of
    Hz x Wx pixels (the padded grid: Hz = nz, Wx = nx)."""

    # (real in, real out, padded in, padded out) per layer
    LAYERS = [(N_IN, WIDTH, 16, 32)] + [(WIDTH, WIDTH, 32, 32)] * (DEPTH - 2) + [(WIDTH, N_OUT, 32, 16)]

    def __init__(self, Hz: int, Wx: int, seed: int = 0, device: int = 0, use_tc: bool = False):
        torch = _torch()
        self.use_tc = use_tc
        if Hz % 32:
            raise ValueError("Hz must be a multiple of 32")
        self.Hz, self.Wx, self.npix = Hz, Wx, Hz * Wx
        self.dev = torch.device("cuda", device)
        self.lib = _lib.load()
        rng = np.random.default_rng(seed)
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.W, self.b, self.mW, self.vW, self.mb, self.vb, self.gW, self.gb = ([] for _ in range(8))
        self.frag, self.frag_t = [], []
        for k, (ci, co, cip, cop) in enumerate(self.LAYERS):
            w = np.zeros((9, cip, cop), dtype=np.float32)
            std = np.sqrt(2.0 / (9 * ci)) * (0.1 if k == DEPTH - 1 else 1.0)
            w[:, :ci, :co] = rng.normal(0.0, std, (9, ci, co))
            self.W.append(torch.from_numpy(w).to(self.dev))
            self.b.append(torch.zeros(cop, **f32))
            for lst, shape in ((self.mW, w.shape), (self.vW, w.shape), (self.gW, w.shape), (self.mb, (cop,)),
                               (self.vb, (cop,)), (self.gb, (cop,))):
                lst.append(torch.zeros(shape, **f32))
            nfrag = 9 * (cip // 16) * (cop // 8) * 32
            self.frag.append(torch.empty(nfrag * 2, dtype=torch.int32, device=self.dev))
            self.frag_t.append(torch.empty(9 * (cop // 16) * (cip // 8) * 32 * 2, dtype=torch.int32, device=self.dev)
                               if cop % 16 == 0 and k > 0 else None)
        bf = dict(dtype=torch.bfloat16, device=self.dev)
        self.x0 = torch.zeros((self.npix, 16), **bf)
        self.z = [torch.zeros((self.npix, cop), **bf) for (_, _, _, cop) in self.LAYERS[:-1]]
        self.y = [torch.zeros((self.npix, cop), **bf) for (_, _, _, cop) in self.LAYERS[:-1]]
        self.out = torch.zeros((self.npix, 16), **f32)
        self.dz = [torch.zeros((self.npix, cop), **bf) for (_, _, _, cop) in self.LAYERS]
        self.ntiles = int(self.lib.fwigb_cnn_tile_count(Hz, Wx))
        self.part = torch.zeros(self.ntiles * 9 * 32 * 32, **f32)
        self.chunk = 1024
        self.bpart = torch.zeros(((self.npix + self.chunk - 1) // self.chunk) * 32, **f32)
        self.lpart = torch.zeros((self.npix + 255) // 256, **f32)
        self.target = torch.zeros((self.npix, N_OUT), **f32)
        self.mask = torch.zeros(self.npix, **f32)
        # tcgen05 operand packs: forward (layers with 32 outputs) and data gradient (layers 1..)
        self.tc = [torch.empty(9 * cip // 8 * 32 * 4, dtype=torch.int32, device=self.dev) if cop == 32 else None
                   for (_, _, cip, cop) in self.LAYERS]
        self.tc_t = [torch.empty(9 * cop // 8 * 32 * 4, dtype=torch.int32, device=self.dev) if k > 0 else None
                     for k, (_, _, cip, cop) in enumerate(self.LAYERS)]
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.step = 0
        self.pack()

    # -- plumbing
    def _s(self):
        return _torch().cuda.current_stream(self.dev).cuda_stream

    @staticmethod
    def _p(t):
        return None if t is None else t.data_ptr()

    def _ck(self, rc):
        if rc != 0:
            raise _lib.FwiError(rc, "CNN kernel launch failed")

    def to_image(self, chans: np.ndarray, c_pad: int, dtype):
        """(C, nz, nx) numpy -> device [npix][c_pad] in the kernels' layout."""
        torch = _torch()
        c = chans.shape[0]
        a = np.zeros((self.Wx, self.Hz, c_pad), dtype=np.float32)
        a[:, :, :c] = np.transpose(chans, (2, 1, 0))
        return torch.from_numpy(a.reshape(self.npix, c_pad)).to(device=self.dev, dtype=dtype)

    def from_image(self, t, c: int) -> np.ndarray:
        """Device [npix][C] -> (c, nz, nx) float64 numpy."""
        a = t.float().cpu().numpy().reshape(self.Wx, self.Hz, -1)[:, :, :c]
        return np.transpose(a, (2, 1, 0)).astype(np.float64)

    def pack(self) -> None:
        """Fragment-ordered BF16 copies of the FP32 weights (forward, and
        transposed for the data gradient)."""
        s = self._s()
        for k, (_, _, cip, cop) in enumerate(self.LAYERS):
            self._ck(self.lib.fwigb_cnn_pack_weights(self._p(self.W[k]), cip, cop, cip, cop, 0,
                                                     self._p(self.frag[k]), s))
            if self.frag_t[k] is not None:
                self._ck(self.lib.fwigb_cnn_pack_weights(self._p(self.W[k]), cip, cop, cip, cop, 1,
                                                         self._p(self.frag_t[k]), s))
            if self.tc[k] is not None:
                self._ck(self.lib.fwigb_cnn_pack_weights_tc(self._p(self.W[k]), cip, cop, cip, cop, 0,
                                                            self._p(self.tc[k]), s))
            if self.tc_t[k] is not None:
                self._ck(self.lib.fwigb_cnn_pack_weights_tc(self._p(self.W[k]), cip, cop, cip, cop, 1,
                                                            self._p(self.tc_t[k]), s))

    # -- network
    def forward(self, x_dev=None):
        """Runs the network on x_dev (or the staged input self.x0); returns the
        FP32 output [npix][16] (first 3 channels meaningful)."""
        s = self._s()
        x = self.x0 if x_dev is None else x_dev
        for k, (_, _, cip, cop) in enumerate(self.LAYERS):
            if k < DEPTH - 1:
                if self.use_tc:
                    self._ck(self.lib.fwigb_cnn_conv3x3_tc(self._p(x), self.Hz, self.Wx, cip, EPI_GELU,
                                                           self._p(self.tc[k]), self._p(self.b[k]),
                                                           self._p(self.y[k]), self._p(self.z[k]), None,
                                                           self._p(self.err), s))
                else:
                    self._ck(self.lib.fwigb_cnn_conv3x3(self._p(x), self.Hz, self.Wx, cip, cop, EPI_GELU,
                                                        self._p(self.frag[k]), self._p(self.b[k]),
                                                        self._p(self.y[k]), None, self._p(self.z[k]), None, s))
                x = self.y[k]
            else:
                self._ck(self.lib.fwigb_cnn_conv3x3(self._p(x), self.Hz, self.Wx, cip, cop, EPI_LINEAR_F32,
                                                    self._p(self.frag[k]), self._p(self.b[k]), None,
                                                    self._p(self.out), None, None, s))
        return self.out

    def backward(self, dy) -> None:
        """Gradients of all weights and biases from dL/d(output) dy (BF16
        [npix][16]), after forward on the same input; into self.gW / self.gb."""
        s = self._s()
        dz = dy
        for k in range(DEPTH - 1, -1, -1):
            _, _, cip, cop = self.LAYERS[k]
            xin = self.x0 if k == 0 else self.y[k - 1]
            self._ck(self.lib.fwigb_cnn_wgrad_partials(self._p(xin), self._p(dz), self.Hz, self.Wx, cip, cop,
                                                       self._p(self.part), s))
            self._ck(self.lib.fwigb_cnn_reduce_partials(self._p(self.part), self.ntiles, 9 * cip * cop,
                                                        self._p(self.gW[k]), s))
            self._ck(self.lib.fwigb_cnn_bias_partials(self._p(dz), self.npix, cop, self.chunk, self._p(self.bpart),
                                                      s))
            nb = (self.npix + self.chunk - 1) // self.chunk
            self._ck(self.lib.fwigb_cnn_reduce_partials(self._p(self.bpart), nb, cop, self._p(self.gb[k]), s))
            if k > 0:  # data gradient through the previous layer's GELU
                if self.use_tc:
                    self._ck(self.lib.fwigb_cnn_conv3x3_tc(self._p(dz), self.Hz, self.Wx, cop, EPI_DGELU,
                                                           self._p(self.tc_t[k]), None, self._p(self.dz[k - 1]),
                                                           None, self._p(self.z[k - 1]), self._p(self.err), s))
                else:
                    self._ck(self.lib.fwigb_cnn_conv3x3(self._p(dz), self.Hz, self.Wx, cop, cip, EPI_DGELU,
                                                        self._p(self.frag_t[k]), None, self._p(self.dz[k - 1]),
                                                        None, None, self._p(self.z[k - 1]), s))
                dz = self.dz[k - 1]

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        s = self._s()
        self.step += 1
        for k in range(DEPTH):
            for w, g, m, v in ((self.W[k], self.gW[k], self.mW[k], self.vW[k]),
                               (self.b[k], self.gb[k], self.mb[k], self.vb[k])):
                self._ck(self.lib.fwigb_cnn_adam(self._p(w), self._p(g), self._p(m), self._p(v), w.numel(), lr,
                                                 beta1, beta2, eps, self.step, s))
        self.pack()

    def loss_and_grad(self, out) -> float:
        """Masked MSE of the output against the staged target; leaves
        dL/d(output) in self.dz[-1]."""
        torch = _torch()
        s = self._s()
        cnt = float(self.mask.sum().item()) * N_OUT
        self._ck(self.lib.fwigb_cnn_mse_grad(self._p(out), self._p(self.target), self._p(self.mask), self.npix, 16,
                                             N_OUT, 1.0 / max(cnt, 1.0), self._p(self.dz[-1]), self._p(self.lpart), s))
        return float(torch.sum(self.lpart).item()) / max(cnt, 1.0)

    # -- data
    def stage(self, feats: np.ndarray, target: Optional[np.ndarray] = None, mask: Optional[np.ndarray] = None):
        torch = _torch()
        self.x0.copy_(self.to_image(feats, 16, torch.bfloat16))
        if target is not None:
            self.target.copy_(self.to_image(target, N_OUT, torch.float32))
        if mask is not None:
            self.mask.copy_(torch.from_numpy(np.ascontiguousarray(mask.T.reshape(-1), dtype=np.float32)).to(self.dev))

    def train(self, samples: Sequence[tuple], epochs: int, lr: float = 1e-3, seed: int = 0,
              log: Optional[List[float]] = None) -> List[float]:
        """Adam on (features, target, mask) samples, one sample per step,
        shuffled each epoch. Returns the mean loss of every epoch."""
        rng = np.random.default_rng(seed)
        hist = []
        for _ in range(epochs):
            tot = 0.0
            for i in rng.permutation(len(samples)):
                f, t, m = samples[i]
                self.stage(f, t, m)
                out = self.forward()
                tot += self.loss_and_grad(out)
                self.backward(self.dz[-1])
                self.adam(lr)
            hist.append(tot / max(len(samples), 1))
            if log is not None:
                log.append(hist[-1])
        return hist

    def evaluate(self, samples: Sequence[tuple]) -> float:
        tot = 0.0
        for f, t, m in samples:
            self.stage(f, t, m)
            tot += self.loss_and_grad(self.forward())
        return tot / max(len(samples), 1)

    def predict(self, feats: np.ndarray) -> np.ndarray:
        """Network output (3, nz, nx) for the features (5, nz, nx), in the
        units of the input channels."""
        self.stage(feats)
        return self.from_image(self.forward(), N_OUT)

    def precondition(self, g_lambda, g_mu, g_den, illum, mask) -> np.ndarray:
        """Preconditioned lambda / mu / rho gradients (3, nz, nx): each
        gradient times exp of its predicted log-gain, zero outside the mask."""
        out = self.predict(features(g_lambda, g_mu, g_den, illum, mask))
        gain = np.exp(np.clip(out, -30.0, 5.0))
        return np.stack([g_lambda, g_mu, g_den]) * gain * mask

    def state(self) -> dict:
        return {f"W{k}": self.W[k].cpu().numpy() for k in range(DEPTH)} | \
               {f"b{k}": self.b[k].cpu().numpy() for k in range(DEPTH)}

    def tc_error(self) -> int:
        """Error bits the tcgen05 kernels raised (bit 1: a bounded wait gave up)."""
        return int(self.err.item())

    def load_state(self, st: dict) -> None:
        torch = _torch()
        for k in range(DEPTH):
            self.W[k].copy_(torch.from_numpy(np.asarray(st[f"W{k}"], dtype=np.float32)))
            self.b[k].copy_(torch.from_numpy(np.asarray(st[f"b{k}"], dtype=np.float32)))
        self.pack()


def benchmark_convs(Hz: int = 352, Wx: int = 832, reps: int = 50, device: int = 0) -> dict:
    """Tensor throughput of the 32 -> 32 channel convolution (forward, GELU)
    on one Hz x Wx image: tcgen05 and warp-level mma.sync kernels, CUDA
    events on the current stream, 2 * 9 * 32 * 32 flops per pixel."""
    torch = _torch()
    net = CnnPreconditioner(Hz, Wx, seed=0, device=device)
    x = torch.randn(net.npix, 32, device=net.dev).to(torch.bfloat16)
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    s = net._s()
    flops = 2.0 * 9 * 32 * 32 * net.npix
    out = {"image": [Hz, Wx], "flops_per_call": flops}
    for name in ("tcgen05", "mma_sync"):
        def call():
            if name == "tcgen05":
                net._ck(net.lib.fwigb_cnn_conv3x3_tc(x.data_ptr(), Hz, Wx, 32, EPI_GELU, net.tc[1].data_ptr(),
                                                     net.b[1].data_ptr(), y.data_ptr(), z.data_ptr(), None,
                                                     net.err.data_ptr(), s))
            else:
                net._ck(net.lib.fwigb_cnn_conv3x3(x.data_ptr(), Hz, Wx, 32, 32, EPI_GELU, net.frag[1].data_ptr(),
                                                  net.b[1].data_ptr(), y.data_ptr(), None, z.data_ptr(), None, s))
        for _ in range(5):
            call()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            call()
        e1.record()
        torch.cuda.synchronize()
        us = e0.elapsed_time(e1) * 1e3 / reps
        out[name] = {"us_per_call": us, "tflops": flops / us / 1e6}
    out["tc_error"] = net.tc_error()
    return out

