"""The BF16 tensor-core CNN kernels (csrc/cnn.cu) against a plain PyTorch
FP32 reference of the same ops on the same BF16-rounded operands.

Tolerances (relative L2): outputs stored in BF16 (8-bit mantissa) 1e-2;
FP32 outputs and FP32 weight gradients (FP32 accumulation of exactly
representable BF16 products, only the summation order differs) 1e-4."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

H, W = 64, 40  # Hz (multiple of 32), Wx (a ragged last tile of 8)


def _setup(fw):
    import torch
    from fwiflow_gb300.precond import CnnPreconditioner

    # FP32 reference: no TF32 rounding inside cuDNN / cuBLAS.
    torch.backends.cudnn.allow_tf32 = False
    torch.backends.cuda.matmul.allow_tf32 = False
    net = CnnPreconditioner(H, W, seed=3)
    torch.manual_seed(0)
    return net, torch


def _torch_img(t, c):
    """Kernel layout [x*Hz + z][C] -> torch NCHW with H = x, W = z (FP32)."""
    return t.float().reshape(W, H, -1)[:, :, :c].permute(2, 0, 1).unsqueeze(0)


def _torch_w(w, ci, co):
    """W[tap = ky*3 + kx][ci][co] -> torch (co, ci, kH = kx, kW = ky)."""
    import torch

    a = w[:, :ci, :co].reshape(3, 3, ci, co)  # [ky][kx][ci][co]
    return a.permute(3, 2, 1, 0).contiguous().to(torch.float32)


def _gelu(x):
    import torch

    return 0.5 * x * (1.0 + torch.erf(x / np.sqrt(2.0)))


def test_forward_layers_match_torch(gpu_lib, fw):
    net, torch = _setup(fw)
    F = torch.nn.functional
    x = torch.randn(5, H, W).numpy()
    net.stage(x)
    out = net.forward()
    ref = _torch_img(net.x0, 16)
    for k, (ci, co, cip, cop) in enumerate(net.LAYERS):
        wq = net.W[k].to(torch.bfloat16).float()
        zr = F.conv2d(ref, _torch_w(wq, cip, cop), bias=net.b[k][:cop], padding=1)
        if k < len(net.LAYERS) - 1:
            assert rel(_torch_img(net.z[k], cop).cpu(), zr.cpu()) < 1e-2, k
            assert rel(_torch_img(net.y[k], cop).cpu(), _gelu(zr).cpu()) < 1e-2, k
            ref = _torch_img(net.y[k], cop)  # continue from the kernel's own BF16 activations
        else:
            assert rel(_torch_img(out, co).cpu(), zr[:, :co].cpu()) < 1e-4


def test_backward_matches_torch_autograd(gpu_lib, fw):
    net, torch = _setup(fw)
    F = torch.nn.functional
    net.stage(torch.randn(5, H, W).numpy(), torch.randn(3, H, W).numpy(), np.ones((H, W)))
    out = net.forward()
    net.loss_and_grad(out)
    dy = net.dz[-1].clone()
    net.backward(dy)
    L = len(net.LAYERS)
    # Each layer in isolation on the kernel's own inputs and incoming gradient.
    for k in range(L):
        ci, co, cip, cop = net.LAYERS[k]
        xin = _torch_img(net.x0 if k == 0 else net.y[k - 1], cip).clone().requires_grad_(True)
        wq = _torch_w(net.W[k].to(torch.bfloat16).float(), cip, cop).requires_grad_(True)
        bq = net.b[k][:cop].clone().requires_grad_(True)
        z = F.conv2d(xin, wq, bias=bq, padding=1)
        g_out = _torch_img(dy if k == L - 1 else net.dz[k], cop)
        z.backward(g_out)
        gw_ref = wq.grad.permute(3, 2, 1, 0).reshape(9, cip, cop)  # back to [tap][ci][co]
        assert rel(net.gW[k].cpu(), gw_ref.cpu()) < 1e-4, ("dW", k)
        assert rel(net.gb[k][:cop].cpu(), bq.grad.cpu()) < 1e-4, ("db", k)
        if k > 0:  # data gradient through the previous layer's GELU
            zp = _torch_img(net.z[k - 1], cip)
            dgelu = 0.5 * (1.0 + torch.erf(zp / np.sqrt(2.0))) + zp * torch.exp(-0.5 * zp * zp) / np.sqrt(2 * np.pi)
            ref_dz = xin.grad * dgelu
            assert rel(_torch_img(net.dz[k - 1], cip).cpu(), ref_dz.cpu()) < 1e-2, ("dX", k)


def test_training_reduces_the_loss(gpu_lib, fw):
    """Fit a fixed smooth map of the inputs (the pseudo-Hessian target of
    random gradients and a positive illumination) on 4 samples."""
    from fwiflow_gb300.precond import features, pseudo_hessian_target

    net, torch = _setup(fw)
    rng = np.random.default_rng(1)
    zz, xx = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    mask = np.zeros((H, W))
    mask[4:-4, 4:-4] = 1.0
    samples = []
    for k in range(4):
        g = [rng.standard_normal((H, W)) for _ in range(3)]
        illum = np.exp(-((zz - 10.0 - 5 * k) ** 2 + (xx - 20.0) ** 2) / 300.0) + 0.05
        samples.append((features(*g, illum, mask), pseudo_hessian_target(*g, illum, mask), mask))
    before = net.evaluate(samples)
    net.train(samples, epochs=40, lr=2e-3)
    after = net.evaluate(samples)
    assert after < 0.5 * before, (before, after)


def test_tcgen05_convolutions_match_mma_sync(gpu_lib, fw):
    """The tcgen05 convolutions (tensor-memory accumulators) against the
    warp-level mma.sync ones, which match PyTorch above: same weights and
    input, every layer's pre-activation / activation and every data gradient
    (BF16, 1e-2), the FP32 output (1e-3); no kernel raised its error bit.
    The image height (96) is not a multiple of the 128-depth tcgen05 tile."""
    import torch
    from fwiflow_gb300.precond import CnnPreconditioner

    Hz, Wx = 96, 37
    a = CnnPreconditioner(Hz, Wx, seed=5, use_tc=True)
    b = CnnPreconditioner(Hz, Wx, seed=5, use_tc=False)
    torch.manual_seed(1)
    x = torch.randn(5, Hz, Wx).numpy()
    t = torch.randn(3, Hz, Wx).numpy()
    m = np.ones((Hz, Wx))
    for net in (a, b):
        net.stage(x, t, m)
        out = net.forward()
        net.loss_and_grad(out)
        net.backward(net.dz[-1])
    torch.cuda.synchronize()
    assert a.tc_error() == 0
    for k in range(len(a.z)):
        assert rel(a.z[k].float().cpu(), b.z[k].float().cpu()) < 1e-2, ("z", k)
        assert rel(a.y[k].float().cpu(), b.y[k].float().cpu()) < 1e-2, ("y", k)
    assert rel(a.out.cpu(), b.out.cpu()) < 1e-3
    for k in range(len(a.dz) - 1):
        assert rel(a.dz[k].float().cpu(), b.dz[k].float().cpu()) < 1e-2, ("dz", k)
    for k in range(len(a.gW)):
        assert rel(a.gW[k].cpu(), b.gW[k].cpu()) < 1e-2, ("dW", k)
