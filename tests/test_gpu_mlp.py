"""Surrogate kernels against plain PyTorch FP32 references of the same ops.

The GEMM is a tcgen05 BF16 kernel with FP32 accumulation: with BF16 inputs
every product is exact in FP32, so it matches torch's FP32 matmul of the same
BF16 values up to summation order (tolerance 1e-5 of the largest |entry|);
BF16 outputs are compared at one BF16 rounding (2^-8 relative).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BF16_REL = 2.0 ** -7     # two roundings (the kernel's and the reference's) of a bf16 value


def _rand(shape, seed, scale=1.0):
    import torch

    g = torch.Generator(device="cpu").manual_seed(seed)
    return (torch.randn(shape, generator=g) * scale).to(torch.bfloat16).cuda()


def _close_bf16(got, want, rel=BF16_REL):
    got, want = got.float(), want.float()
    err = (got - want).abs()
    tol = rel * want.abs() + rel * want.abs().max() * 1e-2 + 1e-30
    assert bool((err <= tol).all()), float((err / (want.abs() + 1e-30)).max())


@pytest.mark.parametrize("E,M,N,K", [(1, 128, 256, 256), (1, 300, 256, 256), (1, 1, 16, 64), (3, 257, 48, 128),
                                     (2, 1000, 256, 512)])
def test_gemm_f32_matches_torch(cuda, E, M, N, K):
    import torch
    from excalibur_tool_gb300.surrogate import kernels as Kn

    a, b = _rand((E, M, K), 1), _rand((E, N, K), 2)
    c = torch.full((E, M, N), float("nan"), device="cuda")
    Kn.gemm(a, b, epilogue="f32", c=c)
    ref = torch.bmm(a.float(), b.float().transpose(1, 2))
    torch.cuda.synchronize()
    assert torch.isfinite(c).all()
    assert float((c - ref).abs().max()) <= 1e-5 * float(ref.abs().max())
    assert Kn.error_count() == 0


def test_gemm_bias_silu_and_transpose(cuda):
    import torch
    from excalibur_tool_gb300.surrogate import kernels as Kn

    E, M, N, K = 2, 200, 256, 256
    a, b = _rand((E, M, K), 3), _rand((E, N, K), 4, 0.1)
    bias = torch.randn(E, N, device="cuda") * 0.1
    z = torch.empty((E, M, N), dtype=torch.bfloat16, device="cuda")
    h = torch.empty_like(z)
    ldt = 256
    ht = torch.zeros((E, N, ldt), dtype=torch.bfloat16, device="cuda")
    Kn.gemm(a, b, epilogue="bias_silu", bias=bias, c=z, c2=h, ct=ht)
    zr = torch.bmm(a.float(), b.float().transpose(1, 2)) + bias[:, None, :]
    torch.cuda.synchronize()
    _close_bf16(z, zr)
    zq = z.float()
    _close_bf16(h, zq * torch.sigmoid(zq))
    assert torch.equal(ht[:, :, :M], h.transpose(1, 2))


def test_gemm_dsilu(cuda):
    import torch
    from excalibur_tool_gb300.surrogate import kernels as Kn

    E, M, N, K = 1, 333, 256, 256
    a, b = _rand((E, M, K), 5), _rand((E, N, K), 6, 0.1)
    zin = _rand((E, M, N), 7)
    d = torch.empty((E, M, N), dtype=torch.bfloat16, device="cuda")
    dt = torch.zeros((E, N, 384), dtype=torch.bfloat16, device="cuda")
    Kn.gemm(a, b, epilogue="dsilu", z_in=zin, c=d, ct=dt)
    zf = zin.float()
    sg = torch.sigmoid(zf)
    ref = torch.bmm(a.float(), b.float().transpose(1, 2)) * (sg * (1 + zf * (1 - sg)))
    torch.cuda.synchronize()
    _close_bf16(d, ref)
    assert torch.equal(dt[:, :, :M], d.transpose(1, 2))


@pytest.mark.parametrize("K,N,shared_a", [(256, 256, False), (256, 256, True), (128, 48, False)])
def test_gemm_many_tiles(cuda, K, N, shared_a):
    """More row tiles than the GPU holds at once (3 members x 313 tiles, the last one ragged),
    every epilogue against torch, and an A shared by the members (the first inference layer)."""
    import torch
    from excalibur_tool_gb300.surrogate import kernels as Kn

    E, M = 3, 40_000                                    # 3 x 313 tiles >= 4 x 152
    a = _rand((M, K), 11) if shared_a else _rand((E, M, K), 11)
    b = _rand((E, N, K), 12, 0.1)
    af = a.float().expand(E, M, K) if shared_a else a.float()
    acc = torch.bmm(af, b.float().transpose(1, 2))
    c = torch.full((E, M, N), float("nan"), device="cuda")
    Kn.gemm(a, b, epilogue="f32", c=c)
    torch.cuda.synchronize()
    assert torch.isfinite(c).all() and float((c - acc).abs().max()) <= 1e-5 * float(acc.abs().max())
    bias = torch.randn(E, N, device="cuda") * 0.1
    z = torch.empty((E, M, N), dtype=torch.bfloat16, device="cuda")
    h = torch.empty_like(z)
    ht = torch.zeros((E, N, M + 64), dtype=torch.bfloat16, device="cuda")
    Kn.gemm(a, b, epilogue="bias_silu", bias=bias, c=z, c2=h, ct=ht)
    torch.cuda.synchronize()
    _close_bf16(z, acc + bias[:, None, :])
    zq = z.float()
    _close_bf16(h, zq * torch.sigmoid(zq))
    assert torch.equal(ht[:, :, :M], h.transpose(1, 2)) and not bool(ht[:, :, M:].any())
    if not shared_a:
        zin = _rand((E, M, N), 13)
        d = torch.empty((E, M, N), dtype=torch.bfloat16, device="cuda")
        dt = torch.zeros((E, N, M), dtype=torch.bfloat16, device="cuda")
        Kn.gemm(a, b, epilogue="dsilu", z_in=zin, c=d, ct=dt)
        zf = zin.float()
        sg = torch.sigmoid(zf)
        torch.cuda.synchronize()
        _close_bf16(d, acc * (sg * (1 + zf * (1 - sg))))
        assert torch.equal(dt, d.transpose(1, 2))
    assert Kn.error_count() == 0


def test_gemm_split_k_weight_gradient(cuda):
    """dW = dZ^T . X with K = batch rows, split over CTAs and reduced."""
    import torch
    from excalibur_tool_gb300.surrogate import kernels as Kn

    E, R, C, K, S = 2, 256, 256, 4096, 16
    a, b = _rand((E, R, K), 8), _rand((E, C, K), 9)
    part = torch.empty((E, S, R, C), device="cuda")
    Kn.gemm(a, b, epilogue="splitk", c=part, k_splits=S)
    out = torch.empty((E, R, C), device="cuda")
    Kn.reduce_splits(part, out)
    ref = torch.bmm(a.float(), b.float().transpose(1, 2))
    torch.cuda.synchronize()
    assert float((out - ref).abs().max()) <= 1e-5 * float(ref.abs().max())


def test_features_match_formula(cuda):
    import torch
    from excalibur_tool_gb300.surrogate import kernels as Kn

    n, npad, nf = 1000, 1024, 64
    rng = np.random.default_rng(0)
    dirs = np.stack([rng.uniform(1.3, 1.8, n), rng.uniform(-0.2, 0.2, n)], 1)
    center, scale = (1.55, 0.0), (1 / 0.25, 1 / 0.2)
    out = torch.full((npad, 4 * nf), 7.0, dtype=torch.bfloat16, device="cuda")
    Kn.features(torch.as_tensor(dirs).cuda(), npad, nf, center, scale, out)
    u = (dirs[:, 0] - center[0]) * scale[0]
    v = (dirs[:, 1] - center[1]) * scale[1]
    k = np.arange(1, nf + 1)
    ref = np.concatenate([np.sin(np.pi * k * u[:, None]), np.cos(np.pi * k * u[:, None]),
                          np.sin(np.pi * k * v[:, None]), np.cos(np.pi * k * v[:, None])], 1)
    got = out.float().cpu().numpy()
    assert np.abs(got[:n] - ref).max() <= 2 ** -8 + 1e-5
    assert (got[n:] == 0).all()


def test_head_forward_backward_matches_autograd(cuda):
    import torch
    from excalibur_tool_gb300.surrogate import kernels as Kn

    E, M, W, NO = 2, 777, 256, 4
    h = _rand((E, M, W), 10)
    z = _rand((E, M, W), 11)
    w = torch.randn(E, NO, W, device="cuda") * 0.05
    b = torch.randn(E, NO, device="cuda") * 0.1
    t = torch.randn(M, NO, device="cuda")
    y = torch.empty(E, M, NO, device="cuda")
    dh = torch.empty((E, M, W), dtype=torch.bfloat16, device="cuda")
    dht = torch.zeros((E, W, 800), dtype=torch.bfloat16, device="cuda")
    dw = torch.zeros(E, NO, W, device="cuda")
    db = torch.zeros(E, NO, device="cuda")
    loss = torch.zeros(E, device="cuda")
    Kn.head(h, w, b, y=y, targets=t, z=z, dh=dh, dht=dht, dw=dw, db=db, loss=loss)
    # reference: torch autograd in FP32 on the same BF16 inputs
    hf = h.float().requires_grad_(True)
    wf = w.clone().requires_grad_(True)
    bf = b.clone().requires_grad_(True)
    yr = torch.einsum("emk,enk->emn", hf, wf) + bf[:, None, :]
    lr = ((yr - t[None]) ** 2).mean(dim=(1, 2))
    lr.sum().backward()
    zf = z.float()
    sg = torch.sigmoid(zf)
    dref = hf.grad * (sg * (1 + zf * (1 - sg)))
    torch.cuda.synchronize()
    assert float((y - yr).abs().max()) <= 1e-4 * float(yr.abs().max())
    assert torch.allclose(loss / (M * NO), lr.detach(), rtol=1e-4)
    assert torch.allclose(dw, wf.grad, rtol=1e-3, atol=1e-6)
    assert torch.allclose(db, bf.grad, rtol=1e-3, atol=1e-7)
    _close_bf16(dh, dref)
    assert torch.equal(dht[:, :, :M], dh.transpose(1, 2))


def test_row_sums_and_adam(cuda):
    import torch
    from excalibur_tool_gb300.surrogate import kernels as Kn

    x = _rand((256, 1000), 12)
    out = torch.empty(256, device="cuda")
    Kn.row_sums(x, 900, out)
    torch.cuda.synchronize()
    assert torch.allclose(out, x.float()[:, :900].sum(1), rtol=1e-4, atol=1e-3)

    E, R, Cc = 2, 16, 32
    p = torch.randn(E * R * Cc, device="cuda")
    g = torch.randn_like(p)
    m1 = torch.randn_like(p) * 0.1
    m2 = torch.rand_like(p) * 0.1
    ref_p, ref_m1, ref_m2 = p.clone(), m1.clone(), m2.clone()
    pb = torch.empty(E * R * Cc, dtype=torch.bfloat16, device="cuda")
    pt = torch.empty(E * R * Cc, dtype=torch.bfloat16, device="cuda")
    Kn.adam(p, g, m1, m2, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, t=5, p_bf16=pb, pt_bf16=pt, shape=(R, Cc))
    ref_m1 = 0.9 * ref_m1 + 0.1 * g
    ref_m2 = 0.999 * ref_m2 + 0.001 * g * g
    ref_p = ref_p - 1e-3 * (ref_m1 / (1 - 0.9 ** 5)) / (torch.sqrt(ref_m2 / (1 - 0.999 ** 5)) + 1e-8)
    torch.cuda.synchronize()
    assert torch.allclose(p, ref_p, rtol=1e-5, atol=1e-6)
    assert torch.equal(pb, p.to(torch.bfloat16))
    assert torch.equal(pt.view(E, Cc, R), pb.view(E, R, Cc).transpose(1, 2))
