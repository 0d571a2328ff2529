"""The surrogate's training step against PyTorch autograd, and the sky-map pipeline end to end."""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_round(x):
    import torch

    return x + (x.to(torch.bfloat16).float() - x).detach()     # forward rounding, identity gradient


def test_gradients_match_autograd(cuda):
    """One forward/backward of the project's kernels == FP32 autograd of the same BF16 network."""
    import torch
    from excalibur_tool_gb300.surrogate.model import SkySurrogate

    torch.manual_seed(0)
    m = SkySurrogate(n_members=2, seed=3)
    for b in m.b:                                   # non-zero biases exercise the bias gradient
        b.copy_(torch.randn_like(b) * 0.1)
    m.b_head.copy_(torch.randn_like(m.b_head) * 0.1)
    B = 512
    rng = np.random.default_rng(0)
    uv = torch.as_tensor(rng.uniform(-1, 1, (B, 2)), device="cuda")
    t = torch.randn(B, 4, device="cuda")
    buf = m._buffers(B, 4)
    m.forward_backward(uv, t, buf)
    x0 = m._features(uv, B).float()
    torch.cuda.synchronize()
    for e in range(m.E):
        ws = [m.wb[l][e].float().clone().requires_grad_(True) for l in range(m.depth)]
        bs = [m.b[l][e].clone().requires_grad_(True) for l in range(m.depth)]
        wh = m.w_head[e].clone().requires_grad_(True)
        bh = m.b_head[e].clone().requires_grad_(True)
        h = x0
        for l in range(m.depth):
            z = _bf16_round(h @ ws[l].t() + bs[l])
            h = _bf16_round(z * torch.sigmoid(z))
        y = h @ wh.t() + bh
        loss = ((y - t) ** 2).mean()
        loss.backward()
        pairs = [(buf["gw"][l][e], ws[l].grad) for l in range(m.depth)] + \
                [(buf["gb"][l][e], bs[l].grad) for l in range(m.depth)] + \
                [(buf["gwh"][e], wh.grad), (buf["gbh"][e], bh.grad)]
        for got, want in pairs:
            got, want = got.flatten(), want.flatten()
            cos = float(torch.nn.functional.cosine_similarity(got, want, dim=0))
            rel = float((got - want).norm() / want.norm())
            assert cos > 0.999 and rel < 0.05, (cos, rel)
        assert abs(float(buf["loss"][e]) / (B * 4) - float(loss)) <= 1e-3 * float(loss)


def test_sky_map_pipeline_small(cuda):
    """Train on rays of a 32^3 lens + random field, fill a 128^2 map, audit it."""
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.surrogate.model import SkySurrogate
    from excalibur_tool_gb300.surrogate.sky import (ExitGeometry, Patch, born_features, compose, fill_sky_map,
                                                    observer_terms, traced_quantities, training_set)

    wl = workloads.flrw_patch(32, 2, device="cuda")
    cfg = dataclasses.replace(wl.cfg, precision="mixed")
    cz = workloads.lcdm()
    patch = Patch((cz._eta_at_a1, *workloads.OBSERVER), tuple(workloads.LENS - workloads.OBSERVER), 10.0)
    uv, y, feats, info = training_set(wl.metric, patch, 32768, cfg, seed=1)
    assert info["kept"] == 32768 and y.shape == (32768, 6) and feats.shape == (32768, 8)
    m = SkySurrogate(n_members=4, n_out=6, seed=0)
    rep = m.fit(uv, y, steps=400, batch=4096, lr=2e-3, log_every=50, extra=feats)
    first, last = rep.loss_curve[0][1], rep.loss_curve[-1][1]
    assert all(l1 < 0.3 * l0 for l0, l1 in zip(first, last)), (first, last)
    # held-out rays: the composed redshift tracks the traced one far better than the straight line does
    geo = ExitGeometry(patch, cfg.stop_box)
    hold = np.random.default_rng(9).uniform(-1, 1, (2048, 2))
    learned_ref, ref = traced_quantities(wl.metric, patch, hold, cfg, geo)
    import torch

    hf = born_features(wl.metric, patch, torch.as_tensor(hold, device="cuda"), cfg.stop_box).cpu().numpy()
    # the first-order line integrals explain the deflection and the exit offsets
    for j, col in ((1, 0), (2, 1), (4, 4), (5, 5)):
        cc = np.corrcoef(hf[:, j], learned_ref[:, col])[0, 1]
        assert abs(cc) > 0.9, (j, cc)
    mean, _ = m.predict(hold, extra=hf)
    terms = observer_terms(wl.metric, patch)
    pred = compose(wl.metric, patch, geo, hold, mean, terms)
    straight = compose(wl.metric, patch, geo, hold, np.zeros_like(mean), terms)
    assert np.median(np.abs(pred[:, 0] - ref[:, 0])) < 0.5 * np.median(np.abs(straight[:, 0] - ref[:, 0]))
    out, report = fill_sky_map(m, wl.metric, patch, cfg, n_side=128, std_threshold=1e-5, audit_fraction=0.05)
    assert out.shape == (128 * 128, 4) and np.isfinite(out).all()
    assert report["audit_pixels"] > 0 and report["pixels"] == 128 * 128
