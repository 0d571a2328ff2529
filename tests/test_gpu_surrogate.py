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


def test_gradients_match_fp64_cpu_reference(cuda):
    """One forward/backward of the project's kernels against the FP64 CPU reference
    (oracle/surrogate_ref.py) of the same network, on the kernels' own bf16 features.

    Tolerances, from what bf16 storage and fp32 sums leave: the reference rounds to bf16 at
    the kernels' storage points (Z, H, dZ) and is otherwise exact, so the kernels differ from it
    by their fp32 accumulation (~1e-6 relative per sum) and by the bf16 roundings that this moves
    across a midpoint (about 2e-6 / 2^-8 = 3e-4 of the stored values, each by one bf16 ulp,
    2^-8). Over a weight gradient (a sum of 512 products) that is well under 2e-3 of its norm;
    a wrong bias, SiLU-derivative or head term is off by O(1). Against the exact-arithmetic
    gradient (no bf16 rounding), storage alone puts the kernels ~2^-8 away, so the bf16
    reference must be the much closer of the two."""
    import torch
    from excalibur_tool_gb300.surrogate.model import SkySurrogate
    from oracle import surrogate_ref as R

    torch.manual_seed(0)
    m = SkySurrogate(n_members=2, seed=3)
    for b in m.b:
        b.copy_(torch.randn_like(b) * 0.1)
    m.b_head.copy_(torch.randn_like(m.b_head) * 0.1)
    B = 512
    rng = np.random.default_rng(0)
    uv = torch.as_tensor(rng.uniform(-1, 1, (B, 2)), device="cuda")
    t = torch.randn(B, 4, device="cuda")
    buf = m._buffers(B, 4)
    m.forward_backward(uv, t, buf)
    x0 = m._features(uv, B).double().cpu().numpy()
    torch.cuda.synchronize()
    # the features: bf16 of the float64 formula, but where the fp32 phase (k u rounded to fp32,
    # ~1.2e-5 absolute in sin for k = 64) moves a value across a bf16 rounding midpoint
    f64 = R.features(uv.cpu().numpy(), m.nf)
    mism = x0 != R.bf16_round(f64)
    assert mism.mean() < 1e-2 and np.all(np.abs(x0 - f64) <= 2.0 ** -8 * np.abs(f64) + 3e-5)
    tt = t.double().cpu().numpy()
    for e in range(m.E):
        W = [m.wb[l][e].double().cpu().numpy() for l in range(m.depth)]
        bb = [m.b[l][e].double().cpu().numpy() for l in range(m.depth)]
        Wh, bh = m.w_head[e].double().cpu().numpy(), m.b_head[e].double().cpu().numpy()
        ref = R.forward_backward(x0, W, bb, Wh, bh, tt, bf16=True)
        exact = R.forward_backward(x0, W, bb, Wh, bh, tt, bf16=False)
        got = {"gw": [buf["gw"][l][e].double().cpu().numpy() for l in range(m.depth)],
               "gb": [buf["gb"][l][e].double().cpu().numpy() for l in range(m.depth)],
               "gwh": buf["gwh"][e].double().cpu().numpy(), "gbh": buf["gbh"][e].double().cpu().numpy()}
        pairs = [(got["gw"][l], ref["gw"][l], exact["gw"][l], f"gw{l}") for l in range(m.depth)] + \
                [(got["gb"][l], ref["gb"][l], exact["gb"][l], f"gb{l}") for l in range(m.depth)] + \
                [(got["gwh"], ref["gwh"], exact["gwh"], "gwh"), (got["gbh"], ref["gbh"], exact["gbh"], "gbh")]
        for g, r, x, name in pairs:
            rel = np.linalg.norm(g - r) / np.linalg.norm(r)
            rel_exact = np.linalg.norm(g - x) / np.linalg.norm(x)
            assert rel <= 2e-3, (e, name, rel)
            assert rel <= 0.5 * rel_exact or rel <= 1e-5, (e, name, rel, rel_exact)
        assert abs(float(buf["loss"][e]) - ref["loss"]) <= 1e-5 * ref["loss"]


def test_fused_inference_matches_layer_by_layer(cuda):
    """exc_mlp_infer (the whole forward pass of every member in one kernel, activations kept in
    shared memory) against the layer-by-layer kernels: the hidden activations take the same
    bf16 roundings, so only the head's fp32 sum differs in order -- agreement to ~1e-6 of the
    outputs' scale; several tiles per CTA and a row count that is not a multiple of 128."""
    import torch
    from excalibur_tool_gb300.surrogate.model import SkySurrogate

    torch.manual_seed(1)
    m = SkySurrogate(n_members=3, seed=7, n_out=6)
    for b in m.b:
        b.copy_(torch.randn_like(b) * 0.1)
    m.b_head.copy_(torch.randn_like(m.b_head) * 0.1)
    rng = np.random.default_rng(3)
    for n in (1000, 152 * 128 * 3 + 77):
        uv = torch.as_tensor(rng.uniform(-1, 1, (n, 2)), device="cuda")
        a = m.predict_members(uv, fused=True)
        b = m.predict_members(uv, fused=False)
        torch.cuda.synchronize()
        scale = float(b.abs().max())
        assert a.shape == b.shape and bool(torch.isfinite(a).all())
        assert float((a - b).abs().max()) <= 1e-5 * scale, (n, float((a - b).abs().max()), scale)
    from excalibur_tool_gb300 import _native as N
    import ctypes as C

    cnt = C.c_uint32(0)
    N.check(N.load().exc_mlp_error_count(C.byref(cnt)), "exc_mlp_error_count")
    assert cnt.value == 0


@pytest.mark.parametrize("E,depth,n_out,m", [(1, 1, 1, 128), (3, 1, 8, 152 * 128 * 2 + 128), (2, 2, 3, 1280),
                                           (5, 3, 6, 152 * 128 * 2), (4, 4, 7, 152 * 128 + 256)])
def test_fused_inference_shapes_match_layer_by_layer(cuda, E, depth, n_out, m):
    """exc_mlp_infer for other ensemble sizes, depths and head widths (one layer a member -- every
    layer is a head --, fewer tiles than SMs, several tiles per CTA) against the layer-by-layer
    kernels on random operands: the same bf16 activations, the head summed in another order."""
    import torch
    from excalibur_tool_gb300.surrogate import kernels as Kn

    g = torch.Generator(device="cuda").manual_seed(E * 100 + depth * 10 + n_out)
    x = (torch.rand((m, 256), generator=g, device="cuda") * 2 - 1).to(torch.bfloat16)
    w = (torch.randn((depth, E, 256, 256), generator=g, device="cuda") * 0.08).to(torch.bfloat16)
    b = torch.randn((depth, E, 256), generator=g, device="cuda") * 0.1
    wh = torch.randn((E, n_out, 256), generator=g, device="cuda") * 0.1
    bh = torch.randn((E, n_out), generator=g, device="cuda") * 0.1
    y = torch.full((E, m, n_out), float("nan"), device="cuda")
    Kn.infer(x, w, b, wh, bh, y)
    inp = x
    for l in range(depth):
        o = torch.empty((E, m, 256), dtype=torch.bfloat16, device="cuda")
        Kn.gemm(inp, w[l].contiguous(), epilogue="bias_silu", bias=b[l].contiguous(), c2=o)
        inp = o
    yr = torch.empty((E, m, n_out), device="cuda")
    Kn.head(inp, wh, bh, y=yr)
    torch.cuda.synchronize()
    scale = float(yr.abs().max())
    assert bool(torch.isfinite(y).all())
    assert float((y - yr).abs().max()) <= 1e-5 * scale, float((y - yr).abs().max())
    from excalibur_tool_gb300 import _native as N
    import ctypes as C

    cnt = C.c_uint32(0)
    N.check(N.load().exc_mlp_error_count(C.byref(cnt)), "exc_mlp_error_count")
    assert cnt.value == 0


def test_graphed_training_equals_eager(cuda):
    """Training steps replayed from a captured CUDA graph (one multi-tensor Adam launch reading
    the step's schedule on the device) follow the eager loop (same batches, per-tensor Adam
    launches with host scalars). The head kernel sums its weight gradients with float atomics,
    so two eager runs already differ in the last bits; the graphed run must differ from the
    eager one no more than a second eager run does, within a small factor."""
    import torch
    from excalibur_tool_gb300.surrogate.model import SkySurrogate

    rng = np.random.default_rng(4)
    uv = rng.uniform(-1, 1, (3000, 2))
    y = np.stack([np.sin(3 * uv[:, 0]) * uv[:, 1], uv[:, 0] ** 2, np.cos(2 * uv[:, 1]), uv[:, 0] * uv[:, 1]], 1)
    runs = []
    for graph in (False, False, True):
        m = SkySurrogate(n_members=2, seed=5)
        w0 = [p.clone() for p in m.params()]
        # 40 steps of 512 rows: 16 eager, 16 replayed from the graph, 8 eager (the remainder),
        # an epoch boundary every 5 steps
        rep = m.fit(uv, y, steps=40, batch=512, lr=3e-3, log_every=10, graph=graph, graph_steps=16)
        torch.cuda.synchronize()
        assert rep.steps == 40 and len(rep.loss_curve) >= 4
        runs.append(([p.clone() for p in m.params()], w0, rep.final_loss))
    (e1, w0, l1), (e2, _, _), (g, _, lg) = runs
    for a, b, c, p0 in zip(e1, e2, g, w0):
        moved = float((a - p0).norm())
        noise = float((a - b).norm())
        assert moved > 0
        assert float((c - a).norm()) <= 10 * noise + 1e-3 * moved
    assert np.allclose(lg, l1, rtol=0.05)


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


def _patch_metric(n, seed, slow):
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.core.constants import one_Mpc
    from excalibur_tool_gb300.grid.grid import Grid
    from excalibur_tool_gb300.grid.interpolator import Interpolator
    from excalibur_tool_gb300.grid.interpolator_4d_fast import InterpolatorFast
    from excalibur_tool_gb300.metrics.perturbed_flrw_metric_fast import PerturbedFLRWMetricFast
    from excalibur_tool_gb300.objects.fields import lens_plus_grf

    cz = workloads.lcdm()
    phi = lens_plus_grf(n, workloads.BOX, workloads.LENS_MASS, 5 * one_Mpc, workloads.LENS, seed=seed)
    grid = Grid((n,) * 3, (workloads.BOX / n,) * 3, (0.0, 0.0, 0.0))
    grid.add_field("Phi", phi)
    ip = Interpolator(grid) if slow else InterpolatorFast(grid, boundary="periodic")
    return PerturbedFLRWMetricFast(cz.a_of_eta, grid, ip, adot_of_eta=cz.adot_of_eta)


def test_smooth_gradient_map_is_learnable(cuda):
    """The base-node gradient of the fast interpolators makes the traced redshift map rough
    at the pixel scale (RK4 stage points switch cells as the direction moves); the slow
    Interpolator's continuous gradient does not, and on its map the surrogate's held-out
    redshift error falls below 1e-7."""
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.core.constants import one_Mpc
    from excalibur_tool_gb300.surrogate.model import SkySurrogate
    from excalibur_tool_gb300.surrogate.sky import (ExitGeometry, Patch, compose, observer_terms,
                                                    traced_quantities, training_set)
    from excalibur_tool_gb300.trace import TraceConfig

    cz = workloads.lcdm()
    patch = Patch((cz._eta_at_a1, *workloads.OBSERVER), tuple(workloads.LENS - workloads.OBSERVER), 10.0)
    hi = 980 * one_Mpc   # inside the slow class's bounds [0, 63 spacings) of a 64^3 grid
    dl = workloads.DLAMBDA
    cfg = TraceConfig(stepper="rk4", precision="fp64_fast", dt=dl, dt_min=dl, dt_max=dl, max_steps=2 ** 62,
                      max_iter=100_000, stop_box=((0, 0, 0), (hi, hi, hi)), a_stop=0.5)
    geo = ExitGeometry(patch, cfg.stop_box)
    t = (np.arange(1024) + 0.5) / 1024 * 2 - 1
    A, B = np.meshgrid(t[480:544], t[480:544], indexing="ij")
    block = np.stack([A.reshape(-1), B.reshape(-1)], 1)
    rough = {}
    for slow in (False, True):
        metric = _patch_metric(64, 1, slow)
        _, v = traced_quantities(metric, patch, block, cfg, geo)
        z = v[:, 0].reshape(64, 64)
        assert np.isfinite(z).all()
        d2 = np.concatenate([(z[2:] - 2 * z[1:-1] + z[:-2]).ravel(), (z[:, 2:] - 2 * z[:, 1:-1] + z[:, :-2]).ravel()])
        rough[slow] = float(np.sqrt(np.mean(d2 ** 2)))
    print("adjacent-pixel second differences of z (rms): base-node", rough[False], "slow", rough[True])
    assert rough[False] > 10 * rough[True]
    metric = _patch_metric(64, 1, True)
    uv, y, _, info = training_set(metric, patch, 65536, cfg, seed=1)
    assert info["kept"] == 65536
    m = SkySurrogate(n_members=4, n_out=6, seed=0)
    m.fit(uv, y, steps=3000, batch=8192, lr=2e-3, log_every=500)
    hold = np.random.default_rng(9).uniform(-1, 1, (4096, 2))
    _, ref = traced_quantities(metric, patch, hold, cfg, geo)
    mean, _ = m.predict(hold)
    pred = compose(metric, patch, geo, hold, mean, observer_terms(metric, patch))
    err = np.abs(pred[:, 0] - ref[:, 0])
    print("held-out |dz|: median", np.median(err), "p95", np.percentile(err, 95), "max", err.max())
    assert np.median(err) < 1e-7
