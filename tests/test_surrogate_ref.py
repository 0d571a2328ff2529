"""The FP64 CPU reference of the surrogate (oracle/surrogate_ref.py) pinned on the CPU: its
bfloat16 rounding against torch's, and its hand-written backward pass against torch float64
autograd of the same network (with and without the bfloat16 rounding points)."""
import numpy as np

from oracle import surrogate_ref as R


def test_bf16_round_matches_torch():
    import torch

    rng = np.random.default_rng(0)
    x = (rng.standard_normal(200_000) * 10.0 ** rng.integers(-8, 8, 200_000)).astype(np.float32).astype(np.float64)
    x[:4] = [0.0, -0.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8]      # exact ties: to even
    want = torch.from_numpy(x).float().to(torch.bfloat16).double().numpy()
    assert np.array_equal(R.bf16_round(x), want)


def _net(rng, depth=3, width=16, n_out=4, B=24):
    W = [rng.uniform(-0.5, 0.5, (width, width)) for _ in range(depth)]
    b = [rng.normal(0, 0.1, width) for _ in range(depth)]
    Wh = rng.uniform(-0.3, 0.3, (n_out, width))
    bh = rng.normal(0, 0.1, n_out)
    x0 = rng.uniform(-1, 1, (B, width))
    t = rng.normal(0, 1, (B, n_out))
    return x0, W, b, Wh, bh, t


def _autograd(x0, W, b, Wh, bh, t, bf16):
    import torch

    def rnd(v):
        if not bf16:
            return v
        return v + (torch.from_numpy(R.bf16_round(v.detach().numpy())) - v).detach()

    ws = [torch.tensor(w, requires_grad=True) for w in W]
    bs = [torch.tensor(v, requires_grad=True) for v in b]
    wh, bhh = torch.tensor(Wh, requires_grad=True), torch.tensor(bh, requires_grad=True)
    h = torch.tensor(x0)
    for w, v in zip(ws, bs):
        z = rnd(h @ w.t() + v)
        h = rnd(z * torch.sigmoid(z))
    y = h @ wh.t() + bhh
    loss = ((y - torch.tensor(t)) ** 2).mean()
    loss.backward()
    return ([w.grad.numpy() for w in ws], [v.grad.numpy() for v in bs], wh.grad.numpy(), bhh.grad.numpy(),
            float(loss.detach()) * t.size)


def test_backward_matches_float64_autograd():
    """Exact arithmetic: the reference's gradients equal autograd's to float64 rounding. With the
    bfloat16 points, autograd sees the rounding as identity in the backward pass (straight-through)
    while the kernels also round dZ; so that comparison is of the forward and the head only."""
    rng = np.random.default_rng(1)
    net = _net(rng)
    ref = R.forward_backward(*net, bf16=False)
    gw, gb, gwh, gbh, loss = _autograd(*net, bf16=False)
    for a, b_ in zip(ref["gw"] + ref["gb"] + [ref["gwh"], ref["gbh"]], gw + gb + [gwh, gbh]):
        assert np.allclose(a, b_, rtol=1e-12, atol=1e-15 * np.abs(b_).max())
    assert abs(ref["loss"] - loss) <= 1e-12 * loss
    ref16 = R.forward_backward(*net, bf16=True)
    _, _, gwh16, gbh16, loss16 = _autograd(*net, bf16=True)
    assert abs(ref16["loss"] - loss16) <= 1e-12 * loss16
    assert np.allclose(ref16["gwh"], gwh16, rtol=1e-12, atol=1e-15) and np.allclose(ref16["gbh"], gbh16, rtol=1e-12)


def test_features_formula():
    uv = np.array([[0.25, -0.5], [0.0, 1.0]])
    f = R.features(uv, 2)
    assert f.shape == (2, 8)
    assert np.allclose(f[0], [np.sin(np.pi / 4), np.sin(np.pi / 2), np.cos(np.pi / 4), np.cos(np.pi / 2),
                              np.sin(-np.pi / 2), np.sin(-np.pi), np.cos(-np.pi / 2), np.cos(-np.pi)])
