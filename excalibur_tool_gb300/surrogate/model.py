"""Ensemble MLP surrogate: sky direction -> (dz, time delay, deflection x, deflection y).

Network (per member): Fourier features of the tangent-plane direction (u, v) in
[-1, 1]^2 (sin/cos(pi k u), sin/cos(pi k v), k = 1..64: 256 features) -> 4
hidden layers of width 256 with SiLU -> linear head of 4 outputs. Weights are
FP32 master copies with BF16 working copies (and transposed BF16 copies for the
backward GEMMs); every forward, backward and optimiser step runs in the
project's kernels (surrogate/kernels.py -> exc_mlp.cu: tcgen05 BF16 GEMMs with
FP32 accumulation). torch only allocates, indexes batches and copies layouts.

Targets are fitted in two parts: a quadratic baseline in (u, v) solved once by
FP64 least squares on the host (it carries the smooth geometric variation, e.g.
of the background redshift across the patch), and the network learning the
residual, normalised to unit variance per output. Ensemble members differ in
their initial weights and batch order; their spread is the disagreement
indicator that sends a direction back to the tracer.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

from . import kernels as K

N_OUT_MAX = 8


def _baseline_design(uv: np.ndarray, extra: Optional[np.ndarray] = None) -> np.ndarray:
    """Columns of the least-squares baseline: a quadratic in (u, v) plus optional
    per-direction features (e.g. first-order line integrals along the ray)."""
    u, v = uv[:, 0], uv[:, 1]
    cols = [np.ones_like(u), u, v, u * u, u * v, v * v]
    if extra is not None:
        cols += [extra[:, k] for k in range(extra.shape[1])]
    return np.stack(cols, 1)


@dataclasses.dataclass
class TrainReport:
    steps: int
    batch: int
    final_loss: list
    seconds: float
    loss_curve: list


class SkySurrogate:
    def __init__(self, n_members: int = 4, n_freq: int = 64, width: int = 256, depth: int = 4, n_out: int = 4,
                 seed: int = 0, device="cuda"):
        import torch

        if width != 256 or 4 * n_freq != 256:
            raise ValueError("the kernels are built for width 256 and 64 frequencies (256 features)")
        if not 1 <= n_out <= N_OUT_MAX:
            raise ValueError(f"n_out must be in [1, {N_OUT_MAX}]")
        self.E, self.nf, self.W, self.depth, self.n_out = n_members, n_freq, width, depth, n_out
        self.device = torch.device(device)
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.w, self.b = [], []
        fan_in = 4 * n_freq
        for _ in range(depth):
            bound = math.sqrt(6.0 / fan_in)     # He-uniform for SiLU
            self.w.append(((torch.rand(self.E, width, fan_in, generator=g) * 2 - 1) * bound).to(self.device))
            self.b.append(torch.zeros(self.E, width, device=self.device))
            fan_in = width
        self.w_head = ((torch.rand(self.E, n_out, width, generator=g) * 2 - 1) * math.sqrt(1.0 / width)).to(
            self.device)
        self.b_head = torch.zeros(self.E, n_out, device=self.device)
        self._sync_bf16()
        self.baseline = np.zeros((6, n_out))
        self.n_extra = 0
        self.t_mean = np.zeros(n_out)
        self.t_std = np.ones(n_out)
        self._adam = None
        self._t = 0

    # ------------------------------------------------------------ weights
    def _sync_bf16(self):
        import torch

        self.wb = [w.to(torch.bfloat16).contiguous() for w in self.w]
        self.wtb = [w.transpose(1, 2).contiguous().to(torch.bfloat16) for w in self.w]

    def params(self):
        return self.w + self.b + [self.w_head, self.b_head]

    # ------------------------------------------------------------ features
    def _features(self, uv, n_pad):
        import torch

        x = torch.empty((n_pad, 4 * self.nf), dtype=torch.bfloat16, device=self.device)
        K.features(uv, n_pad, self.nf, (0.0, 0.0), (1.0, 1.0), x)
        return x

    # ------------------------------------------------------------ targets
    def set_normalisation(self, uv: np.ndarray, targets: np.ndarray, extra: Optional[np.ndarray] = None):
        A = _baseline_design(uv, extra)
        # columns scaled to unit norm for the solve (the features span many decades)
        self._col_scale = np.maximum(np.linalg.norm(A, axis=0), 1e-300)
        coef, *_ = np.linalg.lstsq(A / self._col_scale, targets, rcond=None)
        self.baseline = coef / self._col_scale[:, None]
        self.n_extra = 0 if extra is None else extra.shape[1]
        resid = targets - A @ self.baseline
        self.t_mean = resid.mean(0)
        self.t_std = resid.std(0) + 1e-300
        self._norm_key = None   # the device copies used by prediction are made again

    def _normalise(self, uv: np.ndarray, targets: np.ndarray, extra: Optional[np.ndarray] = None) -> np.ndarray:
        return ((targets - _baseline_design(uv, extra) @ self.baseline - self.t_mean) / self.t_std).astype(np.float32)

    # ------------------------------------------------------------ training
    def _buffers(self, B: int, k_splits: int = 32):
        import torch

        E, W, dev, bf = self.E, self.W, self.device, torch.bfloat16
        S = min(k_splits, B // 64)
        return {
            "Z": [torch.empty((E, B, W), dtype=bf, device=dev) for _ in range(self.depth)],
            "H": [torch.empty((E, B, W), dtype=bf, device=dev) for _ in range(self.depth)],
            "HT": [torch.empty((E, W, B), dtype=bf, device=dev) for _ in range(self.depth - 1)],
            "dZ": [torch.zeros((E, B, W), dtype=bf, device=dev) for _ in range(self.depth)],
            "dZT": [torch.zeros((E, W, B), dtype=bf, device=dev) for _ in range(self.depth)],
            "S": S,
            "part": torch.empty((E, S, W, W), device=dev),
            "gw": [torch.empty_like(w) for w in self.w],
            "gb": [torch.empty_like(b) for b in self.b],
            "gwh": torch.empty_like(self.w_head),
            "gbh": torch.empty_like(self.b_head),
            "loss": torch.zeros(E, device=dev),
        }

    def forward_backward(self, uv_b, t_b, buf):
        """Gradients of the mean-squared error of every member on one batch (uv_b [B, 2]
        float64 and normalised targets t_b [B, 4] float32, device tensors; B a multiple of
        128) into buf["gw"], buf["gb"], buf["gwh"], buf["gbh"]; buf["loss"] gets the
        per-member sums of squared errors."""
        B = uv_b.shape[0]
        x0 = self._features(uv_b, B)
        x0t = x0.t().contiguous()                      # layout for the first layer's weight gradient
        Z, H, HT, dZ, dZT = buf["Z"], buf["H"], buf["HT"], buf["dZ"], buf["dZT"]
        inp = x0
        for l in range(self.depth):
            K.gemm(inp, self.wb[l], epilogue="bias_silu", bias=self.b[l], c=Z[l], c2=H[l],
                   ct=HT[l] if l < self.depth - 1 else None)
            inp = H[l]
        buf["gwh"].zero_()
        buf["gbh"].zero_()
        buf["loss"].zero_()
        K.head(H[-1], self.w_head, self.b_head, targets=t_b, z=Z[-1], dh=dZ[-1], dht=dZT[-1], dw=buf["gwh"],
               db=buf["gbh"], loss=buf["loss"])
        for l in range(self.depth - 1, -1, -1):
            K.gemm(dZT[l], x0t if l == 0 else HT[l - 1], epilogue="splitk", c=buf["part"], k_splits=buf["S"])
            K.reduce_splits(buf["part"], buf["gw"][l])
            K.row_sums(dZT[l], B, buf["gb"][l])
            if l > 0:
                K.gemm(dZ[l], self.wtb[l], epilogue="dsilu", z_in=Z[l - 1], c=dZ[l - 1], ct=dZT[l - 1])

    def _schedule(self, steps, lr, lr_final, beta1=0.9, beta2=0.999):
        """[steps, 3] float32 {lr_t, 1/(1-beta1^t), 1/(1-beta2^t)}: the values the eager step
        passes to exc_mlp_adam (lr_t rounded to float32; the corrections in float32 powf, as
        the library computes them)."""
        out = np.empty((steps, 3), dtype=np.float32)
        one, b1, b2 = np.float32(1.0), np.float32(beta1), np.float32(beta2)
        for step in range(steps):
            t = np.float32(self._t + 1 + step)
            out[step, 0] = np.float32(lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * step / max(1, steps - 1))))
            out[step, 1] = one / (one - np.power(b1, t))
            out[step, 2] = one / (one - np.power(b2, t))
        return out

    def fit(self, uv: np.ndarray, targets: np.ndarray, steps: int = 3000, batch: int = 8192, lr: float = 2e-3,
            lr_final: float = 2e-5, seed: int = 1, k_splits: int = 16, log_every: int = 100,
            extra: Optional[np.ndarray] = None, graph: bool = True, graph_steps: int = 16) -> TrainReport:
        """Train every member on (uv [n, 2] in [-1, 1]^2, targets [n, n_out]) with Adam and a cosine
        schedule; `extra` [n, k] are per-direction baseline features (the same must be given to
        prediction).

        With `graph` (default), `graph_steps` consecutive training steps -- forward, backward and
        Adam, about forty kernels each -- are captured once in a CUDA graph and replayed: the host
        fills a chunk of batches and the steps' learning rates and bias corrections into static
        device buffers, then issues one graph launch, so the step time is the GPU's and not the
        host's launch rate. The steps are the eager loop's, batch for batch and value for value."""
        if graph:
            return self._fit_graphed(uv, targets, steps, batch, lr, lr_final, seed, k_splits, log_every, extra,
                                     graph_steps)
        import time

        import torch

        if batch % 128:
            raise ValueError("batch must be a multiple of 128")
        n = uv.shape[0]
        self.set_normalisation(uv, targets, extra)
        dev = self.device
        uv_d = torch.as_tensor(np.ascontiguousarray(uv, dtype=np.float64), device=dev)
        t_d = torch.as_tensor(self._normalise(uv, targets, extra), device=dev)
        B = batch
        buf = self._buffers(B, k_splits)
        if self._adam is None:
            self._adam = [(torch.zeros_like(p), torch.zeros_like(p)) for p in self.params()]
        gen = torch.Generator(device="cpu").manual_seed(seed)
        perm = torch.randperm(n, generator=gen).to(dev)
        pos = 0
        curve = []
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for step in range(steps):
            if pos + B > n:
                perm = torch.randperm(n, generator=gen).to(dev)
                pos = 0
            idx = perm[pos:pos + B]
            pos += B
            self.forward_backward(uv_d[idx], t_d[idx].contiguous(), buf)
            self._t += 1
            lr_t = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * step / max(1, steps - 1)))
            grads = buf["gw"] + buf["gb"] + [buf["gwh"], buf["gbh"]]
            for i, (p, g) in enumerate(zip(self.params(), grads)):
                m1, m2 = self._adam[i]
                if i < self.depth:
                    K.adam(p, g, m1, m2, lr=lr_t, beta1=0.9, beta2=0.999, eps=1e-8, t=self._t,
                           p_bf16=self.wb[i], pt_bf16=self.wtb[i], shape=(p.shape[1], p.shape[2]))
                else:
                    K.adam(p, g, m1, m2, lr=lr_t, beta1=0.9, beta2=0.999, eps=1e-8, t=self._t)
            if log_every and (step % log_every == 0 or step == steps - 1):
                curve.append((step, (buf["loss"] / (B * self.n_out)).cpu().tolist()))
        torch.cuda.synchronize(dev)
        secs = time.perf_counter() - t0
        return TrainReport(steps, B, curve[-1][1] if curve else [], secs, curve)

    def _fit_graphed(self, uv, targets, steps, batch, lr, lr_final, seed, k_splits, log_every, extra, K_steps):
        import time

        import torch

        if batch % 128:
            raise ValueError("batch must be a multiple of 128")
        if K_steps < 1:
            raise ValueError("graph_steps must be >= 1")
        n = uv.shape[0]
        self.set_normalisation(uv, targets, extra)
        dev = self.device
        uv_d = torch.as_tensor(np.ascontiguousarray(uv, dtype=np.float64), device=dev)
        t_d = torch.as_tensor(self._normalise(uv, targets, extra), device=dev)
        B = batch
        buf = self._buffers(B, k_splits)
        if self._adam is None:
            self._adam = [(torch.zeros_like(p), torch.zeros_like(p)) for p in self.params()]
        sched_all = torch.as_tensor(self._schedule(steps, lr, lr_final), device=dev)
        K_steps = min(K_steps, max(1, steps))
        uv_c = torch.empty((K_steps * B, 2), dtype=torch.float64, device=dev)
        t_c = torch.empty((K_steps * B, t_d.shape[1]), dtype=torch.float32, device=dev)
        sched_c = torch.empty((K_steps, 3), dtype=torch.float32, device=dev)
        gen = torch.Generator(device="cpu").manual_seed(seed)
        state = {"perm": torch.randperm(n, generator=gen).to(dev), "pos": 0}

        def batch_index():   # the eager loop's batch order
            if state["pos"] + B > n:
                state["perm"] = torch.randperm(n, generator=gen).to(dev)
                state["pos"] = 0
            idx = state["perm"][state["pos"]:state["pos"] + B]
            state["pos"] += B
            return idx

        def fill(step0, k):
            idx = torch.cat([batch_index() for _ in range(k)])
            torch.index_select(uv_d, 0, idx, out=uv_c[:k * B])
            torch.index_select(t_d, 0, idx, out=t_c[:k * B])
            sched_c[:k].copy_(sched_all[step0:step0 + k])

        grads = buf["gw"] + buf["gb"] + [buf["gwh"], buf["gbh"]]
        groups = []
        for i, (p, g) in enumerate(zip(self.params(), grads)):
            m1, m2 = self._adam[i]
            if i < self.depth:
                groups.append((p, g, m1, m2, self.wb[i], self.wtb[i], (p.shape[1], p.shape[2])))
            else:
                groups.append((p, g, m1, m2, None, None, None))

        def one_step(j):
            self.forward_backward(uv_c[j * B:(j + 1) * B], t_c[j * B:(j + 1) * B], buf)
            K.adam_multi(groups, sched_c[j], beta1=0.9, beta2=0.999, eps=1e-8)   # every tensor, one launch

        curve = []
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        step, g = 0, None
        while step < steps:
            k = min(K_steps, steps - step)
            fill(step, k)
            if k == K_steps and g is None and step > 0:
                # captured after one eager chunk has run (kernels loaded, attributes set)
                g = torch.cuda.CUDAGraph()
                side = torch.cuda.Stream(dev)
                side.wait_stream(torch.cuda.current_stream(dev))
                with torch.cuda.graph(g, stream=side):
                    for j in range(K_steps):
                        one_step(j)
            if k == K_steps and g is not None:
                g.replay()
            else:
                for j in range(k):
                    one_step(j)
                    if log_every and step == 0 and j == 0:
                        curve.append((0, (buf["loss"] / (B * self.n_out)).cpu().tolist()))
            self._t += k
            step += k
            if log_every and (step // log_every != (step - k) // log_every or step == steps):
                curve.append((step - 1, (buf["loss"] / (B * self.n_out)).cpu().tolist()))
        torch.cuda.synchronize(dev)
        secs = time.perf_counter() - t0
        return TrainReport(steps, B, curve[-1][1] if curve else [], secs, curve)

    # ------------------------------------------------------------ inference
    def predict_members(self, uv, extra=None, fused: bool = True):
        """Every member's outputs [E, m, n_out] (physical units, float64, on the device) for
        directions uv ([m, 2] float64 device tensor) and their baseline features `extra`
        ([m, k] device tensor, as given to fit). `fused`: the whole forward pass in one kernel
        (exc_mlp_infer, activations kept on chip); otherwise layer by layer through HBM (the
        training kernels' forward path; the same roundings, the head summed in another order)."""
        import torch

        m = uv.shape[0]
        mp = ((m + 127) // 128) * 128
        E, W, dev, bf = self.E, self.W, self.device, torch.bfloat16
        y = torch.empty((E, mp, self.n_out), device=dev)
        inp = self._features(uv, mp)
        if fused:
            # the layers' bf16 weights and biases stacked [depth, E, ...] for the one launch (2 MB,
            # copied each call: training updates the per-layer tensors in place)
            K.infer(inp, torch.stack(self.wb).contiguous(), torch.stack(self.b).contiguous(), self.w_head,
                    self.b_head, y)
        else:
            ha = torch.empty((E, mp, W), dtype=bf, device=dev)
            hb = torch.empty((E, mp, W), dtype=bf, device=dev)
            for l in range(self.depth):
                o = ha if l % 2 == 0 else hb
                K.gemm(inp, self.wb[l], epilogue="bias_silu", bias=self.b[l], c2=o)
                inp = o
            K.head(inp, self.w_head, self.b_head, y=y)
        # undo the target normalisation (six-term quadratic baseline + per-output scale)
        u, v = uv[:, 0], uv[:, 1]
        cols = [torch.ones_like(u), u, v, u * u, u * v, v * v]
        if self.n_extra:
            if extra is None or extra.shape[1] != self.n_extra:
                raise ValueError(f"this model was fitted with {self.n_extra} baseline features")
            cols += [extra[:, k].double() for k in range(self.n_extra)]
        design = torch.stack(cols, 1)
        # the normalisation's device copies, made once per fit (no host copy, and so no
        # synchronisation, on each call)
        key = (id(self.baseline), id(self.t_std), id(self.t_mean))
        if getattr(self, "_norm_key", None) != key:
            self._norm_dev = tuple(torch.as_tensor(a, device=dev) for a in (self.baseline, self.t_std, self.t_mean))
            self._norm_key = key
        baseline, scale, shift = self._norm_dev
        base = design @ baseline
        return y[:, :m].double() * scale + shift + base[None]

    def predict(self, uv: np.ndarray, chunk: int = 1 << 20, return_members: bool = False,
                extra: Optional[np.ndarray] = None):
        """Ensemble mean and standard deviation [n, n_out] (physical units) for directions uv [n, 2]."""
        import torch

        means, stds, mems = [], [], []
        for s in range(0, uv.shape[0], chunk):
            uvd = torch.as_tensor(np.ascontiguousarray(uv[s:s + chunk], dtype=np.float64), device=self.device)
            ex = None if extra is None else torch.as_tensor(np.ascontiguousarray(extra[s:s + chunk]),
                                                            device=self.device)
            y = self.predict_members(uvd, ex)
            means.append(y.mean(0).cpu().numpy())
            stds.append(y.std(0, unbiased=False).cpu().numpy())
            if return_members:
                mems.append(y.cpu().numpy())
        mean, std = np.concatenate(means), np.concatenate(stds)
        return (mean, std, np.concatenate(mems, axis=1)) if return_members else (mean, std)
