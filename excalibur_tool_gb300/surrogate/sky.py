"""Surrogate-filled sky maps: train on traced rays, predict every pixel, audit, fall back.

One potential field, one observer, one square tangent-plane patch, rays traced
backward to the exit of the box. The map holds, per pixel, the redshift z at the
box-face crossing, the time-delay excess tau and the deflection (alpha_x,
alpha_y) on the patch basis.

Why the crossing: the tracer stops at the first accepted step outside the box, so
its raw end point (and with it a(eta) and Phi there) moves in whole steps from
one direction to the next -- a saw-tooth of ~1e-4 in z that no smooth model can
follow. The crossing values (final state extrapolated back to the face along its
own velocity, a fraction of one 0.5 Mpc step) are smooth in the direction.

What the network learns (6 outputs): the crossing point's two in-face offsets
from the straight-line crossing, the conformal-time delay of the crossing
behind the straight-line light travel time, tau, alpha_x and alpha_y -- all
smooth integrals along the ray. The redshift is then composed exactly from the
grid and the a(eta) table at the predicted crossing (one metric evaluation per
pixel, exc_metric_tensor): z = a_obs / a(eta_c) - 1 + (Phi_obs - Phi(x_c)) / c^2,
so the small-scale structure of Phi on the exit face, which 64 Fourier
frequencies cannot resolve, never has to be learned.

Optional baseline features: the straight ray's first-order (Born) line
integrals -- Shapiro delay and its moments, deflection, transverse offset at the
face, geometric delay (exc_born_patch, one gather loop per ray) -- can enter the
model's least-squares baseline (`fit(..., extra=)`). They explain the deflection
and exit offsets to a correlation of 0.99, but not the conformal-time delay that
sets z (the reference's FLRW-fast right-hand side lets u^0 drift off the null
cone by ~17 % over 1000 Mpc, a smooth path-history effect), and with them the
network's redshift error is larger (median 3e-7 against 1.8e-7 on the 20 deg
patch), so the default pipeline leaves them out.

How smooth the target is depends on the interpolator. With the fast
interpolators' base-node gradient (piecewise constant per cell), each RK4 stage
point that crosses a cell face as the direction moves changes that step's
increment by a finite amount, so the traced z is rough at the pixel scale: on
the 20 deg patch of a 128^3 field at 4096^2 pixels, adjacent-pixel second
differences of the FP64-traced z are ~2e-7 rms, growing like the square root of
the pixel separation (a random walk of small jumps). No smooth model reaches
1e-7 there; the ensemble reaches ~1.4e-7 median. The slow Interpolator's
gradient (trilinear blend of corner differences) is continuous, the map is
smooth (second differences ~4e-9) and the same pipeline reaches a median
|dz| of ~7e-9 with 99.99 % of audited pixels within 1e-7.

Pipeline: `training_set` traces seeded uniform-random patch positions;
`SkySurrogate.fit` trains the ensemble; `fill_sky_map` predicts all pixel
centres, sends pixels whose ensemble spread in z exceeds `std_threshold` to the
tracer (fallback) and traces a seeded `audit_fraction` of the others to state
the map's accuracy.
"""
from __future__ import annotations

import dataclasses
import time
from typing import Optional

import numpy as np

from ..core.constants import c, one_Mpc
from ..observables import lensing as L
from ..photon.photons import Photons
from ..trace import TraceConfig, trace_batch
from .model import SkySurrogate

N_LEARNED = 6
MAP_OUTPUTS = ("z", "time_delay", "alpha_x", "alpha_y")


@dataclasses.dataclass
class Patch:
    """Observer (eta, x, y, z), axis and angular size of a square tangent-plane patch."""
    origin: tuple
    axis: tuple
    patch_deg: float


class ExitGeometry:
    """Straight-line exit of the patch's rays from the stop box, and the tracer's crossing."""

    def __init__(self, patch: Patch, box):
        self.patch = patch
        self.o = np.asarray(patch.origin, dtype=float)
        self.k, self.e1, self.e2 = Photons.patch_basis(patch.axis)
        self.half = np.tan(np.deg2rad(patch.patch_deg / 2.0))
        self.lo = np.asarray(box[0], dtype=float)
        self.hi = np.asarray(box[1], dtype=float)

    def directions(self, uv):
        d = self.k[None] + (uv[:, :1] * self.half) * self.e1[None] + (uv[:, 1:2] * self.half) * self.e2[None]
        return d / np.linalg.norm(d, axis=1)[:, None]

    def straight(self, uv):
        """(axis index, distance t*, point p*) of the straight ray's first box face."""
        d = self.directions(uv)
        with np.errstate(divide="ignore", invalid="ignore"):
            face = np.where(d > 0, self.hi[None], self.lo[None])
            t = np.where(d != 0, (face - self.o[None, 1:4]) / d, np.inf)
        ax = np.argmin(t, axis=1)
        ts = t[np.arange(len(t)), ax]
        return ax, ts, self.o[None, 1:4] + ts[:, None] * d

    def crossing(self, state):
        """(axis index, eta_c, x_c) of the tracer's final state taken back to the face it crossed."""
        x = state[:, 1:4]
        out_hi, out_lo = x >= self.hi[None], x < self.lo[None]
        viol = np.where(out_hi, x - self.hi[None], 0.0) + np.where(out_lo, self.lo[None] - x, 0.0)
        ax = np.argmax(viol, axis=1)
        rows = np.arange(len(x))
        face = np.where(out_hi[rows, ax], self.hi[ax], self.lo[ax])
        dl = (x[rows, ax] - face) / state[rows, 5 + ax]
        eta_c = state[:, 0] - dl * state[:, 4]
        x_c = x - dl[:, None] * state[:, 5:8]
        return ax, eta_c, x_c

    @staticmethod
    def in_face(ax):
        """The two coordinate indices spanning the face normal to axis ax."""
        return np.stack([(ax + 1) % 3, (ax + 2) % 3], 1)


def _deflection(obs, e1, e2):
    v0 = np.stack([L.col(obs, "v0x"), L.col(obs, "v0y"), L.col(obs, "v0z")], 1)
    v1 = np.stack([L.col(obs, "v1x"), L.col(obs, "v1y"), L.col(obs, "v1z")], 1)
    d = v1 / np.linalg.norm(v1, axis=1)[:, None] - v0 / np.linalg.norm(v0, axis=1)[:, None]
    return d @ e1, d @ e2


def redshift_at_t(metric, eta, x, a_obs, phi_obs_c2):
    """z = a_obs / a(eta) - 1 + Phi_obs / c^2 - Phi(x) / c^2 for device tensors eta [n], x [n, 3]:
    one exc_metric_tensor evaluation per point (g00 = -a^2 (1 + 2 phi) c^2, g11 = a^2 (1 - 2 phi))."""
    import torch

    from .._evaluate import metric_diag

    pts = torch.cat([eta[:, None], x], 1).contiguous()
    g, st = metric_diag(metric, pts)
    A = -g[:, 0] / float(c) ** 2
    B = g[:, 1]
    a2 = 0.5 * (A + B)
    phi = (A - B) / (4.0 * a2)
    z = a_obs / torch.sqrt(a2) - 1.0 + (phi_obs_c2 - phi)
    return torch.where(st == 0, z, torch.full_like(z, float("nan")))


def redshift_at(metric, eta, x, a_obs, phi_obs_c2):
    import torch

    dev = torch.device("cuda")
    return redshift_at_t(metric, torch.as_tensor(np.asarray(eta, dtype=np.float64), device=dev),
                         torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev), a_obs, phi_obs_c2).cpu().numpy()


def observer_terms(metric, patch: Patch):
    """a_obs and Phi_obs / c^2 at the observer."""
    eta0, x0 = np.array([patch.origin[0]]), np.asarray(patch.origin[1:4], dtype=float)[None]
    from .._evaluate import metric_diag
    import torch

    g, _ = metric_diag(metric, torch.as_tensor(np.concatenate([eta0[:, None], x0], 1)).cuda())
    g = g.cpu().numpy()
    A, B = -g[0, 0] / float(c) ** 2, g[0, 1]
    a2 = 0.5 * (A + B)
    return float(np.sqrt(a2)), float((A - B) / (4.0 * a2))


def traced_quantities(metric, patch: Patch, uv, cfg: TraceConfig, geo: ExitGeometry):
    """Trace the rays at patch positions uv; returns (learned targets [n, 6], map values [n, 4])
    with NaN rows for rays that did not leave the box through their straight-line face."""
    import torch

    from .. import _native as N

    states = Photons(metric).generate_patch_points(uv, patch.origin, patch.axis, patch.patch_deg)
    r = trace_batch(metric, states, cfg)
    torch.cuda.synchronize()
    st, obs, status = r.state.cpu().numpy(), r.obs.cpu().numpy(), r.status.cpu().numpy()
    ax_s, t_s, p_s = geo.straight(uv)
    ax_c, eta_c, x_c = geo.crossing(st)
    ok = (status == N.PH_LEFT_BOX) & (ax_c == ax_s)
    rows = np.arange(len(uv))
    f = ExitGeometry.in_face(ax_s)
    off = (x_c[rows[:, None], f] - p_s[rows[:, None], f]) / one_Mpc
    deta = (patch.origin[0] - t_s / float(c)) - eta_c
    ax_, ay_ = _deflection(obs, geo.e1, geo.e2)
    tau = L.time_delay_excess(obs)
    learned = np.stack([off[:, 0], off[:, 1], deta, tau, ax_, ay_], 1)
    a_obs, phi_obs = observer_terms(metric, patch)
    z = redshift_at(metric, eta_c, x_c, a_obs, phi_obs)
    values = np.stack([z, tau, ax_, ay_], 1)
    learned[~ok] = np.nan
    values[~ok] = np.nan
    return learned, values


def compose_t(metric, patch: Patch, geo: ExitGeometry, uv, learned, obs_terms):
    """Map values [..., n, 4] from learned outputs [..., n, 6] on the device (uv [n, 2] device
    tensor; leading dimensions, e.g. ensemble members, broadcast)."""
    import torch

    dev = learned.device
    k, e1, e2 = (torch.as_tensor(v, device=dev) for v in (geo.k, geo.e1, geo.e2))
    o = torch.as_tensor(geo.o, device=dev)
    lo, hi = torch.as_tensor(geo.lo, device=dev), torch.as_tensor(geo.hi, device=dev)
    d = k[None] + (uv[:, :1] * geo.half) * e1[None] + (uv[:, 1:2] * geo.half) * e2[None]
    d = d / torch.linalg.norm(d, dim=1, keepdim=True)
    face = torch.where(d > 0, hi[None], lo[None])
    t = torch.where(d != 0, (face - o[None, 1:4]) / d, torch.full_like(d, float("inf")))
    ts, ax = torch.min(t, dim=1)
    ps = o[None, 1:4] + ts[:, None] * d
    lead = learned.shape[:-2]
    ps = ps.expand(*lead, *ps.shape)
    f1 = ((ax + 1) % 3).expand(*lead, ax.shape[0])[..., None]
    f2 = ((ax + 2) % 3).expand(*lead, ax.shape[0])[..., None]
    x = ps.clone()
    x.scatter_add_(-1, f1, learned[..., 0:1] * one_Mpc)
    x.scatter_add_(-1, f2, learned[..., 1:2] * one_Mpc)
    eta = patch.origin[0] - ts / float(c) - learned[..., 2]
    z = redshift_at_t(metric, eta.reshape(-1), x.reshape(-1, 3), *obs_terms).reshape(eta.shape)
    return torch.stack([z, learned[..., 3], learned[..., 4], learned[..., 5]], -1)


def compose(metric, patch: Patch, geo: ExitGeometry, uv, learned, obs_terms):
    """Map values [n, 4] from learned outputs [n, 6] (host arrays; one member or the mean)."""
    import torch

    dev = torch.device("cuda")
    return compose_t(metric, patch, geo, torch.as_tensor(np.asarray(uv, dtype=np.float64), device=dev),
                     torch.as_tensor(np.asarray(learned, dtype=np.float64), device=dev), obs_terms).cpu().numpy()


def born_features(metric, patch: Patch, uv, box, step=None):
    """[n, 8] first-order line integrals along the straight rays at patch positions uv
    ([n, 2] float64 device tensor); see exc_born_patch in include/excalibur_mlp.h."""
    import ctypes as C

    import torch

    from .. import _native as N

    dev = uv.device
    desc = metric.descriptor(dev, split=True)
    f0 = desc.struct.fields[0]
    k, e1, e2 = Photons.patch_basis(patch.axis)
    a = N.ExcBornArgs()
    a.n = int(uv.shape[0])
    uvc = uv.contiguous()
    a.uv = uvc.data_ptr()
    for i in range(3):
        a.origin[i] = float(patch.origin[1 + i])
        a.axis[i], a.e1[i], a.e2[i] = k[i], e1[i], e2[i]
        a.box_lo[i], a.box_hi[i] = float(box[0][i]), float(box[1][i])
    a.half = float(np.tan(np.deg2rad(patch.patch_deg / 2.0)))
    a.step = float(step if step is not None else 0.5 * min(f0.spacing[i] for i in range(3)))
    a.c = float(c)
    out = torch.empty((a.n, 8), dtype=torch.float64, device=dev)
    a.out = out.data_ptr()
    N.check(N.load().exc_born_patch(C.byref(desc.struct), C.byref(a), N.stream_handle(dev)), "exc_born_patch")
    return out


def training_set(metric, patch: Patch, n: int, cfg: TraceConfig, seed: int = 1):
    """(uv, learned targets, Born features, info) for n seeded uniform patch positions."""
    import torch

    geo = ExitGeometry(patch, cfg.stop_box)
    rng = np.random.default_rng(seed)
    uv = rng.uniform(-1.0, 1.0, size=(n, 2))
    t0 = time.perf_counter()
    learned, _ = traced_quantities(metric, patch, uv, cfg, geo)
    t_trace = time.perf_counter() - t0
    feats = born_features(metric, patch, torch.as_tensor(uv, device="cuda"), cfg.stop_box).cpu().numpy()
    ok = np.isfinite(learned).all(1) & np.isfinite(feats).all(1)
    return uv[ok], learned[ok], feats[ok], {"rays": n, "kept": int(ok.sum()), "trace_s": t_trace}


def pixel_centres(n_side: int) -> np.ndarray:
    t = (np.arange(n_side) + 0.5) / n_side * 2 - 1
    A, B = np.meshgrid(t, t, indexing="ij")
    return np.stack([A.reshape(-1), B.reshape(-1)], 1)


def pixel_centres_t(n_side: int, device, start: int = 0, stop: Optional[int] = None):
    """Rows start..stop of pixel_centres(n_side) built on the device (the same float64
    operations, so the same values)."""
    import torch

    stop = n_side * n_side if stop is None else stop
    i = torch.arange(start, stop, device=device, dtype=torch.int64)
    t = lambda j: (j.to(torch.float64) + 0.5) / n_side * 2 - 1
    return torch.stack([t(torch.div(i, n_side, rounding_mode="floor")), t(i % n_side)], 1)


def fill_sky_map(model: SkySurrogate, metric, patch: Patch, cfg: TraceConfig, n_side: int = 4096,
                 std_threshold: float = 1e-7, audit_fraction: float = 0.01, audit_seed: int = 5,
                 chunk: int = 1 << 20):
    """The n_side^2 map [pixels, 4] of (z, tau, alpha_x, alpha_y) and a report.

    Pixels whose ensemble spread in z exceeds std_threshold (or whose prediction is
    not finite) are traced with `cfg` instead; a seeded audit_fraction of the rest
    is traced as well and compared with the surrogate."""
    import torch

    geo = ExitGeometry(patch, cfg.stop_box)
    obs_terms = observer_terms(metric, patch)
    uv = pixel_centres(n_side)
    n = len(uv)
    t0 = time.perf_counter()
    # the pixel centres are made on the device and the map stays there until one copy at the end
    out_d = torch.empty((n, 4), dtype=torch.float64, device=model.device)
    zstd_d = torch.empty(n, dtype=torch.float64, device=model.device)
    for s in range(0, n, chunk):
        uvc = pixel_centres_t(n_side, model.device, s, min(s + chunk, n))
        ex = born_features(metric, patch, uvc, cfg.stop_box) if model.n_extra else None
        y = model.predict_members(uvc, ex)                               # [E, m, 6] on the device
        members = compose_t(metric, patch, geo, uvc, y, obs_terms)       # [E, m, 4]
        out_d[s:s + chunk] = compose_t(metric, patch, geo, uvc, y.mean(0), obs_terms)
        zstd_d[s:s + chunk] = members[..., 0].std(0, unbiased=False)
    out, zstd = out_d.cpu().numpy(), zstd_d.cpu().numpy()
    del out_d, zstd_d
    t_pred = time.perf_counter() - t0
    fallback = ~(zstd <= std_threshold) | ~np.isfinite(out).all(1)
    t1 = time.perf_counter()
    fb = np.nonzero(fallback)[0]
    for s in range(0, len(fb), chunk):
        sel = fb[s:s + chunk]
        out[sel] = traced_quantities(metric, patch, uv[sel], cfg, geo)[1]
    t_fb = time.perf_counter() - t1
    rng = np.random.default_rng(audit_seed)
    kept = np.nonzero(~fallback)[0]
    n_audit = int(round(audit_fraction * len(kept)))
    audit = np.sort(rng.choice(kept, n_audit, replace=False)) if n_audit else np.zeros(0, dtype=np.int64)
    t2 = time.perf_counter()
    ref = np.concatenate([traced_quantities(metric, patch, uv[audit[s:s + chunk]], cfg, geo)[1]
                          for s in range(0, len(audit), chunk)]) if len(audit) else np.zeros((0, 4))
    t_audit = time.perf_counter() - t2
    good = np.isfinite(ref).all(1)
    err = np.abs(out[audit][good] - ref[good])
    rep = {
        "pixels": int(n), "fallback_pixels": int(fallback.sum()), "fallback_fraction": float(fallback.mean()),
        "std_threshold": std_threshold, "audit_pixels": int(len(audit)),
        "predict_s": t_pred, "fallback_trace_s": t_fb, "audit_trace_s": t_audit,
        "total_s": time.perf_counter() - t0, "tracer_precision": cfg.precision,
    }
    if len(err):
        # what a lower spread threshold would have done: the share of pixels it sends to the tracer,
        # and the largest error among the audited pixels it would still have kept
        zs_a = zstd[audit][good]
        rep["threshold_tradeoff"] = [
            {"std_threshold": t, "fallback_fraction": float((~(zstd <= t) | ~np.isfinite(out).all(1)).mean()),
             "audit_kept": int((zs_a <= t).sum()),
             "audit_max_abs_dz_kept": float(err[zs_a <= t, 0].max()) if (zs_a <= t).any() else None,
             "audit_fraction_within_1e-7_kept": float((err[zs_a <= t, 0] <= 1e-7).mean()) if (zs_a <= t).any() else None}
            for t in sorted({std_threshold, 5e-8, 3e-8, 2e-8, 1e-8, 5e-9}, reverse=True) if t <= std_threshold]
        rep.update({
            "audit_max_abs_dz": float(err[:, 0].max()), "audit_p99_abs_dz": float(np.percentile(err[:, 0], 99)),
            "audit_median_abs_dz": float(np.median(err[:, 0])),
            "audit_fraction_within_1e-7": float((err[:, 0] <= 1e-7).mean()),
            "audit_median_rel_time_delay": float(np.median(err[:, 1] / np.abs(ref[good][:, 1]))),
            "audit_max_abs_deflection": float(np.hypot(err[:, 2], err[:, 3]).max()),
        })
    return out, rep
