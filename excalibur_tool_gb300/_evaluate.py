"""Small batched device evaluations behind the reference's scalar methods.

Each helper runs one kernel of libexcalibur_gb300.so (exc_geodesic_rhs,
exc_metric_tensor, exc_eval_cosmology, exc_null_init, exc_null_error) on a
batch of points; the reference-facing classes call them with batches of one
or many. Nothing here evaluates physics on the host.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _device():
    import torch

    if not torch.cuda.is_available():
        raise N.NativeError("a CUDA device is required (the tracer has no host fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def _as_batch(x, width):
    import torch

    t = torch.as_tensor(np.asarray(x, dtype=np.float64) if not isinstance(x, torch.Tensor) else x,
                        dtype=torch.float64)
    single = t.ndim == 1
    if single:
        t = t[None]
    if t.shape[1] != width:
        raise ValueError(f"expected {width} components, got {t.shape[1]}")
    return t, single


def geodesic_rhs(metric, state, precision="fp64", field_index=None):
    import torch

    dev = _device()
    s, single = _as_batch(state, 8)
    s = s.to(dev).contiguous()
    n = s.shape[0]
    out = torch.empty_like(s)
    status = torch.empty(n, dtype=torch.int32, device=dev)
    desc = metric.descriptor(dev)
    lib = N.load()
    N.check(lib.exc_geodesic_rhs(C.byref(desc.struct), N.PRECISION[precision], N.ptr(s), N.ptr(out),
                                 N.ptr(status), N.ptr(field_index), n, N.stream_handle(dev)), "exc_geodesic_rhs")
    return (out[0], status[0]) if single else (out, status)


def metric_diag(metric, x, field_index=None):
    import torch

    dev = _device()
    xs, single = _as_batch(x, 4)
    xs = xs.to(dev).contiguous()
    n = xs.shape[0]
    g = torch.empty((n, 4), dtype=torch.float64, device=dev)
    status = torch.empty(n, dtype=torch.int32, device=dev)
    desc = metric.descriptor(dev)
    lib = N.load()
    N.check(lib.exc_metric_tensor(C.byref(desc.struct), N.ptr(xs), N.ptr(g), N.ptr(status), N.ptr(field_index),
                                  n, N.stream_handle(dev)), "exc_metric_tensor")
    return (g[0], status[0]) if single else (g, status)


def null_init(metric, states, sign=-1.0, field_index=None):
    """Overwrite u^0 of `states` ([N, 8] float64 CUDA tensor) in place from the null condition."""
    import torch

    dev = states.device
    n = states.shape[0]
    status = torch.empty(n, dtype=torch.int32, device=dev)
    desc = metric.descriptor(dev)
    lib = N.load()
    N.check(lib.exc_null_init(C.byref(desc.struct), N.ptr(states), float(sign), N.ptr(status),
                              N.ptr(field_index), n, N.stream_handle(dev)), "exc_null_init")
    return status


def null_error(metric, states, field_index=None):
    import torch

    dev = _device()
    s, single = _as_batch(states, 8)
    s = s.to(dev).contiguous()
    n = s.shape[0]
    rel = torch.empty(n, dtype=torch.float64, device=dev)
    status = torch.empty(n, dtype=torch.int32, device=dev)
    desc = metric.descriptor(dev)
    lib = N.load()
    N.check(lib.exc_null_error(C.byref(desc.struct), N.ptr(s), N.ptr(rel), N.ptr(status), N.ptr(field_index),
                               n, N.stream_handle(dev)), "exc_null_error")
    return (rel[0], status[0]) if single else (rel, status)


def eval_cosmology(cosmo, eta, which):
    """a(eta) or adot(eta) of an LCDM_Cosmology on the device; scalar in, float out."""
    import torch
    from .trace import base_metric_struct

    dev = _device()
    scalar = np.isscalar(eta) or (isinstance(eta, np.ndarray) and eta.ndim == 0)
    e = torch.as_tensor(np.atleast_1d(np.asarray(eta, dtype=np.float64))).to(dev)
    n = e.shape[0]
    a = torch.empty(n, dtype=torch.float64, device=dev)
    adot = torch.empty(n, dtype=torch.float64, device=dev)
    m = base_metric_struct(N.METRIC_FLRW)
    tab = cosmo.device_table(dev)
    m.cosmology = N.COSMO_TABLE
    m.a_table = tab.data_ptr()
    m.a_table_n = tab.shape[0]
    m.eta_min = cosmo.eta_min
    m.eta_step = cosmo.eta_step
    m.H0, m.omega_m, m.omega_r = cosmo.H0, cosmo.Omega_m, cosmo.Omega_r
    m.omega_k, m.omega_lambda = cosmo.Omega_k, cosmo.Omega_lambda
    lib = N.load()
    N.check(lib.exc_eval_cosmology(C.byref(m), N.ptr(e), N.ptr(a), N.ptr(adot), n, N.stream_handle(dev)),
            "exc_eval_cosmology")
    r = (a if which == "a" else adot).cpu().numpy()
    return float(r[0]) if scalar else r
