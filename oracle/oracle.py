"""ctypes wrapper of liboracle.so -- TEST INFRASTRUCTURE ONLY (the checker).

`Spacetime` describes a metric with plain numpy arrays; `oracle_*` functions
fill the same ExcMetric / ExcTraceArgs structs as the GPU library, with host
pointers, and run the C restatement of the reference (exc_oracle.c).
"""
from __future__ import annotations

import contextlib
import ctypes as C
import dataclasses
import os
from typing import Optional

import numpy as np

from excalibur_tool_gb300 import _native as N
from excalibur_tool_gb300.core import constants as K

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.oracle_trace.argtypes = [C.POINTER(N.ExcMetric), C.POINTER(N.ExcTraceArgs), C.c_int]
        L.oracle_rhs.argtypes = [C.POINTER(N.ExcMetric), P, P, P, P, C.c_int64]
        L.oracle_interp.argtypes = [C.POINTER(N.ExcField), P, P, P, C.c_int64]
        L.oracle_cosmology.argtypes = [C.POINTER(N.ExcMetric), P, P, P, C.c_int64]
        L.oracle_metric_tensor.argtypes = [C.POINTER(N.ExcMetric), P, P, P, P, C.c_int64]
        L.oracle_null_init.argtypes = [C.POINTER(N.ExcMetric), P, C.c_double, P, P, C.c_int64]
        L.oracle_null_error.argtypes = [C.POINTER(N.ExcMetric), P, P, P, P, C.c_int64]
        L.oracle_step.argtypes = [C.POINTER(N.ExcMetric), C.c_int, C.c_int, P, C.c_double, C.c_double, C.c_double,
                                  P, P, P]
        L.oracle_set_power_mode.argtypes = [C.c_int]
        L.oracle_power.argtypes = [P, P, C.c_int64, C.c_int]
        L.oracle_power_mode.restype = C.c_int
        _lib = L
    return _lib


@contextlib.contextmanager
def power_mode(mode):
    """Evaluate x**3 and x**4 with glibc pow() ("libm", the reference's `**`, the default) or with
    the CUDA library's double-double power ("dd") inside the block."""
    L = lib()
    prev = L.oracle_power_mode()
    L.oracle_set_power_mode({"libm": 0, "dd": 1}[mode])
    try:
        yield
    finally:
        L.oracle_set_power_mode(prev)


def power(x, p=3, mode="libm"):
    """x**p (p = 3 or 4) elementwise with glibc pow() or the double-double power."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    with power_mode(mode):
        lib().oracle_power(_p(x), _p(out), x.size, int(p))
    return out


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


@dataclasses.dataclass
class FieldSpec:
    data: np.ndarray
    spacing: tuple
    origin: tuple
    boundary: str = "periodic"
    gradient: str = "base_node"         # "base_node" | "trilinear" (the slow Interpolator)
    shift: tuple = (0.0, 0.0, 0.0)      # query offset of a shifted interpolator (runner local coords)


@dataclasses.dataclass
class Spacetime:
    """Plain-array description of a metric (both the oracle and the GPU tests build from it)."""
    kind: str                           # "flrw" | "schwarzschild"
    fields: list = dataclasses.field(default_factory=list)
    cosmology: str = "static"           # "static" | "table" | "table_fd"
    a_grid: Optional[np.ndarray] = None
    eta_min: float = 0.0
    eta_step: float = 1.0
    H0: float = 0.0
    omega: tuple = (0.0, 0.0, 0.0, 0.0)  # (m, r, k, lambda)
    analytical: bool = False
    free_time: bool = True
    mass: float = 0.0
    radius: float = 0.0
    center: tuple = (0.0, 0.0, 0.0)

    def struct(self):
        """ExcMetric with host pointers (keep `self` alive while it is used)."""
        m = N.ExcMetric()
        m.kind = N.METRIC_FLRW if self.kind == "flrw" else N.METRIC_SCHWARZSCHILD
        m.c, m.c2, m.c4 = K.C_F64, K.C2_F64, K.C4_F64
        m.two_over_c2 = 2 / K.c ** 2
        m.analytical = int(self.analytical)
        m.free_time = int(self.free_time)
        m.mass, m.radius = float(self.mass), float(self.radius)
        m.r_s = 2.0 * K.G * self.mass / (K.c * K.c) if self.kind == "schwarzschild" else 0.0
        for i in range(3):
            m.center[i] = float(self.center[i])
        m.cosmology = {"static": N.COSMO_STATIC, "table": N.COSMO_TABLE, "table_fd": N.COSMO_TABLE_FD}[self.cosmology]
        if self.a_grid is not None:
            self._a = np.ascontiguousarray(self.a_grid, dtype=np.float64)
            m.a_table = self._a.ctypes.data
            m.a_table_n = self._a.shape[0]
        m.eta_min, m.eta_step, m.H0 = float(self.eta_min), float(self.eta_step), float(self.H0)
        m.omega_m, m.omega_r, m.omega_k, m.omega_lambda = (float(v) for v in self.omega)
        self._fields = []
        for i, f in enumerate(self.fields):
            arr = np.ascontiguousarray(f.data)
            self._fields.append(arr)
            m.fields[i] = field_struct(arr, f.spacing, f.origin, f.boundary, f.gradient, f.shift)
        m.n_fields = len(self.fields)
        return m


def field_struct(arr, spacing, origin, boundary, gradient="base_node", shift=(0.0, 0.0, 0.0)):
    fs = N.ExcField()
    for d in range(3):
        fs.shift[d] = float(shift[d])
    fs.data = arr.ctypes.data
    fs.dtype = N.DTYPE_F32 if arr.dtype == np.float32 else N.DTYPE_F64
    fs.ndim = arr.ndim
    fs.boundary = N.BOUNDARY[boundary]
    fs.grad_mode = N.GRAD[gradient]
    for d in range(arr.ndim):
        fs.n[d] = arr.shape[d]
        fs.spacing[d] = float(spacing[d])
        fs.origin[d] = float(origin[d])
    return fs


def interp(field: FieldSpec, pts4):
    arr = np.ascontiguousarray(field.data)
    fs = field_struct(arr, field.spacing, field.origin, field.boundary, field.gradient, field.shift)
    pts = np.ascontiguousarray(pts4, dtype=np.float64)
    n = pts.shape[0]
    out = np.empty((n, 5))
    status = np.empty(n, dtype=np.int32)
    lib().oracle_interp(C.byref(fs), _p(pts), _p(out), _p(status), n)
    return out, status


def rhs(st: Spacetime, states, field_index=None):
    m = st.struct()
    s = np.ascontiguousarray(states, dtype=np.float64)
    out = np.empty_like(s)
    status = np.empty(s.shape[0], dtype=np.int32)
    lib().oracle_rhs(C.byref(m), _p(s), _p(out), _p(status), _p(field_index), s.shape[0])
    return out, status


def cosmology(st: Spacetime, eta):
    m = st.struct()
    e = np.ascontiguousarray(eta, dtype=np.float64)
    a = np.empty_like(e)
    ad = np.empty_like(e)
    lib().oracle_cosmology(C.byref(m), _p(e), _p(a), _p(ad), e.shape[0])
    return a, ad


def metric_tensor(st: Spacetime, x, field_index=None):
    m = st.struct()
    xs = np.ascontiguousarray(x, dtype=np.float64)
    g = np.empty((xs.shape[0], 4))
    status = np.empty(xs.shape[0], dtype=np.int32)
    lib().oracle_metric_tensor(C.byref(m), _p(xs), _p(g), _p(status), _p(field_index), xs.shape[0])
    return g, status


def null_init(st: Spacetime, states, sign=-1.0, field_index=None):
    m = st.struct()
    s = np.array(states, dtype=np.float64, copy=True)
    status = np.empty(s.shape[0], dtype=np.int32)
    lib().oracle_null_init(C.byref(m), _p(s), float(sign), _p(status), _p(field_index), s.shape[0])
    return s, status


def null_error(st: Spacetime, states, field_index=None):
    m = st.struct()
    s = np.ascontiguousarray(states, dtype=np.float64)
    rel = np.empty(s.shape[0])
    status = np.empty(s.shape[0], dtype=np.int32)
    lib().oracle_null_error(C.byref(m), _p(s), _p(rel), _p(status), _p(field_index), s.shape[0])
    return rel, status


def step(st: Spacetime, state, dt, stepper="rk4", tableau="reference", rtol=1e-9, atol=1e-13):
    m = st.struct()
    s = np.ascontiguousarray(state, dtype=np.float64)
    out = np.empty(8)
    dtn = np.empty(1)
    acc = np.empty(1, dtype=np.int32)
    rc = lib().oracle_step(C.byref(m), N.STEPPER[stepper], N.TABLEAU[tableau], _p(s), float(dt), float(rtol),
                           float(atol), _p(out), _p(dtn), _p(acc))
    return out, float(dtn[0]), bool(acc[0]), rc


@dataclasses.dataclass
class OracleResult:
    state: np.ndarray
    status: np.ndarray
    n_steps: np.ndarray
    n_iter: np.ndarray
    dt: np.ndarray
    obs: Optional[np.ndarray]
    records: Optional[np.ndarray]
    n_records: Optional[np.ndarray]


def trace(st: Spacetime, states, cfg, field_index=None, threads=1):
    """Run the C restatement of Integrator.integrate_single over every photon.

    `cfg` is an excalibur_tool_gb300.trace.TraceConfig (only its numbers are read)."""
    m = st.struct()
    n = states.shape[0]
    s = np.array(states, dtype=np.float64, copy=True)
    status = np.empty(n, dtype=np.int32)
    nsteps = np.empty(n, dtype=np.int32)
    niter = np.empty(n, dtype=np.int32)
    dts = np.full(n, float(cfg.dt))
    obs = np.empty((n, N.OBS_N)) if cfg.observables else None
    records = nrec = None
    cols = 14 if st.kind == "flrw" else 12
    if cfg.record_every is not None:
        from excalibur_tool_gb300.trace import _default_max_records
        mr = cfg.max_records if cfg.max_records > 0 else _default_max_records(cfg)
        records = np.full((n, mr, cols), np.nan)
        nrec = np.empty(n, dtype=np.int32)
    fidx = None if field_index is None else np.ascontiguousarray(field_index, dtype=np.int32)
    a = N.ExcTraceArgs()
    a.n_photons = n
    a.state, a.status, a.n_steps, a.n_iter, a.dt_state = (s.ctypes.data, status.ctypes.data, nsteps.ctypes.data,
                                                          niter.ctypes.data, dts.ctypes.data)
    a.field_index = fidx.ctypes.data if fidx is not None else None
    a.obs = obs.ctypes.data if obs is not None else None
    a.records = records.ctypes.data if records is not None else None
    a.n_records = nrec.ctypes.data if nrec is not None else None
    a.record_every = int(cfg.record_every or 0)
    a.max_records = records.shape[1] if records is not None else 0
    a.record_cols = cols
    a.stepper, a.tableau = N.STEPPER[cfg.stepper], N.TABLEAU[cfg.tableau]
    a.renormalize_every = int(cfg.renormalize_every)
    flags = 0
    if cfg.stop_box is not None:
        flags |= N.STOP_BOX
        for i in range(3):
            a.box_lo[i], a.box_hi[i] = float(cfg.stop_box[0][i]), float(cfg.stop_box[1][i])
        if getattr(cfg, "stop_face", False):
            flags |= N.STOP_FACE
    if cfg.a_stop is not None:
        flags |= N.STOP_A
        a.a_stop = float(cfg.a_stop)
    a.stop_flags = flags
    a.obs_flags = (N.OBS_ENDPOINTS | N.OBS_PATH | (N.OBS_ISW if cfg.isw else 0)) if obs is not None else 0
    a.dt, a.dt_min, a.dt_max, a.rtol, a.atol = (float(cfg.dt), float(cfg.dt_min), float(cfg.dt_max),
                                                float(cfg.rtol), float(cfg.atol))
    a.max_iter, a.max_steps = int(cfg.max_iter), int(cfg.max_steps)
    for i in range(3):
        a.lens_center[i] = float(cfg.lens_center[i])
    lib().oracle_trace(C.byref(m), C.byref(a), int(threads))
    return OracleResult(s, status, nsteps, niter, dts, obs, records, nrec)
