"""Batched tracing: the one call every reference-facing API ends in.

`trace_batch(metric, states, cfg)` packs the metric, grids and cosmology
table into the C ABI structs (include/excalibur_gb300.h) and runs
`exc_trace` on the current CUDA stream. It replaces the per-photon Python
loop of `Integrator.integrate_single` / `Integrator.integrate`
(excalibur/integration/integrator.py:218-476) with one persistent launch.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from .core import constants as K


@dataclasses.dataclass(frozen=True)
class TraceConfig:
    """Everything `Integrator.integrate_single` takes, plus the added stops.

    Defaults are the reference's: RK45 with rtol=1e-9, atol=1e-13,
    dt clipped to [1e14, 1e17] s, max_iter=10000 (integrator.py:167-178, :261).
    """

    stepper: str = "rk45"            # "rk4" | "rk45" | "leapfrog4"
    tableau: str = "reference"       # RK45 weights: "reference" (665/1287) | "fehlberg"
    precision: str = "fp64"          # "fp64" (reference order) | "fp64_fast" | "mixed" | "mixed_raw" | "retrace"
    dt: float = 1e-3
    dt_min: float = 1e14
    dt_max: float = 1e17
    rtol: float = 1e-9
    atol: float = 1e-13
    max_iter: int = 10_000
    max_steps: int = 100             # the "steps" stop value
    stop_box: Optional[tuple] = None  # ((lo_x, lo_y, lo_z), (hi_x, hi_y, hi_z)): stop on exit
    stop_face: bool = False           # with stop_box (FLRW): the last step is shortened to end on the face
    a_stop: Optional[float] = None   # stop once a(eta) <= a_stop (FLRW)
    renormalize_every: int = 0
    record_every: Optional[int] = None   # None = no records; else reference semantics
    max_records: int = 0
    observables: bool = True
    isw: bool = False
    lens_center: tuple = (0.0, 0.0, 0.0)
    block_size: int = 0
    blocks_per_sm: int = 0
    staging: str = "cache"           # FP64 tracers' a(eta) table: "cache" (read-only cache) | "shared" (shared memory)
    use_queue: bool = True
    deadline_cycles: int = 0

    def validate(self):
        if self.stepper not in N.STEPPER:
            raise ValueError(f"Integrator '{self.stepper}' not supported. Available: {list(N.STEPPER)}")
        if self.tableau not in N.TABLEAU:
            raise ValueError(f"tableau must be one of {list(N.TABLEAU)}")
        if self.precision not in N.PRECISION:
            raise ValueError(f"precision must be one of {list(N.PRECISION)}")
        if self.record_every is not None and self.record_every < 0:
            raise ValueError("record_every must be >= 0")
        if self.renormalize_every < 0:
            raise ValueError("renormalize_every must be >= 0")
        if self.max_iter < 0 or self.max_steps < 0:
            raise ValueError("max_iter and max_steps must be >= 0")
        if not math.isfinite(self.dt):
            raise ValueError("dt must be finite")
        if self.stop_face and self.stop_box is None:
            raise ValueError("stop_face needs stop_box")
        if self.staging not in N.STAGING:
            raise ValueError(f"staging must be one of {list(N.STAGING)}")
        return self


@dataclasses.dataclass
class TraceResult:
    state: "torch.Tensor"            # [N, 8] float64, final (last accepted) state
    status: "torch.Tensor"           # [N] int32, EXC_PH_* codes
    n_steps: "torch.Tensor"          # [N] int32 accepted steps
    n_iter: "torch.Tensor"           # [N] int32 iterations (accepted + rejected)
    dt: "torch.Tensor"               # [N] float64 final dt
    obs: Optional["torch.Tensor"] = None       # [N, 20] float64
    records: Optional["torch.Tensor"] = None   # [N, max_records, cols]
    n_records: Optional["torch.Tensor"] = None

    def obs_dict(self):
        o = self.obs
        return {name: o[:, i] for i, name in enumerate(N.OBS_COLS)}


class MetricDescriptor:
    """An ExcMetric plus the device tensors its pointers refer to."""

    def __init__(self, struct: N.ExcMetric, keepalive: list, record_cols: int, kind: int):
        self.struct = struct
        self.keepalive = keepalive
        self.record_cols = record_cols
        self.kind = kind


def base_metric_struct(kind: int) -> N.ExcMetric:
    m = N.ExcMetric()
    m.kind = kind
    m.c = K.C_F64
    m.c2 = K.C2_F64
    m.c4 = K.C4_F64
    m.two_over_c2 = 2 / K.c ** 2      # exact rational 2/c**2 rounded once (Python int / int)
    return m


def field_struct(data, shape, spacing, origin, boundary: str, split: bool = False,
                 gradient: str = "base_node", shift=None) -> N.ExcField:
    import torch

    f = N.ExcField()
    if split:
        if data.dtype != torch.float32:
            raise TypeError("split planes must be float32")
        f.dtype = N.DTYPE_F32X2
    elif data.dtype == torch.float64:
        f.dtype = N.DTYPE_F64
    elif data.dtype == torch.float32:
        f.dtype = N.DTYPE_F32
    else:
        raise TypeError(f"field dtype must be float64 or float32, got {data.dtype}")
    if not data.is_contiguous():
        raise ValueError("field data must be C-contiguous")
    if boundary not in N.BOUNDARY:
        raise ValueError("boundary must be one of: 'error', 'clamp', 'periodic'")
    if gradient not in N.GRAD:
        raise ValueError("gradient must be 'base_node' or 'trilinear'")
    f.data = data.data_ptr()
    f.ndim = len(shape)
    f.boundary = N.BOUNDARY[boundary]
    f.grad_mode = N.GRAD[gradient]
    for d in range(len(shape)):
        f.n[d] = int(shape[d])
        f.spacing[d] = float(spacing[d])
        f.origin[d] = float(origin[d])
    if shift is not None:
        for d in range(3):
            f.shift[d] = float(shift[d])
    return f


def _check_device_tensor(t, dtype, shape_tail, name):
    import torch

    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if t.device.type != "cuda":
        raise ValueError(f"{name} must live on a CUDA device (got {t.device})")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if tuple(t.shape[1:]) != tuple(shape_tail):
        raise ValueError(f"{name} must have shape [N, {', '.join(map(str, shape_tail))}]")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def trace_batch(metric, states, cfg: TraceConfig, *, field_index=None, dt=None, out=None,
                queue=None, abort_flag=None, stream=None, check_field_index=True) -> TraceResult:
    """Trace every photon of `states` ([N, 8] float64 on a CUDA device) in one launch.

    `metric` is any of the package's metric classes (it provides `descriptor(device)`).
    `states` is not modified; the result holds fresh tensors (or `out`'s).
    `check_field_index=False` skips the range check of `field_index` (a device reduction and
    a host synchronisation) for callers that built it in range; the kernel still gives an
    out-of-range photon the status EXC_PH_BAD_FIELD.
    """
    import torch

    cfg.validate()
    _check_device_tensor(states, torch.float64, (8,), "states")
    dev = states.device
    n = states.shape[0]
    desc = metric.descriptor(dev, split=cfg.precision in ("mixed", "mixed_raw", "retrace"))
    if out is None:
        st = states.clone()
        status = torch.empty(n, dtype=torch.int32, device=dev)
        nsteps = torch.empty(n, dtype=torch.int32, device=dev)
        niter = torch.empty(n, dtype=torch.int32, device=dev)
        dts = torch.empty(n, dtype=torch.float64, device=dev)
        obs = torch.empty((n, N.OBS_N), dtype=torch.float64, device=dev) if cfg.observables else None
    else:
        st, status, nsteps, niter, dts, obs = (out.state, out.status, out.n_steps, out.n_iter, out.dt, out.obs)
        st.copy_(states)
    if dt is None:
        dts.fill_(float(cfg.dt))
    else:
        dts.copy_(dt)
    records = nrec = None
    if cfg.record_every is not None:
        mr = cfg.max_records if cfg.max_records > 0 else _default_max_records(cfg)
        records = torch.empty((n, mr, desc.record_cols), dtype=torch.float64, device=dev)
        nrec = torch.empty(n, dtype=torch.int32, device=dev)
    if field_index is not None:
        if field_index.dtype != torch.int32 or field_index.device != dev or field_index.shape != (n,):
            raise ValueError("field_index must be an int32 [N] tensor on the states' device")
        nf = desc.struct.n_fields
        if check_field_index and n and (int(field_index.min()) < 0 or int(field_index.max()) >= nf):
            raise ValueError(f"field_index values must lie in [0, {nf})")
    res = TraceResult(st, status, nsteps, niter, dts, obs, records, nrec)
    res.field_index = field_index
    _launch(desc, res, cfg, queue=queue, abort_flag=abort_flag, stream=stream)
    return res


def _make_args(desc, res, cfg: TraceConfig, queue=None, abort_flag=None) -> N.ExcTraceArgs:
    """ExcTraceArgs pointing at `res`'s tensors."""
    n = res.state.shape[0]
    st, status, nsteps, niter, dts, obs = res.state, res.status, res.n_steps, res.n_iter, res.dt, res.obs
    records, nrec = res.records, res.n_records
    field_index = getattr(res, "field_index", None)

    a = N.ExcTraceArgs()
    a.n_photons = n
    a.state = st.data_ptr()
    a.status = status.data_ptr()
    a.n_steps = nsteps.data_ptr()
    a.n_iter = niter.data_ptr()
    a.dt_state = dts.data_ptr()
    a.field_index = field_index.data_ptr() if field_index is not None else None
    a.obs = obs.data_ptr() if obs is not None else None
    a.records = records.data_ptr() if records is not None else None
    a.n_records = nrec.data_ptr() if nrec is not None else None
    a.record_every = int(cfg.record_every or 0)
    a.max_records = records.shape[1] if records is not None else 0
    a.record_cols = desc.record_cols
    a.stepper = N.STEPPER[cfg.stepper]
    a.tableau = N.TABLEAU[cfg.tableau]
    a.precision = N.PRECISION[cfg.precision]
    a.renormalize_every = int(cfg.renormalize_every)
    flags = 0
    if cfg.stop_box is not None:
        flags |= N.STOP_BOX
        lo, hi = cfg.stop_box
        for i in range(3):
            a.box_lo[i] = float(lo[i])
            a.box_hi[i] = float(hi[i])
        if cfg.stop_face:
            flags |= N.STOP_FACE
    if cfg.a_stop is not None:
        flags |= N.STOP_A
        a.a_stop = float(cfg.a_stop)
    a.stop_flags = flags
    a.obs_flags = (N.OBS_ENDPOINTS | N.OBS_PATH | (N.OBS_ISW if cfg.isw else 0)) if obs is not None else 0
    a.block_size = int(cfg.block_size)
    a.blocks_per_sm = int(cfg.blocks_per_sm)
    a.staging = N.STAGING[cfg.staging]
    a.dt = float(cfg.dt)
    a.dt_min = float(cfg.dt_min)
    a.dt_max = float(cfg.dt_max)
    a.rtol = float(cfg.rtol)
    a.atol = float(cfg.atol)
    a.max_iter = int(cfg.max_iter)
    a.max_steps = int(cfg.max_steps)
    for i in range(3):
        a.lens_center[i] = float(cfg.lens_center[i])
    a.queue = queue.data_ptr() if queue is not None else None
    a.abort_flag = abort_flag.data_ptr() if abort_flag is not None else None
    a.deadline_cycles = int(cfg.deadline_cycles)
    return a


def _launch(desc, res, cfg: TraceConfig, *, queue=None, abort_flag=None, stream=None):
    """Call exc_trace on `res`'s tensors on `stream`."""
    import torch

    dev = res.state.device
    s = torch.cuda.current_stream(dev) if stream is None else stream
    if queue is None and cfg.use_queue:
        with torch.cuda.stream(s):
            queue = torch.zeros(2, dtype=torch.int64, device=dev)
    a = _make_args(desc, res, cfg, queue, abort_flag)
    lib = N.load()
    with torch.cuda.device(dev):
        N.check(lib.exc_trace(C.byref(desc.struct), C.byref(a), C.c_void_p(s.cuda_stream)), "exc_trace")
    res._keepalive = (desc, queue)
    return res


def retrace(metric, res: TraceResult, cfg: TraceConfig, *, stream=None) -> TraceResult:
    """The FP64 pass of the guarded mixed tracer over `res` in place: photons that a
    "mixed_raw" trace handed back (status "retrace") are traced by the FP64 tracer;
    every other photon's outputs are left as they are."""
    cfg = dataclasses.replace(cfg, precision="retrace").validate()
    desc = metric.descriptor(res.state.device, split=True)
    return _launch(desc, res, cfg, stream=stream)


def trace_pipelined(metric, batches: Sequence, cfg: TraceConfig, *, side_stream=None) -> list:
    """Guarded mixed tracing of several batches with the re-traces overlapped.

    Each batch's mixed launch runs on the current stream; its FP64 re-trace of the
    handed-back rays (a few percent, each as long as a full FP64 trajectory) runs on
    `side_stream` after an event, so it overlaps the next batches' mixed launches.
    The current stream waits for the side stream before returning; results are
    those of precision "mixed" (identical per photon)."""
    import torch

    if cfg.precision not in ("mixed", "mixed_raw"):
        raise ValueError("trace_pipelined runs the mixed tracer")
    raw = dataclasses.replace(cfg, precision="mixed_raw")
    main = torch.cuda.current_stream(batches[0].device)
    side = side_stream or torch.cuda.Stream(batches[0].device)
    out = []
    for b in batches:
        r = trace_batch(metric, b, raw)
        ev = torch.cuda.Event()
        ev.record(main)
        side.wait_event(ev)
        for t in (r.state, r.status, r.n_steps, r.n_iter, r.dt, r.obs):
            if t is not None:
                t.record_stream(side)
        retrace(metric, r, cfg, stream=side)
        out.append(r)
    done = torch.cuda.Event()
    done.record(side)
    main.wait_event(done)
    return out


_TUNE_CACHE: dict = {}


def autotune(metric, states, cfg: TraceConfig, *, field_index=None, sample: Optional[int] = None, seed: int = 0,
             time_box_cycles: int = 1_000_000_000, use_cache: bool = True) -> TraceConfig:
    """`cfg` with the (block_size, blocks_per_sm, staging) that exc_autotune measured fastest.

    By default every trial traces the whole batch (in a seeded shuffled order), so
    the score -- steps tried per second -- includes the wave quantisation and the
    tail of the batch as it will run; each trial is time-boxed (`time_box_cycles`
    SM clock cycles, ~0.5 s), which turns the score into the steady-state rate for
    batches too large to finish in the box. `sample` traces a random subset
    instead. Plans are cached per device, metric kind, stepper, tableau,
    precision, grid dtype, number of fields and batch size."""
    import torch

    dev = states.device
    desc = metric.descriptor(dev, split=cfg.precision in ("mixed", "mixed_raw", "retrace"))
    key = (torch.cuda.get_device_name(dev), desc.kind, cfg.stepper, cfg.tableau, cfg.precision,
           int(desc.struct.fields[0].dtype), int(desc.struct.n_fields), int(states.shape[0]))
    if use_cache and key in _TUNE_CACHE:
        b, p = _TUNE_CACHE[key][:2]
        return dataclasses.replace(cfg, block_size=b, blocks_per_sm=p, staging=_TUNE_CACHE[key][6])
    n = states.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    idx = torch.randperm(n, generator=g)[:min(sample or n, n)].to(dev)
    pristine = states[idx].contiguous()
    fidx = field_index[idx].contiguous() if field_index is not None else None
    m = pristine.shape[0]
    res = TraceResult(pristine.clone(), torch.empty(m, dtype=torch.int32, device=dev),
                      torch.empty(m, dtype=torch.int32, device=dev), torch.empty(m, dtype=torch.int32, device=dev),
                      torch.empty(m, dtype=torch.float64, device=dev),
                      torch.empty((m, N.OBS_N), dtype=torch.float64, device=dev) if cfg.observables else None)
    res.field_index = fidx
    queue = torch.zeros(2, dtype=torch.int64, device=dev) if cfg.use_queue else None
    a = _make_args(desc, res, dataclasses.replace(cfg, deadline_cycles=int(time_box_cycles)), queue)
    a.dt_state = None
    plan = N.ExcLaunchPlan()
    lib = N.load()
    with torch.cuda.device(dev):
        N.check(lib.exc_autotune(C.byref(desc.struct), C.byref(a), C.c_void_p(pristine.data_ptr()), C.byref(plan),
                                 N.stream_handle(dev)), "exc_autotune")
    names = {v: k for k, v in N.STAGING.items()}
    trials = [(plan.trial_block[i], plan.trial_blocks_per_sm[i], names[plan.trial_staging[i]], plan.trial_ms[i],
               plan.trial_rate[i]) for i in range(plan.n_trials)]
    staging = names[plan.staging]
    _TUNE_CACHE[key] = (plan.block_size, plan.blocks_per_sm, plan.best_ms, trials, plan.best_rate, m, staging)
    return dataclasses.replace(cfg, block_size=plan.block_size, blocks_per_sm=plan.blocks_per_sm, staging=staging)


def tune_report() -> dict:
    return {str(k): {"block_size": v[0], "blocks_per_sm": v[1], "staging": v[6], "best_ms": v[2], "trials": v[3],
                     "best_rate": v[4], "sample": v[5]} for k, v in _TUNE_CACHE.items()}


class CapturedTrace:
    """A trace of a fixed-size batch captured once in a CUDA graph and replayed.

    The graph holds the copy of the input states into the result buffer, the dt
    reset, the work-queue reset and the exc_trace launch(es) (two for the guarded
    mixed tracer), so one replay is one graph launch with no host work between
    kernels. `run(states)` copies new inputs into the static input buffer first."""

    def __init__(self, metric, states, cfg: TraceConfig, *, field_index=None):
        import torch

        cfg.validate()
        if cfg.record_every is not None:
            raise ValueError("records are not captured")
        dev = states.device
        n = states.shape[0]
        self.cfg = cfg
        self.desc = metric.descriptor(dev, split=cfg.precision in ("mixed", "mixed_raw", "retrace"))
        self.inputs = states.clone()
        self.field_index = field_index.clone() if field_index is not None else None
        self.res = TraceResult(states.clone(), torch.empty(n, dtype=torch.int32, device=dev),
                               torch.empty(n, dtype=torch.int32, device=dev),
                               torch.empty(n, dtype=torch.int32, device=dev),
                               torch.empty(n, dtype=torch.float64, device=dev),
                               torch.empty((n, N.OBS_N), dtype=torch.float64, device=dev) if cfg.observables else None)
        self.res.field_index = self.field_index
        self.queue = torch.zeros(2, dtype=torch.int64, device=dev) if cfg.use_queue else None
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):              # eager run: loads the kernels before capture
            self._body()
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._body()

    def _body(self):
        self.res.state.copy_(self.inputs)
        self.res.dt.fill_(float(self.cfg.dt))
        _launch(self.desc, self.res, self.cfg, queue=self.queue)

    def run(self, states=None) -> TraceResult:
        if states is not None:
            self.inputs.copy_(states)
        self.graph.replay()
        return self.res


def _default_max_records(cfg: TraceConfig) -> int:
    # initial + one per recorded step + final
    n = min(cfg.max_steps, cfg.max_iter)
    if cfg.record_every in (None, 0):
        return 2
    return n // cfg.record_every + 3
