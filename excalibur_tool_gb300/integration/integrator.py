"""Integrators and the integration driver (excalibur/integration/integrator.py).

Same classes and signatures as the reference. What changes is where the work
runs: `Integrator.integrate` traces every photon in one persistent GPU launch
(`trace.trace_batch` -> `exc_trace`) instead of a Python loop over
`integrate_single`; `integrate_single` is the same launch with one photon.
The steppers' `step()` run one step through the same kernel.

`integrate` keeps the reference's per-mode contract (integrator.py:434-476):
* "sequential": every photon is integrated as `integrate_single` with its
  defaults (record_every=1: a history row per accepted step, the quantity
  columns one record late, the final record) and updated in order; the first
  photon that fails raises ValueError, as the reference's loop does, leaving
  the photons after it untouched; returns len(photons).
* "parallel" / "chunked": the same launch; a photon that succeeded is updated
  in place, a photon that failed keeps its input state and history; returns
  the number of successes. (The reference's chunked mode puts the integrated
  copies back into the Photons container; its parallel mode discards the
  pool's copies and only counts them.)
The photons are traced together in persistent launches (chunked so that the
recorded rows of one launch stay under 1 GiB of device memory) instead of one
process per photon or chunk; `n_workers` and `chunk_size` are kept for the
signature and select nothing.

Other differences, deliberate: stop modes "steps" as in the reference; "a"
stops once a(eta) <= value, and "box" at the first exit from the grid box (the
reference's "a", "redshift" and "chi" read attributes its Photon never sets,
integrator.py:204-211, so they cannot work there).
"""
from __future__ import annotations

import os

import numpy as np

from .. import _native as N
from ..trace import TraceConfig, trace_batch


class _Stepper:
    name = ""

    def step(self, metric, state, dt, rtol=1e-9, atol=1e-13):
        """One step on the GPU: returns (new_state, dt_new, accepted)."""
        import torch

        cfg = TraceConfig(stepper=self.name, dt=dt, dt_min=abs(dt), dt_max=abs(dt), rtol=rtol, atol=atol,
                          max_iter=1, max_steps=1, observables=False, use_queue=False,
                          tableau=getattr(self, "tableau", "reference"))
        s = torch.as_tensor(np.asarray(state, dtype=np.float64)[None]).cuda()
        r = trace_batch(metric, s, cfg)
        st = int(r.status[0])
        if st in N.FAILED_STATUSES:
            raise ValueError(f"step failed: {N.STATUS_NAMES.get(st, st)}")
        accepted = int(r.n_steps[0]) == 1
        return r.state[0].cpu().numpy(), float(r.dt[0]), accepted


class RK4(_Stepper):
    """Classic RK4 (integrator.py:9-22)."""
    name = "rk4"


class Leapfrog4(_Stepper):
    """Forest-Ruth 4th-order symplectic (integrator.py:24-90)."""
    name = "leapfrog4"


class RK45Adaptive(_Stepper):
    """Embedded RK4(5) with the reference's weights (integrator.py:93-152);
    `tableau="fehlberg"` uses Fehlberg's 6656/12825 instead of 665/1287."""
    name = "rk45"

    def __init__(self, tableau="reference"):
        if tableau not in ("reference", "fehlberg"):
            raise ValueError("tableau must be 'reference' or 'fehlberg'")
        self.tableau = tableau
        # the tableau the kernels step with, as arrays for callers that read it: stage
        # coefficients B (lower triangular), 5th-order weights C5, embedded 4th-order weights C4
        self.B = np.zeros((6, 6))
        self.B[1, :1] = [1 / 4]
        self.B[2, :2] = [3 / 32, 9 / 32]
        self.B[3, :3] = [1932 / 2197, -7200 / 2197, 7296 / 2197]
        self.B[4, :4] = [439 / 216, -8, 3680 / 513, -845 / 4104]
        self.B[5, :5] = [-8 / 27, 2, -3544 / 2565, 1859 / 4104, -11 / 40]
        c5_2 = 665 / 1287 if tableau == "reference" else 6656 / 12825
        self.C5 = np.array([16 / 135, 0, c5_2, 28561 / 56430, -9 / 50, 2 / 55])
        self.C4 = np.array([25 / 216, 0, 1408 / 2565, 2197 / 4104, -1 / 5, 0])


class Integrator:
    STOP_MODES = {"steps", "redshift", "a", "chi", "box"}
    INTEGRATORS = {"rk45": RK45Adaptive, "rk4": RK4, "leapfrog4": Leapfrog4}

    def __init__(self, metric, dt=1e-3, mode="sequential", integrator="rk45", rtol=1e-9, atol=1e-13,
                 dt_min=1e14, dt_max=1e17, n_workers=None, chunk_size=50, *, precision="fp64",
                 tableau="reference", max_iter=10_000, device=None):
        self.metric = metric
        self.dt = dt
        self.mode = mode
        self.rtol = rtol
        self.atol = atol
        self.dt_min = dt_min
        self.dt_max = dt_max
        self.chunk_size = chunk_size
        # the reference's default worker count (integrator.py:188); it selects nothing here
        self.n_workers = n_workers if n_workers is not None else max(1, (os.cpu_count() or 1) - 1)
        if integrator.lower() not in self.INTEGRATORS:
            raise ValueError(f"Integrator '{integrator}' not supported. Available: {list(self.INTEGRATORS.keys())}")
        self.integrator_name = integrator.lower()
        self.integrator = self.INTEGRATORS[self.integrator_name]()
        self.precision = precision
        self.tableau = tableau
        self.max_iter = max_iter
        self.device = device

    # ------------------------------------------------------------ config
    def config(self, stop_mode="steps", stop_value=100, *, record_every=None, renormalize_every=0,
               observables=True, **kw) -> TraceConfig:
        if stop_mode not in self.STOP_MODES:
            raise ValueError(f"stop_mode must be one of {self.STOP_MODES}")
        max_steps = int(stop_value) if stop_mode == "steps" else 2 ** 62
        a_stop = kw.pop("a_stop", None)
        stop_box = kw.pop("stop_box", None)
        if stop_mode == "a":
            a_stop = float(stop_value)
        elif stop_mode == "box":
            stop_box = stop_value if stop_value is not None else self._grid_box()
        elif stop_mode in ("redshift", "chi"):
            raise NotImplementedError(
                f"stop_mode '{stop_mode}' is not available (the reference's Photon never defines it); "
                "use 'a' (scale factor) or 'box'")
        return TraceConfig(stepper=self.integrator_name, tableau=self.tableau, precision=self.precision,
                           dt=float(self.dt), dt_min=float(self.dt_min), dt_max=float(self.dt_max),
                           rtol=float(self.rtol), atol=float(self.atol), max_iter=int(self.max_iter),
                           max_steps=max_steps, stop_box=stop_box, a_stop=a_stop,
                           renormalize_every=int(renormalize_every), record_every=record_every,
                           observables=observables, **kw)

    def _grid_box(self):
        g = getattr(self.metric, "grid", None)
        if g is None:
            raise ValueError("stop_mode='box' needs a metric with a grid, or an explicit ((lo), (hi)) box")
        lo = np.asarray(g.origin[:3], dtype=float)
        hi = lo + np.asarray(g.shape[:3], dtype=float) * np.asarray(g.spacing[:3], dtype=float)
        return (tuple(lo), tuple(hi))

    def _device(self):
        import torch

        if not torch.cuda.is_available():
            raise N.NativeError("a CUDA device is required (the tracer has no host fallback)")
        return torch.device(self.device) if self.device is not None else torch.device("cuda", torch.cuda.current_device())

    def _prepare_state(self, state):
        internal = getattr(self.metric, "internal_coords", None)
        input_coords = getattr(self.metric, "input_coords", None)
        if internal == "spherical" and input_coords == "cartesian":
            state = self.metric.cartesian_state_to_spherical(state)
        return state

    # --------------------------------------------------- batched API
    def trace(self, states, stop_mode="steps", stop_value=100, *, field_index=None, **cfg_kw):
        """Trace a [N, 8] float64 CUDA tensor of states; returns a TraceResult (device tensors)."""
        return trace_batch(self.metric, states, self.config(stop_mode, stop_value, **cfg_kw), field_index=field_index)

    def integrate_batch(self, states_host, stop_mode="steps", stop_value=100, *, field_index=None,
                        out_host=None, **cfg_kw):
        """End-to-end batch call on HOST arrays: copy in, trace, copy results back.

        `states_host` is a [N, 8] float64 array or (pinned) CPU tensor. Returns a
        dict of host arrays: state, status, n_steps and obs (when enabled).
        """
        import torch

        dev = self._device()
        src = states_host if isinstance(states_host, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(states_host, dtype=np.float64))
        d_states = src.to(dev, non_blocking=True)
        res = trace_batch(self.metric, d_states, self.config(stop_mode, stop_value, **cfg_kw),
                          field_index=field_index)
        if out_host is None:
            out_host = {"state": torch.empty(res.state.shape, dtype=torch.float64, pin_memory=True),
                        "status": torch.empty(res.status.shape, dtype=torch.int32, pin_memory=True),
                        "n_steps": torch.empty(res.n_steps.shape, dtype=torch.int32, pin_memory=True)}
            if res.obs is not None:
                out_host["obs"] = torch.empty(res.obs.shape, dtype=torch.float64, pin_memory=True)
        out_host["state"].copy_(res.state, non_blocking=True)
        out_host["status"].copy_(res.status, non_blocking=True)
        out_host["n_steps"].copy_(res.n_steps, non_blocking=True)
        if res.obs is not None and "obs" in out_host:
            out_host["obs"].copy_(res.obs, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()
        return out_host

    # ---------------------------------------------- reference-facing API
    _RECORD_BYTES_PER_LAUNCH = 1 << 30

    def _trace_recorded(self, plist, stop_mode, stop_value, record_every, renormalize_every):
        """Trace `plist` with records; yields (photon, status, rows [n, cols], final [8]) in order,
        in launches whose record buffers stay under _RECORD_BYTES_PER_LAUNCH."""
        import torch

        dev = self._device()
        cfg = self.config(stop_mode, stop_value, record_every=record_every, renormalize_every=renormalize_every,
                          observables=False)
        from ..trace import _default_max_records

        cols = 12 if getattr(self.metric, "internal_coords", None) == "spherical" else 14
        per_photon = _default_max_records(cfg) * cols * 8
        chunk = max(1, self._RECORD_BYTES_PER_LAUNCH // per_photon)
        for lo in range(0, len(plist), chunk):
            part = plist[lo:lo + chunk]
            states = np.stack([self._prepare_state(np.concatenate([p.x, p.u])) for p in part])
            res = trace_batch(self.metric, torch.as_tensor(states, device=dev), cfg)
            status = res.status.cpu().numpy()
            nrec = res.n_records.cpu().numpy()
            final = res.state.cpu().numpy()
            records = res.records.cpu().numpy()
            for i, p in enumerate(part):
                yield p, int(status[i]), records[i, :min(int(nrec[i]), records.shape[1])], final[i]

    @staticmethod
    def _apply(photon, rows, final):
        """Update `photon` as integrate_single does: x, u, the history rows, the quantities.

        A row recorded before the first quantity evaluation (the initial record, and the first
        step's: the reference records before it evaluates, integrator.py:387-394) carries the
        photon's quantities at call time -- none for a new photon (8 columns)."""
        q0 = np.asarray(photon.quantities, dtype=float)
        for row in rows:
            if np.isnan(row[8:]).all():
                photon.history.append(np.concatenate([row[:8], q0]))
            else:
                photon.history.append(row)
        photon.x = final[:4].copy()
        photon.u = final[4:].copy()

    def integrate_single(self, photon, stop_mode="steps", stop_value=100, *, record_every: int = 1,
                         trace_norm: bool = False, renormalize_every: int = 0):
        """Integrator.integrate_single (integrator.py:218-409): mutates `photon`
        (x, u, quantities, history, norm_history) exactly as the reference does."""
        if record_every < 0:
            raise ValueError("record_every must be >= 0")
        if renormalize_every < 0:
            raise ValueError("renormalize_every must be >= 0")
        if stop_mode not in self.STOP_MODES:
            raise ValueError(f"stop_mode must be one of {self.STOP_MODES}")
        if trace_norm and not hasattr(photon, "norm_history"):
            photon.norm_history = []
        _, st, rows, final = next(self._trace_recorded([photon], stop_mode, stop_value, record_every,
                                                       renormalize_every))
        norm_rows = None
        if trace_norm:
            # the reference appends the relative null error at the initial state, after every
            # accepted step (after its renormalisation) and once more at the end
            # (integrator.py:343-345, 384-385, 406-407): the rows of a record_every=1 trace of
            # the same trajectory, which also stops, without a final row, where a failure raises
            norm_rows = rows if record_every == 1 else next(self._trace_recorded(
                [photon], stop_mode, stop_value, 1, renormalize_every))[2]
        self._finish_single(photon, st, rows, final, record_every, norm_rows)
        return photon

    def _finish_single(self, photon, st, rows, final, record_every=1, norm_rows=None):
        from .._evaluate import null_error

        self._apply(photon, rows, final)
        if norm_rows is not None and len(norm_rows):
            rel, _ = null_error(self.metric, np.ascontiguousarray(np.asarray(norm_rows)[:, :8]))
            photon.norm_history.extend(np.atleast_1d(rel.cpu().numpy()).tolist())
        if st in N.FAILED_STATUSES:
            # the reference evaluated the quantities at its last recorded state before it failed
            # (integrator.py:387-394); they are in no record yet
            if record_every and len(rows) > 1:
                try:
                    photon.quantities = np.asarray(self.metric.metric_physical_quantities(rows[-1][:4]))
                except ValueError:
                    pass
            raise ValueError(f"integration failed: {N.STATUS_NAMES.get(st, st)}")
        photon.quantities = rows[-1][8:] if len(rows) else np.array([])

    def integrate(self, photons, stop_mode="steps", stop_value=100, verbose=True):
        """Integrator.integrate (integrator.py:434-476), with the reference's per-mode results
        (module docstring): "sequential" updates every photon like integrate_single, raises on
        the first failure and returns len(photons); "parallel" / "chunked" update the photons
        that succeeded and return their count."""
        if stop_mode not in self.STOP_MODES:
            raise ValueError(f"stop_mode must be one of {self.STOP_MODES}")
        if self.mode not in ("sequential", "parallel", "chunked"):
            raise ValueError("Unknown mode. Use 'sequential', 'parallel', or 'chunked'.")
        plist = list(photons)
        traced = self._trace_recorded(plist, stop_mode, stop_value, 1, 0)
        if self.mode == "sequential":
            for p, st, rows, final in traced:
                self._finish_single(p, st, rows, final)
            return len(photons)
        if verbose:
            if self.mode == "parallel":
                print(f"Parallel integration with {self.n_workers} workers...")
            else:
                n_chunks = (len(plist) + self.chunk_size - 1) // self.chunk_size
                print(f"Chunked mode: {n_chunks} chunks of size {self.chunk_size}")
        ok = 0
        for p, st, rows, final in traced:
            if st in N.FAILED_STATUSES:
                continue
            self._finish_single(p, st, rows, final)
            ok += 1
        return ok
