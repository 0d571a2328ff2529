"""`torch.ops.excalibur_gb.trace`: the batched tracer as a PyTorch custom operator.

A thin wrapper of `trace.trace_batch` (and so of the C ABI's `exc_trace`) for callers that
compose PyTorch operators: its schema holds only tensors and plain numbers, the spacetime
being passed by a handle from `register_metric` (metric objects hold device grids and tables
that an operator schema cannot carry). A fake (meta) implementation gives the output shapes
without running anything, so the operator can be traced by PyTorch's graph tools; the real
implementation launches the persistent kernel on the current stream.

    h = register_metric(metric)
    state, status, n_steps = torch.ops.excalibur_gb.trace(states, h, "rk4", "fp64", dl, dl, dl,
                                                          2000, 10_000, 1e-9, 1e-13, [], [], 0.0)
"""
from __future__ import annotations

import itertools
import threading
from typing import List, Tuple

import torch

_LOCK = threading.Lock()
_METRICS = {}
_NEXT = itertools.count(1)


def register_metric(metric) -> int:
    """A handle for `metric` (any of the package's metric classes) to pass to the operator."""
    with _LOCK:
        h = next(_NEXT)
        _METRICS[h] = metric
    return h


def release_metric(handle: int) -> None:
    with _LOCK:
        _METRICS.pop(int(handle), None)


def _metric(handle: int):
    with _LOCK:
        m = _METRICS.get(int(handle))
    if m is None:
        raise ValueError(f"unknown metric handle {handle} (register_metric first)")
    return m


@torch.library.custom_op("excalibur_gb::trace", mutates_args=())
def trace(states: torch.Tensor, metric: int, stepper: str, precision: str, dt: float, dt_min: float,
          dt_max: float, max_steps: int, max_iter: int, rtol: float, atol: float, box_lo: List[float],
          box_hi: List[float], a_stop: float) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Trace `states` [N, 8] float64 (CUDA) through the registered metric: final states [N, 8],
    status [N] int32 (EXC_PH_*), accepted steps [N] int32. `box_lo`/`box_hi` empty = no box stop;
    `a_stop` <= 0 = no a(eta) stop; other arguments as in TraceConfig."""
    from .trace import TraceConfig, trace_batch

    if (len(box_lo) == 0) != (len(box_hi) == 0) or len(box_lo) not in (0, 3):
        raise ValueError("box_lo and box_hi must both be empty or both have 3 entries")
    cfg = TraceConfig(stepper=stepper, precision=precision, dt=dt, dt_min=dt_min, dt_max=dt_max,
                      max_steps=max_steps, max_iter=max_iter, rtol=rtol, atol=atol,
                      stop_box=(tuple(box_lo), tuple(box_hi)) if box_lo else None,
                      a_stop=a_stop if a_stop > 0 else None, observables=False)
    r = trace_batch(_metric(metric), states.contiguous(), cfg)
    return r.state, r.status, r.n_steps


@trace.register_fake
def _trace_fake(states, metric, stepper, precision, dt, dt_min, dt_max, max_steps, max_iter, rtol, atol, box_lo,
                box_hi, a_stop):
    n = states.shape[0]
    return (torch.empty_like(states), states.new_empty((n,), dtype=torch.int32),
            states.new_empty((n,), dtype=torch.int32))
