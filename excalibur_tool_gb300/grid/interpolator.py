"""The reference's slow interpolator (excalibur/grid/interpolator.py:4-206), on the GPU.

Same API as the reference class -- `interpolate`, `gradient`,
`time_derivative`, `value_and_gradient`, `value_gradient_and_time_derivative`
-- with every evaluation done by the CUDA library (`exc_interp`) and the
tracer reading the same ExcField (grad_mode EXC_GRAD_TRILINEAR) inside its
fused RHS:

* value: trilinear over the cell of rel = (x - origin) / spacing, ValueError
  unless rel is in [0, n-1) on every spatial axis (:36-43); 4-D grids blend
  the two snapshots around t quadrilinearly (time index clipped to
  [0, nt-2], weight not clipped, no time bounds check, :26-31);
* gradient: the trilinear blend of the central differences at the cell's
  eight corners, base index clipped to [1, n-2] (:88-158) -- smooth across
  cell faces, unlike the base-node gradient of the fast classes; 4-D grids
  take it on the snapshot nearest in time (:92-96);
* time derivative (4-D): central difference of the snapshots either side of
  clip(floor(rel_t), 1, nt-2) (:160-174); 0.0 on 3-D grids (:200-203).

One deliberate difference: `gradient` and `time_derivative` called on their
own raise outside the bounds, where the reference's extrapolate from the
clipped cell; through `value_gradient_and_time_derivative` (what the metrics
call) the reference raises first in `interpolate`, so the two agree there.
"""
from __future__ import annotations

import numpy as np

from .interpolator_4d_fast import InterpolatorFast


class Interpolator(InterpolatorFast):
    gradient_mode = "trilinear"

    def __init__(self, grid, field_dtype=None):
        # the slow class has one bounds rule; "error" is its ExcField boundary
        super().__init__(grid, "error", field_dtype)

    def _eval(self, x, field, t):
        if self.is_4d and t is None:
            # the reference's 3-D path on a 4-D field slices whole time columns
            # (grid/interpolator.py:47-50); only the t-given form is defined here
            raise ValueError("4D grid: you must pass t")
        p = [float(x[0]), float(x[1]), float(x[2]), float(t if t is not None else 0.0)]
        val, grad, dtd, status = self.evaluate([p], field)
        if int(status[0]) != 0:
            raise ValueError(f"Position {x} outside grid bounds")
        return float(val[0]), np.array(grad[0].tolist()), float(dtd[0])

    def interpolate(self, x, field, t=None):
        return self._eval(x, field, t)[0]

    def gradient(self, x, field, t=None):
        return self._eval(x, field, t)[1]

    def time_derivative(self, x, field, t):
        if not self.is_4d:
            raise ValueError("Time derivative only available for 4D grids")
        return self._eval(x, field, t)[2]

    def value_and_gradient(self, x, field, t=None):
        v, g, _ = self._eval(x, field, t)
        return v, g

    def value_gradient_and_time_derivative(self, x, field, t=None):
        v, g, d = self._eval(x, field, t)
        return v, g, (d if self.is_4d else 0.0)
