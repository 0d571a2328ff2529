"""Legacy fast interpolator (excalibur/grid/interpolator_fast.py:277-364).

The reference's older class ignores its `boundary` argument and always
applies the strict interior check rel in [1, n-2) with the base-node central
difference (`fused_interpolation_gradient`, :119-192) -- the same arithmetic
as the production interpolator's "error" mode, which is what this class runs.
"""
from __future__ import annotations

from .interpolator_4d_fast import InterpolatorFast as _Interp4D


class InterpolatorFast(_Interp4D):
    def __init__(self, grid, boundary="clamp", field_dtype=None):
        super().__init__(grid, "error", field_dtype)
        self.requested_boundary = boundary
