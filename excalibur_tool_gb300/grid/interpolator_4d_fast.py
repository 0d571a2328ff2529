"""Production interpolator (excalibur/grid/interpolator_4d_fast.py:409-533).

Trilinear Phi plus the base-node central-difference gradient, boundary modes
"error" (strict interior, ValueError outside), "clamp" and "periodic"
(default), 3-D fields or 4-D time snapshots (linear in time, dPhi/dt from the
two snapshots). Evaluation runs on the GPU (`exc_interp`); the tracer reads
the same descriptor inside its fused RHS.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .. import _native as N


class InterpolatorFast:
    gradient_mode = "base_node"   # central difference at the cell's base node
    shift = None                  # query offset (shifted_interpolator); None = query x itself

    def __init__(self, grid, boundary: str = "periodic", field_dtype=None):
        if boundary not in ("error", "clamp", "periodic"):
            raise ValueError("boundary must be one of: 'error', 'clamp', 'periodic'")
        self.grid = grid
        self.is_4d = len(grid.shape) == 4
        self.boundary = boundary
        self.field_dtype = field_dtype
        self.origin = np.array(grid.origin, dtype=np.float64)
        self.spacing = np.array(grid.spacing, dtype=np.float64)
        self.shape = np.array(grid.shape, dtype=np.int64)
        if self.is_4d:
            if self.origin.shape[0] != 4 or self.spacing.shape[0] != 4 or self.shape.shape[0] != 4:
                raise ValueError("4D grid requires origin/spacing/shape of length 4")
        else:
            if self.origin.shape[0] < 3 or self.spacing.shape[0] < 3 or self.shape.shape[0] < 3:
                raise ValueError("3D grid requires origin/spacing/shape of length >= 3")

    # ---- descriptor used by the tracer and exc_interp --------------------
    def field_struct(self, field, device, split=False):
        """ExcField for `field` on `device`. With `split`, a float64 grid is passed
        as two float32 planes (hi, lo) for the mixed-precision tracer."""
        from ..trace import field_struct

        t = self.grid.device_field(field, device, self.field_dtype)
        nd = 4 if self.is_4d else 3
        if split and str(t.dtype) == "torch.float64":
            planes = self.grid.device_field_split(field, device)
            f = field_struct(planes, self.shape[:nd], self.spacing[:nd], self.origin[:nd], self.boundary,
                             split=True, gradient=self.gradient_mode, shift=self.shift)
            return f, planes
        return field_struct(t, self.shape[:nd], self.spacing[:nd], self.origin[:nd], self.boundary,
                            gradient=self.gradient_mode, shift=self.shift), t

    # ---- batched evaluation ----------------------------------------------
    def evaluate(self, points, field="Phi", device="cuda"):
        """points [N, 3] or [N, 4] (x, y, z[, t]) -> (val [N], grad [N, 3], dtd [N], status [N])."""
        import torch

        pts = torch.as_tensor(points, dtype=torch.float64)
        if pts.ndim == 1:
            pts = pts[None]
        n = pts.shape[0]
        p4 = torch.zeros((n, 4), dtype=torch.float64)
        p4[:, : min(4, pts.shape[1])] = pts[:, :4].cpu() if pts.device.type != "cpu" else pts[:, :4]
        p4 = p4.to(device)
        out = torch.empty((n, 5), dtype=torch.float64, device=device)
        status = torch.empty(n, dtype=torch.int32, device=device)
        f, keep = self.field_struct(field, device)
        lib = N.load()
        N.check(lib.exc_interp(C.byref(f), N.ptr(p4), N.ptr(out), N.ptr(status), n, N.stream_handle(device)),
                "exc_interp")
        return out[:, 0], out[:, 1:4], out[:, 4], status

    def value_gradient_and_time_derivative(self, x, field, t=None):
        if self.is_4d and t is None:
            raise ValueError("4D grid: you must pass t for time interpolation/derivative")
        p = [float(x[0]), float(x[1]), float(x[2]), float(t if t is not None else 0.0)]
        val, grad, dtd, status = self.evaluate([p], field)
        if int(status[0]) != 0:
            raise ValueError(f"Point {x} outside grid bounds (boundary='{self.boundary}')")
        g = grad[0].tolist()
        return float(val[0]), (g[0], g[1], g[2]), float(dtd[0])

    def interpolate(self, x, field, t=None):
        if self.is_4d and t is None:
            raise ValueError("4D grid: you must pass t to interpolate")
        return self.value_gradient_and_time_derivative(x, field, t if self.is_4d else 0.0)[0]

    def gradient(self, x, field, t=None):
        if self.is_4d and t is None:
            raise ValueError("4D grid: you must pass t to gradient")
        return self.value_gradient_and_time_derivative(x, field, t if self.is_4d else 0.0)[1]

    def value_and_gradient(self, x, field, t=None):
        if self.is_4d and t is None:
            raise ValueError("4D grid: you must pass t to value_and_gradient")
        v, g, _ = self.value_gradient_and_time_derivative(x, field, t if self.is_4d else 0.0)
        return v, g


def shifted_interpolator(base, shift):
    """`base` queried at x + shift: the comparison runners' _ShiftedInterpolator
    (_excalibur_runs/excalibur_run_compare_schwarzschild_vs_flrw.py:39-56), which lets them
    integrate in observer-local coordinates against a grid laid out in absolute ones.

    Returns a copy of `base` sharing its grid (and the grid's device copy); the offset
    travels in ExcField.shift, so the tracer and `evaluate` both add it on the device with
    one float64 addition per component, as the reference's wrapper does on the host."""
    import copy

    ip = copy.copy(base)
    sh = np.asarray(shift, dtype=np.float64).reshape(-1)
    if sh.shape[0] != 3 or not np.all(np.isfinite(sh)):
        raise ValueError("shift must be three finite numbers")
    ip.shift = sh.copy()
    return ip
