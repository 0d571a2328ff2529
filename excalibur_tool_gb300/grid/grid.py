"""Potential grids (excalibur/grid/grid.py:57-112).

`Grid(shape, spacing, origin)` holds named fields exactly like the reference
(C-order [i, j, k] arrays, or [i, j, k, t] with time innermost). A field is
uploaded to the GPU once per (device, dtype) and stays resident; the tracer
reads it in place. POSIX shared memory (the reference's `shared=True`, used
to feed CPU worker pools) has no role on one GPU and is accepted but ignored.
"""
from __future__ import annotations

import numpy as np


class Grid:
    def __init__(self, shape, spacing, origin=(0, 0, 0), cycle=False):
        self.shape = np.array(shape)
        self.spacing = np.array(spacing, dtype=float)
        self.origin = np.array(origin, dtype=float)
        self.fields = {}
        self.cycle = cycle
        self._device = {}

    def add_field(self, name, data, shared=False):
        """Register a field; `data` is a numpy array or a torch tensor of this grid's shape."""
        if tuple(data.shape) != tuple(int(s) for s in self.shape):
            raise ValueError("field shape does not match the grid shape")
        self.fields[name] = data
        for key in [k for k in self._device if k[0] == name]:
            del self._device[key]

    def get_value(self, name, i, j, k):
        return self.fields[name][i, j, k]

    def physical_position(self, indices):
        return self.origin + indices * self.spacing

    def indices_from_position(self, position):
        relative_pos = (np.array(position) - self.origin) / self.spacing
        indices = np.floor(relative_pos).astype(int)
        if self.cycle:
            indices = indices % self.shape
        return indices

    def device_field(self, name, device, dtype=None):
        """The field as a contiguous tensor on `device` (uploaded once, then cached)."""
        import torch

        data = self.fields[name]
        if dtype is None:
            dtype = data.dtype if isinstance(data, torch.Tensor) else torch.from_numpy(np.asarray(data[:0])).dtype
        elif not isinstance(dtype, torch.dtype):          # numpy dtype or "float32"-style name
            dtype = torch.from_numpy(np.zeros(0, dtype=np.dtype(dtype))).dtype
        key = (name, str(torch.device(device)), dtype)
        t = self._device.get(key)
        if t is None:
            if isinstance(data, torch.Tensor):
                t = data.to(device=device, dtype=dtype).contiguous()
            else:
                t = torch.as_tensor(np.ascontiguousarray(data)).to(device=device, dtype=dtype).contiguous()
            self._device[key] = t
        return t

    def device_field_split(self, name, device):
        """A float64 field as interleaved float32 pairs (hi, lo) per node, hi =
        float32(x) and lo = float32(x - hi), flattened, cached on `device`."""
        import torch

        key = (name, str(torch.device(device)), "f32x2")
        t = self._device.get(key)
        if t is None:
            d = self.device_field(name, device, torch.float64)
            hi = d.to(torch.float32)
            lo = (d - hi.to(torch.float64)).to(torch.float32)
            t = torch.stack([hi.reshape(-1), lo.reshape(-1)], dim=1).reshape(-1).contiguous()
            self._device[key] = t
        return t

    def reconnect_shared(self):
        """A worker's re-attachment of the shared-memory fields (grid.py:99-106): no field is held
        in shared memory here, so there is nothing to re-attach."""

    def close_shared(self):
        pass
