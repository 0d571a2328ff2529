"""Schwarzschild metric, internal spherical coordinates (t, r, theta, phi).

Mirrors excalibur/metrics/schwarzschild_metric_fast.py:160-325. The RHS
(`_schw_accel_analytical` :104-157 / `_schw_accel_tensorial` :12-101 with the
guards of `geodesic_equations` :253-303) runs on the GPU. Photon states given
in cartesian coordinates (coords="cartesian") are converted once on entry by
`cartesian_state_to_spherical`, as the reference's integrator does
(integrator.py:247-255).
"""
from __future__ import annotations

import numpy as np

from .. import _native as N
from ..core import constants as K
from ..core.coordinates import cartesian_to_spherical, cartesian_velocity_to_spherical
from .base_metric import Metric


class SchwarzschildMetricFast(Metric):
    record_cols = 12

    def __init__(self, mass, radius, center=np.array([0.5, 0.5, 0.5]) * K.one_Gpc, analytical_geodesics=False,
                 free_time_geodesic=True, coords="cartesian"):
        self.mass = float(mass)
        self.radius = float(radius)
        self.center = np.asarray(center, dtype=float)
        self.r_s = 2.0 * K.G * self.mass / (K.c * K.c)
        self.analytical_geodesics = bool(analytical_geodesics)
        self.free_time_geodesic = bool(free_time_geodesic)
        if coords not in ("cartesian", "spherical"):
            raise ValueError("coords must be 'cartesian' or 'spherical'")
        self.input_coords = coords
        self.internal_coords = "spherical"
        self._desc = {}

    def descriptor(self, device, split=False):
        import torch
        from ..trace import MetricDescriptor, base_metric_struct

        key = str(torch.device(device))
        d = self._desc.get(key)
        if d is None:
            m = base_metric_struct(N.METRIC_SCHWARZSCHILD)
            m.analytical = int(self.analytical_geodesics)
            m.free_time = int(self.free_time_geodesic)
            m.mass, m.radius, m.r_s = self.mass, self.radius, self.r_s
            for i in range(3):
                m.center[i] = float(self.center[i])
            d = MetricDescriptor(m, [], self.record_cols, N.METRIC_SCHWARZSCHILD)
            self._desc[key] = d
        return d

    def metric_tensor(self, x):
        from .._evaluate import metric_diag

        g, _ = metric_diag(self, x)
        return np.diag(g.cpu().numpy())

    def christoffel(self, x):
        """Gamma for (t, r, theta, phi) with r from the lens centre (schwarzschild_metric_fast.py:203-250)."""
        t, r, theta, phi = (float(v) for v in x)
        if not (np.isfinite(r) and np.isfinite(theta) and np.isfinite(phi)):
            raise ValueError("Non-finite (r,theta,phi) in SchwarzschildMetric")
        r = max(r, self.radius) if r <= self.radius else r
        if r <= self.r_s:
            raise ValueError("Photon inside the Schwarzschild radius, stopping integration")
        G, M, c, rs = K.G, self.mass, K.c, self.r_s
        denom = c ** 2 * r - 2 * G * M
        Gm = np.zeros((4, 4, 4))
        Gm[0, 1, 0] = Gm[0, 0, 1] = G * M / (r * denom)
        Gm[1, 0, 0] = G * M * (c ** 2 * r - 2 * G * M) / (c ** 2 * r ** 3)
        Gm[1, 1, 1] = -G * M / (r * denom)
        Gm[1, 2, 2] = -(r - rs)
        Gm[1, 3, 3] = -(r - rs) * (np.sin(theta) ** 2)
        Gm[2, 1, 2] = Gm[2, 2, 1] = 1.0 / r
        Gm[2, 3, 3] = -np.sin(theta) * np.cos(theta)
        Gm[3, 1, 3] = Gm[3, 3, 1] = 1.0 / r
        Gm[3, 2, 3] = Gm[3, 3, 2] = np.cos(theta) / np.sin(theta)
        return Gm

    def geodesic_equations(self, state):
        from .._evaluate import geodesic_rhs

        if self.input_coords == "cartesian":
            state = self.cartesian_state_to_spherical(state)
        out, st = geodesic_rhs(self, state)
        if st.ndim == 0:
            if int(st) == N.PH_HORIZON:
                raise ValueError("Photon inside the Schwarzschild radius, stopping integration")
            if int(st) != 0:
                raise ValueError("Numerical failure in Schwarzschild fast acceleration (near horizon / poles)")
            return out.cpu().numpy()
        return out, st

    def metric_physical_quantities(self, state):
        r = float(state[1])
        return np.array([r, self.mass, self.radius, self.r_s], dtype=float)

    def cartesian_state_to_spherical(self, state):
        """(t, x, y, z, dt, dx, dy, dz) -> (t, r, theta, phi, dt, dr, dtheta, dphi), lens-centred (:310-325)."""
        t, x, y, z, dtdl, dxdl, dydl, dzdl = state
        X = x - self.center[0]
        Y = y - self.center[1]
        Z = z - self.center[2]
        r, theta, phi = cartesian_to_spherical(X, Y, Z)
        drdl, dthetadl, dphidl = cartesian_velocity_to_spherical(X, Y, Z, dxdl, dydl, dzdl)
        return np.array([t, r, theta, phi, dtdl, drdl, dthetadl, dphidl], dtype=float)
