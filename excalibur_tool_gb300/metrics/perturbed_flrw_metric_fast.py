"""Perturbed FLRW metric in Newtonian gauge (Psi = Phi), fast form.

Mirrors excalibur/metrics/perturbed_flrw_metric_fast.py:102-282. The
geodesic right-hand side (a, adot from the cosmology table, trilinear Phi and
base-node gradient from the grid, the inlined Christoffel contraction of
`compute_tensorial_acceleration` :7-76 or the closed form
`compute_analytical_acceleration` :78-99) runs on the GPU; this class only
describes the spacetime to the kernels.

Several potential realisations can share one launch: pass
`extra_interpolators` (one per extra field) and give each photon a
`field_index` when tracing.
"""
from __future__ import annotations

import numpy as np

from .. import _native as N
from ..core import constants as K
from ..core.cosmology import resolve_cosmology, COSMO_STATIC
from .base_metric import Metric


class PerturbedFLRWMetricFast(Metric):
    record_cols = 14

    def __init__(self, a_of_eta, grid, interpolator, analytical_geodesics=False, adot_of_eta=None,
                 field="Phi", extra_interpolators=()):
        self.analytical_geodesics = analytical_geodesics
        self.a_of_eta = a_of_eta
        self.adot_of_eta = adot_of_eta
        self.grid = grid
        self.interp = interpolator
        self.field = field
        self.extra_interpolators = list(extra_interpolators)
        self.cosmology, self.cosmology_mode = resolve_cosmology(a_of_eta, adot_of_eta)
        self._desc = {}

    # ---- device descriptor ----------------------------------------------
    def descriptor(self, device, split=False):
        """ExcMetric for `device`; `split` passes float64 grids as float32 hi/lo planes
        (what the mixed-precision tracer reads)."""
        import torch
        from ..trace import MetricDescriptor, base_metric_struct

        key = (str(torch.device(device)), bool(split))
        d = self._desc.get(key)
        if d is not None:
            return d
        m = base_metric_struct(N.METRIC_FLRW)
        m.analytical = int(bool(self.analytical_geodesics))
        m.cosmology = self.cosmology_mode
        keep = []
        if self.cosmology_mode != COSMO_STATIC:
            cz = self.cosmology
            tab = cz.device_table(device)
            keep.append(tab)
            m.a_table = tab.data_ptr()
            m.a_table_n = tab.shape[0]
            m.eta_min, m.eta_step = float(cz.eta_min), float(cz.eta_step)
            m.H0 = float(cz.H0)
            m.omega_m, m.omega_r = float(cz.Omega_m), float(cz.Omega_r)
            m.omega_k, m.omega_lambda = float(cz.Omega_k), float(cz.Omega_lambda)
        interps = [self.interp] + self.extra_interpolators
        if len(interps) > N.EXC_MAX_FIELDS:
            raise ValueError(f"at most {N.EXC_MAX_FIELDS} potential fields per launch")
        for i, ip in enumerate(interps):
            f, t = ip.field_struct(self.field, device, split=split)
            m.fields[i] = f
            keep.append(t)
        m.n_fields = len(interps)
        d = MetricDescriptor(m, keep, self.record_cols, N.METRIC_FLRW)
        self._desc[key] = d
        return d

    def invalidate(self):
        self._desc.clear()

    # ---- reference-facing methods (device-evaluated) ----------------------
    def metric_tensor(self, x):
        from .._evaluate import metric_diag

        g, st = metric_diag(self, x)
        if int(st) != 0:
            raise ValueError(f"Point {x} outside grid bounds (boundary='{self.interp.boundary}')")
        return np.diag(g.cpu().numpy())

    def geodesic_equations(self, state):
        """d/dlambda (x, u) for one state [8] or a batch [N, 8] (GPU)."""
        from .._evaluate import geodesic_rhs

        out, st = geodesic_rhs(self, state)
        if st.ndim == 0:
            if int(st) != 0:
                raise ValueError(f"geodesic RHS failed ({N.STATUS_NAMES.get(int(st), st)}) at {state}")
            return out.cpu().numpy()
        return out, st

    def metric_physical_quantities(self, state):
        """[a, Phi, dPhi/dx, dPhi/dy, dPhi/dz, dPhi/deta] at (eta, x, y, z) (:275-282)."""
        eta = float(state[0])
        pos = state[1:4]
        a = float(self.a_of_eta(eta))
        phi, grad, phi_dot = self.interp.value_gradient_and_time_derivative(pos, self.field, eta)
        return np.array([a, phi, *grad, phi_dot])

    def christoffel(self, x):
        """Gamma^mu_{nu sigma} with the fast metric's normalisation (:143-188)."""
        eta = float(x[0])
        a = float(self.a_of_eta(eta))
        adot = float(self.adot_of_eta(eta)) if callable(self.adot_of_eta) else 0.0
        phi, grad_phi, phi_dot = self.interp.value_gradient_and_time_derivative(x[1:4], self.field, eta)
        c = K.c
        g0, g1, g2 = (gp / (c ** 2) for gp in grad_phi)
        psi = phi / (c ** 2)
        psi_dot = phi_dot / (c ** 2)
        G = np.zeros((4, 4, 4))
        G[0, 0, 0] = 1 / c ** 2 * psi_dot
        G[1, 0, 0], G[2, 0, 0], G[3, 0, 0] = g0 / a ** 2, g1 / a ** 2, g2 / a ** 2
        G[1, 1, 1] = -1 / c ** 2 * grad_phi[0]
        G[2, 2, 2] = -1 / c ** 2 * grad_phi[1]
        G[3, 3, 3] = -1 / c ** 2 * grad_phi[2]
        g0ii = a * adot / c ** 2 + 2 * a * adot / c ** 4 * (phi + psi) - a ** 2 / c ** 4 * phi_dot
        G[0, 1, 1] = G[0, 2, 2] = G[0, 3, 3] = g0ii
        G[0, 0, 1] = G[0, 1, 0] = g0 / c ** 2
        G[0, 0, 2] = G[0, 2, 0] = g1 / c ** 2
        G[0, 0, 3] = G[0, 3, 0] = g2 / c ** 2
        h = adot / a - phi_dot / c ** 2
        G[1, 1, 0] = G[1, 0, 1] = G[2, 2, 0] = G[2, 0, 2] = G[3, 3, 0] = G[3, 0, 3] = h
        G[1, 2, 2] = G[1, 3, 3] = g0 / c ** 2
        G[2, 1, 1] = G[2, 3, 3] = g1 / c ** 2
        G[3, 1, 1] = G[3, 2, 2] = g2 / c ** 2
        G[1, 1, 2] = G[1, 2, 1] = -g1 / c ** 2
        G[1, 1, 3] = G[1, 3, 1] = -g2 / c ** 2
        G[2, 2, 1] = G[2, 1, 2] = -g0 / c ** 2
        G[2, 2, 3] = G[2, 3, 2] = -g2 / c ** 2
        G[3, 3, 1] = G[3, 1, 3] = -g0 / c ** 2
        G[3, 3, 2] = G[3, 2, 3] = -g1 / c ** 2
        return G
