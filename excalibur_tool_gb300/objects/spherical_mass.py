"""Analytic lens potentials sampled onto grids (host-side field construction).

`spherical_mass.potential` and `spherical_mass_nfw.potential` follow
excalibur/objects/spherical_mass.py:9-49 and :125-171 (SI, m^2/s^2).
Field construction happens once, before tracing, as in the reference runner
(`_excalibur_runs/excalibur_run_compare_schwarzschild_vs_flrw_impact_parameter.py:462-467`).
"""
import numpy as np

from ..core.constants import G


class spherical_mass:
    def __init__(self, mass, radius, center=np.array([0.5, 0.5, 0.5])):
        self.G = G
        self.mass = mass
        self.radius = radius
        self.center = center
        self.x0, self.y0, self.z0 = self.center

    def contains(self, x, y, z):
        return (x - self.x0) ** 2 + (y - self.y0) ** 2 + (z - self.z0) ** 2 <= self.radius ** 2

    def density(self, x, y, z):
        """M / (4/3 pi R^3) inside the sphere, 0 outside (spherical_mass.py:24-27)."""
        d2 = (x - self.x0) ** 2 + (y - self.y0) ** 2 + (z - self.z0) ** 2
        return np.where(d2 <= self.radius ** 2, self.mass / (4 / 3 * np.pi * self.radius ** 3), 0.0)

    def mass_enclosed(self, x, y, z):
        """M (r/R)^3 inside, M outside; 1-D x, y, z span a grid (spherical_mass.py:51-70)."""
        x, y, z = np.asarray(x), np.asarray(y), np.asarray(z)
        if x.ndim == 1 and y.ndim == 1 and z.ndim == 1:
            X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
        else:
            X, Y, Z = np.broadcast_arrays(x, y, z)
        r = np.sqrt((X - self.x0) ** 2 + (Y - self.y0) ** 2 + (Z - self.z0) ** 2)
        out = np.full(r.shape, float(self.mass))
        inside = r <= self.radius
        out[inside] = self.mass * (r[inside] / self.radius) ** 3
        return out

    def potential(self, x, y, z):
        x, y, z = np.asarray(x), np.asarray(y), np.asarray(z)
        if x.ndim == 1 and y.ndim == 1 and z.ndim == 1:
            X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
        else:
            X, Y, Z = np.broadcast_arrays(x, y, z)
        r = np.sqrt((X - self.x0) ** 2 + (Y - self.y0) ** 2 + (Z - self.z0) ** 2)
        r = np.where(r == 0, 1e-10, r)
        pot = np.empty_like(r, dtype=float)
        inside = r < self.radius
        pot[inside] = -self.G * self.mass * (3 * self.radius ** 2 - r[inside] ** 2) / (2 * self.radius ** 3)
        pot[~inside] = -self.G * self.mass / r[~inside]
        return pot

    def potential_grid(self, shape, spacing, origin=(0.0, 0.0, 0.0), device="cuda"):
        """`potential` on the nodes origin + i * spacing of a C-order grid, built on the GPU
        (exc_spherical_mass_grid): the same values, bit for bit, as
        potential(*np.meshgrid(*[np.linspace(o, o + n * s, n, endpoint=False)], indexing="ij"))
        whenever s is the linspace step (stop - start) / n. Returns a float64 tensor."""
        import ctypes as C

        import torch

        from .. import _native as N

        n = (C.c_int64 * 3)(*[int(v) for v in shape])
        dbl3 = lambda v: (C.c_double * 3)(*[float(x) for x in v])
        out = torch.empty(tuple(int(v) for v in shape), dtype=torch.float64, device=device)
        # the reference's scalar subexpressions, in its own (Python float) arithmetic
        neg_gm = -self.G * self.mass
        three_r2 = 3 * self.radius ** 2
        two_r3 = 2 * self.radius ** 3
        N.check(N.load().exc_spherical_mass_grid(n, dbl3(origin), dbl3(spacing),
                                                 dbl3((self.x0, self.y0, self.z0)), float(self.radius),
                                                 float(neg_gm), float(three_r2), float(two_r3), N.ptr(out),
                                                 N.stream_handle(device)), "exc_spherical_mass_grid")
        return out


class spherical_mass_nfw:
    def __init__(self, mass, radius, concentration, center=np.array([0.5, 0.5, 0.5])):
        self.G = G
        self.mass = mass
        self.radius = radius
        self.center = center
        self.x0, self.y0, self.z0 = self.center
        self.concentration = concentration
        self.Rs = self.radius / self.concentration
        self.rho0 = self.compute_rho0_nfw()

    def compute_rho0_nfw(self):
        """M / (4 pi Rs^3 (ln(1 + c) - c / (1 + c))) (spherical_mass.py:139-144)."""
        c = self.concentration
        return self.mass / (4 * np.pi * self.Rs ** 3 * (np.log(1 + c) - c / (1 + c)))

    def contains(self, x, y, z):
        return (x - self.x0) ** 2 + (y - self.y0) ** 2 + (z - self.z0) ** 2 <= self.radius ** 2

    def _r(self, x, y, z):
        return np.sqrt((x - self.x0) ** 2 + (y - self.y0) ** 2 + (z - self.z0) ** 2)

    def density(self, x, y, z):
        """rho0 / ((r/Rs) (1 + r/Rs)^2), r = 0 taken as 1e-10 (spherical_mass.py:150-153)."""
        r = self._r(x, y, z)
        r = np.where(r == 0, 1e-10, r)
        return self.rho0 / ((r / self.Rs) * (1 + r / self.Rs) ** 2)

    def potential(self, x, y, z):
        """-4 pi G rho0 Rs^2 ln(1 + r/Rs) / (r/Rs) (spherical_mass.py:155-161), the logarithmic
        factor formed first as there."""
        r = self._r(x, y, z)
        r = np.where(r == 0, 1e-10, r)
        xrel = r / self.Rs
        factor = np.log(1 + xrel) / xrel
        return -4 * np.pi * self.G * self.rho0 * self.Rs ** 2 * factor

    def mass_enclosed(self, x, y, z):
        """4 pi rho0 Rs^3 (ln(1 + r/Rs) - (r/Rs) / (1 + r/Rs)) (spherical_mass.py:163-171)."""
        xrel = self._r(x, y, z) / self.Rs
        return 4 * np.pi * self.rho0 * self.Rs ** 3 * (np.log(1 + xrel) - xrel / (1 + xrel))
