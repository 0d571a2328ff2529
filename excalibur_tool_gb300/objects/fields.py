"""Synthetic potential fields for the benchmark workloads (not in the reference).

* Plummer-softened point mass: Phi = -G M / sqrt(r^2 + eps^2) (SI).
* Gaussian random field with P(k) ~ |k|^-3 on the periodic FFT grid, k = 0
  removed, rescaled to a target rms of Phi/c^2 (dimensionless), seeded with
  numpy.random.default_rng(seed).

Nodes sit at origin + i * L / n, like the reference runner's
`np.linspace(0, L, N, endpoint=False)` grid.
"""
from __future__ import annotations

import numpy as np

from ..core.constants import G, c


def node_coords(n, box):
    return np.arange(n, dtype=np.float64) * (box / n)


def plummer_potential(n, box, mass, softening, center, dtype=np.float64):
    x = node_coords(n, box)
    dx2 = (x - center[0]) ** 2
    dy2 = (x - center[1]) ** 2
    dz2 = (x - center[2]) ** 2
    r2 = dx2[:, None, None] + dy2[None, :, None] + dz2[None, None, :]
    return (-G * mass / np.sqrt(r2 + softening ** 2)).astype(dtype)


def gaussian_random_field(n, box, seed, rms=1e-5, spectral_index=-3.0, dtype=np.float64):
    """Dimensionless Phi/c^2 realisation with P(k) ~ k^spectral_index and the given rms."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((n, n, n))
    wk = np.fft.rfftn(white)
    k1 = 2 * np.pi * np.fft.fftfreq(n, d=box / n)
    kz = 2 * np.pi * np.fft.rfftfreq(n, d=box / n)
    k2 = k1[:, None, None] ** 2 + k1[None, :, None] ** 2 + kz[None, None, :] ** 2
    amp = np.zeros_like(k2)
    nz = k2 > 0
    amp[nz] = k2[nz] ** (spectral_index / 4.0)      # sqrt(P) = |k|^(index/2)
    field = np.fft.irfftn(wk * amp, s=(n, n, n), axes=(0, 1, 2))
    field *= rms / field.std()
    return field.astype(dtype)


def lens_plus_grf(n, box, mass, softening, center, seed, rms=1e-5, dtype=np.float64, with_grf=True):
    """Phi_SI = Plummer + c^2 * GRF (the workloads' potential)."""
    phi = plummer_potential(n, box, mass, softening, center, np.float64)
    if with_grf:
        phi = phi + float(c) ** 2 * gaussian_random_field(n, box, seed, rms)
    return phi.astype(dtype)
