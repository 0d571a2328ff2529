"""Background cosmology: the a(eta) table the device kernels read.

Mirrors excalibur/core/cosmology.py. The host builds the same regular
conformal-time table as the reference (`_build_eta_grid_fast`,
cosmology.py:130-159: 2000-point log-spaced a-grid from 1e-4, eta(a) by
`scipy.integrate.quad`, resampled with `np.interp` onto 5000 regular eta
points) and the present-day conformal time `_eta_at_a1`
(`_build_eta_to_a_interpolator`, cosmology.py:163-185: 500-point grid,
lower quad limit 1e-6, argmin |a-1|). The table, `eta_min`, `eta_step` and
the density parameters are uploaded verbatim; the device evaluates
a(eta) (`a_interp_numba`, cosmology.py:8-25) and adot = a^2 H0 E(z)
(`adot_of_eta`, cosmology.py:84-93) itself, so a(eta) agrees with the
reference by construction. Scalar/array evaluation from Python goes through
the device (`exc_eval_cosmology`), never a host restatement.
"""
from __future__ import annotations

import numpy as np

from .constants import one_pc

COSMO_STATIC = 0
COSMO_TABLE = 1       # table a(eta) + analytic adot (reference adot_of_eta)
COSMO_TABLE_FD = 2    # table a(eta) + central-difference adot (perturbed_flrw_metric_fast.py:204-210)


class LCDM_Cosmology:
    """Flat/curved LCDM background (excalibur/core/cosmology.py:39-66).

    H0 is given in km/s/Mpc and stored in s^-1 exactly as the reference does
    (`H0 * 1000 / (1e6 * one_pc)`, cosmology.py:59).
    """

    kind = COSMO_TABLE

    def __init__(self, H0, Omega_m, Omega_r, Omega_lambda, Omega_k=0):
        self.H0_original = H0
        self.H0 = H0 * 1000 / (1e6 * one_pc)
        self.Omega_m = Omega_m
        self.Omega_lambda = Omega_lambda
        self.Omega_r = Omega_r
        self.Omega_k = Omega_k
        self._build_eta_at_a1()
        self._build_eta_grid_fast()
        self._device_table = {}

    @classmethod
    def from_table(cls, H0_si, Omega_m, Omega_r, Omega_lambda, Omega_k, eta_min, eta_step, a_grid, eta_at_a1):
        """Rebuild from a saved table (bypasses the quad integration, e.g. to reuse
        a table produced on another machine)."""
        obj = cls.__new__(cls)
        obj.H0_original = H0_si * (1e6 * one_pc) / 1000
        obj.H0 = float(H0_si)
        obj.Omega_m, obj.Omega_r, obj.Omega_lambda, obj.Omega_k = Omega_m, Omega_r, Omega_lambda, Omega_k
        obj.a_grid = np.asarray(a_grid, dtype=np.float64)
        obj.N_eta = obj.a_grid.shape[0]
        obj.eta_min = float(eta_min)
        obj.eta_step = float(eta_step)
        obj.eta_max = obj.eta_min + obj.eta_step * (obj.N_eta - 1)
        obj.eta_grid = np.linspace(obj.eta_min, obj.eta_max, obj.N_eta)
        obj._eta_at_a1 = float(eta_at_a1)
        obj._device_table = {}
        return obj

    # -- host-side construction (setup, not the traced path) --------------
    def E(self, z):
        """Normalised Hubble rate, same expression as cosmology.py:69-71."""
        return np.sqrt(self.Omega_m * (1 + z) ** 3 + self.Omega_r * (1 + z) ** 4
                       + self.Omega_k * (1 + z) ** 2 + self.Omega_lambda)

    def _eta_integrand(self, a):
        return 1.0 / (a * a * self.H0 * self.E(1 / a - 1))

    def _build_eta_grid_fast(self):
        from scipy.integrate import quad

        a_values = np.logspace(-4, 0.5, 2000)
        eta_values = np.zeros_like(a_values)
        for i, a in enumerate(a_values):
            val, _ = quad(self._eta_integrand, a_values[0], a)
            eta_values[i] = val
        self.eta_min = float(eta_values[0])
        self.eta_max = float(eta_values[-1])
        self.N_eta = 5000
        self.eta_grid = np.linspace(self.eta_min, self.eta_max, self.N_eta)
        self.a_grid = np.interp(self.eta_grid, eta_values, a_values)
        self.eta_step = (self.eta_max - self.eta_min) / (self.N_eta - 1)

    def _build_eta_at_a1(self):
        from scipy.integrate import quad

        def integrand(a_val):
            return 1.0 / (a_val ** 2 * self.H0 * self.E(1.0 / a_val - 1.0))

        a_values = np.logspace(-4, 0.5, 500)
        eta_values = np.zeros_like(a_values)
        for i, a_val in enumerate(a_values):
            val, _ = quad(integrand, 1e-6, a_val)
            eta_values[i] = val
        idx = np.argmin(np.abs(a_values - 1.0))
        self._eta_at_a1 = float(eta_values[idx])

    # -- device-facing ----------------------------------------------------
    def device_table(self, device):
        """The a(eta) table as a float64 tensor resident on `device`."""
        import torch

        key = str(device)
        if key not in self._device_table:
            self._device_table[key] = torch.as_tensor(self.a_grid, dtype=torch.float64).to(device)
        return self._device_table[key]

    def a_of_eta(self, eta):
        """a(eta) evaluated on the GPU (cosmology.py:199-206)."""
        from .._evaluate import eval_cosmology
        return eval_cosmology(self, eta, "a")

    def adot_of_eta(self, eta):
        """da/deta = a^2 H0 E(z) evaluated on the GPU (cosmology.py:84-93)."""
        from .._evaluate import eval_cosmology
        return eval_cosmology(self, eta, "adot")

    def H_of_eta(self, eta):
        a = self.a_of_eta(eta)
        z = 1.0 / a - 1.0
        return self.H0 * self.E(z) / a ** 2

    # -- host helpers of the reference's class (setup, not the traced path) --
    def H_of_z(self, z):
        """H0 E(z) in s^-1 (cosmology.py:74-76)."""
        return self.H0 * self.E(z)

    def a_of_z(self, z):
        """1 / (1 + z) (cosmology.py:95-97)."""
        return 1.0 / (1.0 + z)

    def a_of_t(self, t):
        """Scale factor at cosmic time t [s] (cosmology.py:99-128): t(a) = (1/H0) integral from 0
        to a of da' / (a' E(1/a' - 1)) by quad, and a refined from 1 by a <- a t / t(a) until
        |t(a) - t| < 1e-6 s or 100 updates. Scalar in, float out; arrays elementwise."""
        from scipy.integrate import quad

        def t_of_a(a):
            return quad(lambda x: 1.0 / (x * self.E(1.0 / x - 1.0)), 0, a)[0] / self.H0

        t = np.asarray(t, dtype=float)
        out = np.empty(t.shape if t.ndim else (1,))
        for i, tv in enumerate(np.atleast_1d(t)):
            a = 1.0
            for _ in range(100):
                ta = t_of_a(a)
                if abs(ta - tv) < 1e-6:
                    break
                a *= tv / ta
            out[i] = a
        return float(out[0]) if t.ndim == 0 else out


class StaticCosmology:
    """a(eta) = 1, adot = 0 (excalibur/core/cosmology.py:236-257)."""

    kind = COSMO_STATIC
    H0 = 0.0
    Omega_m = Omega_r = Omega_k = Omega_lambda = 0.0
    eta_min = 0.0
    eta_step = 1.0
    _eta_at_a1 = 0.0

    def a_of_eta(self, eta):
        if isinstance(eta, np.ndarray):
            return np.ones_like(eta, dtype=float)
        return 1.0

    def adot_of_eta(self, eta):
        if isinstance(eta, np.ndarray):
            return np.zeros_like(eta, dtype=float)
        return 0.0

    def a_and_adot(self, eta):
        return self.a_of_eta(eta), self.adot_of_eta(eta)


def resolve_cosmology(a_of_eta, adot_of_eta):
    """Map the reference's callables onto a device cosmology mode.

    The reference metric takes bound methods (`cosmo.a_of_eta`,
    `cosmo.adot_of_eta`) and picks: `a_and_adot` if the a-callable has it,
    else analytic adot if given, else a central difference
    (perturbed_flrw_metric_fast.py:197-210). Only callables bound to the two
    cosmology classes above can be evaluated on the device; anything else is
    rejected loudly rather than evaluated on the host.
    """
    owner = getattr(a_of_eta, "__self__", None)
    if isinstance(a_of_eta, StaticCosmology):
        owner = a_of_eta
    if isinstance(owner, StaticCosmology):
        return owner, COSMO_STATIC
    if isinstance(owner, LCDM_Cosmology):
        if adot_of_eta is None:
            return owner, COSMO_TABLE_FD
        adot_owner = getattr(adot_of_eta, "__self__", None)
        if adot_owner is not owner or getattr(adot_of_eta, "__name__", "") != "adot_of_eta":
            raise NotImplementedError(
                "adot_of_eta must be the adot_of_eta method of the same LCDM_Cosmology "
                "(arbitrary Python callables cannot run inside the device kernel)")
        return owner, COSMO_TABLE
    raise NotImplementedError(
        "a_of_eta must be a bound method of LCDM_Cosmology or StaticCosmology; "
        f"got {a_of_eta!r} (arbitrary Python callables cannot run inside the device kernel)")
