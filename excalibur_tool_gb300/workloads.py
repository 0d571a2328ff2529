"""The benchmark workloads, built from seeded synthetic inputs.

* lens_cone (1,024 rays): Schwarzschild point mass 1e15 Msun at the centre
  (500, 500, 500) Mpc of a 1000 Mpc box, observer at (0, 500, 500) Mpc, 32x32
  polar grid of directions in a 5 deg half-angle cone, RK4 with
  dlambda = 0.5 Mpc / c, 2,000 steps.
* flrw_patch (65,536 rays): perturbed FLRW (LCDM, Omega_m = 0.3, h = 0.7) with
  Phi on a 128^3 float64 grid over 1000 Mpc = Plummer sphere (1e15 Msun,
  softening 5 Mpc) + Gaussian random field (P(k) ~ k^-3, rms Phi/c^2 = 1e-5,
  seed 2); 256x256 directions in a 10 x 10 deg patch; RK4 with
  deta = 0.5 Mpc, until box exit or a <= 0.5.
* flrw_patch_fp32grid: the same construction on a 512^3 float32 grid,
  2048 x 2048 directions in a 20 x 20 deg patch (seed 4).
* multi_field: the lens alone (Plummer, no random field) on a 256^3 float64 grid
  with 1,048,576 full-sky directions (numpy default_rng(3)), plus 16 random-field
  realisations (seeds 1..16, grid 64^3 / 128^3 / 256^3 for seed mod 3 = 0 / 1 / 2)
  with the 65,536-ray patch each, all traced in one launch with adaptive RK45
  (Fehlberg weights, rtol 1e-8, atol 1e-12, dt clipped to [1e10, 1e17] s, at most
  20,000 tried steps per ray).

Inputs are resident on the GPU when the builders return.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .core.constants import c, one_Mpc, one_Msun, G
from .core.cosmology import LCDM_Cosmology
from .grid.grid import Grid
from .grid.interpolator_4d_fast import InterpolatorFast
from .metrics.perturbed_flrw_metric_fast import PerturbedFLRWMetricFast
from .metrics.schwarzschild_metric_fast import SchwarzschildMetricFast
from .objects.fields import gaussian_random_field, lens_plus_grf, plummer_potential
from .photon.photons import Photons
from .trace import TraceConfig

BOX = 1000 * one_Mpc
LENS = np.array([500.0, 500.0, 500.0]) * one_Mpc
OBSERVER = np.array([0.0, 500.0, 500.0]) * one_Mpc
LENS_MASS = 1e15 * one_Msun
DLAMBDA = 0.5 * one_Mpc / c

_COSMO = None


def lcdm():
    global _COSMO
    if _COSMO is None:
        _COSMO = LCDM_Cosmology(70, 0.3, 0.0, 0.7)
    return _COSMO


@dataclasses.dataclass
class Workload:
    name: str
    metric: object
    states: "torch.Tensor"
    cfg: TraceConfig
    info: dict
    field_index: "torch.Tensor" = None


def flrw_patch(n_grid=128, n_side=256, patch_deg=10.0, seed=2, field_dtype=np.float64, precision="fp64",
               device="cuda", with_grf=True):
    import torch

    cz = lcdm()
    phi = lens_plus_grf(n_grid, BOX, LENS_MASS, 5 * one_Mpc, LENS, seed=seed, dtype=field_dtype, with_grf=with_grf)
    grid = Grid((n_grid,) * 3, (BOX / n_grid,) * 3, (0.0, 0.0, 0.0))
    grid.add_field("Phi", phi)
    interp = InterpolatorFast(grid, boundary="periodic")
    metric = PerturbedFLRWMetricFast(cz.a_of_eta, grid, interp, adot_of_eta=cz.adot_of_eta)
    ph = Photons(metric)
    states = ph.generate_patch_grid(n_side, [cz._eta_at_a1, *OBSERVER], LENS - OBSERVER, patch_deg)
    cfg = TraceConfig(stepper="rk4", precision=precision, dt=DLAMBDA, dt_min=DLAMBDA, dt_max=DLAMBDA,
                      max_steps=2 ** 62, max_iter=100_000, stop_box=((0, 0, 0), (BOX, BOX, BOX)), a_stop=0.5,
                      lens_center=tuple(LENS))
    info = {"grid": f"{n_grid}^3 {np.dtype(field_dtype).name}", "photons": n_side * n_side,
            "patch_deg": patch_deg, "seed": seed, "grid_bytes": int(phi.nbytes)}
    return Workload(f"flrw_patch_{n_grid}", metric, states.to(device), cfg, info)


def flrw_patch_rk45(n_grid=512, n_side=2048, patch_deg=20.0, seed=4, field_dtype=np.float32, precision="fp64",
                    rtol=1e-8, atol=1e-12, dt_min=1e10, dt_max=20 * DLAMBDA, device="cuda"):
    """The precision workload traced with the adaptive stepper: the patch of flrw_patch read
    through the reference's slow Interpolator (grid/interpolator.py: its gradient, the trilinear
    blend of corner differences, is continuous across cell faces; the base-node gradient of
    InterpolatorFast jumps at every face, where an adaptive step shrinks to its floor), RK45 with
    Fehlberg's weights at rtol / atol, the step free in [dt_min, dt_max], and the box stop landing
    on the face (stop_face), so that the end point does not depend on the step sequence. The slow
    class reads no further than its last node: the box ends 1.5 cells inside it."""
    import torch

    from .grid.interpolator import Interpolator

    cz = lcdm()
    phi = lens_plus_grf(n_grid, BOX, LENS_MASS, 5 * one_Mpc, LENS, seed=seed, dtype=field_dtype)
    grid = Grid((n_grid,) * 3, (BOX / n_grid,) * 3, (0.0, 0.0, 0.0))
    grid.add_field("Phi", phi)
    metric = PerturbedFLRWMetricFast(cz.a_of_eta, grid, Interpolator(grid), adot_of_eta=cz.adot_of_eta)
    ph = Photons(metric)
    states = ph.generate_patch_grid(n_side, [cz._eta_at_a1, *OBSERVER], LENS - OBSERVER, patch_deg)
    hi = (n_grid - 1.5) * BOX / n_grid
    cfg = TraceConfig(stepper="rk45", tableau="fehlberg", rtol=rtol, atol=atol, precision=precision, dt=DLAMBDA,
                      dt_min=dt_min, dt_max=dt_max, max_steps=2 ** 62, max_iter=100_000,
                      stop_box=((0, 0, 0), (hi, hi, hi)), stop_face=True, a_stop=0.5, lens_center=tuple(LENS))
    info = {"grid": f"{n_grid}^3 {np.dtype(field_dtype).name}", "photons": n_side * n_side, "patch_deg": patch_deg,
            "seed": seed, "grid_bytes": int(phi.nbytes), "interpolator": "slow Interpolator (trilinear gradient)",
            "stepper": f"RK45 Fehlberg rtol {rtol:g} atol {atol:g}, dt in [{dt_min:g}, {dt_max:g}] s",
            "stop": f"box face at {hi / one_Mpc:.2f} Mpc"}
    return Workload(f"flrw_patch_rk45_{n_grid}", metric, states.to(device), cfg, info)


def lens_cone(n_theta=32, n_phi=32, cone_deg=5.0, n_steps=2000, precision="fp64", device="cuda"):
    from .core.coordinates import cartesian_to_spherical

    rs = 2 * G * LENS_MASS / c ** 2
    metric = SchwarzschildMetricFast(LENS_MASS, rs * (1 + 1e-6), center=LENS, coords="spherical",
                                     analytical_geodesics=True, free_time_geodesic=True)
    origin = np.array([0.0, *cartesian_to_spherical(*(OBSERVER - LENS))])
    ph = Photons(metric)
    states = ph.generate_polar_grid(n_theta, n_phi, origin, LENS - OBSERVER, np.deg2rad(cone_deg))
    cfg = TraceConfig(stepper="rk4", precision=precision, dt=DLAMBDA, dt_min=DLAMBDA, dt_max=DLAMBDA,
                      max_steps=n_steps, max_iter=n_steps)
    return Workload("lens_cone", metric, states.to(device), cfg, {"photons": n_theta * n_phi})


def multi_field(main_n=256, n_sky=1 << 20, n_side=256, seeds=tuple(range(1, 17)), sizes=(64, 128, 256),
                tableau="fehlberg", rtol=1e-8, atol=1e-12, precision="fp64", device="cuda"):
    import torch

    from ._evaluate import null_init

    cz = lcdm()
    grids, interps = [], []
    g0 = Grid((main_n,) * 3, (BOX / main_n,) * 3, (0.0, 0.0, 0.0))
    g0.add_field("Phi", plummer_potential(main_n, BOX, LENS_MASS, 5 * one_Mpc, LENS))
    interps.append(InterpolatorFast(g0, boundary="periodic"))
    for sd in seeds:
        n = sizes[sd % 3]
        g = Grid((n,) * 3, (BOX / n,) * 3, (0.0, 0.0, 0.0))
        g.add_field("Phi", float(c) ** 2 * gaussian_random_field(n, BOX, sd, 1e-5))
        interps.append(InterpolatorFast(g, boundary="periodic"))
    metric = PerturbedFLRWMetricFast(cz.a_of_eta, g0, interps[0], adot_of_eta=cz.adot_of_eta,
                                     extra_interpolators=interps[1:])
    ph = Photons(metric)
    origin = [cz._eta_at_a1, *OBSERVER]
    sky = ph.generate_full_sky(n_sky, origin, seed=3)
    patch = ph.generate_patch_grid(n_side, origin, LENS - OBSERVER, 10.0)
    states = torch.cat([sky] + [patch] * len(seeds)).to(device).contiguous()
    fidx = torch.cat([torch.zeros(n_sky, dtype=torch.int32)] +
                     [torch.full((patch.shape[0],), i + 1, dtype=torch.int32) for i in range(len(seeds))]).to(device)
    st = null_init(metric, states, -1.0, field_index=fidx)        # u^0 from each photon's own field
    if int((st != 0).sum()):
        raise ValueError("null initialisation failed")
    # dt floor 1e10 s: the reference's 1e14 s floor (0.97 Mpc) would pin rejected steps at the floor, where a
    # step that straddles a cell face (base-node gradient jump) never meets rtol, until max_iter
    cfg = TraceConfig(stepper="rk45", tableau=tableau, precision=precision, dt=DLAMBDA, dt_min=1e10, dt_max=1e17,
                      rtol=rtol, atol=atol, max_steps=2 ** 62, max_iter=20_000,
                      stop_box=((0, 0, 0), (BOX, BOX, BOX)), a_stop=0.5, lens_center=tuple(LENS))
    info = {"photons": int(states.shape[0]), "sky_photons": n_sky, "patch_photons": int(patch.shape[0]),
            "fields": 1 + len(seeds), "grids": [main_n] + [sizes[sd % 3] for sd in seeds]}
    return Workload("multi_field", metric, states, cfg, info, field_index=fidx)
