"""Schwarzschild-vs-FLRW comparison runs on the GPU.

A drop-in for the reference's comparison runners
(_excalibur_runs/excalibur_run_compare_schwarzschild_vs_flrw.py and its
_impact_parameter twin), the unit of work of the parameter sweeps: one lens (mass M, radius R)
at the centre of a box of side L, an observer at distance D along -x, the same bundle of
photons traced backwards through the analytic Schwarzschild metric and through a perturbed
FLRW metric whose potential is the lens sampled on an N^3 grid, each with RK4 / RK45 /
Leapfrog4 for the same number of steps, trajectories recorded every `record_every` steps.

What is the reference's and kept as is (main(), :305-547):
* geometry: lens at (L/2)^3; D clamped to L/2 - L/N; observer and lens clipped into
  [L/N, (N-2) L/N]; step dlambda = (L/N / steps_per_cell) / c; n_steps = ceil(2 D / (c dlambda))
  (the requested n_steps is overridden, :341-360);
* Schwarzschild: spherical coordinates centred on the lens, analytical geodesics, dt clipped to
  [|dl|/1e6, |dl|] for RK45 and to |dl| otherwise (:374-384);
* FLRW: static cosmology (a = 1) or LCDM(70, 0.3, 0, 0.7); Phi = spherical_mass(M, R, lens)
  on the grid nodes i L/N; the fast (base-node) or slow (trilinear) interpolator; with
  `flrw_local_coords` the photons start at observer-local positions and the interpolator is
  queried at x + observer (ExcField.shift), output positions shifted back (:452-532);
* photons: the cone grid (plain runner, any `sampling`) or impact-parameter bins with seed 0
  (the impact runner when sampling == "impact"), directions in the cartesian basis;
* failures: the plain runner keeps an empty trajectory for a Schwarzschild photon that
  raised (horizon, non-finite state) and lets an FLRW failure end the run; the impact runner
  keeps the history up to the failure for both (:245-300 of each file).

Both traces are single persistent launches of `exc_trace` (trace_batch) with on-device
records; the per-photon loop of `_integrate_all` and its Python history lists are gone.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

from .. import _native as N
from ..core.constants import c, one_Mpc, one_Msun
from ..core.coordinates import cartesian_to_spherical
from ..core.cosmology import LCDM_Cosmology, StaticCosmology
from ..grid.grid import Grid
from ..grid.interpolator import Interpolator
from ..grid.interpolator_4d_fast import InterpolatorFast, shifted_interpolator
from ..metrics.perturbed_flrw_metric_fast import PerturbedFLRWMetricFast
from ..metrics.schwarzschild_metric_fast import SchwarzschildMetricFast
from ..objects.spherical_mass import spherical_mass
from ..photon.photons import Photons
from .analyze import TrajectoryStats, trajectory_stats


@dataclasses.dataclass(frozen=True)
class RunConfig:
    """The runner's RunConfig (excalibur_run_compare_schwarzschild_vs_flrw.py:59-84), SI units."""
    mass: float
    radius: float
    obs_to_lens_distance: float
    n_photons: int
    cone_angle_deg: float
    n_steps: int
    integrator: str
    mode: str
    output_dir: str
    static: bool
    flrw_grid_N: int
    flrw_grid_size: float
    record_every: int
    flrw_fast: bool
    progress_every: int
    steps_per_cell: float
    flrw_local_coords: bool
    trace_norm: bool
    renormalize_every: int
    sampling: str
    b_min: float
    b_max: float
    b_nbins: int
    b_nperbin: int


def run_config(*, mass_msun=1e15, radius_mpc=3.0, distance_mpc=500.0, n_photons=200, cone_angle_deg=10.0,
               n_steps=5000, integrator="rk4", mode="sequential", sampling="cone", b_min_mpc=0.5,
               b_max_mpc=10.0, b_nbins=10, b_nperbin=50, static=False, flrw_grid_N=256,
               flrw_grid_size_mpc=1000.0, output_dir="_data/output", record_every=50, no_flrw_fast=False,
               progress_every=10, steps_per_cell=3.0, flrw_local_coords=False, trace_norm=False,
               renormalize_every=0) -> RunConfig:
    """RunConfig from the runner's command-line options and defaults (:87-231), in its units
    (Msun, Mpc, degrees)."""
    if integrator not in ("rk4", "rk45", "leapfrog4"):
        raise ValueError("integrator must be one of: rk4, rk45, leapfrog4")
    if sampling not in ("cone", "impact"):
        raise ValueError("sampling must be 'cone' or 'impact'")
    return RunConfig(mass=mass_msun * one_Msun, radius=radius_mpc * one_Mpc,
                     obs_to_lens_distance=distance_mpc * one_Mpc, n_photons=int(n_photons),
                     cone_angle_deg=float(cone_angle_deg), n_steps=int(n_steps), integrator=integrator, mode=mode,
                     output_dir=output_dir, static=bool(static), flrw_grid_N=int(flrw_grid_N),
                     flrw_grid_size=flrw_grid_size_mpc * one_Mpc, record_every=int(record_every),
                     flrw_fast=not bool(no_flrw_fast), progress_every=int(progress_every),
                     steps_per_cell=float(steps_per_cell), flrw_local_coords=bool(flrw_local_coords),
                     trace_norm=bool(trace_norm), renormalize_every=int(renormalize_every), sampling=sampling,
                     b_min=b_min_mpc * one_Mpc, b_max=b_max_mpc * one_Mpc, b_nbins=int(b_nbins),
                     b_nperbin=int(b_nperbin))


@dataclasses.dataclass
class RunGeometry:
    lens_center: np.ndarray      # absolute cartesian (m)
    observer: np.ndarray         # absolute cartesian (m)
    obs_to_lens_distance: float  # after the clamp (m)
    clamped: bool
    dlambda: float               # affine step (s)
    n_steps: int                 # steps actually run
    cone_angle: float            # rad
    b_edges: Optional[np.ndarray]
    n_photons_effective: int


def geometry(cfg: RunConfig) -> RunGeometry:
    """Observer, lens, step and step count exactly as the runner computes them (:308-370)."""
    L, N_ = cfg.flrw_grid_size, cfg.flrw_grid_N
    lens = np.array([0.5 * L, 0.5 * L, 0.5 * L], dtype=float)
    max_D = 0.5 * L - (L / N_)
    clamped = cfg.obs_to_lens_distance > max_D
    D = float(max_D) if clamped else float(cfg.obs_to_lens_distance)
    observer = lens + np.array([-D, 0.0, 0.0], dtype=float)
    cell = L / N_
    inner_min, inner_max = 1.0 * cell, (N_ - 2.0) * cell
    observer = np.clip(observer, inner_min, inner_max)
    lens = np.clip(lens, inner_min, inner_max)
    travel = 2.0 * D
    dx_target = (L / float(N_)) / float(cfg.steps_per_cell)
    dlambda = dx_target / c
    n_steps = max(int(np.ceil(travel / dx_target)), 1)
    if cfg.sampling == "impact":
        b_edges = np.linspace(cfg.b_min, cfg.b_max, cfg.b_nbins + 1)
        n_eff = cfg.b_nbins * cfg.b_nperbin
    else:
        b_edges, n_eff = None, cfg.n_photons
    return RunGeometry(lens_center=lens, observer=observer, obs_to_lens_distance=D, clamped=bool(clamped),
                       dlambda=dlambda, n_steps=n_steps, cone_angle=float(np.deg2rad(cfg.cone_angle_deg)),
                       b_edges=b_edges, n_photons_effective=n_eff)


def _photons(metric, cfg: RunConfig, geo: RunGeometry, origin, central, impact_runner: bool, checks):
    ph = Photons(metric, defer_checks=checks is not None)
    if checks is not None:
        checks.append(ph)
    if impact_runner and cfg.sampling == "impact":
        return ph.generate_impact_parameter_bins(origin, central, geo.b_edges, cfg.b_nperbin,
                                                 direction_basis="cartesian", seed=0, u0_sign=-1.0)
    n = geo.n_photons_effective if impact_runner else cfg.n_photons
    return ph.generate_cone_grid(n_photons=n, origin=origin, central_direction=central,
                                 cone_angle=geo.cone_angle, direction_basis="cartesian")


def schwarzschild_setup(cfg: RunConfig, geo: RunGeometry, impact_runner: bool = False, checks=None):
    """(metric, initial states [n, 8] on the GPU, dt_min, dt_max) of the Schwarzschild leg (:372-414).
    With a list `checks`, the generator does not wait for the GPU: its Photons object is
    appended there and `check_generated()` on it raises what the generator would have."""
    if cfg.integrator == "rk45":
        dt_min, dt_max = abs(geo.dlambda) / 1e6, abs(geo.dlambda)
    else:
        dt_min = dt_max = abs(geo.dlambda)
    metric = SchwarzschildMetricFast(mass=cfg.mass, radius=cfg.radius, center=geo.lens_center, coords="spherical",
                                     analytical_geodesics=True)
    origin = np.array([0.0, *cartesian_to_spherical(*(geo.observer - geo.lens_center))], dtype=float)
    states = _photons(metric, cfg, geo, origin, geo.lens_center - geo.observer, impact_runner, checks)
    return metric, states, dt_min, dt_max


def flrw_potential(cfg: RunConfig, geo: RunGeometry, device=None):
    """spherical_mass(M, R, lens).potential on the nodes i L/N (:474-479): a numpy array with
    device=None (the runner's own host construction), else the same grid built on `device`
    by exc_spherical_mass_grid (bit-identical, a float64 tensor)."""
    N_, L = cfg.flrw_grid_N, cfg.flrw_grid_size
    lens = spherical_mass(mass=cfg.mass, radius=cfg.radius, center=geo.lens_center)
    if device is not None:
        d = L / N_                       # numpy.linspace's step (stop - start) / num
        return lens.potential_grid((N_, N_, N_), (d, d, d), (0.0, 0.0, 0.0), device=device)
    x = np.linspace(0, L, N_, endpoint=False)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    return lens.potential(X, Y, Z)


def flrw_setup(cfg: RunConfig, geo: RunGeometry, impact_runner: bool = False, phi: Optional[np.ndarray] = None,
               checks=None):
    """(metric, initial states, x_offset) of the FLRW leg (:449-532). x_offset is the
    observer position when the run integrates in local coordinates, else None."""
    cosmo = StaticCosmology() if cfg.static else LCDM_Cosmology(H0=70, Omega_m=0.3, Omega_r=0.0, Omega_lambda=0.7)
    N_, L = cfg.flrw_grid_N, cfg.flrw_grid_size
    d = L / N_
    grid = Grid(shape=(N_, N_, N_), spacing=(d, d, d), origin=(0.0, 0.0, 0.0))
    grid.add_field("Phi", flrw_potential(cfg, geo, device="cuda") if phi is None else phi)
    base = InterpolatorFast(grid) if cfg.flrw_fast else Interpolator(grid)
    shift = geo.observer if cfg.flrw_local_coords else None
    interp = shifted_interpolator(base, shift) if shift is not None else base
    metric = PerturbedFLRWMetricFast(a_of_eta=cosmo.a_of_eta, adot_of_eta=cosmo.adot_of_eta, grid=grid,
                                     interpolator=interp)
    eta0 = float(getattr(cosmo, "_eta_at_a1", 0.0))
    obs_state = (geo.observer - shift) if shift is not None else geo.observer
    lens_state = (geo.lens_center - shift) if shift is not None else geo.lens_center
    states = _photons(metric, cfg, geo, np.array([eta0, *obs_state], dtype=float), lens_state - obs_state,
                      impact_runner, checks)
    return metric, states, shift


@dataclasses.dataclass
class LegResult:
    trajectories: np.ndarray     # [n_photons, n_records, cols] float64, NaN-padded like the runner's files
    status: np.ndarray           # [n_photons] EXC_PH_*
    n_steps: np.ndarray
    stats: Optional[TrajectoryStats]   # None when no photon kept a trajectory


@dataclasses.dataclass
class CompareResult:
    config: RunConfig
    geometry: RunGeometry
    schwarzschild: LegResult
    flrw: LegResult
    # Set when a leg kept no trajectory at all: the reference's analyzer cannot reduce a file
    # of empty trajectories (it indexes their columns) and the job ends without a per-run table.
    error: Optional[str] = None


def reduce_leg(trajectories, status, n_steps, lens_center, *, is_spherical: bool) -> LegResult:
    stats = (trajectory_stats(trajectories, lens_center, is_spherical=is_spherical)
             if trajectories.shape[1] > 0 else None)
    return LegResult(trajectories, status, n_steps, stats)


def compare_result(cfg, geo, s: LegResult, f: LegResult) -> CompareResult:
    err = None
    for name, leg in (("Schwarzschild", s), ("FLRW", f)):
        if leg.stats is None:
            counts = np.bincount(leg.status, minlength=len(N.STATUS_NAMES))
            why = ", ".join(f"{N.STATUS_NAMES[i]} {int(k)}" for i, k in enumerate(counts) if k)
            err = f"every photon of the {name} leg failed ({why}): no trajectory to analyse"
            break
    return CompareResult(cfg, geo, s, f, err)


def trace_config(cfg: RunConfig, geo: RunGeometry, dt_min: float, dt_max: float):
    from ..trace import TraceConfig

    return TraceConfig(stepper=cfg.integrator, dt=geo.dlambda, dt_min=dt_min, dt_max=dt_max,
                       max_steps=geo.n_steps, record_every=cfg.record_every,
                       renormalize_every=cfg.renormalize_every, observables=False)


_FAILED = (N.PH_HORIZON, N.PH_NONFINITE, N.PH_OUTSIDE_GRID)


def leg_trajectories(res, x_offset, *, empty_failed: bool, fail_on_error: bool, label: str) -> tuple:
    """Stack one leg's records into the runner's NaN-padded array (padded to the longest photon)."""
    from ..records import trajectories_from_result

    status = res.status.cpu().numpy()
    failed = np.isin(status, _FAILED)
    if fail_on_error and failed.any():
        i = int(np.argmax(failed))
        raise RuntimeError(f"[{label}] photon {i + 1} failed ({N.STATUS_NAMES.get(int(status[i]), status[i])})")
    tr = trajectories_from_result(res, x_offset)
    n_rec = res.n_records.cpu().numpy().astype(np.int64)
    if empty_failed:
        tr[failed] = np.nan
        n_rec = np.where(failed, 0, n_rec)
    keep = int(n_rec.max()) if n_rec.size else 0
    return np.ascontiguousarray(tr[:, :keep]), status


def run(cfg: RunConfig, *, impact_runner: Optional[bool] = None) -> CompareResult:
    """Both legs of one comparison run, reduced with the analyzer's statistics (`error` set,
    and the statistics of the empty leg None, when a leg kept no trajectory at all)."""
    import torch

    from ..trace import trace_batch

    if impact_runner is None:
        impact_runner = cfg.sampling == "impact"
    geo = geometry(cfg)
    sm, s_states, dt_min, dt_max = schwarzschild_setup(cfg, geo, impact_runner)
    fm, f_states, shift = flrw_setup(cfg, geo, impact_runner)
    s_res = trace_batch(sm, s_states, trace_config(cfg, geo, dt_min, dt_max))
    f_res = trace_batch(fm, f_states, trace_config(cfg, geo, abs(geo.dlambda), abs(geo.dlambda)))
    torch.cuda.synchronize()
    s_tr, s_st = leg_trajectories(s_res, None, empty_failed=not impact_runner, fail_on_error=False,
                                  label="Schwarzschild")
    f_tr, f_st = leg_trajectories(f_res, shift, empty_failed=False, fail_on_error=not impact_runner, label="FLRW")
    s = reduce_leg(s_tr, s_st, s_res.n_steps.cpu().numpy(), geo.lens_center, is_spherical=True)
    f = reduce_leg(f_tr, f_st, f_res.n_steps.cpu().numpy(), geo.lens_center, is_spherical=False)
    return compare_result(cfg, geo, s, f)
