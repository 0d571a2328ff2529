"""Per-photon statistics of comparison-run trajectories and the per-run CSV.

Restates `_trajectory_stats` (_postprocessing/analyze_compare_trajectories.py:115-200) over a
whole stacked trajectory array at once, and the analyzer's per-run table (:330-368):

* positions: cartesian columns 1..3, or for the spherical (Schwarzschild) rows
  (r sin th cos ph, r sin th sin ph, r cos th) + lens centre (:84-94, :122-128);
* cartesian spatial velocity: columns 5..7, or the spherical rates through the
  e_r / e_theta / e_phi basis (:97-112);
* path length: sum over consecutive finite records of |x_{k+1} - x_k|, positions taken
  relative to the lens centre (:139-152);
* min_r / final_r: nanmin and last of |x - lens centre| (:154-160);
* bending angle: arccos(clip(v0_hat . v1_hat)) of the first and last finite velocities
  (:162-178);
* speed: |v_cart| / |u^0| (:180-186).

The arithmetic follows numpy's own evaluation order so that the results are bit-identical
to the reference analyzer: row norms over the last axis, pairwise sums per photon, and the
bending angle's norms and dot products through the inner dot routine numpy uses for 1-D
vectors (BLAS: a plain 3-term sum does not round the same way), for all photons at once.
The trajectories arrive NaN-padded to the longest photon, as the runners write them.
"""
from __future__ import annotations

import csv
import dataclasses
import os

import numpy as np

from ..core.constants import G, c

CSV_HEADER = ["photon", "S_n_records", "S_path_length_m", "S_min_r_m", "S_bend_rad",
              "F_n_records", "F_path_length_m", "F_min_r_m", "F_bend_rad", "delta_bend_rad"]


@dataclasses.dataclass
class TrajectoryStats:
    """One array per `TrajStats` field (analyze_compare_trajectories.py:74-83), [n_photons] each."""
    n_records: np.ndarray
    finite_fraction: np.ndarray
    path_length: np.ndarray
    min_r: np.ndarray
    final_r: np.ndarray
    bending_angle_rad: np.ndarray
    speed_mean: np.ndarray
    speed_max: np.ndarray

    def table(self) -> np.ndarray:
        """[n_photons, 8] in field order."""
        return np.column_stack([getattr(self, f.name).astype(np.float64) for f in dataclasses.fields(self)])


def _positions_velocities(trajs, lens_center, is_spherical):
    u = trajs[..., 4:8]
    if is_spherical:
        r, th, ph = trajs[..., 1], trajs[..., 2], trajs[..., 3]
        sth = np.sin(th)
        xyz_rel = np.stack([r * sth * np.cos(ph), r * sth * np.sin(ph), r * np.cos(th)], axis=-1)
        xyz = xyz_rel if lens_center is None else xyz_rel + lens_center
        dr, dth, dph = u[..., 1], u[..., 2], u[..., 3]
        cth, sph, cph = np.cos(th), np.sin(ph), np.cos(ph)
        vx = dr * (sth * cph) + (r * dth) * (cth * cph) + (r * sth * dph) * (-sph)
        vy = dr * (sth * sph) + (r * dth) * (cth * sph) + (r * sth * dph) * (cph)
        vz = dr * (cth) + (r * dth) * (-sth)
        v = np.stack([vx, vy, vz], axis=-1)
    else:
        xyz = trajs[..., 1:4]
        v = u[..., 1:4]
    return xyz, v, u


def _row_norm(a):
    # numpy.linalg.norm(a, axis=-1): sqrt of the sum of squares along the last axis
    return np.sqrt(np.add.reduce(a * a, axis=-1))


def _dots(a, b):
    """Row-wise dot products of [n, 3] arrays through numpy's vector-vector matmul, which
    evaluates each one with the same inner dot routine (BLAS) as numpy.dot on 1-D vectors,
    so the sums round exactly as the reference's per-photon calls do."""
    return np.matmul(a[:, None, :], b[:, :, None])[:, 0, 0]


def _bend(v):
    """Bending angles of [n_photons, n_records, 3] cartesian velocities (:162-178): the angle
    between the unit vectors (v / numpy.linalg.norm(v), zero below 1e-30) of each photon's
    first and last finite velocity; 0 with fewer than two records or two finite ones."""
    n_ph, n_rec = v.shape[0], v.shape[1]
    if n_rec < 2:
        return np.zeros(n_ph)
    finite = np.isfinite(v).all(axis=2)
    i0 = np.argmax(finite, axis=1)
    i1 = n_rec - 1 - np.argmax(finite[:, ::-1], axis=1)
    ok = finite.any(axis=1) & (i1 > i0)
    rows = np.arange(n_ph)
    v0 = np.where(ok[:, None], v[rows, i0], 1.0)
    v1 = np.where(ok[:, None], v[rows, i1], 1.0)

    def unit(x):
        n = np.sqrt(_dots(x, x))[:, None]
        return np.where(n < 1e-30, x * 0.0, x / np.where(n < 1e-30, 1.0, n))

    ang = np.arccos(np.clip(_dots(unit(v0), unit(v1)), -1.0, 1.0))
    return np.where(ok, ang, 0.0)


def trajectory_stats(trajs, lens_center=None, *, is_spherical: bool) -> TrajectoryStats:
    """Statistics of every photon of `trajs` [n_photons, n_records, n_cols] (float64, NaN-padded).

    `lens_center` (3,) in metres or None; `is_spherical` selects the Schwarzschild
    (t, r, theta, phi) reading of the position columns."""
    trajs = np.asarray(trajs, dtype=np.float64)
    if trajs.ndim != 3:
        raise ValueError("trajs must be [n_photons, n_records, n_cols]")
    n_ph, n_rec = trajs.shape[0], trajs.shape[1]
    lc = None if lens_center is None else np.asarray(lens_center, dtype=np.float64)
    xyz, v, u = _positions_velocities(trajs, lc, is_spherical)
    with np.errstate(invalid="ignore", divide="ignore"):
        finite_fraction = (np.isfinite(trajs).all(axis=2).mean(axis=1) if n_rec else np.zeros(n_ph))
        xyz_path = xyz if lc is None else xyz - lc
        if n_rec >= 2:
            ok = np.isfinite(xyz_path).all(axis=2)
            seg_ok = ok[:, 1:] & ok[:, :-1]
            seg_len = _row_norm(xyz_path[:, 1:] - xyz_path[:, :-1])
            path = np.ascontiguousarray(np.where(seg_ok, seg_len, 0.0)).sum(axis=1)
        else:
            path = np.full(n_ph, np.nan)
        rr = _row_norm(xyz_path)
        rr = np.where(np.isfinite(rr), rr, np.nan)
        # numpy's nanmin / nanmax / nanmean, computed as numpy computes them (fmin/fmax
        # reductions; sum of the non-NaN values over their count) but without the warnings
        # those emit for all-NaN rows: the warnings filters are process-wide, and rows are
        # reduced on several threads at once
        min_r = np.fmin.reduce(rr, axis=1) if n_rec else np.full(n_ph, np.nan)
        final_r = rr[:, -1] if n_rec else np.full(n_ph, np.nan)
        vmag = _row_norm(v)
        detadl = u[..., 0]
        denom = np.where(np.abs(detadl) > 0, np.abs(detadl), np.nan)
        speed = vmag / denom
        nan = np.isnan(speed)
        speed_mean = np.where(nan, 0.0, speed).sum(axis=1) / (~nan).sum(axis=1)
        speed_max = np.fmax.reduce(speed, axis=1) if n_rec else np.full(n_ph, np.nan)
    bend = _bend(v)
    return TrajectoryStats(n_records=np.full(n_ph, n_rec, dtype=np.int64), finite_fraction=finite_fraction,
                           path_length=path, min_r=min_r, final_r=final_r, bending_angle_rad=bend,
                           speed_mean=speed_mean, speed_max=speed_max)


def deflection_theory(min_r, mass_kg):
    """alpha = 4 G M / (c^2 b) with b = min_r, NaN where b is not finite and positive (:202-212)."""
    b = np.asarray(min_r, dtype=float)
    alpha = np.full_like(b, np.nan, dtype=float)
    ok = np.isfinite(b) & (b > 0)
    alpha[ok] = (4.0 * G * float(mass_kg)) / (c ** 2 * b[ok])
    return alpha


def per_run_rows(s: TrajectoryStats, f: TrajectoryStats):
    """The analyzer's CSV rows (:330-368): photon, S_* and F_* stats, FLRW - Schwarzschild bend."""
    n = min(len(s.n_records), len(f.n_records))
    delta = f.bending_angle_rad - s.bending_angle_rad
    rows = []
    for i in range(n):
        rows.append([i, int(s.n_records[i]), float(s.path_length[i]), float(s.min_r[i]),
                     float(s.bending_angle_rad[i]), int(f.n_records[i]), float(f.path_length[i]),
                     float(f.min_r[i]), float(f.bending_angle_rad[i]), float(delta[i])])
    return rows


def write_per_run_csv(path: str, s: TrajectoryStats, f: TrajectoryStats) -> str:
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(path, "w", newline="") as fp:
        w = csv.writer(fp)
        w.writerow(CSV_HEADER)
        w.writerows(per_run_rows(s, f))
    return path
