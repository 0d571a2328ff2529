"""CPU restatement of the redshift-map post-processing: the checker of csrc/exc_maps.cu.

Test infrastructure: only tests/ import this module. Pure Python loops over one photon at a
time, for the small record stacks the tests use.

What it restates, operation for operation:
  * _postprocessing/compute_redshift_map.py:30-51 (load_trajectories): a record row holding a
    NaN in any column is dropped before anything else;
  * compute_redshift_map.py:98-171 (compute_redshift_map): photons with fewer than two rows
    left keep zeros; the others get the components of
  * excalibur/observables/redshift.py:165-399 (RedshiftCalculator, trajectories with >= 14
    columns): z_H = a_obs / a_em - 1 (:177); z_SW = (Phi_obs - Phi_em) / c**2 (:220);
    z_ISW = -simpson(Phi_dot * c**2, x=eta) / c**2 (:255, :271); the Doppler term
    (v_obs . n - v_em . n) / c with n the unit endpoint displacement (:300-312), zero without a
    velocity field; z_v = 0; z_total and z_total_exact (:393-398);
  * compute_redshift_map.py:54-95 (extract_sky_positions): the unit spatial velocity of each
    photon's first row, their mean direction, and the tangent-plane projection.

Third-party arithmetic restated from its published algorithm:
  * scipy.integrate.simpson (scipy >= 1.11; 1.18.1 here): composite Simpson for irregular
    spacing over the first N - 1 (odd N) or N - 2 (even N) intervals, and for even N >= 4 the
    correction of the last interval from Cartwright (2017), with the zero-denominator guards of
    scipy's `np.true_divide(..., where=den != 0)` (the cube of the last spacing: `cube` below);
    two samples are a trapezoid;
  * numpy's pairwise summation (np.sum of a contiguous float64 array): blocks of fewer than
    eight terms summed in order, blocks of up to 128 with eight partial sums, longer ones
    split at n/2 rounded down to a multiple of 8.
tests/test_redshift_map_oracle.py pins both against scipy and numpy: bit for bit, but for the
even-count Simpson's last-interval cube (within an ulp of that weight).
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np


def np_sum(a, lo: int = 0, n: int | None = None) -> float:
    """np.sum of a[lo:lo + n] (float64, contiguous)."""
    if n is None:
        n = len(a) - lo
    return 0.0 + _pairwise(a, lo, n)


def _pairwise(a, lo, n):
    if n < 8:
        res = -0.0
        for i in range(n):
            res += float(a[lo + i])
        return res
    if n <= 128:
        r = [float(a[lo + j]) for j in range(8)]
        i = 8
        while i < n - (n % 8):
            for j in range(8):
                r[j] += float(a[lo + i + j])
            i += 8
        res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]))
        while i < n:
            res += float(a[lo + i])
            i += 1
        return res
    n2 = n // 2
    n2 -= n2 % 8
    return _pairwise(a, lo, n2) + _pairwise(a, lo + n2, n - n2)


def _fma(a: float, b: float, c: float) -> float:
    """a * b + c rounded once (an infinity or a NaN among the operands propagates as IEEE
    arithmetic does)."""
    if not (math.isfinite(a) and math.isfinite(b) and math.isfinite(c)):
        return a * b + c
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def cube(x: float) -> float:
    """x**3 as the kernel forms it: the exact square split by an FMA (Dekker), times x in
    double-double, rounded at the end. scipy's `h[1] ** 3` is numpy's float64 power, which is
    libm's pow on most builds (correctly rounded but for rare near-halfway cases) and a SIMD
    routine within an ulp of it on AVX-512 x86 builds; this form agrees with the correctly
    rounded cube except near halfway cases, so the even-count Simpson here is within an ulp of
    the last interval's weight of scipy's on any platform."""
    p = x * x
    e = _fma(x, x, -p)
    hi = p * x
    lo = _fma(p, x, -hi) + e * x
    return hi + lo


def _div0(num, den):
    """np.true_divide(num, den, out=zeros, where=den != 0)."""
    return num / den if den != 0.0 else 0.0


def _basic_simpson_terms(y, x, stop):
    """The per-pair terms of scipy's irregular-spacing Simpson over pairs starting at 0, 2, ...
    below `stop`."""
    out = []
    for k in range(0, stop, 2):
        h0 = float(x[k + 1]) - float(x[k])
        h1 = float(x[k + 2]) - float(x[k + 1])
        hsum = h0 + h1
        hprod = h0 * h1
        h0divh1 = _div0(h0, h1)
        t0 = float(y[k]) * (2.0 - _div0(1.0, h0divh1))
        t1 = float(y[k + 1]) * (hsum * _div0(hsum, hprod))
        t2 = float(y[k + 2]) * (2.0 - h0divh1)
        out.append(hsum / 6.0 * ((t0 + t1) + t2))
    return out


def simpson(y, x) -> float:
    """scipy.integrate.simpson(y, x=x) for 1-D float64 y and x of the same length."""
    n = len(y)
    if n % 2 == 1:
        return np_sum(_basic_simpson_terms(y, x, n - 2))
    if n == 2:
        last_dx = float(x[-1]) - float(x[-2])
        return 0.0 + (0.0 + 0.5 * last_dx * (float(y[-1]) + float(y[-2])))
    result = np_sum(_basic_simpson_terms(y, x, n - 3))
    h0 = float(x[-2]) - float(x[-3])
    h1 = float(x[-1]) - float(x[-2])
    alpha = _div0(2 * h1 ** 2 + 3 * h0 * h1, 6 * (h1 + h0))
    beta = _div0(h1 ** 2 + 3.0 * h0 * h1, 6 * h0)
    eta = _div0(1 * cube(h1), 6 * h0 * (h0 + h1))
    result += alpha * float(y[-1]) + beta * float(y[-2]) - eta * float(y[-3])
    return result + 0.0


def clean_rows(states: np.ndarray) -> np.ndarray:
    return states[~np.isnan(states).any(axis=1)]


def _dot3(a, b):
    """np.dot of two 3-vectors (and the square under np.linalg.norm): BLAS ddot, which on x86-64
    (OpenBLAS with FMA) forms a0*b0 and fuses a1*b1, then a2*b2, into it."""
    return _fma(float(a[2]), float(b[2]), _fma(float(a[1]), float(b[1]), float(a[0]) * float(b[0])))


# output columns, as csrc/exc_maps.cu writes them (EXC_RS_* in include/excalibur_gb300.h)
COLUMNS = ("z_H", "z_SW", "z_ISW", "z_D", "z_total", "z_total_exact", "Phi_obs", "Phi_em", "a_obs", "a_em",
           "eta_obs", "eta_em", "x_obs0", "x_obs1", "x_obs2", "x_em0", "x_em1", "x_em2", "n_rows",
           "path", "chord", "time_delay", "td_kept")
_C = {k: i for i, k in enumerate(COLUMNS)}


def time_delay_kept(tr: np.ndarray) -> bool:
    """compute_time_delay_map.py:76-92 (load_trajectories): a photon is kept when it has a clean
    row and every clean |x|, |y|, |z| < 1e26 m and |eta| < 3e18 s."""
    if len(tr) == 0:
        return False
    return bool(np.max(np.abs(tr[:, 1:4])) < 1e26 and np.max(np.abs(tr[:, 0])) < 3e18)


def time_delay(tr: np.ndarray, c: float):
    """compute_time_delays (compute_time_delay_map.py:244-310) for one clean trajectory:
    (time_delay, path, chord); zeros below two rows. The path is summed segment by segment in
    row order from 0.0 (compute_travel_time_deflected, :97-126); the straight path is the
    chord |x_last - x_first| (compute_travel_time_straight returns the distance it is given)."""
    if len(tr) < 2:
        return 0.0, 0.0, 0.0
    path = 0.0
    for i in range(len(tr) - 1):
        d = [float(tr[i + 1, 1 + k]) - float(tr[i, 1 + k]) for k in range(3)]
        path += math.sqrt(_dot3(d, d))
    X = [float(tr[-1, 1 + k]) - float(tr[0, 1 + k]) for k in range(3)]
    chord = math.sqrt(_dot3(X, X))
    return path / c - chord / c, path, chord


def redshift_row(states: np.ndarray, c: float, v_obs=None, v_em=None) -> np.ndarray:
    """The output row of one photon's NaN-padded record block [n_rows, n_cols >= 14]."""
    out = np.zeros(len(COLUMNS))
    tr = clean_rows(states)
    m = len(tr)
    out[_C["n_rows"]] = m
    out[6:18] = np.nan
    out[_C["td_kept"]] = 1.0 if time_delay_kept(tr) else 0.0
    out[_C["time_delay"]], out[_C["path"]], out[_C["chord"]] = time_delay(tr, c)
    if m >= 1:
        out[10], out[11] = tr[0, 0], tr[-1, 0]
        out[12:15], out[15:18] = tr[0, 1:4], tr[-1, 1:4]
        out[6], out[7] = tr[0, 9], tr[-1, 9]
        out[8], out[9] = tr[0, 8], tr[-1, 8]
    if m < 2:
        return out
    c2 = c ** 2
    z_h = (float(tr[0, 8]) / float(tr[-1, 8])) - 1.0
    z_sw = (float(tr[0, 9]) - float(tr[-1, 9])) / c2
    dphi = [float(p) * c2 for p in tr[:, 13]]
    z_isw = -simpson(dphi, tr[:, 0]) / c2
    z_d = 0.0
    if v_obs is not None:
        d = [float(tr[-1, 1 + k]) - float(tr[0, 1 + k]) for k in range(3)]
        nrm = math.sqrt(_dot3(d, d))
        nh = [d[k] / nrm for k in range(3)]
        z_d = (_dot3([float(v) for v in v_obs], nh) - _dot3([float(v) for v in v_em], nh)) / c
    z_v = 0.0
    out[0:4] = z_h, z_sw, z_isw, z_d
    out[4] = z_h + z_sw + z_isw + z_d + z_v
    out[5] = ((1 + z_h) * (1 + z_sw) * (1 + z_isw) * (1 + z_d) * (1 + z_v)) - 1.0
    return out


def redshift_rows(records: np.ndarray, c: float, v_obs=None, v_em=None) -> np.ndarray:
    return np.stack([redshift_row(records[i], c, None if v_obs is None else v_obs[i],
                                  None if v_em is None else v_em[i]) for i in range(len(records))])


def sky_positions(records: np.ndarray):
    """(x_proj, y_proj, used) of extract_sky_positions over the photons with at least one row
    left (`used`, a boolean mask: the reference's arrays cover only those photons)."""
    dirs, used = [], np.zeros(len(records), bool)
    for i in range(len(records)):
        tr = clean_rows(records[i])
        if len(tr) < 1:
            continue
        u = [float(v) for v in tr[0, 5:8]]
        nrm = math.sqrt(_dot3(u, u))
        dirs.append([u[k] / nrm for k in range(3)])
        used[i] = True
    dirs = np.array(dirs)
    mean = [0.0, 0.0, 0.0]
    for d in dirs:                       # np.mean(axis=0): rows accumulated in order
        for k in range(3):
            mean[k] += d[k]
    mean = [m / len(dirs) for m in mean]
    nrm = math.sqrt(_dot3(mean, mean))
    mean = [m / nrm for m in mean]
    up = [0.0, 0.0, 1.0] if abs(mean[2]) < 0.9 else [1.0, 0.0, 0.0]
    ud = _dot3(up, mean)
    bx = [up[k] - ud * mean[k] for k in range(3)]
    nb = math.sqrt(_dot3(bx, bx))
    bx = [b / nb for b in bx]
    by = [mean[1] * bx[2] - mean[2] * bx[1], mean[2] * bx[0] - mean[0] * bx[2], mean[0] * bx[1] - mean[1] * bx[0]]
    xp, yp = np.zeros(len(dirs)), np.zeros(len(dirs))
    for i, d in enumerate(dirs):
        ct = _dot3(d, mean)
        th = math.acos(min(max(ct, -1.0), 1.0))
        if th > 1e-10:
            ip = [d[k] - ct * mean[k] for k in range(3)]
            ni = math.sqrt(_dot3(ip, ip))
            ip = [v / ni for v in ip]
            xp[i] = _dot3(ip, bx) * th
            yp[i] = _dot3(ip, by) * th
    return xp, yp, used


def bin_mean(x, y, v, nx: int, ny: int, extent):
    """Pixel means of scattered samples: pixel (j, i) with i = floor((x - x0) / (x1 - x0) * nx)
    and j likewise from y, a sample at the upper edge falling in the last pixel, samples
    outside the extent or with a NaN skipped. Returns (mean [ny, nx] with NaN where empty,
    count [ny, nx])."""
    x0, x1, y0, y1 = extent
    s = np.zeros((ny, nx))
    cnt = np.zeros((ny, nx), np.int64)
    for xi, yi, vi in zip(x, y, v):
        if not (np.isfinite(xi) and np.isfinite(yi) and np.isfinite(vi)):
            continue
        if xi < x0 or xi > x1 or yi < y0 or yi > y1:
            continue
        i = min(int(math.floor((xi - x0) / (x1 - x0) * nx)), nx - 1)
        j = min(int(math.floor((yi - y0) / (y1 - y0) * ny)), ny - 1)
        s[j, i] += vi
        cnt[j, i] += 1
    with np.errstate(invalid="ignore", divide="ignore"):
        mean = np.where(cnt > 0, s / np.maximum(cnt, 1), np.nan)
    return mean, cnt
