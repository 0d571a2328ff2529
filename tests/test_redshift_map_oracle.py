"""The redshift-map oracle (oracle/redshift_map.py) against scipy, numpy and the package's
RedshiftCalculator (itself the reference's class on a trajectory's rows), bit for bit."""
import numpy as np
import pytest

from oracle import redshift_map as O
from excalibur_tool_gb300.core.constants import c
from excalibur_tool_gb300.observables.redshift import RedshiftCalculator


def _irregular(rng, n, dup=False):
    x = np.cumsum(rng.uniform(0.1, 2.0, n)) * 1e14 + 4.6e17
    if dup and n > 3:
        x[n // 2] = x[n // 2 - 1]          # a zero-length interval (scipy's where= guards)
    return x


def test_np_sum_matches_numpy():
    rng = np.random.default_rng(1)
    for n in list(range(0, 140)) + [255, 256, 257, 1000, 1031, 4100]:
        a = rng.standard_normal(n) * 10.0 ** rng.integers(-6, 6, n)
        assert O.np_sum(a) == np.sum(a), n


def test_simpson_matches_scipy():
    from scipy.integrate import simpson

    rng = np.random.default_rng(2)
    for n in list(range(1, 70)) + [128, 129, 257, 258, 301, 1000]:
        for dup in (False, True):
            x = _irregular(rng, n, dup)
            y = rng.standard_normal(n) * 1e-3
            got, want = O.simpson(y, x), float(simpson(y, x=x))
            if n % 2 == 1 or n == 2:
                assert got == want, (n, dup, got, want)
            else:
                # the last interval's x**3: numpy's power against a double-double cube
                scale = float(np.sum(np.abs(y) * np.gradient(x)))
                assert abs(got - want) <= 4e-16 * scale, (n, dup, got, want)


def test_cube_is_correctly_rounded_off_halfway():
    from fractions import Fraction

    rng = np.random.default_rng(6)
    x = rng.uniform(1e13, 2e14, 3000)
    bad = sum(O.cube(float(v)) != float(Fraction(float(v)) ** 3) for v in x)
    assert bad <= 3


def _records(rng, n_photons=40, n_rows=60, lag=True, lengths=None):
    """NaN-padded FLRW record stacks: ragged lengths (0, 1, 2, 3, ... rows), the first row's
    quantity columns NaN like the runners' histories (lag=True), a NaN row in the middle."""
    rec = np.full((n_photons, n_rows, 14), np.nan)
    for i in range(n_photons):
        if lengths is not None:
            m = lengths[i]
        else:
            m = i if i < 6 else int(rng.integers(2, n_rows + 1))
        eta = 4.6e17 - np.cumsum(rng.uniform(0.5, 1.5, m)) * 1e14
        rec[i, :m, 0] = eta
        rec[i, :m, 1:4] = rng.uniform(0, 3e24, 3) + np.cumsum(rng.normal(0, 1e21, (m, 3)), axis=0)
        rec[i, :m, 4] = -1.0
        rec[i, :m, 5:8] = rng.normal(0, 1, 3) * 1e5 + np.array([-3e8, 0, 0])
        rec[i, :m, 8] = 1.0 / (1.0 + np.linspace(0, 0.3, m))
        rec[i, :m, 9] = rng.normal(0, 1e-6, m)
        rec[i, :m, 10:13] = rng.normal(0, 1e-9, (m, 3))
        rec[i, :m, 13] = rng.normal(0, 1e-24, m)
        if lag and m > 0:
            rec[i, 0, 8:] = np.nan
        if m > 8 and i % 5 == 0:
            rec[i, m // 2, 3] = np.nan
    return rec


def test_redshift_rows_match_the_calculator():
    rng = np.random.default_rng(3)
    rec = _records(rng)
    rows = O.redshift_rows(rec, c)
    for i in range(len(rec)):
        tr = O.clean_rows(rec[i])
        if len(tr) < 2:
            assert np.all(rows[i, :6] == 0.0)
            continue
        r = RedshiftCalculator(tr).compute_all_components()
        for k, name in enumerate(("z_H", "z_SW", "z_ISW", "z_D", "z_total", "z_total_exact")):
            assert rows[i, k] == r[name], (i, name)
        assert rows[i, O.COLUMNS.index("n_rows")] == len(tr)


def test_doppler_matches_the_calculator():
    rng = np.random.default_rng(4)
    rec = _records(rng, n_photons=12, lag=False)
    v = rng.normal(0, 3e5, (12, 2, 3))
    rows = O.redshift_rows(rec, c, v[:, 0], v[:, 1])
    for i in range(6, 12):
        tr = O.clean_rows(rec[i])
        calls = iter([v[i, 0], v[i, 1]])
        r = RedshiftCalculator(tr, velocity_func=lambda *a: next(calls)).compute_all_components()
        if _numpy_dot_is_fma_sequence():
            assert rows[i, 3] == r["z_D"] and rows[i, 4] == r["z_total"]
        else:
            # another BLAS orders the 3-term dot differently: an ulp or two
            assert abs(rows[i, 3] - r["z_D"]) <= 1e-15 * abs(r["z_D"]) + 1e-30
            assert abs(rows[i, 4] - r["z_total"]) <= 1e-15 * abs(r["z_total"])


def _numpy_dot_is_fma_sequence():
    """Whether this numpy's 3-vector dot is the product a0*b0 with a1*b1 and a2*b2 fused into it
    in order (OpenBLAS's ddot on x86-64), the form the oracle and the kernels restate."""
    rng = np.random.default_rng(9)
    a, b = rng.standard_normal((2, 2000, 3)) * 10.0 ** rng.integers(-3, 3, (2, 2000, 3))
    return all(float(np.dot(a[i], b[i])) == O._dot3(a[i], b[i]) for i in range(len(a)))


def test_time_delays_match_the_reference_script():
    """tests/golden/time_delays.npz: compute_time_delay_map.py's own load_trajectories and
    compute_time_delays on synthetic record blocks (ragged, NaN holes, photons its loader drops
    at 1e26 m, 3e18 s and infinity, one just below both limits). The oracle's table keeps the
    same photons and gives their path, chord and delay bit for bit."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "time_delays.npz"))
    rows = O.redshift_rows(g["records"], c)
    kept = rows[:, O.COLUMNS.index("td_kept")] == 1.0
    assert np.array_equal(kept, g["kept"]) and kept.sum() == len(g["time_delays"])
    got = {k: rows[kept, O.COLUMNS.index(k)] for k in ("time_delay", "path", "chord")}
    if _numpy_dot_is_fma_sequence():
        assert np.array_equal(got["time_delay"], g["time_delays"])
        assert np.array_equal(got["path"], g["distances_deflected"])
        assert np.array_equal(got["chord"], g["distances_straight"])
    else:
        for k, ref in (("time_delay", "time_delays"), ("path", "distances_deflected"),
                       ("chord", "distances_straight")):
            assert np.allclose(got[k], g[ref], rtol=1e-14, atol=1e-3), k
    assert np.any(got["time_delay"] > 0) and np.any(got["time_delay"] == 0.0)


def test_sky_positions_match_numpy():
    rng = np.random.default_rng(5)
    rec = _records(rng)
    xp, yp, used = O.sky_positions(rec)
    trajs = [O.clean_rows(r) for r in rec]
    dirs = np.array([t[0, 5:8] / np.linalg.norm(t[0, 5:8]) for t in trajs if len(t)])
    md = np.mean(dirs, axis=0)
    md /= np.linalg.norm(md)
    assert used.sum() == len(dirs)
    ct = dirs @ md
    th = np.arccos(np.clip(ct, -1, 1))
    ip = dirs - ct[:, None] * md
    ip /= np.linalg.norm(ip, axis=1)[:, None]
    up = np.array([0.0, 0, 1])
    bx = up - up @ md * md
    bx /= np.linalg.norm(bx)
    by = np.cross(md, bx)
    # d - cos(theta) * mean cancels to |d| * theta: relative rounding ~1e-16 / theta**2
    tol = 1e-15 / th
    assert np.all(np.abs(xp - ip @ bx * th) <= tol) and np.all(np.abs(yp - ip @ by * th) <= tol)


def test_bin_mean_small():
    x = np.array([0.0, 0.5, 1.0, 0.99, np.nan, 2.0])
    y = np.array([0.0, 0.5, 1.0, 0.0, 0.0, 0.0])
    v = np.array([1.0, 2.0, 3.0, 4.0, 5.0, 6.0])
    mean, cnt = O.bin_mean(x, y, v, 2, 2, (0.0, 1.0, 0.0, 1.0))
    assert cnt.tolist() == [[1, 1], [0, 2]]
    assert mean[1, 1] == 2.5 and np.isnan(mean[1, 0]) and mean[0, 1] == 4.0


def test_map_frame_and_extent_follow_the_reference():
    """The host pieces of observables.maps: the tangent-plane frame and create_2d_map's square
    extent, against the reference's formulas (compute_redshift_map.py:68-80,
    compute_time_delay_map.py:330-345)."""
    from excalibur_tool_gb300.observables import maps

    for mean in ([-1.0, 0.01, 0.02], [0.1, 0.2, 0.95]):
        m, bx, by = maps.sky_frame(mean)
        ref_m = np.asarray(mean) / np.linalg.norm(mean)
        up = np.array([0.0, 0, 1]) if abs(ref_m[2]) < 0.9 else np.array([1.0, 0, 0])
        ref_bx = up - np.dot(up, ref_m) * ref_m
        ref_bx = ref_bx / np.linalg.norm(ref_bx)
        assert np.array_equal(m, ref_m) and np.array_equal(bx, ref_bx)
        assert np.array_equal(by, np.cross(ref_m, ref_bx))
    x = np.array([-1.0, 3.0, 0.5])
    y = np.array([2.0, 2.5, 2.2])
    x0, x1, y0, y1 = maps.square_extent(x, y)
    assert (x0, x1) == (1.0 - 2.4, 1.0 + 2.4) and (y0, y1) == (2.25 - 2.4, 2.25 + 2.4)
