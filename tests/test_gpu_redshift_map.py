"""Redshift maps on the GPU (csrc/exc_maps.cu) against the oracle (oracle/redshift_map.py):
per-photon components bit for bit, sky positions to the rounding of the mean direction,
binned maps to the order of the atomic sums."""
import numpy as np
import pytest

from oracle import redshift_map as O
from test_redshift_map_oracle import _records
from excalibur_tool_gb300.core.constants import c

pytestmark = pytest.mark.gpu

def _table(rec, **kw):
    from excalibur_tool_gb300.observables import maps

    return maps.redshift_table(rec, **kw).cpu().numpy()


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True)


def test_components_match_oracle(cuda):
    rng = np.random.default_rng(11)
    rec = _records(rng, n_photons=48, n_rows=60)
    got, want = _table(rec), O.redshift_rows(rec, c)
    assert got.shape == want.shape
    assert _same(got, want)


def test_long_histories_match_oracle(cuda):
    """Histories of 250 to 700 rows (Simpson sums of more than 128 pairs: numpy's recursive
    split), odd and even clean counts, a zero-length interval."""
    rng = np.random.default_rng(12)
    rec = _records(rng, n_photons=10, n_rows=700, lag=True,
                   lengths=(699, 700, 257, 258, 300, 301, 513, 514, 640, 641))
    rec[3, 100, 0] = rec[3, 99, 0]
    got, want = _table(rec), O.redshift_rows(rec, c)
    assert _same(got, want)
    assert np.all(got[:, O.COLUMNS.index("n_rows")] >= 250)


def test_doppler_matches_oracle(cuda):
    rng = np.random.default_rng(13)
    rec = _records(rng, n_photons=16, n_rows=40, lag=False)
    v = rng.normal(0, 3e5, (2, 16, 3))
    calls = {}

    def velocity(x, y, z, eta):
        # the endpoint velocities by the endpoint's time
        k = next(i for i in range(16) if eta in (calls.get((i, 0)), calls.get((i, 1))))
        return v[0 if eta == calls[(k, 0)] else 1, k]

    want = O.redshift_rows(rec, c, v[0], v[1])
    for i in range(16):
        tr = O.clean_rows(rec[i])
        if len(tr) >= 2:
            calls[(i, 0)], calls[(i, 1)] = tr[0, 0], tr[-1, 0]
    got = _table(rec, velocity_func=velocity)
    ok = want[:, O.COLUMNS.index("n_rows")] >= 2
    assert _same(got[ok], want[ok]) and np.any(got[ok, 3] != 0.0)


def _golden_time_delays():
    import os

    return np.load(os.path.join(os.path.dirname(__file__), "golden", "time_delays.npz"))


def test_time_delay_columns_match_oracle(cuda):
    """The whole table, time-delay columns included, on the reference script's golden records:
    photons the loader drops (1e26 m, 3e18 s, an infinite position) flagged, the one just below
    both limits kept."""
    rec = _golden_time_delays()["records"]
    got, want = _table(rec), O.redshift_rows(rec, c)
    assert _same(got, want)
    assert got[:, O.COLUMNS.index("td_kept")].tolist() == _golden_time_delays()["kept"].astype(float).tolist()


def test_compute_time_delays_matches_the_reference_script(cuda):
    """maps.compute_time_delays against compute_time_delay_map.py's own outputs on the same
    records (tests/golden/time_delays.npz): delays, deflected and straight distances bit for
    bit; sky positions to CUDA's acos against libm's."""
    from excalibur_tool_gb300.observables import maps

    g = _golden_time_delays()
    delays, dd, ds, (x, y) = maps.compute_time_delays(g["records"])
    assert np.array_equal(delays, g["time_delays"])
    assert np.array_equal(dd, g["distances_deflected"]) and np.array_equal(ds, g["distances_straight"])
    th = np.hypot(g["x_proj"], g["y_proj"])
    tol = 4e-15 * th + 1e-18
    assert np.all(np.abs(x - g["x_proj"]) <= tol) and np.all(np.abs(y - g["y_proj"]) <= tol)


def test_time_delay_depends_on_record_every(cuda):
    """The recorded path is summed over the rows kept, so thinning the rows (record_every)
    shortens it toward the chord, as in the reference; one pass (<= 257 rows) and the scratch
    pass (> 257 rows) give the oracle's values."""
    rng = np.random.default_rng(16)
    rec = _records(rng, n_photons=8, n_rows=520, lag=False, lengths=[520] * 8)
    for every in (1, 2, 4):
        sub = np.ascontiguousarray(rec[:, ::every])
        got, want = _table(sub), O.redshift_rows(sub, c)
        assert _same(got, want), every
    p1 = _table(rec)[:, O.COLUMNS.index("path")]
    p4 = _table(np.ascontiguousarray(rec[:, ::4]))[:, O.COLUMNS.index("path")]
    assert np.all(p4 < p1)


def test_runner_trajectories_map(cuda):
    """The comparison runner's FLRW histories (first rows' quantities NaN, as the runner records
    them) through compute_redshift_map: the components the oracle gives on the same file."""
    from test_compare_runner import job1_config
    from excalibur_tool_gb300.observables import maps
    from excalibur_tool_gb300.runners import compare as R

    res = R.run(job1_config())
    tr = res.flrw.trajectories
    data, (x, y) = maps.compute_redshift_map(tr)
    want = O.redshift_rows(tr, c)
    for k in ("z_H", "z_SW", "z_ISW", "z_D", "z_total"):
        assert np.array_equal(data[k], want[:, O.COLUMNS.index(k)]), k
    assert np.all(want[:, O.COLUMNS.index("n_rows")] >= 2) and np.isfinite(data["z_total"]).all()
    ox, oy, used = O.sky_positions(tr)
    assert len(x) == used.sum() == len(tr)
    th = np.hypot(ox, oy)
    tol = 4e-15 * th + 1e-18
    assert np.all(np.abs(x - ox) <= tol) and np.all(np.abs(y - oy) <= tol)


def test_sky_positions_match_oracle(cuda):
    from excalibur_tool_gb300.observables import maps

    rng = np.random.default_rng(14)
    rec = _records(rng, n_photons=64, n_rows=30)
    xp, yp, used = maps.sky_projection(rec)
    ox, oy, oused = O.sky_positions(rec)
    assert np.array_equal(used.cpu().numpy(), oused)
    x, y = xp.cpu().numpy()[oused], yp.cpu().numpy()[oused]
    # the frame is the reference's to the bit (np.mean on the host); what remains is CUDA's
    # acos against libm's, a couple of ulps of each angle
    th = np.hypot(ox, oy)
    tol = 4e-15 * th + 1e-18
    assert np.all(np.abs(x - ox) <= tol) and np.all(np.abs(y - oy) <= tol)
    assert np.isnan(xp.cpu().numpy()[~oused]).all()


def test_one_photon_sky_map(cuda):
    """A single sample (zero-width range) still bins: a small square about it."""
    from excalibur_tool_gb300.observables import maps

    X, Y, mean, cnt = maps.bin_sky_map(np.array([0.01]), np.array([-0.02]), np.array([3.0]), grid_resolution=8)
    assert cnt.sum() == 1 and np.nanmax(mean) == 3.0
    with pytest.raises(ValueError):
        maps.bin_sky_map(np.array([np.nan]), np.array([0.0]), np.array([1.0]), grid_resolution=8)


def test_bin_sky_map_matches_oracle(cuda):
    from excalibur_tool_gb300.observables import maps

    rng = np.random.default_rng(15)
    n = 200_000
    x, y = rng.normal(0, 1e-3, n), rng.normal(0, 1e-3, n)
    v = rng.normal(1e-4, 1e-5, n)
    x[::97] = np.nan
    v[::89] = np.inf
    ext = maps.square_extent(x[np.isfinite(x)], y[np.isfinite(x)])
    X, Y, mean, cnt = maps.bin_sky_map(x, y, v, grid_resolution=64, extent=ext)
    om, oc = O.bin_mean(x, y, v, 64, 64, ext)
    assert np.array_equal(cnt, oc) and cnt.sum() > 0.95 * n
    both = oc > 0
    assert np.array_equal(np.isnan(mean), ~both)
    assert np.all(np.abs(mean[both] - om[both]) <= 1e-12 * np.abs(om[both]))
    assert X.shape == (64, 64) and X[0, 0] > ext[0] and Y[-1, 0] < ext[3]
