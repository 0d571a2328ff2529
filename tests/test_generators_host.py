"""The reference's cone generators against the reference's own output (tests/golden/generators.npz).

The directions are host arithmetic (the cone grid, the Rodrigues rotation, the cartesian to
spherical velocity conversion); u^0 comes from the device. Here the metric evaluations are
stood in for by the oracle (pinned to the reference bit for bit), so that the host part runs
without a GPU. The batched rotation and normalisation sum in another order than the reference's
per-vector numpy calls: a direction differs by at most an ulp (on ~10 % of the photons), which
the spherical velocity's angular components, ~sin(cone angle) of the radial one, magnify in
relative terms.
"""
import numpy as np
import pytest

from conftest import golden
from helpers import lcdm_spacetime, rel_err, schw_spacetime
from oracle import oracle as O

ONE_MPC = 3.085677581e22


class _OracleMetric:
    """metric_tensor through the oracle, for the generators' host code."""

    def __init__(self, st):
        self.st = st

    def metric_tensor(self, x):
        gd, status = O.metric_tensor(self.st, np.asarray(x, dtype=float)[None])
        assert status[0] == 0
        return np.diag(gd[0])


def _cases(g):
    flrw = lcdm_spacetime(g["field"], float(g["box"]))
    schw = schw_spacetime(1e15 * 1.98847e30, 3 * ONE_MPC)
    obs = np.array([0.01, 0.01, 0.01]) * 1e3 * ONE_MPC
    return {"flrw": (flrw, g["flrw_origin"], [1.0, 0.5, -0.3], 7.0),
            "schw": (schw, g["schw_origin"], g["schw_center"] - obs, 2.0)}


def _column_scaled(a, b):
    scale = np.abs(b).max(axis=0)
    return float((np.abs(a - b) / np.where(scale > 0, scale, 1.0)).max())


def _check(name, got, want):
    assert got.shape == want.shape
    assert np.array_equal(got[:, :4], want[:, :4])
    assert rel_err(got[:, 4], want[:, 4]).max() <= 4.5e-16
    if name == "flrw":
        assert rel_err(got, want).max() <= 4.5e-16
    else:
        # v_theta, v_phi ~ sin(2 deg) v_r: an ulp of the cartesian direction is ~3e-15 of them
        assert _column_scaled(got, want) <= 1e-14


@pytest.mark.parametrize("name", ["flrw", "schw"])
def test_cone_grid_metric_tensor(monkeypatch, capsys, name):
    """generate_cone_grid_metric_tensor (photons.py:159-293): u^0 from the diagonal metric at the
    origin; 49 photons (7 x 7, the theta = 0 row once) in a 7 degree FLRW cone, 4 x 9 in a
    2 degree cone from a spherical Schwarzschild origin with cartesian directions."""
    from excalibur_tool_gb300 import _evaluate
    from excalibur_tool_gb300.photon.photons import Photons

    g = golden("generators.npz")
    st, origin, axis, deg = _cases(g)[name]
    monkeypatch.setattr(_evaluate, "null_error", lambda metric, s: O.null_error(metric.st, np.asarray(s)))
    ph = Photons(_OracleMetric(st))
    out = ph.generate_cone_grid_metric_tensor(49 if name == "flrw" else (4, 9), origin, axis, np.deg2rad(deg),
                                              direction_basis="cartesian")
    _check(name, out, g[f"{name}_cone_mt"])
    assert np.array_equal(ph.states_numpy(), out) and len(ph) == len(out)
    assert "Warning" not in capsys.readouterr().out


@pytest.mark.parametrize("name", ["flrw", "schw"])
def test_cone_grid_directions(name):
    """generate_cone_grid's directions (photons.py:295-424) completed by the oracle's null-condition
    solve against the reference's states: 49 photons in the FLRW cone, 36 (6 x 6) in the
    Schwarzschild one."""
    from excalibur_tool_gb300.photon.photons import Photons

    g = golden("generators.npz")
    st, origin, axis, deg = _cases(g)[name]
    d = Photons._cone_grid_directions(49 if name == "flrw" else 36, axis, np.deg2rad(deg))
    s = np.zeros((len(d), 8))
    s[:, :4] = origin
    s[:, 5:8] = Photons(None)._spatial_from_directions(origin, d, "cartesian")
    out, status = O.null_init(st, s, -1.0)
    assert (status == 0).all()
    _check(name, out, g[f"{name}_cone"])


def test_cone_grid_metric_tensor_reports_violations(monkeypatch, capsys):
    """A photon whose relative null error exceeds 1e-5 is reported, as the reference prints it."""
    from excalibur_tool_gb300 import _evaluate
    from excalibur_tool_gb300.photon.photons import Photons

    g = golden("generators.npz")
    st, origin, axis, deg = _cases(g)["flrw"]
    monkeypatch.setattr(_evaluate, "null_error", lambda metric, s: (np.full(len(s), 2e-5), np.zeros(len(s))))
    Photons(_OracleMetric(st)).generate_cone_grid_metric_tensor((2, 3), origin, axis, np.deg2rad(deg))
    out = capsys.readouterr().out
    assert out.count("null condition violated") == 4


def _photons_with_histories():
    from excalibur_tool_gb300.photon.photon import Photon
    from excalibur_tool_gb300.photon.photons import Photons

    ph = Photons(None)
    rng = np.random.default_rng(8)
    for i, (n_rows, width) in enumerate(((3, 8), (5, 14), (0, 14))):
        p = Photon(rng.standard_normal(4), rng.standard_normal(4), weight=0.5 + i)
        for k in range(n_rows):
            p.history.append(rng.standard_normal(8 if k == 0 else width))
        ph.add_photon(p)
    return ph


def _same_photons(a, b):
    assert len(a) == len(b)
    for p, q in zip(a, b):
        assert np.array_equal(p.x, q.x) and np.array_equal(p.u, q.u) and p.weight == q.weight
        assert len(p.history.states) == len(q.history.states)
        for r, s in zip(p.history.states, q.history.states):
            assert np.array_equal(r, s)


def test_binary_round_trip(tmp_path):
    """save_to_binary / load_from_binary (photons.py:713-780): weights, x, u and ragged history rows."""
    from excalibur_tool_gb300.photon.photons import Photons

    ph = _photons_with_histories()
    path = str(tmp_path / "photons.npz")
    ph.save_to_binary(path)
    back = Photons(None)
    back.load_from_binary(path)
    _same_photons(ph, back)


def test_load_binary_in_the_reference_layout(tmp_path):
    """A file as the reference's writer lays it out (n_photons, and photon_data as a list of dicts
    stored by numpy.savez_compressed) loads."""
    from excalibur_tool_gb300.photon.photons import Photons

    rows = [np.arange(8.0), np.arange(14.0)]
    path = str(tmp_path / "ref.npz")
    np.savez_compressed(path, **{"n_photons": 1, "photon_data": [
        {"weight": 2.0, "initial_position": np.ones(4), "initial_velocity": -np.ones(4), "history_states": rows}]})
    ph = Photons(None)
    ph.load_from_binary(path)
    assert len(ph) == 1 and ph[0].weight == 2.0
    assert np.array_equal(ph[0].x, np.ones(4)) and np.array_equal(ph[0].u, -np.ones(4))
    assert all(np.array_equal(a, b) for a, b in zip(ph[0].history.states, rows))


def test_update_quantities_all():
    ph = _photons_with_histories()
    ph.update_quantities_all(lambda x: np.array([x[0], 2 * x[1]]))
    for p in ph:
        assert np.array_equal(p.quantities, [p.x[0], 2 * p.x[1]])


def test_hdf5_round_trip(tmp_path):
    """save_all_histories / load_from_hdf5 (photons.py:782-910): the runners' per-photon datasets."""
    h5py = pytest.importorskip("h5py")
    from excalibur_tool_gb300.photon.photons import Photons

    ph = _photons_with_histories()
    path = str(tmp_path / "h.h5")
    ph.save_all_histories(path)
    with h5py.File(path, "r") as f:
        assert int(f.attrs["n_photons"]) == 3
        assert f["photon_1_states"].shape == (5, 14) and f["photon_2_states"].shape == (0,)
        assert list(f["photon_info"]["n_states"]) == [3, 5, 0]
    back = Photons(None)
    back.load_from_hdf5(path)
    assert len(back) == 3
    for p, q in zip(ph, back):
        assert p.weight == q.weight
        for r, s in zip(p.history.states, q.history.states):
            assert np.array_equal(r, s)
        if p.history.states:
            assert np.array_equal(q.x, p.history.states[0][:4])


def test_hdf5_needs_h5py(tmp_path):
    """Without h5py the HDF5 calls raise RuntimeError, as the reference's do."""
    try:
        import h5py  # noqa: F401
        pytest.skip("h5py is importable")
    except ImportError:
        pass
    ph = _photons_with_histories()
    with pytest.raises(RuntimeError):
        ph.save_all_histories(str(tmp_path / "h.h5"))
    with pytest.raises(RuntimeError):
        ph.load_from_hdf5(str(tmp_path / "h.h5"))


def _oracle_finish(spacetime):
    """Photons._finish with the oracle's null-condition solve in place of the device's."""

    def finish(self, origins, u_spatial, sign=-1.0):
        s = np.zeros((len(u_spatial), 8))
        s[:, :4] = origins
        s[:, 5:8] = u_spatial
        out, status = O.null_init(spacetime, s, sign)
        assert (status == 0).all()
        self._append_batch(out)
        return out

    return finish


@pytest.mark.parametrize("name", ["flrw", "schw"])
def test_impact_parameter_bins(monkeypatch, name):
    """generate_impact_parameter_bins (photons.py:570-701) against the reference's states, bit for
    bit: 3 FLRW annuli of 5 photons (seed 3) from a cartesian origin, 2 Schwarzschild annuli of 4
    (seed 0) from a spherical one (screen points converted with the reference's scalar r)."""
    from excalibur_tool_gb300.photon.photons import Photons

    g = golden("generators.npz")
    st, origin, _, _ = _cases(g)[name]
    if name == "flrw":
        axis, edges, n, seed = [1.0, 0.2, 0.1], np.linspace(0.1, 2.0, 4) * ONE_MPC, 5, 3
    else:
        obs = np.array([0.01, 0.01, 0.01]) * 1e3 * ONE_MPC
        axis, edges, n, seed = g["schw_center"] - obs, np.linspace(0.5, 10, 3) * ONE_MPC, 4, 0
    monkeypatch.setattr(Photons, "_finish", _oracle_finish(st))
    out = Photons(None).generate_impact_parameter_bins(origin, axis, edges, n, seed=seed)
    assert np.array_equal(out, g[f"{name}_bins"])


def test_cone_random_follows_numpy_global_stream(monkeypatch):
    """generate_cone_random without a seed (photons.py:33-156) draws theta, then phi, photon after
    photon, from numpy's global stream: after np.random.seed(17) its 25 photons are the
    reference's (u^0 > 0), within the cone grid's ulp of direction."""
    from excalibur_tool_gb300.photon.photons import Photons

    g = golden("generators.npz")
    st, origin, axis, deg = _cases(g)["flrw"]
    monkeypatch.setattr(Photons, "_finish", _oracle_finish(st))
    state = np.random.get_state()
    try:
        np.random.seed(17)
        out = Photons(None).generate_cone_random(25, origin, axis, np.deg2rad(deg), direction_basis="cartesian")
    finally:
        np.random.set_state(state)
    want = g["flrw_cone_random"]
    assert (out[:, 4] > 0).all()
    _check("flrw", out, want)
