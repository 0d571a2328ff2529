"""Comparison runner (Schwarzschild vs FLRW) on the CPU: geometry, potential, the analyzer's
statistics and the oracle's traces against the reference's own run of sweep job 1
(tests/golden/compare_job1.npz, written by make_golden.py from the reference's runner and
analyzer), and against the reference's committed per-run table of that job (produced on the
author's machine with numba's fastmath)."""
import hashlib

import numpy as np
import pytest

from conftest import golden
from helpers import rel_err
from excalibur_tool_gb300.runners import analyze as A
from excalibur_tool_gb300.runners import compare as R


def job1_config():
    g = golden("compare_job1.npz")
    argv = [str(a) for a in g["argv"]]
    opt = dict(zip(argv[0::2], argv[1::2]))
    return R.run_config(mass_msun=float(opt["--mass-msun"]), distance_mpc=float(opt["--distance-mpc"]),
                        flrw_grid_N=int(opt["--flrw-grid-N"]), record_every=int(opt["--record-every"]),
                        n_photons=int(opt["--n-photons"]), cone_angle_deg=float(opt["--cone-angle-deg"]),
                        sampling=opt["--sampling"], progress_every=0, static="--static" in argv,
                        flrw_local_coords="--flrw-local-coords" in argv)


def test_geometry_matches_runner():
    from excalibur_tool_gb300.core.constants import one_Mpc

    cfg = job1_config()
    geo = R.geometry(cfg)
    g = golden("compare_job1.npz")
    assert geo.clamped and geo.obs_to_lens_distance / one_Mpc == pytest.approx(500.0 - 1000.0 / 128)  # "D from 500 to 492"
    assert geo.n_steps == 378                                  # "Overriding n_steps 5000 -> 378"
    assert geo.dlambda == 268039388119658.22                   # printed by the reference runner
    assert np.array_equal(geo.lens_center, g["lens_center"])
    assert int(g["n_records"]) == 378 // cfg.record_every + 3  # initial + every 4th step + final


def test_potential_bit_identical():
    cfg = job1_config()
    g = golden("compare_job1.npz")
    phi = R.flrw_potential(cfg, R.geometry(cfg))
    assert tuple(phi.shape) == tuple(g["phi_shape"])
    assert hashlib.sha256(phi.tobytes()).hexdigest() == str(g["phi_sha256"])


def test_stats_bit_identical_to_reference_analyzer():
    g = golden("compare_job1.npz")
    k = g["keep"]
    s = A.trajectory_stats(g["schw_traj"], g["lens_center"], is_spherical=True).table()
    f = A.trajectory_stats(g["flrw_traj"], g["lens_center"], is_spherical=False).table()
    assert np.array_equal(s, g["schw_stats"][k], equal_nan=True)
    assert np.array_equal(f, g["flrw_stats"][k], equal_nan=True)


def test_stats_edge_cases():
    # an empty (failed) photon padded with NaN rows, a single record, a photon at rest
    tr = np.full((3, 4, 14), np.nan)
    tr[1, 0] = np.arange(14.0)
    tr[2, :, :] = 1.0
    st = A.trajectory_stats(tr, np.zeros(3), is_spherical=False)
    assert st.path_length[0] == 0.0 and np.isnan(st.min_r[0]) and st.bending_angle_rad[0] == 0.0
    assert st.path_length[1] == 0.0 and st.bending_angle_rad[1] == 0.0
    assert st.path_length[2] == 0.0 and st.bending_angle_rad[2] == 0.0
    assert list(st.n_records) == [4, 4, 4]
    one = A.trajectory_stats(tr[:, :1], None, is_spherical=False)
    assert np.all(np.isnan(one.path_length))


def _oracle_leg(cfg, geo, states, kind, phi=None, dt_bounds=None):
    """The oracle's records [n, n_rec, 12] and statuses of one runner leg; `dt_bounds` =
    (dt_min, dt_max) of the leg (default both |dlambda|, the fixed-step integrators' bounds)."""
    from excalibur_tool_gb300.trace import TraceConfig
    from oracle import oracle as O
    from oracle.oracle import FieldSpec, Spacetime

    if kind == "schwarzschild":
        st = Spacetime(kind="schwarzschild", mass=cfg.mass, radius=cfg.radius, center=tuple(geo.lens_center),
                       analytical=True)
        shift = None
    else:
        d = cfg.flrw_grid_size / cfg.flrw_grid_N
        shift = geo.observer if cfg.flrw_local_coords else None
        st = Spacetime(kind="flrw", cosmology="static",
                       fields=[FieldSpec(phi, (d, d, d), (0.0, 0.0, 0.0), "periodic",
                                         shift=tuple(shift) if shift is not None else (0.0, 0.0, 0.0))])
    dl = geo.dlambda
    dt_min, dt_max = dt_bounds if dt_bounds is not None else (abs(dl), abs(dl))
    tc = TraceConfig(stepper=cfg.integrator, dt=dl, dt_min=dt_min, dt_max=dt_max, max_steps=geo.n_steps,
                     record_every=cfg.record_every, renormalize_every=cfg.renormalize_every, observables=False)
    r = O.trace(st, states, tc, threads=4)
    tr = r.records[:, : int(r.n_records.max())].copy()
    if shift is not None:
        tr[..., 1:4] += shift
    return tr, r.status


@pytest.fixture(scope="module")
def oracle_job1():
    cfg = job1_config()
    geo = R.geometry(cfg)
    g = golden("compare_job1.npz")
    s_tr, s_st = _oracle_leg(cfg, geo, g["schw_init"], "schwarzschild")
    f_tr, f_st = _oracle_leg(cfg, geo, g["flrw_init"], "flrw", R.flrw_potential(cfg, geo))
    s = A.trajectory_stats(s_tr, geo.lens_center, is_spherical=True).table()
    f = A.trajectory_stats(f_tr, geo.lens_center, is_spherical=False).table()
    return dict(s=s, f=f, s_status=s_st, f_status=f_st, s_tr=s_tr, f_tr=f_tr)


def test_oracle_reproduces_reference_run(oracle_job1):
    """The C oracle, fed the runner's initial states, against the reference's own run."""
    g = golden("compare_job1.npz")
    o = oracle_job1
    assert np.all(o["s_status"] == 0) and np.all(o["f_status"] == 0)
    # FLRW leg: bit-identical records, so identical statistics
    assert np.array_equal(o["f_tr"][g["keep"]], g["flrw_traj"], equal_nan=True)
    assert np.array_equal(o["f"], g["flrw_stats"], equal_nan=True)
    # Schwarzschild leg: the same libm sin/cos as numpy, so bit-identical as well
    assert np.array_equal(o["s_tr"][g["keep"]], g["schw_traj"], equal_nan=True)
    assert np.array_equal(o["s"], g["schw_stats"], equal_nan=True)


def test_reference_table_of_job1(oracle_job1):
    """Against the committed per-run table (numba fastmath on the author's machine): FLRW path
    length and min_r are bit-identical; bend angles agree to arccos's conditioning."""
    g = golden("compare_job1.npz")
    csv = g["csv_author"]
    o = oracle_job1
    assert np.array_equal(csv[:, 1], o["s"][:, 0]) and np.array_equal(csv[:, 5], o["f"][:, 0])
    assert np.array_equal(csv[:, 6], o["f"][:, 2])
    assert np.array_equal(csv[:, 7], o["f"][:, 3])
    assert np.abs(csv[:, 8] - o["f"][:, 5]).max() <= 1e-8
    assert rel_err(csv[:, 2], o["s"][:, 2]).max() <= 1e-13
    assert rel_err(csv[:, 3], o["s"][:, 3], floor=1e20).max() <= 1e-13
    assert np.abs(csv[:, 4] - o["s"][:, 5]).max() <= 1e-7


def test_per_run_csv_layout(tmp_path):
    g = golden("compare_job1.npz")
    k = g["keep"]
    s = A.trajectory_stats(g["schw_traj"], g["lens_center"], is_spherical=True)
    f = A.trajectory_stats(g["flrw_traj"], g["lens_center"], is_spherical=False)
    p = A.write_per_run_csv(str(tmp_path / "per_run" / "job_00001.csv"), s, f)
    rows = np.loadtxt(p, delimiter=",", skiprows=1)
    with open(p) as fp:
        assert fp.readline().strip().split(",") == A.CSV_HEADER
    csv = g["csv_author"][k]
    assert np.array_equal(rows[:, 6:8], csv[:, 6:8])   # FLRW path, min_r as the reference wrote them
    assert np.array_equal(rows[:, 9], rows[:, 8] - rows[:, 4])


# ------------------------------------------------------------------ sweep manifests
def _manifest_runs():
    import os
    from conftest import GOLDEN

    with open(os.path.join(GOLDEN, "manifest_args.txt")) as f:
        for line in f:
            name, *argv = line.split()
            yield name, argv, os.path.join(GOLDEN, name)


def test_manifest_matches_reference_writer(tmp_path):
    from excalibur_tool_gb300.runners import sweep as S

    for name, argv, ref in _manifest_runs():
        out = tmp_path / name
        S.manifest_main(["--out", str(out), *argv])
        assert out.read_text() == open(ref).read(), name


def test_manifest_rows_to_runner_configs():
    from excalibur_tool_gb300.core.constants import one_Mpc, one_Msun
    from excalibur_tool_gb300.runners import sweep as S

    runs = {name: path for name, _, path in _manifest_runs()}
    cone = S.read_jobs(runs["manifest_cone.csv"])
    assert [j.jobid for j in cone] == list(range(16)) and [j.seed for j in cone] == list(range(7, 23))
    assert cone[1].integrator == "leapfrog4" and cone[0].b_nbins == 0
    cfg = S.job_config(cone[3])
    assert cfg.sampling == "cone" and cfg.n_photons == 100 and cfg.cone_angle_deg == 5.0
    assert cfg.mass == 1e13 * one_Msun and cfg.obs_to_lens_distance == 300.0 * one_Mpc
    assert cfg.flrw_grid_N == 128 and cfg.static and cfg.flrw_local_coords and cfg.record_every == 4
    imp = S.read_jobs(runs["manifest_impact.csv"])
    assert len(imp) == 16 and imp[5].bin_id == 1 and imp[5].radius_mpc == 3.0
    assert imp[5].b_nbins == 1 and imp[5].b_nperbin == 30 and imp[5].b_min_mpc == 1.0
    # make_manifest writes no "sampling" column and run_one_job reads a missing one as "cone"
    # (run_one_job.py:75), so the reference runs impact rows as 200-photon cone jobs; kept.
    cfg = S.job_config(imp[5])
    assert cfg.sampling == "cone" and cfg.n_photons == 200 and cfg.cone_angle_deg == 10.0
    assert not cfg.static and cfg.record_every == 8 and cfg.radius == 3.0 * one_Mpc
    # a row that does say "impact" gets the bin, as run_one_job's impact branch passes it
    import dataclasses
    cfg = S.job_config(dataclasses.replace(imp[5], sampling="impact"))
    assert cfg.sampling == "impact" and cfg.b_nbins == 1 and cfg.b_nperbin == 30 and cfg.n_photons == 30
    assert cfg.b_min == 1.0 * one_Mpc and cfg.b_max == 1.5 * one_Mpc
    geo = R.geometry(cfg)
    assert geo.n_photons_effective == 30 and len(geo.b_edges) == 2
    with pytest.raises(SystemExit):
        S.read_job(runs["manifest_impact.csv"], 99)


def test_empty_inputs():
    from excalibur_tool_gb300.runners import sweep as S

    st = A.trajectory_stats(np.zeros((0, 5, 14)), np.zeros(3), is_spherical=False)
    assert st.table().shape == (0, 8)
    st = A.trajectory_stats(np.zeros((0, 5, 12)), np.zeros(3), is_spherical=True)
    assert st.table().shape == (0, 8)
    assert S.run_jobs([]) == {}
