"""Comparison runner and sweep driver on the GPU, against the reference's own run of sweep
job 1 (tests/golden/compare_job1.npz), its committed per-run table, and the oracle."""
import hashlib

import numpy as np
import pytest

from conftest import golden
from helpers import rel_err
from test_compare_runner import _oracle_leg, job1_config
from excalibur_tool_gb300 import _native as N
from excalibur_tool_gb300.runners import compare as R

pytestmark = pytest.mark.gpu


def test_device_potential_bit_identical(cuda):
    from excalibur_tool_gb300.core.constants import one_Mpc, one_Msun
    from excalibur_tool_gb300.objects.spherical_mass import spherical_mass

    cfg = job1_config()
    geo = R.geometry(cfg)
    g = golden("compare_job1.npz")
    phi = R.flrw_potential(cfg, geo, device=cuda).cpu().numpy()
    assert hashlib.sha256(phi.tobytes()).hexdigest() == str(g["phi_sha256"])
    # an uneven grid with an offset origin, the centre on a node (the r == 0 branch) and
    # nodes both inside and outside the radius
    shape, sp, org = (17, 9, 33), (2.5 * one_Mpc, 4.0 * one_Mpc, 1.25 * one_Mpc), (-10 * one_Mpc, 3 * one_Mpc, 0.0)
    centre = np.array([org[0] + 6 * sp[0], org[1] + 4 * sp[1], org[2] + 20 * sp[2]])
    lens = spherical_mass(3e14 * one_Msun, 6 * one_Mpc, centre)
    dev = lens.potential_grid(shape, sp, org, device=cuda).cpu().numpy()
    axes = [np.linspace(o, o + n * s, n, endpoint=False) for o, n, s in zip(org, shape, sp)]
    host = lens.potential(*np.meshgrid(*axes, indexing="ij"))
    assert np.array_equal(dev, host)


def test_shifted_interpolator_queries_x_plus_shift(cuda):
    from excalibur_tool_gb300.grid.grid import Grid
    from excalibur_tool_gb300.grid.interpolator import Interpolator
    from excalibur_tool_gb300.grid.interpolator_4d_fast import InterpolatorFast, shifted_interpolator

    rng = np.random.default_rng(3)
    n, h = 24, 3.7e22
    grid = Grid((n, n, n), (h, h, h), (0.0, 0.0, 0.0))
    grid.add_field("Phi", rng.standard_normal((n, n, n)) * 1e10)
    shift = np.array([2.3e23, 4.1e23, -1.7e23])
    pts = rng.uniform(-0.2 * n * h, 1.2 * n * h, (500, 3)) - shift
    for base in (InterpolatorFast(grid), InterpolatorFast(grid, boundary="clamp"), Interpolator(grid)):
        sh = shifted_interpolator(base, shift)
        a = sh.evaluate(pts)
        b = base.evaluate(pts + shift)          # the reference wrapper: x + shift on the host
        for u, v in zip(a, b):
            assert np.array_equal(u.cpu().numpy(), v.cpu().numpy(), equal_nan=True)
        assert base.shift is None               # the copy carries the shift, the base does not


@pytest.fixture(scope="module")
def job1_gpu(cuda):
    return R.run(job1_config())


def test_job1_matches_reference_run(job1_gpu):
    """The whole runner on the GPU against the reference's run of the same job: FLRW leg
    bit-identical; Schwarzschild leg to CUDA's sin/cos (path length and min_r 1e-13 relative,
    bend angles to arccos's resolution near 1: the cosine moves in steps of 1.1e-16 there, so
    the angle in steps of sqrt(2 * 1.1e-16) = 1.5e-8 rad)."""
    g = golden("compare_job1.npz")
    s, f = job1_gpu.schwarzschild, job1_gpu.flrw
    assert s.trajectories.shape == (381, 97, 12) and f.trajectories.shape == (381, 97, 14)
    assert np.all(s.status == 0) and np.all(f.status == 0)
    assert np.array_equal(f.stats.table(), g["flrw_stats"], equal_nan=True)
    assert np.array_equal(f.trajectories[g["keep"]], g["flrw_traj"], equal_nan=True)
    st, ref = s.stats.table(), g["schw_stats"]
    assert np.array_equal(st[:, 0], ref[:, 0])
    assert rel_err(st[:, 2], ref[:, 2]).max() <= 1e-13
    assert rel_err(st[:, 3], ref[:, 3], floor=1e20).max() <= 1e-12
    assert np.abs(st[:, 5] - ref[:, 5]).max() <= 5e-8
    assert job1_gpu.error is None
    csv = g["csv_author"]
    assert np.array_equal(csv[:, 6], f.stats.path_length) and np.array_equal(csv[:, 7], f.stats.min_r)
    assert np.abs(csv[:, 8] - f.stats.bending_angle_rad).max() <= 1e-8


def test_job1_initial_states_and_oracle(cuda):
    """The GPU-generated initial states against the runner's, and the GPU traces against the
    oracle fed the same states."""
    import torch

    from excalibur_tool_gb300.trace import trace_batch

    cfg = job1_config()
    geo = R.geometry(cfg)
    g = golden("compare_job1.npz")
    sm, ss, dmin, dmax = R.schwarzschild_setup(cfg, geo)
    fm, fs, shift = R.flrw_setup(cfg, geo)
    ss_h, fs_h = ss.cpu().numpy(), fs.cpu().numpy()
    assert rel_err(ss_h, g["schw_init"]).max() <= 4e-16
    assert rel_err(fs_h, g["flrw_init"], floor=1e-300).max() <= 4e-16
    f_res = trace_batch(fm, fs, R.trace_config(cfg, geo, abs(geo.dlambda), abs(geo.dlambda)))
    s_res = trace_batch(sm, ss, R.trace_config(cfg, geo, dmin, dmax))
    torch.cuda.synchronize()
    f_tr, _ = R.leg_trajectories(f_res, shift, empty_failed=False, fail_on_error=True, label="FLRW")
    s_tr, _ = R.leg_trajectories(s_res, None, empty_failed=True, fail_on_error=False, label="S")
    of, _ = _oracle_leg(cfg, geo, fs_h, "flrw", R.flrw_potential(cfg, geo))
    os_, _ = _oracle_leg(cfg, geo, ss_h, "schwarzschild")
    assert np.array_equal(f_tr, of, equal_nan=True)
    assert _scaled_err(s_tr, os_) <= 1e-12


def _scaled_err(a, b):
    """max |a - b| per column over the column's largest |b| (angles near 0, velocities near 0)."""
    scale = np.nanmax(np.abs(b), axis=(0, 1))
    return float(np.nanmax(np.abs(a - b) / np.where(scale > 0, scale, 1.0)))


def _legs_equal(a, b):
    for leg in ("schwarzschild", "flrw"):
        la, lb = getattr(a, leg), getattr(b, leg)
        assert np.array_equal(la.trajectories, lb.trajectories, equal_nan=True)
        assert np.array_equal(la.status, lb.status)
        if la.stats is None:
            assert lb.stats is None
        else:
            assert np.array_equal(la.stats.table(), lb.stats.table(), equal_nan=True)
    assert a.error == b.error


def test_sweep_batched_equals_row_by_row(cuda, tmp_path):
    """Rows sharing a launch give the tables they give alone, bit for bit; the CSVs land where
    run_one_job puts them. The manifest's Leapfrog4 rows lose every Schwarzschild photon to a
    non-finite state (as the oracle does, below), so those rows end without a table."""
    import os

    from conftest import GOLDEN
    from excalibur_tool_gb300.runners import sweep as S

    manifest = os.path.join(GOLDEN, "manifest_cone.csv")
    jobs = S.read_jobs(manifest)
    grouped = S.run_jobs(jobs)
    alone = S.run_jobs(jobs, max_fields=1, streams=1)
    assert sorted(grouped) == list(range(16))
    for j in jobs:
        a = grouped[j.jobid]
        _legs_equal(a, alone[j.jobid])
        assert a.flrw.trajectories.shape[0] == 91                # 10 x 10 cone grid minus 9 duplicate axis rays
        assert (a.error is not None) == (j.integrator == "leapfrog4")
    paths = S.run_sweep(manifest, [2, 4, 5], results=str(tmp_path))
    assert [os.path.basename(p) for p in paths] == ["job_00002.csv", "job_00004.csv"]
    rows = np.loadtxt(paths[1], delimiter=",", skiprows=1)
    st = grouped[4]
    assert np.array_equal(rows[:, 6], st.flrw.stats.path_length)
    assert np.array_equal(rows[:, 4], st.schwarzschild.stats.bending_angle_rad)


def test_sweep_rows_match_oracle(cuda):
    """One RK4 and one Leapfrog4 row of the cone manifest against the oracle, both legs."""
    import os

    from conftest import GOLDEN
    from excalibur_tool_gb300.runners import sweep as S

    jobs = S.read_jobs(os.path.join(GOLDEN, "manifest_cone.csv"))
    got = S.run_jobs([jobs[2], jobs[3]])
    for j in (jobs[2], jobs[3]):
        cfg = S.job_config(j)
        geo = R.geometry(cfg)
        _, fs, _ = R.flrw_setup(cfg, geo)
        _, ss, _, _ = R.schwarzschild_setup(cfg, geo)
        of, _ = _oracle_leg(cfg, geo, fs.cpu().numpy(), "flrw", R.flrw_potential(cfg, geo))
        assert np.array_equal(got[j.jobid].flrw.trajectories, of, equal_nan=True), j.integrator
        os_, ost = _oracle_leg(cfg, geo, ss.cpu().numpy(), "schwarzschild")
        assert np.array_equal(got[j.jobid].schwarzschild.status, ost)
        if j.integrator == "rk4":
            ok = ost == 0
            assert ok.sum() == 90
            gs = got[j.jobid].schwarzschild.trajectories
            assert _scaled_err(gs[ok], os_[ok][:, : gs.shape[1]]) <= 1e-12
        else:
            assert np.all(ost == 6) and got[j.jobid].error.startswith("every photon of the Schwarzschild leg")


def test_impact_runner_matches_oracle(cuda):
    """The impact-parameter runner (sampling "impact": impact-parameter bins, seed 0; a photon
    that fails keeps its history up to the failure) against the oracle fed the same states."""
    cfg = R.run_config(mass_msun=1e14, distance_mpc=300.0, flrw_grid_N=64, record_every=8, sampling="impact",
                       b_min_mpc=0.5, b_max_mpc=3.0, b_nbins=3, b_nperbin=20, n_photons=20, static=True,
                       flrw_local_coords=True, progress_every=0)
    geo = R.geometry(cfg)
    res = R.run(cfg)
    assert res.flrw.trajectories.shape[0] == 60 and res.schwarzschild.trajectories.shape[0] == 60
    _, fs, _ = R.flrw_setup(cfg, geo, impact_runner=True)
    _, ss, _, _ = R.schwarzschild_setup(cfg, geo, impact_runner=True)
    of, fst = _oracle_leg(cfg, geo, fs.cpu().numpy(), "flrw", R.flrw_potential(cfg, geo))
    assert np.array_equal(res.flrw.trajectories, of, equal_nan=True) and np.all(fst == 0)
    os_, sst = _oracle_leg(cfg, geo, ss.cpu().numpy(), "schwarzschild")
    assert np.array_equal(res.schwarzschild.status, sst)
    ok = sst == 0
    gs = res.schwarzschild.trajectories
    if ok.any():
        assert _scaled_err(gs[ok], os_[ok][:, : gs.shape[1]]) <= 1e-12
    # failed photons keep their records up to the failure (not emptied, unlike the plain runner);
    # the state columns of the first record are finite (its quantity columns lag one record)
    for i in np.flatnonzero(~ok):
        assert np.isfinite(gs[i, 0, :8]).all()


def test_rk45_row_matches_oracle(cuda):
    """A manifest row run with the runner's RK45 (rtol 1e-9, atol 1e-13; the Schwarzschild step
    free in [|dl| / 1e6, |dl|], the FLRW step pinned to |dl|) against the oracle fed the same
    states and bounds. On this row the reference's controller accepts no trial step, down to the
    floor: every photon of both legs stops at the 10,000-iteration cap with its initial state,
    here and in the oracle alike. Statuses and accepted steps agree; records to a few ulps on
    the FLRW leg and to 1e-6 (1e-10 on most photons) on the Schwarzschild one, the tolerances
    a run that does take steps needs (one RK45 step differs from the oracle's by <= 4.5e-16; a
    free step control can turn a sin/cos ulp into another step sequence)."""
    import dataclasses
    import os

    from conftest import GOLDEN
    from excalibur_tool_gb300.runners import sweep as S

    job = dataclasses.replace(S.read_jobs(os.path.join(GOLDEN, "manifest_cone.csv"))[0], integrator="rk45")
    got = S.run_jobs([job])[job.jobid]
    cfg = S.job_config(job)
    geo = R.geometry(cfg)
    _, fs, _ = R.flrw_setup(cfg, geo)
    _, ss, dmin, dmax = R.schwarzschild_setup(cfg, geo)
    assert dmin == abs(geo.dlambda) / 1e6 and dmax == abs(geo.dlambda)
    of, fst = _oracle_leg(cfg, geo, fs.cpu().numpy(), "flrw", R.flrw_potential(cfg, geo))
    assert np.array_equal(got.flrw.status, fst)
    gf = got.flrw.trajectories
    assert gf.shape == of.shape and np.array_equal(np.isnan(gf), np.isnan(of))
    assert _scaled_err(gf, of) <= 1e-13
    os_, sst = _oracle_leg(cfg, geo, ss.cpu().numpy(), "schwarzschild", dt_bounds=(dmin, dmax))
    assert np.array_equal(got.schwarzschild.status, sst)
    for leg in (got.flrw, got.schwarzschild):
        assert np.all(leg.status == N.PH_MAX_ITER) and np.all(leg.n_steps == 0)
    failed = np.isin(sst, (N.PH_HORIZON, N.PH_NONFINITE, N.PH_OUTSIDE_GRID))
    if failed.all():
        assert got.error.startswith("every photon of the Schwarzschild leg")
        return
    ok = np.flatnonzero(~failed)
    gs = got.schwarzschild.trajectories
    n = min(gs.shape[1], os_.shape[1])
    scale = np.nanmax(np.abs(os_[ok][:, :n]), axis=(0, 1))
    scale = np.where(scale > 0, scale, 1.0)
    per_photon = np.array([np.nanmax(np.abs(gs[i, :n] - os_[i, :n]) / scale) for i in ok])
    assert per_photon.max() <= 1e-6 and (per_photon <= 1e-10).mean() >= 0.9
