"""GPU parity: the CUDA tracer (through the C ABI) against the reference's
golden vectors and against the C oracle on identical seeded inputs.

Tolerances (the parity target: 1e-12 relative on final state and observables):
* FLRW, parity build ("fp64"): the reference's IEEE operation order with no
  FMA contraction -> bit-identical interpolation/RHS/RK4. The one exception is
  x**3 in adot: the library's correctly rounded double-double cube, where the
  reference's libm pow misrounds 0.09 % of near-halfway cubes by one ulp. The
  oracle run with the same cube (oracle.power_mode("dd")) must therefore equal
  the GPU bit for bit -- states, statuses, step counts and every observable --
  which shows that the cube is the only difference; against the reference's
  arithmetic (the oracle's default libm mode, and the goldens) the tests hold
  1e-12 (1e-13 to 1e-14 where the runs are short).
* Schwarzschild: CUDA's sin/cos differ from glibc's by <= 1-2 ulp, so states
  agree to ~1e-15 per step; well-conditioned rays stay within 1e-12.
* fp64_fast build: FMA contraction and reciprocals; checked at 1e-11.
"""
import numpy as np
import pytest

from conftest import golden
from helpers import gpu_metric, gpu_trace, lcdm_spacetime, rel_err, schw_spacetime
from excalibur_tool_gb300 import _native as N
from excalibur_tool_gb300.trace import TraceConfig
from oracle import oracle as O
from oracle.oracle import FieldSpec

pytestmark = pytest.mark.gpu


def _interp_gpu(field, pts4):
    import torch
    from excalibur_tool_gb300.grid.grid import Grid
    from excalibur_tool_gb300.grid.interpolator_4d_fast import InterpolatorFast

    g = Grid(field.data.shape, field.spacing, field.origin)
    g.add_field("Phi", field.data)
    ip = InterpolatorFast(g, boundary=field.boundary)
    val, grad, dtd, status = ip.evaluate(pts4, "Phi")
    torch.cuda.synchronize()
    out = np.concatenate([val.cpu().numpy()[:, None], grad.cpu().numpy(), dtd.cpu().numpy()[:, None]], axis=1)
    return out, status.cpu().numpy()


@pytest.mark.parametrize("mode", ["periodic", "clamp", "error"])
def test_interp3d_matches_reference(cuda, mode):
    g = golden("interp.npz")
    f = FieldSpec(g["f3"], tuple(g["f3_spacing"]), tuple(g["f3_origin"]), mode)
    pts = np.concatenate([g["pts3"], np.zeros((len(g["pts3"]), 1))], axis=1)
    out, status = _interp_gpu(f, pts)
    ok = g[f"ok3_{mode}"].astype(bool)
    assert np.array_equal(status == 0, ok)
    assert np.array_equal(out[ok], g[f"out3_{mode}"][ok])


@pytest.mark.parametrize("mode", ["periodic", "clamp", "error"])
def test_interp4d_matches_reference(cuda, mode):
    g = golden("interp.npz")
    f = FieldSpec(g["f4"], tuple(g["f4_spacing"]), tuple(g["f4_origin"]), mode)
    out, status = _interp_gpu(f, g["pts4"])
    ok = g[f"ok4_{mode}"].astype(bool)
    assert np.array_equal(status == 0, ok)
    assert np.array_equal(out[ok], g[f"out4_{mode}"][ok])


def test_cosmology_matches_reference(cuda):
    from helpers import golden_lcdm

    cz = golden("cosmology.npz")
    lc = golden_lcdm()
    a = lc.a_of_eta(cz["etas"])
    adot = lc.adot_of_eta(cz["etas"])
    assert np.array_equal(a, cz["a"])
    # adot = a^2 H0 E(z): E sums Omega_m (1+z)^3 (libm pow in the reference) -> <= 2 ulp
    assert rel_err(adot, cz["adot"]).max() <= 4.5e-16
    # ... and the oracle with the library's cube gives the same bits
    with O.power_mode("dd"):
        a_o, adot_o = O.cosmology(lcdm_spacetime(np.zeros((4, 4, 4)), 1.0), cz["etas"])
    assert np.array_equal(a, a_o) and np.array_equal(adot, adot_o)


@pytest.mark.parametrize("variant,cosmo,analytical", [("lcdm_tensorial", "table", False),
                                                      ("lcdm_analytical", "table", True),
                                                      ("lcdm_fd", "table_fd", False),
                                                      ("static_tensorial", "static", False)])
@pytest.mark.parametrize("precision", ["fp64", "fp64_fast"])
def test_flrw_rhs_matches_reference(cuda, variant, cosmo, analytical, precision):
    from excalibur_tool_gb300._evaluate import geodesic_rhs

    g = golden("rhs.npz")
    spec = lcdm_spacetime(g["flrw_field"], float(g["flrw_box"]), cosmology=cosmo, analytical=analytical)
    m = gpu_metric(spec)
    out, st = geodesic_rhs(m, g["flrw_states"], precision=precision)
    out = out.cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    want = g[f"flrw_{variant}"]
    if precision == "fp64":
        # the analytic adot uses x**3 (libm pow in the reference): <= 1 ulp in rare cases
        assert rel_err(out, want).max() <= (0.0 if cosmo != "table" else 4.5e-16)
        with O.power_mode("dd"):
            o, ost = O.rhs(spec, g["flrw_states"])
        assert (ost == 0).all() and np.array_equal(out, o)
    else:
        # reciprocal constants + FMA: ulp-level; the finite-difference adot
        # (a(eta+h) - a(eta-h)) / 2h with h = 1e-6 eta amplifies a's ulps by ~1e6
        scale = np.abs(want).max(axis=0, keepdims=True)
        tol = 1e-10 if cosmo == "table_fd" else 1e-13
        assert (np.abs(out - want) / np.maximum(scale, 1e-300)).max() <= tol


@pytest.mark.parametrize("variant,analytical,free", [("analytical_free", True, True),
                                                     ("analytical_null", True, False),
                                                     ("tensorial", False, True)])
def test_schwarzschild_rhs_matches_reference(cuda, variant, analytical, free):
    from excalibur_tool_gb300._evaluate import geodesic_rhs

    g = golden("rhs.npz")
    M = float(g["schw_mass"])
    spec = schw_spacetime(M, 1.2 * 2 * 6.67430e-11 * M / 299792458 ** 2, analytical=analytical, free_time=free)
    out, st = geodesic_rhs(gpu_metric(spec), g["schw_states"])
    out = out.cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    want = g[f"schw_{variant}"]
    # CUDA sin/cos vs glibc: a few ulp, amplified by cancellation in du1 / du2
    scale = np.abs(want).max(axis=1, keepdims=True)
    assert (np.abs(out - want) / scale).max() <= 1e-14


def test_rk4_integrate_single_records(cuda):
    g = golden("integrate.npz")
    spec = lcdm_spacetime(g["field"], float(g["box"]))
    dt = float(g["dt"])
    for k in range(4):
        rec, ren, nsteps, _ = (int(v) for v in g["cases"][k])
        cfg = TraceConfig(stepper="rk4", dt=dt, dt_min=dt, dt_max=dt, max_steps=nsteps, record_every=rec,
                          renormalize_every=ren, observables=False, precision="fp64")
        r = gpu_trace(spec, g[f"case{k}_init"][None], cfg)
        assert r["status"][0] == 0
        want = g[f"case{k}_records"]
        got = r["records"][0, :r["n_records"][0]]
        assert got.shape == want.shape
        assert np.array_equal(np.isnan(got), np.isnan(want))
        both = ~np.isnan(want)
        assert rel_err(got[both], want[both]).max() <= 1e-14, k
        assert rel_err(r["state"][0], g[f"case{k}_final"]).max() <= 1e-14
        with O.power_mode("dd"):
            o = O.trace(spec, g[f"case{k}_init"][None], cfg)
        assert r["n_records"][0] == o.n_records[0]
        nr = int(o.n_records[0])
        assert np.array_equal(r["records"][0, :nr], o.records[0, :nr], equal_nan=True)
        assert np.array_equal(r["state"], o.state)


def test_rk45_integrate_single(cuda):
    g = golden("integrate.npz")
    spec = lcdm_spacetime(g["field"], float(g["box"]))
    rtol, atol, dmin, dmax = g["case4_tol"]
    dt = float(g["dt"])
    cfg = TraceConfig(stepper="rk45", dt=dt, dt_min=dmin, dt_max=dmax, rtol=rtol, atol=atol, max_steps=30,
                      record_every=1, observables=False)
    r = gpu_trace(spec, g["case4_init"][None], cfg)
    assert r["status"][0] == 0
    # reference y5 is a BLAS product; the step-size control amplifies its ulps (see test_oracle_golden)
    assert rel_err(r["state"][0], g["case4_final"]).max() <= 1e-12
    with O.power_mode("dd"):
        o = O.trace(spec, g["case4_init"][None], cfg)
    assert r["n_records"][0] == o.n_records[0]
    nr = int(o.n_records[0])
    assert np.array_equal(r["records"][0, :nr], o.records[0, :nr], equal_nan=True)
    assert np.array_equal(r["state"], o.state)


def test_leapfrog4_integrate_single(cuda):
    """integrate_single with the Leapfrog4 stepper from the reference's own run (40 fixed steps,
    record_every 1 and 3): the records and final state at the parity bar, and bit-identical to the
    oracle run with the library's correctly rounded cube."""
    g = golden("integrate_lf4.npz")
    spec = lcdm_spacetime(g["field"], float(g["box"]))
    dt = float(g["dt"])
    for k in range(2):
        cfg = TraceConfig(stepper="leapfrog4", dt=dt, dt_min=dt, dt_max=dt, max_steps=40,
                          record_every=int(g["record_every"][k]), observables=False, precision="fp64")
        r = gpu_trace(spec, g[f"case{k}_init"][None], cfg)
        assert r["status"][0] == 0
        want = g[f"case{k}_records"]
        got = r["records"][0, :r["n_records"][0]]
        assert got.shape == want.shape
        assert np.array_equal(np.isnan(got), np.isnan(want))
        both = ~np.isnan(want)
        assert rel_err(got[both], want[both]).max() <= 1e-14, k
        assert rel_err(r["state"][0], g[f"case{k}_final"]).max() <= 1e-14
        with O.power_mode("dd"):
            o = O.trace(spec, g[f"case{k}_init"][None], cfg)
        nr = int(o.n_records[0])
        assert r["n_records"][0] == nr
        assert np.array_equal(r["records"][0, :nr], o.records[0, :nr], equal_nan=True)
        assert np.array_equal(r["state"], o.state)


@pytest.mark.parametrize("name", ["lf4", "rk45", "rk4ren"])
def test_schw_steppers_integrate_single(cuda, name):
    """Six off-pole cone photons through the analytical Schwarzschild metric with
    integrate_single, from the reference's own run: Leapfrog4 (300 fixed steps, record_every 10)
    RK45 (80 iterations, record_every 2) and RK4 renormalised onto the null cone every 7 steps
    (300 steps, record_every 5) give the same records row for row: Leapfrog4 bit for bit, RK45 and
    the renormalised RK4 within the 1e-15 that the reference's BLAS-ordered tensordot and
    u_i g_ij u_j leave (measured on a GB300: 0.0, 4.3e-16 and 4.0e-16, the oracle's own figures)."""
    g = golden("schw_steppers.npz")
    spec = schw_spacetime(float(g["mass"]), float(g["radius"]))
    dl = float(g["dl"])
    if name == "lf4":
        cfg = TraceConfig(stepper="leapfrog4", dt=dl, dt_min=dl, dt_max=dl, max_steps=300,
                          record_every=10, observables=False, precision="fp64")
    elif name == "rk45":
        cfg = TraceConfig(stepper="rk45", dt=dl, dt_min=dl / 50, dt_max=dl, rtol=1e-4, atol=1e12,
                          max_steps=80, record_every=2, observables=False, precision="fp64")
    else:
        cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=300, record_every=5,
                          renormalize_every=7, observables=False, precision="fp64")
    r = gpu_trace(spec, g["states"], cfg)
    assert (r["status"] == 0).all()
    assert np.array_equal(r["n_records"], g[f"{name}_n_records"])
    worst = 0.0
    for i in range(len(g["states"])):
        want = g[f"{name}_records"][i, :g[f"{name}_n_records"][i]]
        got = r["records"][i, :r["n_records"][i]]
        assert np.array_equal(np.isnan(got), np.isnan(want))
        ok = ~np.isnan(want)
        worst = max(worst, rel_err(got[ok], want[ok]).max(),
                    rel_err(r["state"][i], g[f"{name}_final"][i]).max())
    assert worst <= (0.0 if name == "lf4" else 1e-15), worst


def test_steppers_match_oracle(cuda):
    """Single steps of every stepper, GPU vs oracle."""
    g = golden("steps.npz")
    spec = lcdm_spacetime(g["field"], float(g["box"]))
    dt = float(g["dt"])
    for stepper in ("rk4", "leapfrog4", "rk45"):
        cfg = TraceConfig(stepper=stepper, dt=dt, dt_min=dt / 100, dt_max=dt, max_steps=1, max_iter=1,
                          rtol=1e-3, atol=1e-3, observables=False)
        r = gpu_trace(spec, g["states"], cfg)
        o = O.trace(spec, g["states"], cfg)
        assert np.array_equal(r["status"], o.status)
        tol = 0.0 if stepper != "rk45" else 4.5e-16
        assert rel_err(r["state"], o.state).max() <= tol, stepper
        with O.power_mode("dd"):
            o = O.trace(spec, g["states"], cfg)
        assert np.array_equal(r["state"], o.state) and np.array_equal(r["dt"], o.dt), stepper


def test_schw_polar_subset_matches_reference(cuda):
    g = golden("schw_polar_1024.npz")
    spec = schw_spacetime(float(g["mass"]), float(g["radius"]))
    dl = float(g["dl"])
    sel = g["sel"]
    cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=2000, observables=False)
    r = gpu_trace(spec, g["states"][sel], cfg)
    failed = r["status"] >= N.PH_OUTSIDE_GRID
    assert np.array_equal(failed, g["failed"].astype(bool))
    ok = ~failed
    # rays that cross the spherical coordinate pole (phi_j = 0, pi) are ill-conditioned
    # in the reference itself (1-ulp input perturbation -> ~1e-10): compare them looser
    pole = np.isin(sel % 32, (0, 16))
    err = rel_err(r["state"], g["final"]).max(axis=1)
    assert err[ok & ~pole].max() <= 1e-12
    assert err[ok & pole].max() <= 1e-8


def test_flrw_patch_32_matches_reference(cuda):
    g = golden("flrw_patch_32.npz")
    box = float(g["box"])
    spec = lcdm_spacetime(g["field"], box)
    dl = float(g["dl"])
    cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=10000,
                      stop_box=((0, 0, 0), (box, box, box)))
    r = gpu_trace(spec, g["states"], cfg)
    assert (r["status"] == N.PH_LEFT_BOX).all()
    assert np.array_equal(r["n_steps"], g["n_steps"])
    assert rel_err(r["state"], g["final"]).max() <= 1e-13


def test_schw_polar_full_matches_oracle(cuda):
    g = golden("schw_polar_1024.npz")
    spec = schw_spacetime(float(g["mass"]), float(g["radius"]))
    dl = float(g["dl"])
    cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=2000, observables=True)
    r = gpu_trace(spec, g["states"], cfg)
    o = O.trace(spec, g["states"], cfg, threads=8)
    failed = o.status >= N.PH_OUTSIDE_GRID
    assert np.array_equal(r["status"] >= N.PH_OUTSIDE_GRID, failed)
    j = np.arange(1024) % 32
    pole = np.isin(j, (0, 16))
    good = ~failed & ~pole
    assert good.sum() > 900
    assert rel_err(r["state"][good], o.state[good]).max() <= 1e-12
    # observables: deflection inputs, path length and min r
    for col in ("path", "chord", "min_r", "v1x", "v1y", "v1z"):
        i = N.OBS_COLS.index(col)
        assert rel_err(r["obs"][good, i], o.obs[good, i], floor=1.0).max() <= 1e-12, col


def _flrw_patch_case(n_grid, n_side, seed=2, pick=None):
    from excalibur_tool_gb300.objects.fields import lens_plus_grf
    from excalibur_tool_gb300.core.constants import one_Mpc, one_Msun, c

    box = 1000 * one_Mpc
    lens = np.array([500.0, 500.0, 500.0]) * one_Mpc
    phi = lens_plus_grf(n_grid, box, 1e15 * one_Msun, 5 * one_Mpc, lens, seed=seed)
    spec = lcdm_spacetime(phi, box)
    cz = golden("cosmology.npz")
    half = np.tan(np.deg2rad(5.0))
    t = (np.arange(n_side) + 0.5) / n_side * 2 - 1
    A, B = np.meshgrid(t, t, indexing="ij")
    d = np.stack([np.ones_like(A), A * half, B * half], axis=-1).reshape(-1, 3)
    d /= np.linalg.norm(d, axis=1)[:, None]
    if pick is not None:
        d = d[pick]
    st = np.zeros((len(d), 8))
    st[:, 0] = float(cz["eta_at_a1"])
    st[:, 1:4] = np.array([0.0, 500.0, 500.0]) * one_Mpc
    st[:, 5:8] = d * c
    st, status = O.null_init(spec, st, -1.0)
    assert (status == 0).all()
    dl = 0.5 * one_Mpc / c
    cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=10000, max_iter=10000,
                      stop_box=((0, 0, 0), (box, box, box)), lens_center=tuple(lens))
    return spec, st, cfg


_OBS_CHECKED = ("a_obs", "a_em", "phi_obs", "phi_em", "path", "chord", "excess", "min_r", "v1x", "v1y", "v1z")


def _assert_matches_oracle(r, spec, st, cfg, tol):
    """GPU vs the oracle: bit for bit with the library's cube, within `tol` with libm's (the
    reference's arithmetic). The time-delay excess (path - chord without cancellation, ~1e-9
    of the path) is held to 1e-12 of the path length: a 1e-16 state difference moves it by the
    ray's transverse excursion times that, far above its own 1e-12 relative resolution."""
    with O.power_mode("dd"):
        od = O.trace(spec, st, cfg, threads=8)
    for k in ("status", "n_steps", "n_iter"):
        assert np.array_equal(r[k], getattr(od, k)), k
    assert np.array_equal(r["state"], od.state)
    assert np.array_equal(r["obs"], od.obs, equal_nan=True)
    o = O.trace(spec, st, cfg, threads=8)
    assert np.array_equal(r["status"], o.status) and np.array_equal(r["n_steps"], o.n_steps)
    assert rel_err(r["state"], o.state).max() <= tol
    path = o.obs[:, N.OBS_COLS.index("path")]
    for col in _OBS_CHECKED:
        i = N.OBS_COLS.index(col)
        if col == "excess":
            assert (np.abs(r["obs"][:, i] - o.obs[:, i]) <= tol * path).all(), col
        else:
            assert rel_err(r["obs"][:, i], o.obs[:, i]).max() <= tol, col


def test_flrw_patch_grid128_matches_oracle(cuda):
    spec, st, cfg = _flrw_patch_case(128, 24)
    r = gpu_trace(spec, st, cfg)
    _assert_matches_oracle(r, spec, st, cfg, 1e-12)


def test_flrw_patch_subset_matches_oracle(cuda):
    """4,096 seeded pixels of the 256 x 256 patch of the 65,536-ray FLRW workload (128^3 Plummer +
    random-field potential, LCDM, RK4 at 0.5 Mpc to box exit), the benchmark's own geometry."""
    pick = np.sort(np.random.default_rng(22).choice(256 * 256, 4096, replace=False))
    spec, st, cfg = _flrw_patch_case(128, 256, pick=pick)
    r = gpu_trace(spec, st, cfg)
    assert (r["status"] == N.PH_LEFT_BOX).all()
    _assert_matches_oracle(r, spec, st, cfg, 1e-12)


@pytest.mark.parametrize("stepper,gradient", [("rk4", "base_node"), ("rk45", "trilinear")])
def test_box_face_stop_matches_oracle(cuda, stepper, gradient):
    """stop_face: the last step shortened to end on the box face. The FP64 tracer equals the
    oracle's face stop bit for bit (states, statuses, step counts, observables), and every ray
    ends within a small fraction of a step of a face (the shortened step is aimed along the
    velocity; the trajectory's curvature over that step is what remains)."""
    import dataclasses

    from excalibur_tool_gb300.core.constants import one_Mpc

    spec, st, cfg = _flrw_patch_case(32, 8)
    spec.fields[0].gradient = gradient
    hi = 1000 * one_Mpc if gradient == "base_node" else 29.5 * 1000 * one_Mpc / 32   # slow class: inside its nodes
    kw = dict(stop_face=True, stop_box=((0.0, 0.0, 0.0), (hi, hi, hi)))
    if stepper == "rk45":
        kw.update(stepper="rk45", tableau="fehlberg", rtol=1e-8, atol=1e-12, dt_min=1e10, dt_max=20 * cfg.dt,
                  max_iter=20000)
    cfg = dataclasses.replace(cfg, **kw)
    r = gpu_trace(spec, st, cfg)
    with O.power_mode("dd"):
        od = O.trace(spec, st, cfg, threads=8)
    for k in ("status", "n_steps", "n_iter", "state"):
        assert np.array_equal(r[k], getattr(od, k)), k
    assert np.array_equal(r["obs"], od.obs, equal_nan=True)
    assert (r["status"] == N.PH_LEFT_BOX).all()
    x = r["state"][:, 1:4]
    to_face = np.minimum(x, hi - x).min(axis=1)
    assert np.abs(to_face).max() <= (1e-3 if stepper == "rk4" else 0.05) * one_Mpc


def test_flrw_patch_grid128_fast_build_matches_oracle(cuda):
    import dataclasses

    spec, st, cfg = _flrw_patch_case(128, 24)
    cfg = dataclasses.replace(cfg, precision="fp64_fast")
    r = gpu_trace(spec, st, cfg)
    o = O.trace(spec, st, cfg, threads=8)
    assert np.array_equal(r["status"], o.status)
    assert np.array_equal(r["n_steps"], o.n_steps)
    assert rel_err(r["state"], o.state).max() <= 1e-11
    for col in ("a_em", "phi_em", "path", "chord", "min_r", "v1x", "v1y", "v1z"):
        i = N.OBS_COLS.index(col)
        assert rel_err(r["obs"][:, i], o.obs[:, i]).max() <= 1e-10, col


def test_queue_and_static_schedules_agree(cuda):
    import dataclasses

    spec, st, cfg = _flrw_patch_case(32, 12)
    a = gpu_trace(spec, st, dataclasses.replace(cfg, use_queue=True))
    b = gpu_trace(spec, st, dataclasses.replace(cfg, use_queue=False))
    for k in ("state", "status", "n_steps", "obs"):
        assert np.array_equal(a[k], b[k], equal_nan=True)


def test_multi_field_batch_matches_single(cuda):
    """Photons routed to different grids in one launch == separate launches."""
    from excalibur_tool_gb300.objects.fields import lens_plus_grf
    from excalibur_tool_gb300.core.constants import one_Mpc, one_Msun

    spec, st, cfg = _flrw_patch_case(32, 8)
    box = 1000 * one_Mpc
    lens = np.array([500.0, 500.0, 500.0]) * one_Mpc
    f2 = lens_plus_grf(16, box, 1e15 * one_Msun, 5 * one_Mpc, lens, seed=5)
    spec2 = lcdm_spacetime(f2, box)
    both = lcdm_spacetime(spec.fields[0].data, box)
    both.fields.append(spec2.fields[0])
    fidx = (np.arange(len(st)) % 2).astype(np.int32)
    r = gpu_trace(both, st, cfg, field_index=fidx)
    r0 = gpu_trace(spec, st[fidx == 0], cfg)
    r1 = gpu_trace(spec2, st[fidx == 1], cfg)
    assert np.array_equal(r["state"][fidx == 0], r0["state"])
    assert np.array_equal(r["state"][fidx == 1], r1["state"])


def test_failure_statuses(cuda):
    """Outside-grid, horizon and non-finite photons fail with a status, never a trap."""
    from excalibur_tool_gb300.core.constants import one_Mpc, c

    g = golden("rhs.npz")
    spec = lcdm_spacetime(g["flrw_field"], float(g["flrw_box"]), cosmology="table")
    spec.fields[0].boundary = "error"
    st = g["flrw_states"][:4].copy()
    st[0, 1] = -1e30          # outside the strict interior
    st[1, 2] = np.nan         # non-finite position
    dt = 0.1 * one_Mpc / c
    cfg = TraceConfig(stepper="rk4", dt=dt, dt_min=dt, dt_max=dt, max_steps=5)
    r = gpu_trace(spec, st, cfg)
    o = O.trace(spec, st, cfg)
    assert r["status"][0] == N.PH_OUTSIDE_GRID
    assert r["status"][1] == N.PH_NONFINITE
    assert np.array_equal(r["status"], o.status)
    M = float(g["schw_mass"])
    rs = 2 * 6.67430e-11 * M / 299792458 ** 2
    sspec = schw_spacetime(M, 0.5 * rs)
    s2 = g["schw_states"][:2].copy()
    s2[0, 1] = 0.9 * rs       # inside the horizon
    r = gpu_trace(sspec, s2, cfg)
    assert r["status"][0] == N.PH_HORIZON


def test_abort_flag_and_deadline(cuda):
    """Host abort flag and device deadline end the launch with statuses (bounded waits, no hang)."""
    import dataclasses
    import torch
    from excalibur_tool_gb300.trace import trace_batch

    spec, st, cfg = _flrw_patch_case(32, 16)
    m = gpu_metric(spec)
    s = torch.as_tensor(st).cuda()
    flag = torch.ones(1, dtype=torch.int32, device="cuda")
    r = trace_batch(m, s, cfg, abort_flag=flag)
    torch.cuda.synchronize()
    status = r.status.cpu().numpy()
    assert set(np.unique(status)) <= {N.PH_ABORTED, N.PH_NOT_RUN}
    r = trace_batch(m, s, dataclasses.replace(cfg, deadline_cycles=1000))
    torch.cuda.synchronize()
    status = r.status.cpu().numpy()
    assert (status != N.PH_LEFT_BOX).any()
    assert set(np.unique(status)) <= {N.PH_TIMED_OUT, N.PH_NOT_RUN, N.PH_LEFT_BOX}
    # the context stays usable
    r = trace_batch(m, s, cfg)
    torch.cuda.synchronize()
    assert (r.status.cpu().numpy() == N.PH_LEFT_BOX).all()


def test_division_by_launch_constants_is_ieee(cuda):
    """The parity build divides by launch constants (c^2, c^4, grid spacings and their
    doubles, the a(eta) table step) with x * RN(1/c) and Markstein's FMA correction; over
    2^32 quotients per run -- random operands over 2^-200 .. 2^200 and operands placed next to
    rounding midpoints -- it must equal the IEEE quotient bit for bit."""
    import ctypes as C

    import torch
    from excalibur_tool_gb300 import _native as N
    from excalibur_tool_gb300.core import constants as K

    cz = golden("cosmology.npz")
    divs = [K.C2_F64, K.C4_F64, float(cz["eta_step"]), 6.0]   # 6: the redshift table's Simpson terms
    for n in (32, 64, 96, 128, 256, 512):
        h = 1000 * K.one_Mpc / n
        divs += [h, 2.0 * h]
    rng = np.random.default_rng(8)
    divs += list(rng.uniform(1.0, 2.0, 16) * 2.0 ** rng.integers(-60, 90, 16))
    d = torch.as_tensor(np.array(divs), device=cuda)
    bad = torch.zeros(1, dtype=torch.int64, device=cuda)
    L = N.load()
    for seed in (1, 2):
        N.check(L.exc_probe_div_rn(N.ptr(d), len(divs), 1 << 32, seed, N.ptr(bad), N.stream_handle(cuda)),
                "exc_probe_div_rn")
        torch.cuda.synchronize()
        assert int(bad.item()) == 0
