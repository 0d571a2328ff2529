"""Generate the golden vectors by running the REFERENCE implementation.

Runs lmagristella/excalibur-tool's own Python code (its numba-decorated
kernels execute as plain Python through the test-only shim in
oracle/shim/numba) on small seeded inputs and writes the results to
tests/golden/*.npz. Only the machine that holds the reference checkout can
run this (--ref <path> or EXCALIBUR_REF=<path>); the committed .npz files
are what the tests read.

    python tests/golden/make_golden.py --ref <reference checkout> [generator ...]
"""
from __future__ import annotations

import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _reference_path(argv):
    """The reference checkout: `--ref PATH` or the EXCALIBUR_REF environment variable."""
    if "--ref" in argv:
        i = argv.index("--ref")
        path = argv[i + 1]
        del argv[i:i + 2]
        return path
    path = os.environ.get("EXCALIBUR_REF")
    if not path:
        sys.exit("usage: make_golden.py --ref PATH_TO_REFERENCE [generator ...] (or set EXCALIBUR_REF)")
    return path


REF = _reference_path(sys.argv)
sys.path[:0] = [os.path.join(REPO, "oracle", "shim"), REF, REPO]

from excalibur.core.constants import c, G, one_Mpc, one_Msun, one_Gpc  # noqa: E402
from excalibur.core.coordinates import cartesian_to_spherical, cartesian_velocity_to_spherical  # noqa: E402
from excalibur.core.cosmology import LCDM_Cosmology, StaticCosmology  # noqa: E402
from excalibur.grid.grid import Grid  # noqa: E402
from excalibur.grid import interpolator_4d_fast as i4d  # noqa: E402
from excalibur.grid import interpolator_fast as ifast  # noqa: E402
from excalibur.integration.integrator import RK4, RK45Adaptive, Leapfrog4, Integrator  # noqa: E402
from excalibur.metrics.perturbed_flrw_metric_fast import PerturbedFLRWMetricFast  # noqa: E402
from excalibur.metrics.schwarzschild_metric_fast import SchwarzschildMetricFast  # noqa: E402
from excalibur.photon.photons import Photons  # noqa: E402
from excalibur.photon.photon import Photon  # noqa: E402

from excalibur_tool_gb300.objects.fields import lens_plus_grf  # noqa: E402


def _load_file(name, *rel):
    """Import one reference module by path (its package __init__ pulls in matplotlib, absent here)."""
    spec = importlib.util.spec_from_file_location(name, os.path.join(REF, *rel))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def _load_postprocessing():
    return _load_file("analyze_compare_trajectories", "_postprocessing", "analyze_compare_trajectories.py")


RedshiftCalculator = _load_file("excalibur_redshift", "excalibur", "observables", "redshift.py").RedshiftCalculator


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"wrote {name}: " + ", ".join(f"{k}{np.shape(v)}" for k, v in arrays.items()))


# ----------------------------------------------------------------- cosmology
def gen_cosmology():
    cz = LCDM_Cosmology(70, 0.3, 0.0, 0.7)
    rng = np.random.default_rng(11)
    eta_max = cz.eta_min + cz.eta_step * (cz.N_eta - 1)
    etas = np.concatenate([rng.uniform(cz.eta_min, eta_max, 200),
                           [cz.eta_min - 1e15, cz.eta_min, eta_max, eta_max + 1e16, cz._eta_at_a1,
                            cz._eta_at_a1 - 5.1e13, 1e18, 1.2e18]])
    a = np.array([cz.a_of_eta(float(e)) for e in etas])
    adot = np.array([cz.adot_of_eta(float(e)) for e in etas])
    # the class's host helpers: H(z), a(z), and a(t) by its quad-and-update search
    zs = np.array([0.0, 0.5, 1.0, 3.0, 1100.0])
    ts = np.array([1.0e16, 1.0e17, 3.0e17, 4.3e17])
    save("cosmology.npz", a_grid=cz.a_grid, eta_min=cz.eta_min, eta_step=cz.eta_step, N_eta=cz.N_eta,
         eta_at_a1=cz._eta_at_a1, H0=cz.H0, etas=etas, a=a, adot=adot, zs=zs,
         H_of_z=np.array([cz.H_of_z(z) for z in zs]), a_of_z=np.array([cz.a_of_z(z) for z in zs]),
         ts=ts, a_of_t=cz.a_of_t(ts), a_of_t_scalar=cz.a_of_t(3.0e17))
    return cz


# ------------------------------------------------------------- interpolators
def _grid_and_points(shape, spacing, origin, seed, n_pts, lo_frac=-0.3, hi_frac=1.3):
    rng = np.random.default_rng(seed)
    data = rng.standard_normal(shape) * 3.0e4
    g = Grid(shape, spacing, origin)
    g.add_field("Phi", data)
    ext = np.array(shape[:3]) * np.array(spacing[:3])
    pts = np.array(origin[:3]) + rng.uniform(lo_frac, hi_frac, (n_pts, 3)) * ext
    # exact nodes, cell edges and the high corner
    nodes = np.array(origin[:3]) + np.array([[1, 1, 1], [2, 3, 1], [shape[0] - 2, 1, 2], [0, 0, 0],
                                             [shape[0] - 1, shape[1] - 1, shape[2] - 1]]) * np.array(spacing[:3])
    pts = np.concatenate([pts, nodes, -nodes - 0.5 * np.array(spacing[:3])])
    return g, data, pts


def gen_interp():
    out = {}
    shape, spacing, origin = (9, 7, 8), (2.5e22, 3.0e22, 2.0e22), (1.0e22, -4.0e22, 0.0)
    g, data, pts = _grid_and_points(shape, spacing, origin, 3, 300)
    out.update(f3=data, f3_spacing=np.array(spacing), f3_origin=np.array(origin), pts3=pts)
    for mode in ("periodic", "clamp", "error"):
        ip = i4d.InterpolatorFast(g, boundary=mode)
        vals, ok = [], []
        for p in pts:
            try:
                v, gr, dt = ip.value_gradient_and_time_derivative(p, "Phi", 0.0)
                vals.append([v, *gr, dt])
                ok.append(1)
            except Exception:
                vals.append([np.nan] * 5)
                ok.append(0)
        out[f"out3_{mode}"] = np.array(vals)
        out[f"ok3_{mode}"] = np.array(ok)
    legacy = ifast.InterpolatorFast(g)
    vals, ok = [], []
    for p in pts:
        try:
            v, gr, dt = legacy.value_gradient_and_time_derivative(p, "Phi")
            vals.append([v, *gr, dt])
            ok.append(1)
        except Exception:
            vals.append([np.nan] * 5)
            ok.append(0)
    out["out3_legacy"] = np.array(vals)
    out["ok3_legacy"] = np.array(ok)
    # 4-D: three time snapshots
    shape4, spacing4, origin4 = (8, 9, 7, 3), (2.0e22, 2.5e22, 3.0e22, 4.0e15), (0.0, 1.0e22, -2.0e22, 1.0e17)
    rng = np.random.default_rng(5)
    data4 = rng.standard_normal(shape4) * 3.0e4
    g4 = Grid(shape4, spacing4, origin4)
    g4.add_field("Phi", data4)
    pts4 = np.concatenate([np.array(origin4[:3]) + rng.uniform(-0.2, 1.2, (200, 3)) * np.array(shape4[:3]) *
                           np.array(spacing4[:3]),
                           (origin4[3] + rng.uniform(-0.3, 2.3, 200) * spacing4[3])[:, None]], axis=1)
    out.update(f4=data4, f4_spacing=np.array(spacing4), f4_origin=np.array(origin4), pts4=pts4)
    for mode in ("periodic", "clamp", "error"):
        ip = i4d.InterpolatorFast(g4, boundary=mode)
        vals, ok = [], []
        for p in pts4:
            try:
                v, gr, dt = ip.value_gradient_and_time_derivative(p[:3], "Phi", p[3])
                vals.append([v, *gr, dt])
                ok.append(1)
            except Exception:
                vals.append([np.nan] * 5)
                ok.append(0)
        out[f"out4_{mode}"] = np.array(vals)
        out[f"ok4_{mode}"] = np.array(ok)
    save("interp.npz", **out)


def _slow_eval(ip, pts, times=None):
    vals, ok = [], []
    for i, p in enumerate(pts):
        try:
            t = 0.0 if times is None else float(times[i])
            v, gr, dt = ip.value_gradient_and_time_derivative(p, "Phi", t)
            vals.append([v, *gr, dt])
            ok.append(1)
        except ValueError:
            vals.append([np.nan] * 5)
            ok.append(0)
    return np.array(vals), np.array(ok)


def gen_interp_slow(cz):
    """The slow Interpolator (grid/interpolator.py): 3-D float64 and float32
    grids, 4-D grids with three and two snapshots (times inside, outside and on
    half-integers, where np.round goes to even), and RK4 traces through
    PerturbedFLRWMetricFast with that interpolator."""
    from excalibur.grid.interpolator import Interpolator

    out = {}
    shape, spacing, origin = (9, 7, 8), (2.5e22, 3.0e22, 2.0e22), (1.0e22, -4.0e22, 0.0)
    g, data, pts = _grid_and_points(shape, spacing, origin, 13, 300, lo_frac=-0.1, hi_frac=1.1)
    # points in the first and last cells (gradient base clipped to 1 / n-2)
    ext = np.array(shape) * np.array(spacing)
    edge = np.array(origin) + np.array([[0.3, 0.5, 0.2], [0.99, 0.5, 0.5], [0.01, 0.99, 0.5]]) * \
        (np.array(shape) - 1) * np.array(spacing)
    pts = np.concatenate([pts, edge, (np.array(origin) + ext * 0.5)[None]])
    out.update(f3=data, f3_spacing=np.array(spacing), f3_origin=np.array(origin), pts3=pts)
    out["out3"], out["ok3"] = _slow_eval(Interpolator(g), pts)
    g32 = Grid(shape, spacing, origin)
    g32.add_field("Phi", data.astype(np.float32))
    out["out3_f32"], out["ok3_f32"] = _slow_eval(Interpolator(g32), pts)
    rng = np.random.default_rng(17)
    for nt in (3, 2):
        shape4, spacing4, origin4 = (8, 9, 7, nt), (2.0e22, 2.5e22, 3.0e22, 4.0e15), (0.0, 1.0e22, -2.0e22, 1.0e17)
        data4 = rng.standard_normal(shape4) * 3.0e4
        g4 = Grid(shape4, spacing4, origin4)
        g4.add_field("Phi", data4)
        n4 = 200
        p4 = np.array(origin4[:3]) + rng.uniform(-0.1, 1.1, (n4, 3)) * (np.array(shape4[:3]) - 1) * \
            np.array(spacing4[:3])
        rel_t = np.concatenate([rng.uniform(-0.6, nt + 0.4, n4 - 8), [-0.5, 0.5, 1.5, 2.5, 0.0, 1.0, nt - 1.0, 3.5]])
        t4 = origin4[3] + rel_t * spacing4[3]
        o4, k4 = _slow_eval(Interpolator(g4), p4, t4)
        out.update({f"f4_{nt}": data4, f"f4_{nt}_spacing": np.array(spacing4), f"f4_{nt}_origin": np.array(origin4),
                    f"pts4_{nt}": np.column_stack([p4, t4]), f"out4_{nt}": o4, f"ok4_{nt}": k4})
    # RK4 traces through the fast FLRW metric with the slow interpolator
    n, box = 16, 40 * one_Mpc
    rng = np.random.default_rng(19)
    field = rng.standard_normal((n, n, n)) * 1e-5 * c ** 2
    gt = Grid((n, n, n), (box / n,) * 3, (0.0, 0.0, 0.0))
    gt.add_field("Phi", field)
    m = PerturbedFLRWMetricFast(cz.a_of_eta, gt, Interpolator(gt), adot_of_eta=cz.adot_of_eta)
    dt = 0.25 * one_Mpc / c
    eta0 = cz._eta_at_a1
    inits, finals, recs = [], [], []
    for k in range(4):
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        x0 = np.array([eta0, *(rng.uniform(0.35, 0.65, 3) * box)])
        u0 = Photons(m)._solve_u0_from_null_condition(x0, d * c, sign=-1.0)
        p = Photon(x0, np.array([u0, *(d * c)]))
        Integrator(m, dt=dt, integrator="rk4", dt_min=dt, dt_max=dt).integrate_single(p, "steps", 40, record_every=1)
        inits.append(np.concatenate([x0, [u0], d * c]))
        finals.append(np.concatenate([p.x, p.u]))
        recs.append(np.array([np.asarray(h, dtype=float)[:8] for h in p.history.states]))
    out.update(trace_field=field, trace_box=box, trace_dt=dt, trace_init=np.array(inits),
               trace_final=np.array(finals), trace_records=np.array(recs))
    save("interp_slow.npz", **out)


# ----------------------------------------------------------------- RHS
def _flrw_setup(cz, n=16, box=40 * one_Mpc, seed=7, boundary="periodic"):
    rng = np.random.default_rng(seed)
    data = rng.standard_normal((n, n, n)) * 1e-5 * c ** 2
    g = Grid((n, n, n), (box / n,) * 3, (0.0, 0.0, 0.0))
    g.add_field("Phi", data)
    ip = i4d.InterpolatorFast(g, boundary=boundary)
    return g, data, ip


def gen_rhs(cz):
    g, data, ip = _flrw_setup(cz)
    box = 40 * one_Mpc
    rng = np.random.default_rng(21)
    n = 64
    eta0 = cz._eta_at_a1
    states = np.zeros((n, 8))
    states[:, 0] = eta0 + rng.uniform(-3e16, 3e16, n)
    states[:, 1:4] = rng.uniform(0.05, 0.95, (n, 3)) * box
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    states[:, 5:8] = d * c * rng.uniform(0.9, 1.1, (n, 1))
    states[:, 4] = -rng.uniform(0.95, 1.05, n)
    out = {"flrw_field": data, "flrw_box": box, "flrw_states": states}
    static = StaticCosmology()
    variants = {
        "lcdm_tensorial": (cz.a_of_eta, cz.adot_of_eta, False),
        "lcdm_analytical": (cz.a_of_eta, cz.adot_of_eta, True),
        "lcdm_fd": (cz.a_of_eta, None, False),
        "static_tensorial": (static.a_of_eta, static.adot_of_eta, False),
    }
    for name, (af, adf, analytical) in variants.items():
        m = PerturbedFLRWMetricFast(af, g, ip, analytical_geodesics=analytical, adot_of_eta=adf)
        out[f"flrw_{name}"] = np.array([m.geodesic_equations(s) for s in states])
        out[f"flrw_g_{name}"] = np.array([np.diag(m.metric_tensor(s[:4])) for s in states])
    # Schwarzschild: random spherical states away from the poles
    M = 1e15 * one_Msun
    rs = 2 * G * M / c ** 2
    sst = np.zeros((n, 8))
    sst[:, 0] = rng.uniform(0, 1e16, n)
    sst[:, 1] = rs * np.exp(rng.uniform(np.log(1.5), np.log(1e7), n))
    sst[:, 2] = rng.uniform(0.2, np.pi - 0.2, n)
    sst[:, 3] = rng.uniform(-np.pi, np.pi, n)
    sst[:, 4] = -rng.uniform(0.9, 1.2, n)
    sst[:, 5] = c * rng.uniform(-1, 1, n)
    sst[:, 6] = c / sst[:, 1] * rng.uniform(-1, 1, n)
    sst[:, 7] = c / sst[:, 1] * rng.uniform(-1, 1, n)
    out["schw_states"] = sst
    out["schw_mass"] = M
    for name, (an, ft) in {"analytical_free": (True, True), "analytical_null": (True, False),
                           "tensorial": (False, True)}.items():
        m = SchwarzschildMetricFast(M, 1.2 * rs, center=np.zeros(3), analytical_geodesics=an,
                                    free_time_geodesic=ft, coords="spherical")
        out[f"schw_{name}"] = np.array([m.geodesic_equations(s) for s in sst])
        out[f"schw_g_{name}"] = np.array([np.diag(m.metric_tensor(s[:4])) for s in sst])
    save("rhs.npz", **out)


# ---------------------------------------------------------------- steppers
def gen_steps(cz):
    g, data, ip = _flrw_setup(cz, seed=8)
    box = 40 * one_Mpc
    rhs = np.load(os.path.join(HERE, "rhs.npz"))
    states = rhs["flrw_states"][:24]
    m = PerturbedFLRWMetricFast(cz.a_of_eta, g, ip, adot_of_eta=cz.adot_of_eta)
    dt = 0.5 * one_Mpc / c
    out = {"field": data, "box": box, "states": states, "dt": dt}
    out["rk4"] = np.array([RK4().step(m, s, dt)[0] for s in states])
    out["lf4"] = np.array([Leapfrog4().step(m, s, dt)[0] for s in states])
    rk45 = RK45Adaptive()
    res = [rk45.step(m, s, dt, 1e-9, 1e-13) for s in states]
    out["rk45_state"] = np.array([r[0] for r in res])
    out["rk45_dt"] = np.array([r[1] for r in res])
    out["rk45_acc"] = np.array([r[2] for r in res])
    res = [rk45.step(m, s, dt, 1e-3, 1e-3) for s in states]   # loose tolerances: accepted steps
    out["rk45l_state"] = np.array([r[0] for r in res])
    out["rk45l_dt"] = np.array([r[1] for r in res])
    out["rk45l_acc"] = np.array([r[2] for r in res])
    save("steps.npz", **out)


# -------------------------------------------------- integrate_single (records)
def gen_integrate(cz):
    g, data, ip = _flrw_setup(cz, seed=9)
    box = 40 * one_Mpc
    m = PerturbedFLRWMetricFast(cz.a_of_eta, g, ip, adot_of_eta=cz.adot_of_eta)
    dt = 0.25 * one_Mpc / c
    eta0 = cz._eta_at_a1
    rng = np.random.default_rng(31)
    out = {"field": data, "box": box, "dt": dt}
    cases = []
    # RK4, fixed steps, record_every = 1 / 5 / 0, with and without renormalisation
    for k, (rec, ren, nsteps) in enumerate([(1, 0, 40), (5, 0, 57), (0, 0, 40), (1, 3, 40)]):
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        x0 = np.array([eta0, *(rng.uniform(0.3, 0.7, 3) * box)])
        ph = Photons(m)
        ph.photons.append(Photon(x0, np.array([0.0, *(d * c)])))
        u0 = ph._solve_u0_from_null_condition(x0, d * c, sign=-1.0)
        p = Photon(x0, np.array([u0, *(d * c)]))
        integ = Integrator(m, dt=dt, integrator="rk4", dt_min=dt, dt_max=dt)
        integ.integrate_single(p, "steps", nsteps, record_every=rec, renormalize_every=ren)
        hist = p.history.states
        width = max(len(h) for h in hist)
        arr = np.full((len(hist), width), np.nan)
        for i, h in enumerate(hist):
            arr[i, :len(h)] = h
        out[f"case{k}_init"] = np.concatenate([x0, [u0], d * c])
        out[f"case{k}_final"] = np.concatenate([p.x, p.u])
        out[f"case{k}_records"] = arr
        cases.append((rec, ren, nsteps, "rk4"))
    # RK45 (reference tableau) through integrate_single with the dt clip active
    d = np.array([0.6, 0.48, 0.64])
    x0 = np.array([eta0, 0.4 * box, 0.45 * box, 0.5 * box])
    u0 = Photons(m)._solve_u0_from_null_condition(x0, d * c, sign=-1.0)
    p = Photon(x0, np.array([u0, *(d * c)]))
    integ = Integrator(m, dt=dt, integrator="rk45", rtol=1e-6, atol=1e-3, dt_min=dt / 50, dt_max=dt)
    integ.integrate_single(p, "steps", 30, record_every=1)
    hist = p.history.states
    arr = np.full((len(hist), 14), np.nan)
    for i, h in enumerate(hist):
        arr[i, :len(h)] = h
    out["case4_init"] = np.concatenate([x0, [u0], d * c])
    out["case4_final"] = np.concatenate([p.x, p.u])
    out["case4_records"] = arr
    out["case4_tol"] = np.array([1e-6, 1e-3, dt / 50, dt])
    cases.append((1, 0, 30, "rk45"))
    out["cases"] = np.array([[r, e, s, 0 if n == "rk4" else 1] for r, e, s, n in cases])
    save("integrate.npz", **out)


# --------------------------- integrate_single, RK45 (reference tableau), slow Interpolator
def gen_rk45_slow(cz):
    """Integrator(integrator="rk45").integrate_single through PerturbedFLRWMetricFast read with the
    slow Interpolator (continuous trilinear-blended gradient): three photons, 30 iterations,
    record_every 1, tolerances loose enough that trial steps are both accepted and rejected."""
    from excalibur.grid.interpolator import Interpolator

    n, box = 16, 40 * one_Mpc
    rng = np.random.default_rng(23)
    field = rng.standard_normal((n, n, n)) * 1e-5 * c ** 2
    g = Grid((n, n, n), (box / n,) * 3, (0.0, 0.0, 0.0))
    g.add_field("Phi", field)
    m = PerturbedFLRWMetricFast(cz.a_of_eta, g, Interpolator(g), adot_of_eta=cz.adot_of_eta)
    dt = 0.25 * one_Mpc / c
    eta0 = cz._eta_at_a1
    tol = (1e-6, 1e-3, dt / 50, dt)
    out = {"field": field, "box": box, "dt": dt, "tol": np.array(tol)}
    for k in range(3):
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        x0 = np.array([eta0, *(rng.uniform(0.35, 0.65, 3) * box)])
        u0 = Photons(m)._solve_u0_from_null_condition(x0, d * c, sign=-1.0)
        p = Photon(x0, np.array([u0, *(d * c)]))
        Integrator(m, dt=dt, integrator="rk45", rtol=tol[0], atol=tol[1], dt_min=tol[2], dt_max=tol[3]) \
            .integrate_single(p, "steps", 30, record_every=1)
        out[f"case{k}_init"] = np.concatenate([x0, [u0], d * c])
        out[f"case{k}_final"] = np.concatenate([p.x, p.u])
        out[f"case{k}_records"] = _history_array(p)
    save("rk45_slow.npz", **out)


# ------------------------------------- integrate_single with the Leapfrog4 stepper
def gen_integrate_lf4(cz):
    """Integrator(integrator="leapfrog4").integrate_single on the integrate.npz field: two photons,
    40 fixed steps, record_every 1 and 3."""
    g, data, ip = _flrw_setup(cz, seed=9)
    box = 40 * one_Mpc
    m = PerturbedFLRWMetricFast(cz.a_of_eta, g, ip, adot_of_eta=cz.adot_of_eta)
    dt = 0.25 * one_Mpc / c
    eta0 = cz._eta_at_a1
    rng = np.random.default_rng(37)
    out = {"field": data, "box": box, "dt": dt}
    recs = []
    for k, rec in enumerate((1, 3)):
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        x0 = np.array([eta0, *(rng.uniform(0.3, 0.7, 3) * box)])
        u0 = Photons(m)._solve_u0_from_null_condition(x0, d * c, sign=-1.0)
        p = Photon(x0, np.array([u0, *(d * c)]))
        Integrator(m, dt=dt, integrator="leapfrog4", dt_min=dt, dt_max=dt).integrate_single(
            p, "steps", 40, record_every=rec)
        out[f"case{k}_init"] = np.concatenate([x0, [u0], d * c])
        out[f"case{k}_final"] = np.concatenate([p.x, p.u])
        out[f"case{k}_records"] = _history_array(p)
        recs.append(rec)
    out["record_every"] = np.array(recs)
    save("integrate_lf4.npz", **out)


# ------------------------------------------- Integrator.integrate (per mode)
def _history_array(p, width=14):
    hist = p.history.states
    arr = np.full((len(hist), width), np.nan)
    for i, h in enumerate(hist):
        arr[i, :len(h)] = h
    return arr


def gen_integrate_modes(cz):
    """Integrator.integrate on five photons through a strict ("error") grid, the fourth of
    which leaves the grid's interior: sequential mode (records every step, raises at that
    photon, the fifth never integrated) and chunked mode (two workers, chunks of two; the
    failed photon left as it was)."""
    g, data, ip = _flrw_setup(cz, seed=11, boundary="error")
    box = 40 * one_Mpc
    m = PerturbedFLRWMetricFast(cz.a_of_eta, g, ip, adot_of_eta=cz.adot_of_eta)
    dt = 0.25 * one_Mpc / c
    eta0 = cz._eta_at_a1
    rng = np.random.default_rng(41)
    inits = []
    for k in range(5):
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        x0 = np.array([eta0, *(rng.uniform(0.4, 0.6, 3) * box)])
        if k == 3:      # starts next to the strict interior's edge, heading out
            x0[1:4] = [0.85 * box, 0.5 * box, 0.5 * box]
            d = np.array([1.0, 0.0, 0.0])
        u0 = Photons(m)._solve_u0_from_null_condition(x0, d * c, sign=-1.0)
        inits.append(np.concatenate([x0, [u0], d * c]))
    out = {"field": data, "box": box, "dt": dt, "inits": np.array(inits), "n_steps": 40}

    def make():
        ph = Photons(m)
        for s in inits:
            ph.photons.append(Photon(s[:4].copy(), s[4:].copy()))
        return ph

    integ = Integrator(m, dt=dt, mode="sequential", integrator="rk4", dt_min=dt, dt_max=dt)
    ph = make()
    try:
        integ.integrate(ph.photons, "steps", 40, verbose=False)
        raised = 0
    except ValueError:
        raised = 1
    out["seq_raised"] = raised
    for k, p in enumerate(ph.photons):
        out[f"seq{k}_history"] = _history_array(p)
        out[f"seq{k}_final"] = np.concatenate([p.x, p.u])
        out[f"seq{k}_quantities"] = np.asarray(p.quantities, dtype=float)
    integ = Integrator(m, dt=dt, mode="chunked", integrator="rk4", dt_min=dt, dt_max=dt, n_workers=2, chunk_size=2)
    ph = make()
    out["chunked_ok"] = integ.integrate(ph, "steps", 40, verbose=False)
    for k, p in enumerate(ph.photons):
        out[f"chunked{k}_history"] = _history_array(p)
        out[f"chunked{k}_final"] = np.concatenate([p.x, p.u])
    save("integrate_modes.npz", **out)


# ------------------------------------------------ Schwarzschild polar cone, 1,024 rays
def schw_polar_initial_states():
    """1024 photons: Schwarzschild lens (1e15 Msun at the box centre), observer at (0,500,500) Mpc,
    32x32 polar grid theta_i = (i+1/2) 5deg/32, phi_j = 2 pi j/32, rotated onto the lens direction with
    the reference's Rodrigues formula, spherical velocities via cartesian_velocity_to_spherical and
    u^0 from _solve_u0_from_null_condition (sign -1)."""
    M = 1e15 * one_Msun
    rs = 2 * G * M / c ** 2
    lens = np.array([500.0, 500.0, 500.0]) * one_Mpc
    obs = np.array([0.0, 500.0, 500.0]) * one_Mpc
    m = SchwarzschildMetricFast(M, rs * (1 + 1e-6), center=lens, coords="spherical",
                                analytical_geodesics=True, free_time_geodesic=True)
    ph = Photons(m)
    origin = np.array([0.0, *cartesian_to_spherical(*(obs - lens))])
    central = (lens - obs) / np.linalg.norm(lens - obs)
    r0, t0, p0 = origin[1:]
    x0 = r0 * np.sin(t0) * np.cos(p0)
    y0 = r0 * np.sin(t0) * np.sin(p0)
    z0 = r0 * np.cos(t0)
    states = np.zeros((1024, 8))
    for i in range(32):
        th = (i + 0.5) * np.deg2rad(5.0) / 32
        for j in range(32):
            phi = 2 * np.pi * j / 32
            d = np.array([np.sin(th) * np.cos(phi), np.sin(th) * np.sin(phi), np.cos(th)])
            d3 = ph._rotate_to_direction(d, central)
            d3 = d3 / np.linalg.norm(d3)
            us = np.array(cartesian_velocity_to_spherical(x0, y0, z0, *(d3 * c)))
            u0 = ph._solve_u0_from_null_condition(origin, us, sign=-1.0)
            states[i * 32 + j] = np.concatenate([origin, [u0], us])
    return m, states


def gen_schw_polar():
    m, states = schw_polar_initial_states()
    dl = 0.5 * one_Mpc / c
    rng = np.random.default_rng(101)
    sel = np.unique(np.concatenate([[0, 1, 8, 15, 16, 17, 31, 511, 520, 1023],
                                    rng.choice(1024, 30, replace=False)]))
    rk = RK4()
    finals, status, nsteps = [], [], []
    for idx in sel:
        s = states[idx].copy()
        st, k = 0, 0
        try:
            for k in range(2000):
                s, _, _ = rk.step(m, s, dl)
            k = 2000
        except Exception:
            st = 1
        finals.append(s)
        status.append(st)
        nsteps.append(k)
    save("schw_polar_1024.npz", states=states, sel=sel, final=np.array(finals), failed=np.array(status),
         n_steps=np.array(nsteps), dl=dl, mass=m.mass, radius=m.radius)


# -------------------------------- Schwarzschild polar cone: Leapfrog4 and RK45 integrate_single
def gen_schw_steppers():
    """Six off-pole photons of the polar cone through Integrator.integrate_single with the Leapfrog4
    stepper (300 fixed steps, record_every 10), with the reference's RK45 (rtol 1e-4, atol 1e12,
    dt in [dl/50, dl], 80 iterations, record_every 2) and with RK4 renormalised onto the null cone
    every 7 steps (300 fixed steps, record_every 5, with trace_norm: its norm_history, the relative
    null error at the initial state, after every step and at the end)."""
    m, states = schw_polar_initial_states()
    dl = 0.5 * one_Mpc / c
    pick = np.array([1, 9, 100, 333, 700, 1000])
    out = {"dl": dl, "mass": m.mass, "radius": m.radius, "pick": pick, "states": states[pick]}
    for name, kw, n_steps, rec, ren in (
            ("lf4", dict(integrator="leapfrog4", dt_min=dl, dt_max=dl), 300, 10, 0),
            ("rk45", dict(integrator="rk45", rtol=1e-4, atol=1e12, dt_min=dl / 50, dt_max=dl), 80, 2, 0),
            ("rk4ren", dict(integrator="rk4", dt_min=dl, dt_max=dl), 300, 5, 7)):
        finals, recs, norms = [], [], []
        for s in states[pick]:
            p = Photon(s[:4].copy(), s[4:].copy())
            Integrator(m, dt=dl, **kw).integrate_single(p, "steps", n_steps, record_every=rec,
                                                        renormalize_every=ren, trace_norm=bool(ren))
            finals.append(np.concatenate([p.x, p.u]))
            recs.append(_history_array(p, width=12))
            if ren:
                norms.append(np.array(p.norm_history, dtype=float))
        if norms:
            out[f"{name}_norm"] = np.array(norms)
        width = max(r.shape[0] for r in recs)
        arr = np.full((len(recs), width, 12), np.nan)
        for i, r in enumerate(recs):
            arr[i, :r.shape[0]] = r
        out[f"{name}_final"] = np.array(finals)
        out[f"{name}_records"] = arr
        out[f"{name}_n_records"] = np.array([r.shape[0] for r in recs])
    save("schw_steppers.npz", **out)


# ------------------------------------------------ FLRW lens + random-field patch, 32^3
def gen_flrw_patch_32(cz):
    """The lens patch construction on a 32^3 grid: Plummer (1e15 Msun, eps 5 Mpc) + GRF (seed 2, rms 1e-5),
    periodic interpolation, LCDM, observer (0,500,500) Mpc at eta = _eta_at_a1, 6x6 directions in a
    10x10 degree tangent patch, RK4 dl = 0.5 Mpc/c, stop at box exit (after each accepted step)."""
    n, box = 32, 1000 * one_Mpc
    lens = np.array([500.0, 500.0, 500.0]) * one_Mpc
    phi = lens_plus_grf(n, box, 1e15 * one_Msun, 5 * one_Mpc, lens, seed=2)
    g = Grid((n, n, n), (box / n,) * 3, (0.0, 0.0, 0.0))
    g.add_field("Phi", phi)
    ip = i4d.InterpolatorFast(g, boundary="periodic")
    m = PerturbedFLRWMetricFast(cz.a_of_eta, g, ip, adot_of_eta=cz.adot_of_eta)
    eta0 = cz._eta_at_a1
    obs = np.array([0.0, 500.0, 500.0]) * one_Mpc
    half = np.tan(np.deg2rad(5.0))
    k = 6
    t = (np.arange(k) + 0.5) / k * 2 - 1
    states = []
    ph = Photons(m)
    for a in t:
        for b in t:
            d = np.array([1.0, a * half, b * half])
            d /= np.linalg.norm(d)
            x0 = np.array([eta0, *obs])
            u0 = ph._solve_u0_from_null_condition(x0, d * c, sign=-1.0)
            states.append(np.concatenate([x0, [u0], d * c]))
    states = np.array(states)
    dl = 0.5 * one_Mpc / c
    rk = RK4()
    finals, nsteps = [], []
    for s0 in states:
        s = s0.copy()
        steps = 0
        while steps < 10000:
            s, _, _ = rk.step(m, s, dl)
            steps += 1
            if not np.all((s[1:4] >= 0.0) & (s[1:4] < box)):
                break
        finals.append(s)
        nsteps.append(steps)
    save("flrw_patch_32.npz", field=phi, box=box, states=states, final=np.array(finals), n_steps=np.array(nsteps),
         dl=dl)


# ------------------------------------------------------ photon generators
def gen_generators(cz):
    g, data, ip = _flrw_setup(cz, seed=12)
    box = 40 * one_Mpc
    m = PerturbedFLRWMetricFast(cz.a_of_eta, g, ip, adot_of_eta=cz.adot_of_eta)
    eta0 = cz._eta_at_a1
    origin = np.array([eta0, 0.2 * box, 0.3 * box, 0.4 * box])
    ph = Photons(m)
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        ph.generate_cone_grid(n_photons=49, origin=origin, central_direction=[1.0, 0.5, -0.3],
                              cone_angle=np.deg2rad(7), direction_basis="cartesian")
    flrw_cone = np.array([np.concatenate([p.x, p.u]) for p in ph.photons])
    flrw_null = np.array([p.null_condition_relative_error(m) for p in ph.photons])
    ph5 = Photons(m)
    with contextlib.redirect_stdout(io.StringIO()):
        ph5.generate_cone_grid_metric_tensor(n_photons=49, origin=origin, central_direction=[1.0, 0.5, -0.3],
                                             cone_angle=np.deg2rad(7), direction_basis="cartesian")
    flrw_cone_mt = np.array([np.concatenate([p.x, p.u]) for p in ph5.photons])
    ph7 = Photons(m)
    np.random.seed(17)
    with contextlib.redirect_stdout(io.StringIO()):
        ph7.generate_cone_random(n_photons=25, origin=origin, central_direction=[1.0, 0.5, -0.3],
                                 cone_angle=np.deg2rad(7), direction_basis="cartesian")
    flrw_cone_random = np.array([np.concatenate([p.x, p.u]) for p in ph7.photons])
    ph2 = Photons(m)
    ph2.generate_impact_parameter_bins(origin, [1.0, 0.2, 0.1], np.linspace(0.1, 2.0, 4) * one_Mpc, 5, seed=3)
    flrw_bins = np.array([np.concatenate([p.x, p.u]) for p in ph2.photons])
    M = 1e15 * one_Msun
    rs = 2 * G * M / c ** 2
    center = np.array([0.5, 0.5, 0.5]) * one_Gpc
    ms = SchwarzschildMetricFast(M, 3 * one_Mpc, center=center, coords="spherical", analytical_geodesics=True)
    obs = np.array([0.01, 0.01, 0.01]) * one_Gpc
    o_sph = np.array([0.0, *cartesian_to_spherical(*(obs - center))])
    ph3 = Photons(ms)
    ph3.generate_cone_grid(n_photons=36, origin=o_sph, central_direction=center - obs, cone_angle=np.deg2rad(2),
                           direction_basis="cartesian")
    schw_cone = np.array([np.concatenate([p.x, p.u]) for p in ph3.photons])
    schw_null = np.array([p.null_condition_relative_error(ms) for p in ph3.photons])
    ph6 = Photons(ms)
    with contextlib.redirect_stdout(io.StringIO()):
        ph6.generate_cone_grid_metric_tensor(n_photons=(4, 9), origin=o_sph, central_direction=center - obs,
                                             cone_angle=np.deg2rad(2), direction_basis="cartesian")
    schw_cone_mt = np.array([np.concatenate([p.x, p.u]) for p in ph6.photons])
    ph4 = Photons(ms)
    ph4.generate_impact_parameter_bins(o_sph, center - obs, np.linspace(0.5, 10, 3) * one_Mpc, 4, seed=0)
    schw_bins = np.array([np.concatenate([p.x, p.u]) for p in ph4.photons])
    vecs = np.random.default_rng(4).standard_normal((20, 3))
    targets = np.random.default_rng(5).standard_normal((20, 3))
    targets[0] = [0, 0, 1]
    targets[1] = [0, 0, -2]
    rot = np.array([ph._rotate_to_direction(v, t) for v, t in zip(vecs, targets)])
    save("generators.npz", field=data, box=box, flrw_origin=origin, flrw_cone=flrw_cone, flrw_null=flrw_null,
         flrw_bins=flrw_bins, schw_origin=o_sph, schw_center=center, schw_cone=schw_cone, schw_null=schw_null,
         schw_bins=schw_bins, rot_vecs=vecs, rot_targets=targets, rot_out=rot, flrw_cone_mt=flrw_cone_mt,
         schw_cone_mt=schw_cone_mt, flrw_cone_random=flrw_cone_random)


# ------------------------------------------------------------ observables
def gen_observables(cz):
    pp = _load_postprocessing()
    rng = np.random.default_rng(77)
    # a smooth FLRW-like trajectory with 14 columns
    n = 60
    eta = cz._eta_at_a1 - np.linspace(0, 3e16, n)
    xyz = np.cumsum(rng.normal(1.5e22, 1e19, (n, 3)), axis=0)
    u = np.column_stack([-np.ones(n), np.tile([c * 0.6, c * 0.64, c * 0.48], (n, 1))])
    a = np.array([cz.a_of_eta(e) for e in eta])
    phi = rng.normal(0, 1e11, n)
    grad = rng.normal(0, 1e-3, (n, 3))
    phid = rng.normal(0, 1e-7, n)
    traj = np.column_stack([eta, xyz, u, a, phi, grad, phid])
    rc = RedshiftCalculator(traj).compute_all_components()
    red = np.array([rc["z_H"], rc["z_SW"], rc["z_ISW"], rc["z_D"], rc["z_total"], rc["z_total_exact"]])
    cart = pp._trajectory_stats(traj, None, is_spherical=False)
    lens = np.array([5.0, 6.0, 7.0]) * 1e24
    sph = np.column_stack([np.linspace(0, 1e16, n), np.linspace(1e25, 2e25, n),
                           np.linspace(1.2, 1.3, n), np.linspace(-0.5, 0.7, n),
                           -np.ones(n), rng.normal(c, 1e3, n), rng.normal(0, 1e-17, n), rng.normal(0, 1e-17, n)])
    sphs = pp._trajectory_stats(sph, lens, is_spherical=True)
    stats = lambda s: np.array([s.n_records, s.finite_fraction, s.path_length, s.min_r, s.final_r,
                                s.bending_angle_rad, s.speed_mean, s.speed_max])
    # compute_time_delay_map.compute_travel_time_deflected (restated: that module imports h5py/matplotlib)
    pos = traj[:, 1:4]
    path = 0.0
    for i in range(len(pos) - 1):
        path += np.linalg.norm(pos[i + 1] - pos[i])
    delay = path / c - np.linalg.norm(pos[-1] - pos[0]) / c
    theory = pp._deflection_theory_per_photon(np.array([1e22, 2e23, -1.0, np.nan]), 1e15 * one_Msun)
    save("observables.npz", traj=traj, redshift=red, stats_cart=stats(cart), traj_sph=sph, lens=lens,
         stats_sph=stats(sphs), path=path, delay=delay, theory=theory)


# --------------------------------------------- comparison runner (one sweep job)
# The job behind the reference's committed per-run table results_test/per_run/job_00001.csv,
# whose command line is in results_test/logs/job_00001_runner.log.
COMPARE_JOB_ARGV = ["--mass-msun", "20000000000000.0", "--distance-mpc", "500.0", "--flrw-grid-N", "128",
                    "--progress-every", "0", "--record-every", "4", "--sampling", "cone", "--n-photons", "400",
                    "--cone-angle-deg", "10.0", "--static", "--flrw-local-coords"]
COMPARE_KEEP = [1, 40, 97, 190, 300, 380]     # photons whose whole trajectories are kept


def gen_compare_job():
    """Run the reference's comparison runner (excalibur_run_compare_schwarzschild_vs_flrw.py) on
    job 1's command line, capture each photon's initial state as the runner hands it to
    integrate_single, and reduce both trajectory files with the reference's analyzer
    (analyze_compare_trajectories._trajectory_stats). Also keeps the reference's committed CSV
    of the same job (produced on the author's machine with numba's fastmath) for comparison."""
    import contextlib
    import hashlib
    import io
    import tempfile

    pp = _load_postprocessing()
    runner = _load_file("compare_runner", "_excalibur_runs", "excalibur_run_compare_schwarzschild_vs_flrw.py")
    inits, phis = {}, []
    orig_integrate_all, orig_add = runner._integrate_all, runner.Grid.add_field

    def capture(photons, integrator, n_steps, **kw):
        inits[kw["label"]] = np.array([np.concatenate([p.x, p.u]) for p in photons.photons])
        return orig_integrate_all(photons, integrator, n_steps, **kw)

    def add_field(self, name, data):
        phis.append(np.asarray(data))
        return orig_add(self, name, data)

    runner._integrate_all = capture
    runner.Grid.add_field = add_field
    with tempfile.TemporaryDirectory() as tmp:
        old = sys.argv
        sys.argv = ["runner", *COMPARE_JOB_ARGV, "--output-dir", tmp]
        out = io.StringIO()
        try:
            with contextlib.redirect_stdout(out):
                runner.main()
        finally:
            sys.argv = old
            runner._integrate_all, runner.Grid.add_field = orig_integrate_all, orig_add
        text = out.getvalue()
        s_h5 = text.split("Schwarzschild ->")[1].splitlines()[0].strip()
        f_h5 = text.split("FLRW          ->")[1].splitlines()[0].strip()
        s_tr, _ = pp._load_trajectories(s_h5.replace(".h5", ".npz"))
        f_tr, _ = pp._load_trajectories(f_h5.replace(".h5", ".npz"))
    lens = np.asarray(pp.parse_trajectory_filename(s_h5)["mass_position_m"], dtype=float)

    def stats(tr, sph):
        rows = []
        for i in range(tr.shape[0]):
            st = pp._trajectory_stats(tr[i], lens, is_spherical=sph)
            rows.append([st.n_records, st.finite_fraction, st.path_length, st.min_r, st.final_r,
                         st.bending_angle_rad, st.speed_mean, st.speed_max])
        return np.array(rows)

    csv_ref = np.loadtxt(os.path.join(REF, "results_test", "per_run", "job_00001.csv"), delimiter=",", skiprows=1)
    phi = phis[0]
    save("compare_job1.npz", argv=np.array(COMPARE_JOB_ARGV), lens_center=lens,
         schw_init=inits["Schwarzschild"], flrw_init=inits["FLRW"],
         schw_stats=stats(s_tr, True), flrw_stats=stats(f_tr, False),
         keep=np.array(COMPARE_KEEP), schw_traj=s_tr[COMPARE_KEEP], flrw_traj=f_tr[COMPARE_KEEP],
         n_records=np.array(s_tr.shape[1]), phi_sha256=np.array(hashlib.sha256(phi.tobytes()).hexdigest()),
         phi_shape=np.array(phi.shape), csv_author=csv_ref)


def gen_manifest():
    """The reference's manifest writer (make_manifest.py) on a small sweep, both sampling modes."""
    import subprocess
    import tempfile

    script = os.path.join(REF, "_simulations", "_schwarzschild_vs_flrw", "make_manifest.py")
    runs = {
        "manifest_cone.csv": ["--masses", "1e13,2e13", "--distances", "300,500", "--Ns", "64,128",
                              "--sampling", "cone", "--cone-nphotons", "100", "--cone-angle-deg", "5",
                              "--integrators", "rk4,leapfrog4", "--seed0", "7"],
        "manifest_impact.csv": ["--masses", "1e14", "--distances", "200,400", "--Ns", "96",
                                "--b-min", "0.5", "--b-max", "2.5", "--b-nbins", "4", "--b-nperbin", "30",
                                "--radii-mpc", "2,3", "--static", "0", "--record-every", "8"],
    }
    for name, argv in runs.items():
        with tempfile.TemporaryDirectory() as tmp:
            out = os.path.join(tmp, name)
            subprocess.run([sys.executable, script, "--out", out, *argv], check=True, capture_output=True)
            with open(out) as f, open(os.path.join(HERE, name), "w") as g:
                g.write(f.read())
        print(f"wrote {name}")
    with open(os.path.join(HERE, "manifest_args.txt"), "w") as g:
        for name, argv in runs.items():
            g.write(name + " " + " ".join(argv) + "\n")


# ------------------------------------------------------------ time-delay map
def _time_delay_records(rng, n_photons=36, n_rows=48):
    """NaN-padded FLRW record blocks [n, rows, 14] in SI units: ragged lengths (0, 1, 2, 3 rows
    first), a NaN hole, and photons the time-delay loader rejects (a position at 1e26 m, a time at
    3e18 s, an infinite position) or keeps at the edge (just below both limits)."""
    rec = np.full((n_photons, n_rows, 14), np.nan)
    for i in range(n_photons):
        m = i if i < 4 else (n_rows if i < 10 else int(rng.integers(2, n_rows + 1)))
        start = rng.uniform(1e24, 2e24, 3)
        steps = rng.normal(0, 2e20, (m, 3)) + np.array([-1.5e22, 0, 0])
        rec[i, :m, 0] = 4.6e17 - np.arange(m) * 5e13
        rec[i, :m, 1:4] = start + np.cumsum(steps, axis=0)
        rec[i, :m, 4] = -1.0
        rec[i, :m, 5:8] = np.array([-3e8, 0, 0]) + rng.normal(0, 1e5, 3)
        rec[i, :m, 8] = 1.0 / (1.0 + np.linspace(0, 0.2, m))
        rec[i, :m, 9:14] = rng.normal(0, 1e-6, (m, 5))
        if m > 8 and i % 7 == 0:
            rec[i, m // 2, 2] = np.nan
    rec[5, 3, 1] = 1e26
    rec[6, 2, 0] = 3e18
    rec[7, 4, 3] = -np.inf
    rec[8, 1, 2] = np.nextafter(1e26, 0)
    rec[8, 1, 0] = np.nextafter(3e18, 0)
    return rec


def gen_time_delays():
    """compute_time_delay_map.py's own loader and compute_time_delays on synthetic record blocks.
    The module imports h5py and matplotlib at the top (both absent here): stand-in modules serve
    the blocks as a trajectory file and give matplotlib's names, which these functions never call."""
    import types

    rec = _time_delay_records(np.random.default_rng(21))
    files = {"records.h5": rec}

    class _File:
        def __init__(self, name, mode="r"):
            self._rec = files[name]
            self.attrs = {"n_photons": len(self._rec)}

        def __enter__(self):
            return self

        def __exit__(self, *exc):
            return False

        def __contains__(self, key):
            return key.startswith("photon_") and key.endswith("_states")

        def __getitem__(self, key):
            return self._rec[int(key.split("_")[1])]

    h5 = types.ModuleType("h5py")
    h5.File = _File
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    colors = types.ModuleType("matplotlib.colors")
    colors.TwoSlopeNorm = object
    mpl.pyplot, mpl.colors = plt, colors
    saved = {k: sys.modules.get(k) for k in ("h5py", "matplotlib", "matplotlib.pyplot", "matplotlib.colors")}
    sys.modules.update({"h5py": h5, "matplotlib": mpl, "matplotlib.pyplot": plt, "matplotlib.colors": colors})
    try:
        td = _load_file("compute_time_delay_map", "_postprocessing", "compute_time_delay_map.py")
        import contextlib
        import io

        with contextlib.redirect_stdout(io.StringIO()):
            trajs, meta = td.load_trajectories("records.h5")
        delays, dd, ds, (xp, yp) = td.compute_time_delays(trajs, meta)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    # which photons the loader kept, by their first clean row
    firsts = [t[0] for t in trajs]
    kept = np.array([any(len(b := r[~np.isnan(r).any(axis=1)]) and np.array_equal(b[0], f) for f in firsts)
                     for r in rec])
    save("time_delays.npz", records=rec, kept=kept, time_delays=np.asarray(delays),
         distances_deflected=np.asarray(dd), distances_straight=np.asarray(ds), x_proj=xp, y_proj=yp)


# ------------------------------------------------------------ lens mass profiles
def gen_objects():
    """The uniform sphere and the NFW halo of objects/spherical_mass.py: density, potential,
    enclosed mass and containment at points inside, outside and at the centre."""
    sm = _load_file("excalibur_spherical_mass", "excalibur", "objects", "spherical_mass.py")
    centre = np.array([0.5, 0.5, 0.5]) * one_Gpc
    rng = np.random.default_rng(21)
    pts = centre + rng.normal(0.0, 8.0, (64, 3)) * one_Mpc
    pts[0] = centre
    x, y, z = (v.reshape(8, 8) for v in pts.T)      # 2-D: broadcast point by point, no meshgrid
    u = sm.spherical_mass(3e14 * one_Msun, 6 * one_Mpc, centre)
    h = sm.spherical_mass_nfw(1e15 * one_Msun, 2 * one_Mpc, 5.0, centre)
    save("objects.npz", pts=pts, u_mass=u.mass, u_radius=u.radius, u_density=u.density(x, y, z),
         u_potential=u.potential(x, y, z), u_mass_enclosed=u.mass_enclosed(x, y, z), u_contains=u.contains(x, y, z),
         h_mass=h.mass, h_radius=h.radius, h_concentration=h.concentration, h_rho0=h.rho0,
         h_density=h.density(x, y, z), h_potential=h.potential(x, y, z),
         h_mass_enclosed=h.mass_enclosed(x[1:], y[1:], z[1:]), h_contains=h.contains(x, y, z),
         u_grid_axes=pts[:4].T, u_grid_potential=u.potential(*pts[:4].T), u_grid_mass=u.mass_enclosed(*pts[:4].T))


# ------------------------------------------------------------ coordinate conversions
def gen_coordinates():
    """The six conversions of core/coordinates.py on seeded points (the poles and the axis among
    them), velocities, and radii around a Schwarzschild radius."""
    import excalibur.core.coordinates as co
    rng = np.random.default_rng(31)
    xyz = rng.normal(0.0, 1.0, (40, 3)) * one_Mpc
    xyz[0] = [0.0, 0.0, 2.0 * one_Mpc]
    xyz[1] = [0.0, 0.0, -3.0 * one_Mpc]
    xyz[2] = [1.0 * one_Mpc, 0.0, 0.0]
    v = rng.normal(0.0, 1.0, (40, 3)) * c
    sph = np.array(co.cartesian_to_spherical(*xyz.T))
    back = np.array(co.spherical_to_cartesian(*sph))
    vsph = np.array([co.cartesian_velocity_to_spherical(*xyz[i], *v[i]) for i in range(3, 40)])
    rs = 2 * G * 1e15 * one_Msun / c ** 2
    r = np.linspace(1.01, 50.0, 25) * rs
    iso = np.array(co.spherical_to_isotropic_radius(r, rs))
    sch = np.array(co.isotropic_to_spherical_radius(iso, rs))
    centre = np.array([0.5, 0.5, 0.5]) * one_Gpc
    pts = centre + rng.normal(0.0, 10.0, (20, 3)) * one_Mpc
    iso_xyz = np.array(co.cartesian_to_isotropic_radius(pts[:, 0], pts[:, 1], pts[:, 2], centre, rs))
    save("coordinates.npz", xyz=xyz, v=v, sph=sph, back=back, vsph=vsph, rs=rs, r=r, iso=iso, sch=sch,
         centre=centre, pts=pts, iso_xyz=iso_xyz)


GENERATORS = ["cosmology", "interp", "interp_slow", "rhs", "steps", "integrate", "integrate_modes", "generators",
              "observables", "flrw_patch_32", "schw_polar", "compare_job", "manifest", "time_delays",
              "integrate_lf4", "rk45_slow", "schw_steppers", "objects", "coordinates"]

if __name__ == "__main__":
    if not os.path.isdir(REF):
        sys.exit(f"reference checkout not found at {REF}")
    np.seterr(all="ignore")
    which = sys.argv[1:] or GENERATORS
    cz = gen_cosmology() if "cosmology" in which else None
    if cz is None and set(which) & {"interp_slow", "rhs", "steps", "integrate", "integrate_modes", "generators",
                                    "observables", "flrw_patch_32", "integrate_lf4", "rk45_slow"}:
        cz = LCDM_Cosmology(70, 0.3, 0.0, 0.7)
    for name in which:
        if name == "cosmology":
            continue
        fn = globals()["gen_" + name]
        fn(cz) if name in ("interp_slow", "rhs", "steps", "integrate", "integrate_modes", "generators",
                           "observables", "flrw_patch_32", "integrate_lf4", "rk45_slow") else fn()
