"""The reference's own CPU paths, timed: `Integrator(mode="chunked")` and its multiprocessing pool,
and (--persistent) its `PersistentPoolIntegrator`.

Measurement infrastructure: only bench.py's CPU-baseline leg and its `--impl reference` arm run
this, as a process of its own (the pool forks, so the parent must not have touched CUDA). It
imports the UNMODIFIED reference package installed under baseline/_ref (`pip install --target`);
when numba is not importable there it puts the no-op `numba` stand-in of oracle/shim first on
the path, so the reference's `@njit` kernels run as plain Python (and says so in its output).

What is timed is the reference's public path for the flrw_patch workload
(excalibur/integration/integrator.py:452-473): the Φ grid in `Grid` + `InterpolatorFast`
(periodic), `LCDM_Cosmology(70, 0.3, 0, 0.7)`, `PerturbedFLRWMetricFast` with the cosmology's
analytic ȧ, a `Photons` collection of the given initial states, then
`Integrator(metric, dt, mode="chunked", integrator="rk4", dt_min=dt, dt_max=dt,
n_workers=..., chunk_size=...).integrate(photons, "steps", n_steps)` -- pool start-up, pickling,
RK4 and the per-step history records of `integrate_single` included, the metric and grid
construction excluded. The reference has no box-exit stop, so every photon takes `n_steps`
steps (the grid is periodic).

    python oracle/reference_pool.py --inputs IN.npz --out OUT.json [--workers N] [--chunk-size K] [--persistent]

IN.npz: phi [n, n, n] float64 (SI), box (m), states [N, 8], dt (s), n_steps.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _import_reference(ref_dir):
    """Put the installed reference first on the path; the numba stand-in only when the real
    numba cannot be imported. Returns (numba_importable, how the reference's kernels ran)."""
    try:
        import numba  # noqa: F401

        have = True
    except Exception:
        have = False
    sys.path.insert(0, ref_dir)
    if not have:
        sys.path.insert(1, os.path.join(HERE, "shim"))
    return have, ("numba" if have else "plain Python (no-op numba stand-in; numba not importable)")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--inputs", required=True)
    ap.add_argument("--out", required=True)
    ap.add_argument("--ref-dir", default=os.path.join(REPO, "baseline", "_ref"))
    ap.add_argument("--workers", type=int, default=0, help="0: os.cpu_count()")
    ap.add_argument("--chunk-size", type=int, default=0, help="0: photons / workers, rounded up")
    ap.add_argument("--persistent", action="store_true",
                    help="also time PersistentPoolIntegrator (parallel_integrator_persistent.py) on the same photons")
    args = ap.parse_args(argv)
    if not os.path.isdir(os.path.join(args.ref_dir, "excalibur")):
        raise SystemExit(f"reference package not installed under {args.ref_dir}")
    have_numba, kernels = _import_reference(args.ref_dir)

    import numpy as np
    from excalibur.core.cosmology import LCDM_Cosmology
    from excalibur.grid.grid import Grid
    from excalibur.grid.interpolator_4d_fast import InterpolatorFast
    from excalibur.integration.integrator import Integrator
    from excalibur.metrics.perturbed_flrw_metric_fast import PerturbedFLRWMetricFast
    from excalibur.photon.photon import Photon
    from excalibur.photon.photons import Photons

    d = np.load(args.inputs)
    phi, box, states = d["phi"], float(d["box"]), d["states"]
    dt, n_steps = float(d["dt"]), int(d["n_steps"])
    n = phi.shape[0]
    t_setup = time.perf_counter()
    cz = LCDM_Cosmology(70, 0.3, 0.0, 0.7)
    g = Grid((n, n, n), (box / n,) * 3, (0.0, 0.0, 0.0))
    g.add_field("Phi", phi)
    ip = InterpolatorFast(g, boundary="periodic")
    metric = PerturbedFLRWMetricFast(cz.a_of_eta, g, ip, adot_of_eta=cz.adot_of_eta)
    photons = Photons(metric)
    for s in states:
        photons.photons.append(Photon(s[:4].copy(), s[4:].copy()))
    t_setup = time.perf_counter() - t_setup
    workers = args.workers or os.cpu_count() or 1
    chunk = args.chunk_size or max(1, -(-len(states) // workers))
    integ = Integrator(metric, dt=dt, mode="chunked", integrator="rk4", dt_min=dt, dt_max=dt,
                       n_workers=workers, chunk_size=chunk)
    t0 = time.perf_counter()
    ok = integ.integrate(photons, "steps", n_steps, verbose=False)
    wall = time.perf_counter() - t0
    # the "steps" stop: every photon that did not raise took exactly n_steps accepted steps
    steps = int(ok) * n_steps
    persistent = _time_persistent(metric, states, dt, n_steps, workers, chunk, Photons, Photon) \
        if args.persistent else None
    try:
        affinity = len(os.sched_getaffinity(0))
    except AttributeError:
        affinity = None
    out = {"photon_steps_per_s": steps / wall, "rays_per_s": ok / wall, "seconds": wall,
           "photons": int(len(states)), "succeeded": int(ok), "photon_steps": steps, "steps_per_photon": n_steps,
           "workers": workers, "chunk_size": chunk, "os_cpu_count": os.cpu_count(), "affinity": affinity,
           "numba_importable": have_numba, "kernels": kernels, "setup_s": t_setup,
           "python": platform.python_version(), "numpy": np.__version__, "machine": platform.machine(),
           "path": "excalibur.integration.integrator.Integrator(mode='chunked', integrator='rk4').integrate "
                   "(multiprocessing.Pool, fork), reference installed under baseline/_ref"}
    if persistent is not None:
        out["persistent_pool"] = persistent
    with open(args.out, "w") as f:
        json.dump(out, f)


def _time_persistent(metric, states, dt, n_steps, workers, chunk, Photons, Photon):
    """The reference's PersistentPoolIntegrator (excalibur/integration/parallel_integrator_persistent.py:
    130-336): a pool whose workers each rebuild the grid, interpolator_fast.InterpolatorFast and a
    PerturbedFLRWMetricFast with its finite-difference adot once at pool start (not timed), then
    integrate_photons_chunked -> integrator_old.Integrator.integrate(photon, n_steps) per photon
    (timed). Its arithmetic differs from Integrator's (no dt clip, the FD adot, the legacy
    interpolator's strict interior), so it is a rate, not a parity reference. That interpolator
    raises on the grid's outer cells, where the batch's observer sits (x = 0), and the worker
    evaluates the metric before its own try block, so each photon starts two cells further along
    its ray. Steps are counted from the returned history lengths (one record before the first step
    and one per step)."""
    import contextlib
    import io

    import numpy as np
    from excalibur.integration.parallel_integrator_persistent import PersistentPoolIntegrator

    cell = float(np.max(metric.grid.spacing))
    photons = Photons(metric)
    for s in states:
        x = s[:4].copy()
        d = s[5:8] / np.linalg.norm(s[5:8])
        x[1:4] += 2.0 * cell * d
        photons.photons.append(Photon(x, s[4:].copy()))
    t0 = time.perf_counter()
    with contextlib.redirect_stdout(io.StringIO()):
        pool = PersistentPoolIntegrator(metric, dt, n_workers=workers)
    t_start = time.perf_counter() - t0
    try:
        t1 = time.perf_counter()
        with contextlib.redirect_stdout(io.StringIO()):
            n_ok, results = pool.integrate_photons_chunked(photons, n_steps, chunk_size=chunk, verbose=False)
        wall = time.perf_counter() - t1
    finally:
        pool.close()
    steps = int(sum(max(int(r[3]) - 1, 0) for r in results))
    return {"photon_steps_per_s": steps / wall, "seconds": wall, "pool_start_s": t_start, "succeeded": int(n_ok),
            "photon_steps": steps, "workers": workers, "chunk_size": chunk,
            "path": "excalibur.integration.parallel_integrator_persistent.PersistentPoolIntegrator"
                    ".integrate_photons_chunked (multiprocessing.Pool, fork; workers built once)"}


if __name__ == "__main__":
    main()
