"""Parameter sweeps of comparison runs: manifest rows -> batched GPU launches -> per-run CSVs.

The reference runs a sweep as one 1-core Slurm task per manifest row
(_simulations/_schwarzschild_vs_flrw/run_array.slurm:1-19): `run_one_job.py` (:43-243) reads
row `jobid`, runs the comparison runner on it as a subprocess, runs the analyzer on the two
trajectory files it wrote and leaves `results/per_run/job_NNNNN.csv`. The manifest comes from
`make_manifest.py` (:43-249): the product masses x distances x Ns x radii x integrators
(x impact-parameter bins), one row each.

Here the same manifest and the same per-run tables come out of a handful of launches:
* `make_manifest` writes the reference's manifest byte for byte (same columns, order, seeds);
* `read_jobs` / `read_job` read it with run_one_job's defaults for absent columns;
* `job_config` maps a row onto the runner's options exactly as run_one_job builds its
  command line (impact rows pass --n-photons b_nperbin; cone rows their cone options);
* `run_sweep` groups rows whose FLRW legs share every launch-wide setting -- integrator,
  step count, step size, record cadence, cosmology, interpolator -- and traces up to
  EXC_MAX_FIELDS rows' FLRW legs in one persistent launch, each row's potential a separate
  field (built on the device by exc_spherical_mass_grid) with its own observer shift, photons
  tagged with their row's field index. The Schwarzschild legs (one metric per row) are
  launched back to back on the same stream with no host synchronisation between them.
  Every photon's arithmetic is the same as in a run of its own row, so the tables equal
  those of row-by-row runs bit for bit.
"""
from __future__ import annotations

import csv
import dataclasses
import os
from typing import Iterable, List, Optional

import numpy as np

from .. import _native as N
from .analyze import write_per_run_csv
from . import compare as R

IMPACT_HEADER = ["jobid", "mass_msun", "radius_mpc", "distance_mpc", "integrator", "flrw_grid_N", "bin_id",
                 "b_min_mpc", "b_max_mpc", "b_nbins", "b_nperbin", "static", "local", "record_every",
                 "progress_every", "renormalize_every", "n_steps", "steps_per_cell", "flrw_grid_size_mpc", "seed"]
CONE_HEADER = ["jobid", "mass_msun", "radius_mpc", "distance_mpc", "integrator", "flrw_grid_N", "cone_angle_deg",
               "cone_nphotons", "static", "local", "record_every", "progress_every", "renormalize_every", "n_steps",
               "steps_per_cell", "flrw_grid_size_mpc", "seed"]


def _parse_list(s: str) -> List[float]:
    return [float(x.strip()) for x in s.split(",") if x.strip()]


def _parse_str_list(s: str) -> List[str]:
    return [x.strip() for x in s.split(",") if x.strip()]


def make_manifest(out: str, *, masses: str, distances: str, Ns: str, radius_mpc: float = 3.0,
                  integrator: str = "rk4", radii_mpc: Optional[str] = None, integrators: Optional[str] = None,
                  sampling: str = "impact", b_min: Optional[float] = None, b_max: Optional[float] = None,
                  b_nbins: int = 10, cone_angle_deg: float = 10.0, cone_nphotons: int = 200,
                  b_nperbin: int = 200, static: int = 1, local: int = 1, seed0: int = 0, record_every: int = 4,
                  progress_every: int = 0, renormalize_every: int = 0, n_steps: int = 5000,
                  steps_per_cell: float = 3.0, flrw_grid_size_mpc: float = 1000.0) -> int:
    """make_manifest.py's main() (:43-249) with its option names and defaults; the list options
    are its comma-separated strings. Returns the number of rows written."""
    m_list, d_list = _parse_list(masses), _parse_list(distances)
    n_list = [int(x) for x in _parse_list(Ns)]
    r_list = _parse_list(radii_mpc) if radii_mpc else [float(radius_mpc)]
    i_list = _parse_str_list(integrators) if integrators else [str(integrator)]
    os.makedirs(os.path.dirname(out) or ".", exist_ok=True)
    jobid = 0
    if sampling == "impact":
        if b_min is None or b_max is None:
            raise ValueError("impact sampling needs b_min and b_max")
        edges = np.linspace(b_min, b_max, b_nbins + 1)
        if b_max <= b_min:
            raise SystemExit("b-max must be > b-min")
        with open(out, "w", newline="") as fp:
            w = csv.writer(fp)
            w.writerow(IMPACT_HEADER)
            for m in m_list:
                for d in d_list:
                    for n in n_list:
                        for r in r_list:
                            for integ in i_list:
                                for bin_id in range(b_nbins):
                                    w.writerow([jobid, m, r, d, integ, n, bin_id, float(edges[bin_id]),
                                                float(edges[bin_id + 1]), 1, b_nperbin, static, local, record_every,
                                                progress_every, renormalize_every, n_steps, steps_per_cell,
                                                flrw_grid_size_mpc, int(seed0 + jobid)])
                                    jobid += 1
    elif sampling == "cone":
        with open(out, "w", newline="") as fp:
            w = csv.writer(fp)
            w.writerow(CONE_HEADER)
            for m in m_list:
                for d in d_list:
                    for n in n_list:
                        for r in r_list:
                            for integ in i_list:
                                w.writerow([jobid, m, r, d, integ, n, cone_angle_deg, cone_nphotons, static, local,
                                            record_every, progress_every, renormalize_every, n_steps,
                                            steps_per_cell, flrw_grid_size_mpc, int(seed0 + jobid)])
                                jobid += 1
    else:
        raise ValueError("sampling must be 'impact' or 'cone'")
    return jobid


def manifest_main(argv=None) -> int:
    """make_manifest.py's command line (same option names and defaults)."""
    import argparse

    p = argparse.ArgumentParser(description="Write a comparison-sweep manifest CSV")
    p.add_argument("--out", required=True)
    p.add_argument("--masses", required=True)
    p.add_argument("--distances", required=True)
    p.add_argument("--Ns", required=True)
    p.add_argument("--radius-mpc", type=float, default=3.0)
    p.add_argument("--integrator", default="rk4", choices=["rk4", "rk45", "leapfrog4"])
    p.add_argument("--radii-mpc", default=None)
    p.add_argument("--integrators", default=None)
    p.add_argument("--sampling", default="impact", choices=["impact", "cone"])
    p.add_argument("--b-min", type=float, required=False)
    p.add_argument("--b-max", type=float, required=False)
    p.add_argument("--b-nbins", type=int, default=10)
    p.add_argument("--cone-angle-deg", type=float, default=10.0)
    p.add_argument("--cone-nphotons", type=int, default=200)
    p.add_argument("--b-nperbin", type=int, default=200)
    p.add_argument("--static", type=int, default=1, choices=[0, 1])
    p.add_argument("--local", type=int, default=1, choices=[0, 1])
    p.add_argument("--seed0", type=int, default=0)
    p.add_argument("--record-every", type=int, default=4)
    p.add_argument("--progress-every", type=int, default=0)
    p.add_argument("--renormalize-every", type=int, default=0)
    p.add_argument("--n-steps", type=int, default=5000)
    p.add_argument("--steps-per-cell", type=float, default=3.0)
    p.add_argument("--flrw-grid-size-mpc", type=float, default=1000.0)
    a = p.parse_args(argv)
    n = make_manifest(a.out, masses=a.masses, distances=a.distances, Ns=a.Ns, radius_mpc=a.radius_mpc,
                      integrator=a.integrator, radii_mpc=a.radii_mpc, integrators=a.integrators,
                      sampling=a.sampling, b_min=a.b_min, b_max=a.b_max, b_nbins=a.b_nbins,
                      cone_angle_deg=a.cone_angle_deg, cone_nphotons=a.cone_nphotons, b_nperbin=a.b_nperbin,
                      static=a.static, local=a.local, seed0=a.seed0, record_every=a.record_every,
                      progress_every=a.progress_every, renormalize_every=a.renormalize_every,
                      n_steps=a.n_steps, steps_per_cell=a.steps_per_cell,
                      flrw_grid_size_mpc=a.flrw_grid_size_mpc)
    print(f"Wrote {n} jobs to {a.out}")
    return n


@dataclasses.dataclass
class Job:
    """run_one_job.Job (:31-56): one manifest row with the runner's defaults."""
    jobid: int
    mass_msun: float
    distance_mpc: float
    flrw_grid_N: int
    radius_mpc: float = 3.0
    integrator: str = "rk4"
    sampling: str = "cone"
    cone_nphotons: int = 200
    cone_angle_deg: float = 10.0
    bin_id: int = 0
    b_min_mpc: float = 0.0
    b_max_mpc: float = 0.0
    b_nbins: int = 0
    b_nperbin: int = 0
    static: int = 1
    local: int = 1
    record_every: int = 4
    progress_every: int = 0
    renormalize_every: int = 0
    n_steps: int = 5000
    steps_per_cell: float = 3.0
    flrw_grid_size_mpc: float = 1000.0
    seed: int = 0


def _job_from_row(row: dict) -> Job:
    """read_job's parsing (:59-120): the impact columns decide the row kind."""
    common = dict(jobid=int(row["jobid"]), mass_msun=float(row["mass_msun"]),
                  radius_mpc=float(row.get("radius_mpc", 3.0) or 3.0), distance_mpc=float(row["distance_mpc"]),
                  flrw_grid_N=int(row["flrw_grid_N"]), integrator=str(row.get("integrator", "rk4") or "rk4"),
                  sampling=row.get("sampling", "cone"), cone_nphotons=int(row.get("cone_nphotons", 200)),
                  cone_angle_deg=float(row.get("cone_angle_deg", 10.0)), static=int(row.get("static", 1)),
                  local=int(row.get("local", 1)), record_every=int(row.get("record_every", 4) or 4),
                  progress_every=int(row.get("progress_every", 0) or 0),
                  renormalize_every=int(row.get("renormalize_every", 0) or 0),
                  n_steps=int(row.get("n_steps", 5000) or 5000),
                  steps_per_cell=float(row.get("steps_per_cell", 3.0) or 3.0),
                  flrw_grid_size_mpc=float(row.get("flrw_grid_size_mpc", 1000.0) or 1000.0),
                  seed=int(row.get("seed", 0)))
    if all(k in row for k in ("b_min_mpc", "b_max_mpc", "b_nbins", "b_nperbin")):
        common.update(bin_id=int(row.get("bin_id", 0)), b_min_mpc=float(row.get("b_min_mpc", 0.0)),
                      b_max_mpc=float(row.get("b_max_mpc", 0.0)), b_nbins=int(row.get("b_nbins", 0)),
                      b_nperbin=int(row.get("b_nperbin", 0)))
    return Job(**common)


def read_jobs(manifest: str) -> List[Job]:
    with open(manifest, newline="") as fp:
        return [_job_from_row(row) for row in csv.DictReader(fp)]


def read_job(manifest: str, jobid: int) -> Job:
    for job in read_jobs(manifest):
        if job.jobid == int(jobid):
            return job
    raise SystemExit(f"jobid={jobid} not found in {manifest}")


def job_config(job: Job, output_dir: str = os.path.join("_data", "output")) -> R.RunConfig:
    """The runner's RunConfig for `job`, i.e. what run_one_job's command line (:176-232) parses to.
    Impact rows set --sampling impact, their bin and --n-photons b_nperbin; cone rows their
    cone size and angle. A row that is neither has the runner's defaults for those."""
    kw = dict(mass_msun=float(str(job.mass_msun)), radius_mpc=float(str(job.radius_mpc)),
              distance_mpc=float(str(job.distance_mpc)), integrator=str(job.integrator),
              flrw_grid_N=int(job.flrw_grid_N), output_dir=output_dir, progress_every=int(job.progress_every),
              record_every=int(job.record_every), renormalize_every=int(job.renormalize_every),
              n_steps=int(job.n_steps), steps_per_cell=float(str(job.steps_per_cell)),
              flrw_grid_size_mpc=float(str(job.flrw_grid_size_mpc)), static=bool(job.static),
              flrw_local_coords=bool(job.local))
    if str(job.sampling).lower() == "impact":
        kw.update(sampling="impact", b_min_mpc=float(str(job.b_min_mpc)), b_max_mpc=float(str(job.b_max_mpc)),
                  b_nbins=int(job.b_nbins), b_nperbin=int(job.b_nperbin), n_photons=int(job.b_nperbin))
    else:
        kw.update(sampling="cone", n_photons=int(job.cone_nphotons), cone_angle_deg=float(str(job.cone_angle_deg)))
    return R.run_config(**kw)


def _flrw_key(cfg: R.RunConfig, geo: R.RunGeometry):
    # everything a launch shares: ExcTraceArgs fields and the ExcMetric header
    return (cfg.integrator, geo.n_steps, geo.dlambda, cfg.record_every, cfg.renormalize_every, cfg.static,
            cfg.flrw_fast, cfg.flrw_grid_N, cfg.flrw_grid_size)


@dataclasses.dataclass
class _Prepared:
    job: Job
    cfg: R.RunConfig
    geo: R.RunGeometry
    s_metric: object
    s_states: object
    s_dt: tuple
    f_metric: object
    f_states: object
    shift: Optional[np.ndarray]
    checks: list


def _prepare(job: Job, impact_runner: bool) -> _Prepared:
    # no host synchronisation here: the generators' checks wait for the wave's end
    cfg = job_config(job)
    geo = R.geometry(cfg)
    checks = []
    sm, ss, dmin, dmax = R.schwarzschild_setup(cfg, geo, impact_runner, checks=checks)
    fm, fs, shift = R.flrw_setup(cfg, geo, impact_runner, checks=checks)
    return _Prepared(job, cfg, geo, sm, ss, (dmin, dmax), fm, fs, shift, checks)


def _split_leg(res, lo, hi, x_offset, *, empty_failed, fail_on_error, label):
    """One row's slice [lo, hi) of a (possibly shared) trace result, as a stacked array."""
    sub = dataclasses.replace(res, state=res.state[lo:hi], status=res.status[lo:hi], n_steps=res.n_steps[lo:hi],
                              n_iter=res.n_iter[lo:hi], dt=res.dt[lo:hi],
                              records=res.records[lo:hi], n_records=res.n_records[lo:hi], obs=None)
    return R.leg_trajectories(sub, x_offset, empty_failed=empty_failed, fail_on_error=fail_on_error, label=label)


def _finish_row(p: _Prepared, f_res, lo, n, s_res, impact_runner):
    for ph in p.checks:
        ph.check_generated()
    f_tr, f_st = _split_leg(f_res, lo, lo + n, p.shift, empty_failed=False, fail_on_error=not impact_runner,
                            label=f"FLRW job {p.job.jobid}")
    s_tr, s_st = R.leg_trajectories(s_res, None, empty_failed=not impact_runner, fail_on_error=False,
                                    label=f"Schwarzschild job {p.job.jobid}")
    s = R.reduce_leg(s_tr, s_st, s_res.n_steps.cpu().numpy(), p.geo.lens_center, is_spherical=True)
    f = R.reduce_leg(f_tr, f_st, f_res.n_steps[lo:lo + n].cpu().numpy(), p.geo.lens_center, is_spherical=False)
    return p.job.jobid, R.compare_result(p.cfg, p.geo, s, f)


def run_jobs(jobs: Iterable[Job], *, runner: str = "plain", max_fields: int = N.EXC_MAX_FIELDS,
             streams: int = 16, wave_rows: int = 256, threads: Optional[int] = None) -> dict:
    """Trace every job's two legs in grouped launches; returns {jobid: CompareResult}.

    Rows are taken in waves of at most `wave_rows` (bounding the device memory held: each row's
    potential and records). Within a wave, every FLRW launch (up to `max_fields` rows) and every
    Schwarzschild launch goes to one of `streams` CUDA streams in turn, so the small launches of
    a sweep -- a few hundred photons each, bound by the per-step latency of FP64 arithmetic --
    run side by side on the SMs instead of one after another; the host waits once per wave and
    reduces the rows' records on `threads` host threads."""
    import concurrent.futures as cf

    import torch

    from ..trace import trace_batch

    if runner not in ("plain", "impact"):
        raise ValueError("runner must be 'plain' or 'impact'")
    impact_runner = runner == "impact"
    if not 1 <= max_fields <= N.EXC_MAX_FIELDS:
        raise ValueError(f"max_fields must be in [1, {N.EXC_MAX_FIELDS}]")
    jobs = list(jobs)
    if not jobs:
        return {}
    # launch groups from the row parameters alone (no device work yet)
    groups = {}
    for job in jobs:
        cfg = job_config(job)
        groups.setdefault(_flrw_key(cfg, R.geometry(cfg)), []).append(job)
    chunks = [members[c0:c0 + max_fields] for members in groups.values()
              for c0 in range(0, len(members), max_fields)]
    waves, cur = [], []
    for ch in chunks:
        if cur and sum(len(c) for c in cur) + len(ch) > wave_rows:
            waves.append(cur)
            cur = []
        cur.append(ch)
    if cur:
        waves.append(cur)
    main = torch.cuda.current_stream()
    pool = [torch.cuda.Stream() for _ in range(max(1, int(streams)))]
    workers = threads or min(16, os.cpu_count() or 1)
    out = {}
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        for wave in waves:
            launched, k = [], 0
            for chunk_jobs in wave:
                chunk = [_prepare(j, impact_runner) for j in chunk_jobs]
                first = chunk[0]
                interps = [p.f_metric.interp for p in chunk]
                batched = R.PerturbedFLRWMetricFast(a_of_eta=first.f_metric.a_of_eta,
                                                    adot_of_eta=first.f_metric.adot_of_eta, grid=interps[0].grid,
                                                    interpolator=interps[0], extra_interpolators=interps[1:])
                counts = [int(p.f_states.shape[0]) for p in chunk]
                states = torch.cat([p.f_states for p in chunk])
                fidx = torch.cat([torch.full((n,), i, dtype=torch.int32, device=states.device)
                                  for i, n in enumerate(counts)])
                dl = abs(first.geo.dlambda)
                st = pool[k % len(pool)]
                k += 1
                st.wait_stream(main)
                with torch.cuda.stream(st):
                    f_res = trace_batch(batched, states, R.trace_config(first.cfg, first.geo, dl, dl),
                                        field_index=fidx, check_field_index=False)
                s_res = []
                for p in chunk:
                    st = pool[k % len(pool)]
                    k += 1
                    st.wait_stream(main)
                    with torch.cuda.stream(st):
                        s_res.append(trace_batch(p.s_metric, p.s_states, R.trace_config(p.cfg, p.geo, *p.s_dt)))
                # `states` and the rows' inputs are read by the pool streams: keep them alive
                # (the caching allocator would hand their memory to the next row otherwise)
                launched.append((chunk, counts, f_res, s_res, states))
            torch.cuda.synchronize()
            tasks = []
            for chunk, counts, f_res, s_res, _ in launched:
                lo = 0
                for p, n, sr in zip(chunk, counts, s_res):
                    tasks.append(ex.submit(_finish_row, p, f_res, lo, n, sr, impact_runner))
                    lo += n
            for t in tasks:
                jobid, res = t.result()
                out[jobid] = res
    return out


def run_sweep(manifest: str, jobids: Optional[Iterable[int]] = None, *, results: str = "results",
              runner: str = "plain", overwrite: bool = False, max_fields: int = N.EXC_MAX_FIELDS) -> List[str]:
    """run_one_job for many rows at once: writes results/per_run/job_NNNNN.csv for every selected
    row (all rows by default), skipping rows whose table exists unless `overwrite`. A row whose
    Schwarzschild or FLRW leg kept no trajectory gets no table, as in the reference (its
    analyzer fails on the empty file); the paths of the tables that exist are returned."""
    jobs = read_jobs(manifest)
    if jobids is not None:
        wanted = {int(j) for j in jobids}
        missing = wanted - {j.jobid for j in jobs}
        if missing:
            raise SystemExit(f"jobid={min(missing)} not found in {manifest}")
        jobs = [j for j in jobs if j.jobid in wanted]
    os.makedirs(os.path.join(results, "per_run"), exist_ok=True)
    todo, paths = [], []
    for j in jobs:
        path = os.path.join(results, "per_run", f"job_{j.jobid:05d}.csv")
        paths.append(path)
        if overwrite or not os.path.exists(path):
            todo.append(j)
    written = []
    for jobid, res in sorted(run_jobs(todo, runner=runner, max_fields=max_fields).items()):
        path = os.path.join(results, "per_run", f"job_{jobid:05d}.csv")
        if res.error is not None:
            # run_one_job raises here and the row is left without a table
            print(f"[fail] job {jobid}: {res.error}")
            continue
        write_per_run_csv(path, res.schwarzschild.stats, res.flrw.stats)
    return [p for p in paths if os.path.exists(p)]


def main(argv=None):
    import argparse

    p = argparse.ArgumentParser(description="Run manifest rows of a comparison sweep on the GPU")
    p.add_argument("--manifest", required=True)
    p.add_argument("--jobids", default=None, help="comma-separated job ids (default: every row)")
    p.add_argument("--results", default="results")
    p.add_argument("--runner", default="plain", choices=["plain", "impact"])
    p.add_argument("--overwrite", action="store_true")
    a = p.parse_args(argv)
    ids = None if a.jobids is None else [int(x) for x in a.jobids.split(",") if x.strip()]
    for path in run_sweep(a.manifest, ids, results=a.results, runner=a.runner, overwrite=a.overwrite):
        print(f"[ok] {path}")


if __name__ == "__main__":
    main()
