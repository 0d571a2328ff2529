"""Benchmark: photon-steps/s of the backward ray tracer on the FLRW lensing workload.

Workload (one "step" = one pass of the hot path over one batch): 65,536
photons on a 256x256 grid of directions in a 10x10 deg patch, traced
backward with RK4 (deta = 0.5 Mpc) through a perturbed-FLRW (LCDM) metric
whose Phi lives on a 128^3 float64 grid over 1000 Mpc (Plummer lens + seeded
P(k)~k^-3 random field, rms Phi/c^2 = 1e-5) until box exit or a <= 0.5.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The line also carries `precision`: the guarded mixed-precision tracer on the
precision workload (4,194,304 photons, 2048x2048 directions in a 20x20 deg
patch, Phi on a 512^3 float32 grid, seed 4) against the FP64 tracer on a
seeded 65,536-ray subset (numpy default_rng(40)).

Further keys: `roofline.fp64_pipe` (the parity tracer against the FP64 pipe, each
operation kind weighted by its throughput measured with exc_probe_fp64_rates),
`variants`, `batching` (multi-field RK45 launch, autotuned), `surrogate` and
`surrogate_smooth` (learned 4096^2 sky maps on the fast and the slow
interpolator's reading of one field, against tracing every pixel).

`--impl reference` times the CPU oracle (the C restatement of the reference's
integrate_single loop, oracle/exc_oracle.c) on all host threads over the same
workload instead. Under torchrun (N > 1) each rank traces its own batch (weak
scaling, no collective on the data path); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "rays/s & photon-steps/s on 1 GB300: plain FP64 vs mixed/surrogate at |Δz|≤1e-9"
UNIT = "photon-steps/s"
WORKLOAD = ("flrw_patch: 65,536 photons (256x256 directions, 10x10 deg patch) through perturbed FLRW "
            "(LCDM Om=0.3 h=0.7), Phi on a 128^3 float64 grid over 1000 Mpc (Plummer 1e15 Msun eps 5 Mpc + "
            "seeded k^-3 random field, rms 1e-5), RK4 deta = 0.5 Mpc, until box exit or a <= 0.5")
L2_FLUSH_BYTES = 256 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--shard", action="store_true",
                   help="N>1: split one batch of photons across the ranks (strong scaling) instead of a "
                        "batch per rank (weak scaling); the per-rank results are gathered once after timing")
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", default="fp64", choices=["fp64", "fp64_fast", "mixed"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-variants", action="store_true")
    p.add_argument("--side", type=int, default=256, help="directions per side (smaller cases for profiling)")
    p.add_argument("--no-precision", action="store_true", help="skip the 512^3 / 4M-ray precision workload")
    p.add_argument("--precision-side", type=int, default=2048)
    p.add_argument("--precision-rk45-side", type=int, default=1024,
                   help="directions per side of the RK45 precision leg (2048: the full 4,194,304 rays)")
    p.add_argument("--no-surrogate", action="store_true", help="skip the learned sky-map leg")
    p.add_argument("--no-batching", action="store_true", help="skip the multi-field RK45 batching leg")
    p.add_argument("--batching-scale", type=int, default=1,
                   help="run 1/scale of the batching configuration (1: the full 1,048,576 + 16 x 65,536 rays)")
    p.add_argument("--no-sweep", action="store_true", help="skip the comparison-sweep leg")
    p.add_argument("--no-redshift-map", action="store_true",
                   help="skip the redshift-map leg (262,144 recorded 64-row histories)")
    p.add_argument("--profile-gemm", type=int, default=0, metavar="M",
                   help="only time the surrogate's tensor-core GEMM on M rows (for profiling) and exit")
    p.add_argument("--profile-infer", type=int, default=0, metavar="M",
                   help="only time the surrogate's fused forward pass (and the layer-by-layer one) on M rows and exit")
    p.add_argument("--profile-training", type=int, default=0, metavar="STEPS",
                   help="only run STEPS graph-captured surrogate training steps (batch 8192, 4 members, 6 "
                        "outputs, synthetic targets) and exit")
    p.add_argument("--profile-sweep", action="store_true",
                   help="only run the 32-row comparison sweep of the sweep leg once and exit")
    p.add_argument("--profile-redshift-map", type=int, default=0, metavar="N",
                   help="only time the redshift-map kernels on N synthetic 64-row FLRW histories and exit")
    p.add_argument("--profile-batching", type=int, default=0, metavar="SCALE",
                   help="only run the multi-field RK45 launch of the batching leg once at 1/SCALE and exit")
    p.add_argument("--profile-aux", type=int, default=0, metavar="N",
                   help="only run the auxiliary kernels once on N rays (device photon generation, the lens "
                        "potential on a 128^3 grid, the surrogate's Born features) and exit")
    p.add_argument("--profile-rk45-mixed", type=int, default=0, metavar="SIDE",
                   help="only run the mixed RK45 tracer once on SIDE x SIDE rays of the slow-Interpolator "
                        "patch (128^3 float32 grid) and exit")
    p.add_argument("--map-side", type=int, default=4096)
    p.add_argument("--train-steps", type=int, default=8000)
    p.add_argument("--smooth-train-steps", type=int, default=12000,
                   help="training steps of the surrogate on the slow-Interpolator field")
    return p.parse_args()


# ------------------------------------------------------------------ dist
def launch_ranks(n):
    """`--gpus N` run without a launcher (WORLD_SIZE unset): start N ranks of this same command
    under torch.distributed.run on this node (rendezvous on 127.0.0.1) and return its exit code."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__), *sys.argv[1:]]
    return subprocess.call(cmd)


def dist_setup(n):
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if n > 1 and world != n:
        raise SystemExit(f"--gpus {n} but WORLD_SIZE={world}: run under torch.distributed.run with "
                         f"--nproc-per-node {n}, or without a launcher to have bench.py start the ranks")
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if os.environ.get("BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world, device=None):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world, device=None):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as fh:
            for line in fh:
                parts = [s.strip() for s in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        power = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(power) if power else None}


# ------------------------------------------------------------------ peaks
def measured_peaks(device):
    """HBM / bf16 from MEASURED_PEAKS.json (driver-written) plus FP64 / FP32 measured here with cuBLAS."""
    import torch

    peaks = {}
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            peaks.update(json.load(fh))
    res = {}
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    for name, dt, n in (("fp64_tflops", torch.float64, 4096), ("fp32_tflops", torch.float32, 8192)):
        a = torch.randn(n, n, device=device, dtype=dt)
        b = torch.randn(n, n, device=device, dtype=dt)
        for _ in range(2):
            a @ b
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = float("inf")
        for _ in range(5):
            e0.record()
            a @ b
            e1.record()
            torch.cuda.synchronize(device)
            best = min(best, e0.elapsed_time(e1))
        res[name] = 2 * n ** 3 / (best * 1e-3) / 1e12
        del a, b
    torch.backends.cuda.matmul.allow_tf32 = old
    peaks.update(res)
    return peaks


# ncu summary of the trace kernel on this workload (profiles/trace_fp64_flrw_patch.md):
# DRAM bytes per launch from one capture; None until a capture exists.
NCU_TRAFFIC_BYTES = {"fp64": None, "fp64_fast": None, "mixed": None}


# ------------------------------------------------------------------ ours
def run_ours(args, rank, world, local):
    import torch

    from excalibur_tool_gb300 import _native as N
    from excalibur_tool_gb300 import roofline, workloads
    from excalibur_tool_gb300.integration.integrator import Integrator
    from excalibur_tool_gb300.trace import trace_batch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl = workloads.flrw_patch(128, args.side, precision=args.precision, device=dev)
    metric, states, cfg = wl.metric, wl.states, wl.cfg
    n_total = states.shape[0]
    sharded = args.shard and world > 1
    if sharded:
        # strong scaling: this rank traces its contiguous slice of the one batch
        from excalibur_tool_gb300.distributed import shard_range

        lo, hi = shard_range(n_total, rank, world)
        states = states[lo:hi].contiguous()
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    peaks = measured_peaks(dev)
    # the launch schedule measured on this batch by the library's autotuner (untimed; whole-batch
    # trials): with ~1.7 similar trajectories a lane at the occupancy limit, the last wave runs
    # two thirds full, and a lane count nearer two a lane fills it
    from excalibur_tool_gb300.trace import autotune

    t_tune = time.perf_counter()
    cfg = autotune(metric, states, cfg, use_cache=False)
    t_tune = time.perf_counter() - t_tune
    schedule = {"block_size": cfg.block_size, "blocks_per_sm": cfg.blocks_per_sm, "staging": cfg.staging,
                "source": "exc_autotune on this batch", "tune_s": t_tune}

    for _ in range(max(args.warmup, 1)):
        res = trace_batch(metric, states, cfg)
    torch.cuda.synchronize(dev)
    steps_per_batch = int(res.n_steps.sum().item())
    rays = states.shape[0]
    status_counts = np.bincount(res.status.cpu().numpy(), minlength=12).tolist()

    # ---- device-resident timed region ----
    clocks = ClockSampler(local)
    clocks.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize(dev)
    t_wall = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))                      # evict L2 between timed steps
        evs[k][0].record(stream)
        res = trace_batch(metric, states, cfg)
        evs[k][1].record(stream)
    torch.cuda.synchronize(dev)
    barrier(world)
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    dev_s = sum(step_ms) / 1e3
    dev_s_max = max_over_ranks(dev_s, world, dev)
    total_steps = sum_over_ranks(float(steps_per_batch * args.steps), world, dev)
    value = total_steps / dev_s_max
    rays_s = sum_over_ranks(float(rays * args.steps), world, dev) / dev_s_max
    gpu_launches = args.steps                     # one exc_trace kernel per step
    gathered = None
    if sharded:
        # the one collective: the per-photon results, gathered once after the timed region
        from excalibur_tool_gb300.distributed import gather_rows

        full = gather_rows(res.state, n_total)
        gathered = {"rows": int(full.shape[0]), "of": n_total,
                    "all_finite": bool(torch.isfinite(full).all().item())}

    # ---- end to end through the public API: host states in, host results out ----
    integ = Integrator(metric, dt=cfg.dt, integrator="rk4", dt_min=cfg.dt_min, dt_max=cfg.dt_max,
                       precision=args.precision, max_iter=cfg.max_iter)
    host_states = states.cpu().pin_memory()
    out_host = None
    sched_kw = {"block_size": cfg.block_size, "blocks_per_sm": cfg.blocks_per_sm, "staging": cfg.staging}
    for _ in range(max(1, args.warmup)):
        out_host = integ.integrate_batch(host_states, "box", cfg.stop_box, out_host=out_host, a_stop=0.5,
                                         lens_center=cfg.lens_center, **sched_kw)
    barrier(world)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))
        out_host = integ.integrate_batch(host_states, "box", cfg.stop_box, out_host=out_host, a_stop=0.5,
                                         lens_center=cfg.lens_center, **sched_kw)
    torch.cuda.synchronize(dev)
    barrier(world)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    h2d = host_states.numel() * 8
    d2h = sum(t.numel() * t.element_size() for t in out_host.values())
    e2e_steps = int(out_host["n_steps"].sum())
    e2e_value = sum_over_ranks(float(e2e_steps * args.steps), world, dev) / e2e_s

    # ---- roofline of the trace kernel ----
    mean_launch_s = dev_s / args.steps
    flops_launch = steps_per_batch * roofline.FLOPS_PER_RK4_STEP_FLRW
    if args.precision == "mixed":
        bound, peak = "fp32", peaks.get("fp32_tflops")
    else:
        bound, peak = "fp64", peaks.get("fp64_tflops")
    achieved = flops_launch / mean_launch_s / 1e12
    roof = {"bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if peak else None, "traffic": NCU_TRAFFIC_BYTES.get(args.precision),
            "peak_source": f"cuBLAS {'D' if bound == 'fp64' else 'S'}GEMM measured in this run",
            "algorithmic_flops_per_launch": flops_launch, "gather_bytes_per_launch":
                steps_per_batch * roofline.bytes_per_rk4_step(8),
            "hbm_gbs_measured": peaks.get("hbm_gbs")}
    if bound == "fp64":
        roof["fp64_pipe"] = fp64_pipe_roofline(dev, stream, steps_per_batch / mean_launch_s)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "strong" if sharded else "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "fp64_fast": "f64", "mixed": "f32+f64"}[args.precision],
            "data": "synthetic (seeded Plummer + Gaussian random field; patch of directions)",
            "config": {"workload": WORKLOAD, "precision": args.precision, "photons": rays,
                       "photon_steps_per_batch": steps_per_batch, "grid": "128^3 float64 (16.8 MB)",
                       "l2": "flushed between timed steps (256 MiB write); grid itself fits in L2",
                       "parallelism": (f"sharded x{world} (one batch split by photon index)" if sharded
                                       else f"replicas x{world} (independent photon batches)"),
                       "status_counts": status_counts, "schedule": schedule},
            "rays_per_s": rays_s, "wall_s_timed": wall,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "api": "Integrator.integrate_batch(pinned host states) -> pinned host results"},
            "gpu_launches": gpu_launches, "roofline": roof, "clocks": clk}
    if gathered is not None:
        line["gathered"] = gathered

    if not args.no_variants and world == 1:
        line["variants"] = run_variants(args, wl, peaks, dev, stream, value)
    if not args.no_cpu_baseline and world == 1 and rank == 0:
        line["cpu_baseline"] = cpu_baseline(wl, steps_per_batch, res)
        line["parity"] = line["cpu_baseline"].pop("parity", None)
    if not args.no_precision and world == 1:
        del wl, metric, states, res
        torch.cuda.empty_cache()
        line["precision"] = run_precision(args, dev, stream, flush, value)
    if not args.no_batching and world == 1:
        torch.cuda.empty_cache()
        line["batching"] = run_batching(args, dev, stream)
    if not args.no_sweep and world == 1:
        torch.cuda.empty_cache()
        line["sweep"] = run_sweep_leg(args, dev)
    if not args.no_redshift_map and world == 1:
        torch.cuda.empty_cache()
        rm = profile_redshift_map(262144)
        if peaks.get("hbm_gbs"):
            rm["table_frac_of_measured_hbm"] = rm["table_algo_gbs"] / peaks["hbm_gbs"]
        line["redshift_map"] = rm
        torch.cuda.empty_cache()
    if not args.no_surrogate and world == 1:
        torch.cuda.empty_cache()
        line["surrogate"] = run_surrogate(args, dev, stream, peaks, rays_s)
        torch.cuda.empty_cache()
        line["surrogate_smooth"] = run_surrogate_smooth(args, dev)
    if rank == 0:
        print(json.dumps(line), flush=True)


def fp64_pipe_rates(dev, stream):
    """FP64 operations per second of each kind (exc_probe_fp64_rates, no FMA contraction)."""
    import ctypes as C
    import torch

    from excalibur_tool_gb300 import _native as N

    lib = N.load()
    n = int(lib.exc_probe_scratch_len())
    scratch = torch.empty(n, dtype=torch.float64, device=dev)
    out = (C.c_double * 4)()
    N.check(lib.exc_probe_fp64_rates(C.c_void_p(scratch.data_ptr()), n, out, C.c_void_p(stream.cuda_stream)),
            "exc_probe_fp64_rates")
    return {k: out[i] for k, i in N.PROBE.items()}


def fp64_pipe_roofline(dev, stream, photon_steps_per_s):
    """The parity tracer against the FP64 pipe itself: the algorithmic operation mix of a
    photon-step in multiply/add-equivalent slots (divisions, fmod and sqrt weighted by their
    measured cost), times the photon-step rate, over the measured multiply/add rate. Index
    arithmetic, comparisons and conversions are not counted, so this is a lower bound of the
    pipe's occupancy by the algorithm."""
    from excalibur_tool_gb300 import roofline

    rates = fp64_pipe_rates(dev, stream)
    ops = roofline.OPS_PER_RK4_STEP_FLRW
    slots_ieee = roofline.fp64_pipe_slots(ops, rates)
    slots = roofline.fp64_pipe_slots_executed(ops, rates)
    achieved = photon_steps_per_s * slots
    return {"ops_per_photon_step": {**ops, "div_by_launch_constant": roofline.DIV_CONST_PER_RK4_STEP_FLRW},
            "measured_ops_per_s": rates,
            "slot_cost": {**{k: rates["addmul"] / rates[k] for k in ("div", "fmod", "sqrt")},
                          "div_by_launch_constant": roofline.CONST_DIV_SLOTS},
            "slots_per_photon_step": slots, "achieved_slots_per_s": achieved,
            "peak_slots_per_s": rates["addmul"], "frac": achieved / rates["addmul"],
            "frac_if_every_division_were_ieee": photon_steps_per_s * slots_ieee / rates["addmul"],
            "note": "the parity build takes its divisions by launch constants as correctly rounded FMA "
                    "quotients from host reciprocals (1 multiply + 2 FMA, bit-identical to IEEE division, "
                    "checked by exc_probe_div_rn); frac counts them at 3 slots",
            "source": "exc_probe_fp64_rates (multiply/add, IEEE division, sqrt, fmod throughput, --fmad=false)"}


def run_variants(args, wl, peaks, dev, stream, main_value):
    """The other precision builds on the same batch, with their error against the parity build."""
    import dataclasses
    import torch

    from excalibur_tool_gb300 import _native as N
    from excalibur_tool_gb300.trace import trace_batch

    ref = trace_batch(wl.metric, wl.states, dataclasses.replace(wl.cfg, precision="fp64"))
    torch.cuda.synchronize(dev)
    out = {}
    for prec in ("fp64", "fp64_fast", "mixed", "mixed_raw"):
        if prec == args.precision:
            continue
        cfg = dataclasses.replace(wl.cfg, precision=prec)
        from excalibur_tool_gb300.trace import autotune

        cfg = autotune(wl.metric, wl.states, cfg, use_cache=False)    # whole-batch trials, as the headline
        try:
            r = trace_batch(wl.metric, wl.states, cfg)
        except N.NativeError as e:
            out[prec] = {"unavailable": str(e).splitlines()[0][:200]}
            continue
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            r = trace_batch(wl.metric, wl.states, cfg)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        s = e0.elapsed_time(e1) / 3e3
        steps = int(r.n_steps[r.status != N.PH_RETRACE].sum())
        out[prec] = {"photon_steps_per_s": steps / s, "rays_per_s": wl.states.shape[0] / s,
                     f"speedup_vs_{args.precision}": steps / s / main_value,
                     "schedule": {"block_size": cfg.block_size, "blocks_per_sm": cfg.blocks_per_sm}}
        if prec == "mixed":
            # a stream of batches: each batch's FP64 re-traces overlap the next batches' mixed launches
            from excalibur_tool_gb300.trace import trace_pipelined

            nb = 8
            trace_pipelined(wl.metric, [wl.states] * 2, cfg)
            torch.cuda.synchronize(dev)
            e0.record(stream)
            rs = trace_pipelined(wl.metric, [wl.states] * nb, cfg)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            sp = e0.elapsed_time(e1) / 1e3
            out[prec]["pipelined"] = {"batches": nb, "photon_steps_per_s": nb * steps / sp,
                                      "rays_per_s": nb * wl.states.shape[0] / sp,
                                      f"speedup_vs_{args.precision}": nb * steps / sp / main_value,
                                      "note": "re-trace of batch k on a side stream, overlapping batches k+1.."}
        if prec == "mixed_raw":
            # the mixed launch alone: rays handed back for the FP64 re-trace carry no result
            back = r.status == N.PH_RETRACE
            out[prec]["retrace_fraction"] = float(back.float().mean())
            out[prec]["note"] = "photon-steps of handed-back rays not counted; errors over the other rays"
            out[prec].update(errors_vs(ref, r, ~back))
        else:
            out[prec].update(errors_vs(ref, r))
    return out


def run_precision(args, dev, stream, flush, fp64_value):
    """Guarded mixed tracer on the 512^3 float32 / 4M-ray workload; errors against the
    FP64 parity tracer on a seeded 65,536-ray subset of the same rays."""
    import dataclasses
    import torch

    from excalibur_tool_gb300 import _native as N
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.trace import trace_batch

    t0 = time.perf_counter()
    side = args.precision_side
    wl = workloads.flrw_patch(512, side, 20.0, seed=4, field_dtype=np.float32, device=dev)
    build_s = time.perf_counter() - t0
    n = wl.states.shape[0]
    cfg = dataclasses.replace(wl.cfg, precision="mixed")
    r = trace_batch(wl.metric, wl.states, cfg)
    torch.cuda.synchronize(dev)
    steps = int(r.n_steps.sum())
    k = max(2, min(args.steps, 3))
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
    for i in range(k):
        flush.fill_(float(i))
        evs[i][0].record(stream)
        r = trace_batch(wl.metric, wl.states, cfg)
        evs[i][1].record(stream)
    torch.cuda.synchronize(dev)
    sec = sum(a.elapsed_time(b) for a, b in evs) / 1e3 / k
    raw = trace_batch(wl.metric, wl.states, dataclasses.replace(cfg, precision="mixed_raw"))
    torch.cuda.synchronize(dev)
    back = float((raw.status == N.PH_RETRACE).float().mean())
    del raw
    # FP64 parity tracer on the seeded subset
    idx = np.sort(np.random.default_rng(40).choice(n, min(65536, n), replace=False))
    sub = wl.states[torch.as_tensor(idx, device=dev)].contiguous()
    c64 = dataclasses.replace(wl.cfg, precision="fp64")
    r64 = trace_batch(wl.metric, sub, c64)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    r64 = trace_batch(wl.metric, sub, c64)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    s64 = e0.elapsed_time(e1) / 1e3
    steps64 = int(r64.n_steps.sum())

    class _Sub:
        pass

    rs = _Sub()
    ti = torch.as_tensor(idx, device=dev)
    rs.obs, rs.state, rs.status = r.obs[ti], r.state[ti], r.status[ti]
    err = errors_vs(r64, rs)
    err["status_equal"] = bool(torch.equal(rs.status, r64.status))
    err["steps_equal"] = bool(torch.equal(r.n_steps[ti], r64.n_steps))
    mixed_ps = steps / sec
    fp64_ps = steps64 / s64
    return {"workload": f"flrw_patch_512: {n:,} photons ({side}x{side} directions, 20x20 deg patch), Phi on a "
                        "512^3 float32 grid (512 MB, Plummer + seeded random field, seed 4), RK4 deta = 0.5 Mpc",
            "precision": "mixed (FP32 RHS, double-float state, FP64 re-trace of guarded rays)",
            "photon_steps_per_s": mixed_ps, "rays_per_s": n / sec, "ms_per_batch": sec * 1e3,
            "timed_batches": k, "retrace_fraction": back,
            "fp64_subset_photon_steps_per_s": fp64_ps, "speedup_vs_fp64": mixed_ps / fp64_ps,
            "speedup_vs_fp64_patch_value": mixed_ps / fp64_value,
            "errors_vs_fp64_on_subset": {**err, "subset": "65,536 rays, numpy default_rng(40)"},
            "host_field_build_s": build_s,
            "rk45": run_precision_rk45(args, dev, stream, flush)}


def run_precision_rk45(args, dev, stream, flush):
    """The precision workload with the adaptive stepper its configuration names ("FP64 RK45 error
    control"): RK45 (Fehlberg, rtol 1e-8, atol 1e-12) through the slow Interpolator's continuous
    gradient on the 512^3 float32 grid, the box stop on the face; the mixed tracer (FP32 stages,
    double-float state, FP64 error norm and step control) against the FP64 RK45 parity tracer on
    a default_rng(40) subset. Rates are RK45 trial steps per second (six RHS evaluations each)."""
    import dataclasses
    import torch

    from excalibur_tool_gb300 import _native as N
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.trace import trace_batch

    side = args.precision_rk45_side
    wl = workloads.flrw_patch_rk45(512, side, 20.0, seed=4, device=dev)
    n = wl.states.shape[0]
    cfg = dataclasses.replace(wl.cfg, precision="mixed")
    r = trace_batch(wl.metric, wl.states, cfg)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.fill_(1.0)
    e0.record(stream)
    r = trace_batch(wl.metric, wl.states, cfg)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    sec = e0.elapsed_time(e1) / 1e3
    raw = trace_batch(wl.metric, wl.states, dataclasses.replace(cfg, precision="mixed_raw"))
    torch.cuda.synchronize(dev)
    back = float((raw.status == N.PH_RETRACE).float().mean())
    del raw
    idx = np.sort(np.random.default_rng(40).choice(n, min(65536, n), replace=False))
    ti = torch.as_tensor(idx, device=dev)
    sub = wl.states[ti].contiguous()
    c64 = dataclasses.replace(wl.cfg, precision="fp64")
    r64 = trace_batch(wl.metric, sub, c64)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    r64 = trace_batch(wl.metric, sub, c64)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    s64 = e0.elapsed_time(e1) / 1e3

    class _Sub:
        pass

    rs = _Sub()
    rs.obs, rs.state, rs.status = r.obs[ti], r.state[ti], r.status[ti]
    both = (rs.status == N.PH_LEFT_BOX) & (r64.status == N.PH_LEFT_BOX)
    err = errors_vs(r64, rs, both)
    # the FP64 tracer's own sensitivity: the same rays with their initial speed changed by 1e-9
    sub2 = sub.clone()
    sub2[:, 5:8] *= 1.0 + 1e-9
    r64b = trace_batch(wl.metric, sub2, c64)
    torch.cuda.synchronize(dev)
    both2 = both & (r64b.status == N.PH_LEFT_BOX)
    sens = errors_vs(r64, r64b, both2)
    err["rays_compared"] = int(both.sum())
    err["status_counts_mixed"] = np.bincount(rs.status.cpu().numpy(), minlength=12).tolist()
    err["status_counts_fp64"] = np.bincount(r64.status.cpu().numpy(), minlength=12).tolist()
    trials, trials64 = int(r.n_iter.sum()), int(r64.n_iter.sum())
    mixed_ps, fp64_ps = trials / sec, trials64 / s64
    return {"workload": f"flrw_patch_rk45_512: {n:,} photons ({side}x{side} directions, 20x20 deg patch), Phi on "
                        "the 512^3 float32 grid read through the slow Interpolator, RK45 Fehlberg rtol 1e-8 atol "
                        "1e-12, dt in [1e10 s, 10 Mpc/c], box stop on the face 1.5 cells inside the last node",
            "precision": "mixed RK45 (FP32 stages, double-float state, FP64 error norm, step control and "
                         "re-trace of guarded rays)",
            "rk45_trials_per_s": mixed_ps, "accepted_steps_per_s": int(r.n_steps.sum()) / sec,
            "rays_per_s": n / sec, "s_per_batch": sec, "retrace_fraction": back,
            "fp64_subset_rk45_trials_per_s": fp64_ps, "speedup_vs_fp64": mixed_ps / fp64_ps,
            "trials_per_ray": trials / n, "rejected_fraction": 1 - int(r.n_steps.sum()) / max(1, trials),
            "errors_vs_fp64_on_subset": {**err, "subset": f"{len(idx):,} rays, numpy default_rng(40); rays that "
                                                          "left the box in both"},
            "fp64_own_sensitivity": {**sens, "perturbation": "the FP64 parity tracer on the same rays with the "
                                     "initial speed scaled by 1 + 1e-9 (RK45 end points are determined to the "
                                     "method's truncation error: step sequences that part move them by this much)"}}


def run_batching(args, dev, stream):
    """The lens grid (256^3) with 1,048,576 full-sky rays plus 16 random fields (64^3..256^3) with
    65,536 patch rays each: one persistent adaptive-RK45 launch, autotuned, captured in a CUDA graph."""
    import torch

    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.trace import CapturedTrace, autotune, trace_batch, tune_report

    t0 = time.perf_counter()
    scale = args.batching_scale
    wl = workloads.multi_field(n_sky=(1 << 20) // scale, n_side=256 // int(round(scale ** 0.5)), device=dev)
    build_s = time.perf_counter() - t0
    t1 = time.perf_counter()
    tuned = autotune(wl.metric, wl.states, wl.cfg, field_index=wl.field_index, use_cache=False)
    tune_s = time.perf_counter() - t1
    plan = next(iter(tune_report().values()))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # the tuned plan captured once (its constructor runs the batch eagerly, loading the kernels)
    cap = CapturedTrace(wl.metric, wl.states, tuned, field_index=wl.field_index)
    torch.cuda.synchronize(dev)
    k = 1 if scale == 1 else 3
    e0.record(stream)
    for _ in range(k):
        out = cap.run()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    graph_s = e0.elapsed_time(e1) / 1e3 / k
    # one eager launch with the library's default schedule, for comparison
    e0.record(stream)
    r = trace_batch(wl.metric, wl.states, wl.cfg, field_index=wl.field_index)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    default_s = e0.elapsed_time(e1) / 1e3
    del r
    n = wl.states.shape[0]
    steps = out.n_steps.cpu().numpy()
    iters = out.n_iter.cpu().numpy()
    status = out.status.cpu().numpy()
    fidx = wl.field_index.cpu().numpy()
    sky = fidx == 0
    long = steps[sky][steps[sky] > 1]

    def dist(v):
        v = np.asarray(v)
        if not len(v):
            return None
        return {"p05": float(np.percentile(v, 5)), "median": float(np.median(v)), "p95": float(np.percentile(v, 95)),
                "max": int(v.max()), "rays": int(len(v))}

    return {"configuration": "full configuration" if scale == 1 else f"1/{scale} of the configuration",
            "workload": f"lens alone on a 256^3 float64 grid with {(1 << 20) // scale:,} full-sky rays "
                        f"(default_rng(3)) + 16 random fields (seeds 1-16; 64^3/128^3/256^3) x "
                        f"{wl.info['patch_photons']:,} patch rays, adaptive RK45 (Fehlberg weights, rtol 1e-8, "
                        "atol 1e-12, dt in [1e10, 1e17] s) to box exit; one launch"
                        + (f"; 1/{scale} of the 1,048,576 + 16 x 65,536 configuration" if scale > 1 else ""),
            "photons": n, "fields": wl.info["fields"], "host_build_s": build_s,
            "autotune": {"block_size": plan["block_size"], "blocks_per_sm": plan["blocks_per_sm"],
                         "staging": plan["staging"], "knobs": "threads per block x blocks per SM, then the "
                                                              "3 fastest with the a(eta) table in shared memory",
                         "best_steps_tried_per_s": plan["best_rate"], "trials": len(plan["trials"]),
                         "seconds": tune_s, "sample": plan["sample"], "time_box": "1e8 SM cycles per trial",
                         "all_trials": [{"block": t[0], "per_sm": t[1], "staging": t[2], "rate": t[4]}
                                        for t in plan["trials"]]},
            "default_schedule_s": default_s, "graph_replay_s": graph_s,
            "rays_per_s": n / graph_s, "accepted_steps_per_s": float(steps.sum()) / graph_s,
            "rk45_trials_per_s": float(iters.sum()) / graph_s,
            "accepted_steps": {"sky_rays": dist(steps[sky]), "sky_rays_past_the_first_step": dist(long),
                               "random_field_rays": dist(steps[~sky])},
            "tried_steps": {"sky_rays": dist(iters[sky]), "random_field_rays": dist(iters[~sky])},
            "rejected_fraction": float(1 - steps.sum() / max(1, iters.sum())),
            "status_counts": np.bincount(status, minlength=12).tolist(),
            "gpu_launches_per_replay": 1}


SWEEP_MANIFEST = dict(masses="1e13,3e13,1e14,3e14", distances="200,300,400,500", Ns="64,128", sampling="cone",
                      cone_nphotons=200, cone_angle_deg=10.0, integrators="rk4")


def run_sweep_leg(args, dev):
    """A 32-row comparison sweep (4 masses x 4 distances x 2 grid sizes, 183-photon cones, RK4,
    records every 4 steps, static cosmology, local coordinates): every row's Schwarzschild and
    FLRW legs and its per-run statistics, from the manifest to the tables. Timed end to end on
    the host clock (potentials built on the device, photon generation, launches, record copies,
    statistics), grouped launches against one launch per row; the oracle runs one row's two
    legs on the host threads for the CPU rate."""
    import tempfile

    import torch

    from excalibur_tool_gb300.runners import compare as R
    from excalibur_tool_gb300.runners import sweep as S

    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "manifest.csv")
        S.make_manifest(path, **SWEEP_MANIFEST)
        jobs = S.read_jobs(path)
    S.run_jobs(jobs[:2])                        # warm-up: library load, first launches
    torch.cuda.synchronize(dev)
    out = {}
    for name, mf in (("grouped", 32), ("row_by_row", 1)):
        t0 = time.perf_counter()
        res = S.run_jobs(jobs, max_fields=mf)
        torch.cuda.synchronize(dev)
        out[name] = time.perf_counter() - t0
    steps = sum(int(r.schwarzschild.n_steps.sum()) + int(r.flrw.n_steps.sum()) for r in res.values())
    photons = sum(r.flrw.trajectories.shape[0] for r in res.values())
    leg = {"workload": f"{len(jobs)} manifest rows ({SWEEP_MANIFEST['masses']} Msun x {SWEEP_MANIFEST['distances']} "
                       f"Mpc x N {SWEEP_MANIFEST['Ns']}), cone of 200 requested photons (183 traced) per leg, "
                       "RK4, record_every 4, static cosmology, observer-local FLRW coordinates",
           "rows": len(jobs), "photons_per_leg": photons, "photon_steps": steps,
           "grouped_s": out["grouped"], "row_by_row_s": out["row_by_row"],
           "rows_per_s": len(jobs) / out["grouped"], "photon_steps_per_s": steps / out["grouped"],
           "grouping_speedup": out["row_by_row"] / out["grouped"]}
    # the oracle on one row (the largest: 500 Mpc, N = 128), both legs, host threads
    from oracle import oracle as O
    from oracle.oracle import FieldSpec, Spacetime
    from excalibur_tool_gb300.trace import TraceConfig

    job = max(jobs, key=lambda j: (j.distance_mpc, j.flrw_grid_N))
    cfg = S.job_config(job)
    geo = R.geometry(cfg)
    _, ss, _, _ = R.schwarzschild_setup(cfg, geo)
    _, fs, shift = R.flrw_setup(cfg, geo)
    d = cfg.flrw_grid_size / cfg.flrw_grid_N
    phi = R.flrw_potential(cfg, geo)
    tc = TraceConfig(stepper="rk4", dt=geo.dlambda, dt_min=abs(geo.dlambda), dt_max=abs(geo.dlambda),
                     max_steps=geo.n_steps, record_every=cfg.record_every, observables=False)
    th = host_threads()
    t0 = time.perf_counter()
    O.trace(Spacetime(kind="schwarzschild", mass=cfg.mass, radius=cfg.radius, center=tuple(geo.lens_center),
                      analytical=True), ss.cpu().numpy(), tc, threads=th)
    O.trace(Spacetime(kind="flrw", cosmology="static",
                      fields=[FieldSpec(phi, (d, d, d), (0.0, 0.0, 0.0), "periodic", shift=tuple(shift))]),
            fs.cpu().numpy(), tc, threads=th)
    cpu_s = time.perf_counter() - t0
    leg["cpu_oracle_one_row"] = {"seconds": cpu_s, "threads": th, "row": job.jobid,
                                 "photon_steps": 2 * int(ss.shape[0]) * geo.n_steps,
                                 "note": "C restatement of the two legs (no host setup, no statistics)"}
    return leg


def gemm_tflops(dev, stream, m=1 << 20, members=4):
    """One forward layer of the ensemble ([members, m, 256] x [256, 256] BF16, bias + SiLU epilogue)
    timed alone with CUDA events: the surrogate's tensor-core kernel against the bf16 peak."""
    import torch

    from excalibur_tool_gb300.surrogate import kernels as Kn

    a = (torch.randn(m, 256, device=dev) * 0.5).to(torch.bfloat16)
    w = (torch.randn(members, 256, 256, device=dev) * 0.06).to(torch.bfloat16)
    bias = torch.zeros(members, 256, device=dev)
    h = torch.empty((members, m, 256), dtype=torch.bfloat16, device=dev)
    for _ in range(3):
        Kn.gemm(a, w, epilogue="bias_silu", bias=bias, c2=h)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record(stream)
    for _ in range(reps):
        Kn.gemm(a, w, epilogue="bias_silu", bias=bias, c2=h)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    sec = e0.elapsed_time(e1) / 1e3 / reps
    flops = 2.0 * members * m * 256 * 256
    return flops / sec / 1e12, sec, flops


def infer_tflops(dev, stream, m=1 << 20, members=4, depth=4, n_out=6):
    """The fused forward pass (exc_mlp_infer: every member's four 256-wide layers and head, one
    launch) on m feature rows, timed with CUDA events: against the bf16 peak, and beside the
    layer-by-layer path (four GEMM launches and the head kernel through HBM)."""
    import torch

    from excalibur_tool_gb300.surrogate import kernels as Kn

    x = (torch.randn(m, 256, device=dev) * 0.5).to(torch.bfloat16)
    w = (torch.randn(depth, members, 256, 256, device=dev) * 0.06).to(torch.bfloat16)
    b = torch.randn(depth, members, 256, device=dev) * 0.1
    wh = torch.randn(members, n_out, 256, device=dev) * 0.06
    bh = torch.zeros(members, n_out, device=dev)
    y = torch.empty((members, m, n_out), device=dev)
    ha = torch.empty((members, m, 256), dtype=torch.bfloat16, device=dev)
    hb = torch.empty_like(ha)

    def layered():
        inp = x
        for l in range(depth):
            o = ha if l % 2 == 0 else hb
            Kn.gemm(inp, w[l], epilogue="bias_silu", bias=b[l], c2=o)
            inp = o
        Kn.head(inp, wh, bh, y=y)

    def fused():
        Kn.infer(x, w, b, wh, bh, y)

    out = {}
    for name, fn in (("fused", fused), ("layer_by_layer", layered)):
        for _ in range(3):
            fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 5
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        sec = e0.elapsed_time(e1) / 1e3 / reps
        flops = 2.0 * members * m * (depth * 256 * 256 + 256 * n_out)
        out[name] = {"ms": sec * 1e3, "tflops": flops / sec / 1e12, "rows_per_s": m / sec}
    out["rows"], out["members"], out["flops_per_launch"] = m, members, flops
    return out


def _surrogate_map(args, metric, patch, cfg, fp64_rays_s, train_steps, lr=2e-3, strict_threshold=None):
    """Train the BF16 ensemble on 1,048,576 rays traced with `cfg`, fill an n x n map with
    ensemble-spread fallback and a seeded 1 % audit (both traced with `cfg`), and compare
    the map time with tracing every pixel. With `strict_threshold` the map is filled a second
    time with that (lower) spread threshold, which sends more pixels to the tracer."""
    from excalibur_tool_gb300.surrogate.model import SkySurrogate
    from excalibur_tool_gb300.surrogate.sky import fill_sky_map, training_set

    n_train = 1 << 20
    # untimed warm-up of every kernel and torch op on the path (first launches on a fresh
    # process load modules and, for torch's own kernels, may compile them)
    training_set(metric, patch, 8192, cfg, seed=2)
    uv, y, _, info = training_set(metric, patch, n_train, cfg, seed=1)
    tracer_rays_s = n_train / info["trace_s"]
    model = SkySurrogate(n_members=4, n_out=y.shape[1], seed=0, device=torch_device())
    rep = model.fit(uv, y, steps=train_steps, batch=8192, lr=lr, log_every=1000)
    fill_sky_map(model, metric, patch, cfg, n_side=128, std_threshold=1e-7, audit_fraction=0.01, audit_seed=6)
    _, mrep = fill_sky_map(model, metric, patch, cfg, n_side=args.map_side, std_threshold=1e-7,
                           audit_fraction=0.01, audit_seed=5)
    pixels = args.map_side ** 2
    every_pixel_tracer_s = pixels / tracer_rays_s
    every_pixel_fp64_s = pixels / fp64_rays_s
    map_s = mrep["total_s"]
    with_training = map_s + info["trace_s"] + rep.seconds
    step_flops = 11 * 2.0 * 8192 * 256 * 256 * 4
    strict = {}
    if strict_threshold is not None:
        _, srep = fill_sky_map(model, metric, patch, cfg, n_side=args.map_side, std_threshold=strict_threshold,
                               audit_fraction=0.01, audit_seed=5)
        srep.pop("threshold_tradeoff", None)
        s_map = srep["total_s"]
        strict = {"map_strict": {**srep, "speedup_vs_tracing_every_pixel": {
            f"{cfg.precision}_tracer": every_pixel_tracer_s / s_map, "fp64_tracer": every_pixel_fp64_s / s_map,
            "fp64_tracer_incl_training": every_pixel_fp64_s / (s_map + info["trace_s"] + rep.seconds)}}}
    return {
        "train": {"rays": n_train, "trace_s": info["trace_s"], "steps": rep.steps, "batch": rep.batch,
                  "seconds": rep.seconds, "final_loss_normalised": rep.final_loss,
                  "gemm_tflops_in_training_step": step_flops * rep.steps / rep.seconds / 1e12},
        "map": mrep,
        "every_pixel_trace_s": {f"{cfg.precision}_tracer": every_pixel_tracer_s, "fp64_tracer": every_pixel_fp64_s},
        "speedup_vs_tracing_every_pixel": {f"{cfg.precision}_tracer": every_pixel_tracer_s / map_s,
                                           "fp64_tracer": every_pixel_fp64_s / map_s,
                                           "fp64_tracer_incl_training": every_pixel_fp64_s / with_training},
        **strict,
    }


def profile_training(steps):
    """`steps` graph-captured training steps of the surrogate (4 members, 6 outputs, batch 8192)
    on 1,048,576 synthetic smooth targets, after a 32-step warm-up fit."""
    from excalibur_tool_gb300.surrogate.model import SkySurrogate

    rng = np.random.default_rng(4)
    uv = rng.uniform(-1, 1, (1 << 20, 2))
    y = np.stack([np.sin(3 * uv[:, 0]) * uv[:, 1], uv[:, 0] ** 2, np.cos(2 * uv[:, 1]), uv[:, 0] * uv[:, 1],
                  uv[:, 1], uv[:, 0]], 1)
    SkySurrogate(n_members=4, n_out=6, seed=0, device=torch_device()).fit(uv, y, steps=32, batch=8192, log_every=0)
    m = SkySurrogate(n_members=4, n_out=6, seed=0, device=torch_device())
    rep = m.fit(uv, y, steps=steps, batch=8192, log_every=0)
    return {"training_steps": steps, "ms_per_step": 1e3 * rep.seconds / steps, "batch": 8192, "members": 4}


def torch_device():
    import torch

    return torch.device("cuda", torch.cuda.current_device())


def run_surrogate(args, dev, stream, peaks, fp64_rays_s):
    """Learned sky map on the fast interpolators' field (base-node gradient), the batch's FP64
    rate as the every-pixel reference; plus the GEMM rate of one hidden layer."""
    import dataclasses

    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.surrogate.sky import Patch

    wl = workloads.flrw_patch(128, 2, 20.0, seed=1, device=dev)
    cfg = dataclasses.replace(wl.cfg, precision="mixed")
    cz = workloads.lcdm()
    patch = Patch((cz._eta_at_a1, *workloads.OBSERVER), tuple(workloads.LENS - workloads.OBSERVER), 20.0)
    out = {"workload": f"{args.map_side}x{args.map_side} map of a 20x20 deg patch; field: Plummer + random field "
                       "(seed 1) on a 128^3 float64 grid, InterpolatorFast (base-node gradient); training: "
                       "1,048,576 rays (numpy default_rng(1)) traced with the guarded mixed tracer; ensemble of "
                       "4 MLPs (64 Fourier frequencies, 4 x 256 SiLU)"}
    out.update(_surrogate_map(args, wl.metric, patch, cfg, fp64_rays_s, args.train_steps))
    tf_gemm, sec_gemm, fl_gemm = gemm_tflops(dev, stream)
    peak = peaks.get("bf16_tflops")
    out["gemm_kernel"] = {"bound": "tensor", "achieved": tf_gemm, "peak": peak, "unit": "TFLOP/s",
                          "frac": tf_gemm / peak if peak else None, "peak_source": "MEASURED_PEAKS.json bf16 burst",
                          "shape": "4 members x 1,048,576 x 256 x 256, bias + SiLU epilogue",
                          "algorithmic_flops_per_launch": fl_gemm, "ms_per_launch": sec_gemm * 1e3}
    inf = infer_tflops(dev, stream)
    out["inference_kernel"] = {"bound": "tensor", "achieved": inf["fused"]["tflops"], "peak": peak,
                               "unit": "TFLOP/s", "frac": inf["fused"]["tflops"] / peak if peak else None,
                               "peak_source": "MEASURED_PEAKS.json bf16 burst",
                               "shape": "4 members x 1,048,576 rows: four 256 x 256 layers (bias + SiLU) and a "
                                        "6-output head, one launch (exc_mlp_infer)",
                               "ms_per_launch": inf["fused"]["ms"], "layer_by_layer_ms": inf["layer_by_layer"]["ms"],
                               "layer_by_layer_tflops": inf["layer_by_layer"]["tflops"],
                               "algorithmic_flops_per_launch": inf["flops_per_launch"]}
    out["note"] = ("map redshift is taken at the box-face crossing; fallback and audit rays use the guarded mixed "
                   "tracer (|dz| <= 1e-9 of the FP64 tracer). The reference's base-node gradient makes its own "
                   "map rough at the pixel scale: adjacent-pixel second differences of the FP64-traced z are "
                   "~2e-7 rms, so no smooth model reaches 1e-7 on this field (see surrogate_smooth)")
    return out


def run_surrogate_smooth(args, dev):
    """The same pipeline on the same field read through the reference's slow Interpolator
    (grid/interpolator.py, continuous trilinear-blended gradient): training, fallback and audit
    rays traced with the guarded mixed tracer; every-pixel reference = the parity FP64 rate
    measured on a 65,536-ray sample of the same patch, on which the mixed tracer's errors
    against the parity build are stated too."""
    import dataclasses
    import torch

    from excalibur_tool_gb300 import _native as N
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.core.constants import one_Mpc
    from excalibur_tool_gb300.grid.grid import Grid
    from excalibur_tool_gb300.grid.interpolator import Interpolator
    from excalibur_tool_gb300.metrics.perturbed_flrw_metric_fast import PerturbedFLRWMetricFast
    from excalibur_tool_gb300.objects.fields import lens_plus_grf
    from excalibur_tool_gb300.photon.photons import Photons
    from excalibur_tool_gb300.surrogate.sky import Patch, pixel_centres
    from excalibur_tool_gb300.trace import TraceConfig, trace_batch

    cz = workloads.lcdm()
    n = 128
    phi = lens_plus_grf(n, workloads.BOX, workloads.LENS_MASS, 5 * one_Mpc, workloads.LENS, seed=1)
    grid = Grid((n,) * 3, (workloads.BOX / n,) * 3, (0.0, 0.0, 0.0))
    grid.add_field("Phi", phi)
    metric = PerturbedFLRWMetricFast(cz.a_of_eta, grid, Interpolator(grid), adot_of_eta=cz.adot_of_eta)
    # the slow class's bounds are [0, (n-1) spacing): stop at 990 Mpc, inside the last cell
    hi = 990 * one_Mpc
    dl = workloads.DLAMBDA
    cfg = TraceConfig(stepper="rk4", precision="mixed", dt=dl, dt_min=dl, dt_max=dl, max_steps=2 ** 62,
                      max_iter=100_000, stop_box=((0, 0, 0), (hi, hi, hi)), a_stop=0.5,
                      lens_center=tuple(workloads.LENS))
    patch = Patch((cz._eta_at_a1, *workloads.OBSERVER), tuple(workloads.LENS - workloads.OBSERVER), 20.0)
    sample = Photons(metric).generate_patch_points(pixel_centres(256), patch.origin, patch.axis, patch.patch_deg)
    parity = dataclasses.replace(cfg, precision="fp64")
    trace_batch(metric, sample[:4096], parity)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = trace_batch(metric, sample, parity)
    torch.cuda.synchronize()
    fp64_rays_s = sample.shape[0] / (time.perf_counter() - t0)
    trace_batch(metric, sample[:4096], cfg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rm = trace_batch(metric, sample, cfg)
    torch.cuda.synchronize()
    mixed_rays_s = sample.shape[0] / (time.perf_counter() - t0)
    raw = trace_batch(metric, sample, dataclasses.replace(cfg, precision="mixed_raw"))
    retrace = float((raw.status == N.PH_RETRACE).float().mean())
    out = {"workload": f"{args.map_side}x{args.map_side} map of the same 20x20 deg patch and field (seed 1, 128^3 "
                       "float64) read through the slow Interpolator (continuous gradient), box stop at 990 Mpc; "
                       "training, fallback and audit rays traced with the guarded mixed tracer",
           "fp64_parity_rays_per_s": fp64_rays_s,
           "fp64_parity_sample": "65,536 pixel centres (256 x 256) of the patch, one launch",
           "fp64_parity_status_counts": np.bincount(r.status.cpu().numpy(), minlength=12).tolist(),
           "mixed_on_sample": {"rays_per_s": mixed_rays_s, "speedup_vs_fp64": mixed_rays_s / fp64_rays_s,
                               "retrace_fraction": retrace, **errors_vs(r, rm)}}
    # strict: a spread threshold of 1e-8 keeps every audited pixel within 1e-7 (the configured 1e-7
    # threshold leaves ~1e-4 of them above it; the map report's threshold_tradeoff shows the curve)
    out.update(_surrogate_map(args, metric, patch, cfg, fp64_rays_s, args.smooth_train_steps, lr=3.5e-3,
                              strict_threshold=1e-8))
    return out


def errors_vs(ref, r, mask=None):
    """|dz|, relative time-delay and deflection error of `r` against the parity build `ref`."""
    from excalibur_tool_gb300.observables.lensing import deflection_angle, time_delay_excess, redshift_total

    sel = slice(None) if mask is None else mask.cpu().numpy()
    o0 = ref.obs.cpu().numpy()[sel]
    o1 = r.obs.cpu().numpy()[sel]
    z0, z1 = redshift_total(o0), redshift_total(o1)
    t0, t1 = time_delay_excess(o0), time_delay_excess(o1)
    a0, a1 = deflection_angle(o0), deflection_angle(o1)
    return {"max_abs_dz": float(np.nanmax(np.abs(z1 - z0))),
            "max_rel_time_delay": float(np.nanmax(np.abs(t1 - t0) / np.maximum(np.abs(t0), 1e-300))),
            "max_abs_deflection_rad": float(np.nanmax(np.abs(a1 - a0))),
            "max_rel_position": float(np.nanmax(np.abs(r.state.cpu().numpy()[sel, :4] - ref.state.cpu().numpy()[sel, :4]) /
                                                np.maximum(np.abs(ref.state.cpu().numpy()[sel, :4]), 1e-300)))}


# ------------------------------------------------------------------ CPU side
def _oracle_inputs(wl=None):
    """Workload inputs as host arrays for the oracle (built without the GPU library)."""
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.core.constants import c, one_Mpc
    from excalibur_tool_gb300.objects.fields import lens_plus_grf
    from oracle import oracle as O
    from oracle.oracle import FieldSpec, Spacetime

    cz = workloads.lcdm()
    n = 128
    phi = lens_plus_grf(n, workloads.BOX, workloads.LENS_MASS, 5 * one_Mpc, workloads.LENS, seed=2)
    spec = Spacetime(kind="flrw", fields=[FieldSpec(phi, (workloads.BOX / n,) * 3, (0.0, 0.0, 0.0), "periodic")],
                     cosmology="table", a_grid=cz.a_grid, eta_min=cz.eta_min, eta_step=cz.eta_step, H0=cz.H0,
                     omega=(0.3, 0.0, 0.0, 0.7))
    if wl is not None:
        states = wl.states.cpu().numpy()
        cfg = wl.cfg
    else:
        k = np.array([1.0, 0.0, 0.0])
        e1, e2 = np.array([0.0, 1.0, 0.0]), np.array([0.0, 0.0, 1.0])
        half = np.tan(np.deg2rad(5.0))
        t = (np.arange(256) + 0.5) / 256 * 2 - 1
        A, B = np.meshgrid(t, t, indexing="ij")
        d = k[None] + (A.reshape(-1, 1) * half) * e1[None] + (B.reshape(-1, 1) * half) * e2[None]
        d /= np.linalg.norm(d, axis=1)[:, None]
        states = np.zeros((len(d), 8))
        states[:, 0] = cz._eta_at_a1
        states[:, 1:4] = workloads.OBSERVER
        states[:, 5:8] = d * c
        states, _ = O.null_init(spec, states, -1.0)
        from excalibur_tool_gb300.trace import TraceConfig

        B_ = workloads.BOX
        cfg = TraceConfig(stepper="rk4", dt=workloads.DLAMBDA, dt_min=workloads.DLAMBDA, dt_max=workloads.DLAMBDA,
                          max_steps=2 ** 62, max_iter=100_000, stop_box=((0, 0, 0), (B_, B_, B_)), a_stop=0.5,
                          lens_center=tuple(workloads.LENS))
    return spec, states, cfg


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_oracle(spec, states, cfg, threads, target_s=12.0, full=False, result=None):
    """Oracle photon-steps/s on a bounded sample (about target_s of CPU work), or on the whole
    batch (`full`). `result` (a dict) receives the traced sample and its indices."""
    from oracle import oracle as O

    if full:
        n_sample = len(states)
    else:
        probe = states[:: max(1, len(states) // (threads * 8))][: threads * 8]
        t0 = time.perf_counter()
        r = O.trace(spec, probe, cfg, threads=threads)
        dt = time.perf_counter() - t0
        rate = r.n_steps.sum() / dt
        per_photon = r.n_steps.mean()
        n_sample = int(min(len(states), max(threads * 16, target_s * rate / max(per_photon, 1))))
    idx = np.linspace(0, len(states) - 1, n_sample).astype(int)
    t0 = time.perf_counter()
    r = O.trace(spec, states[idx], cfg, threads=threads)
    dt = time.perf_counter() - t0
    if result is not None:
        result["idx"], result["oracle"] = idx, r
    return float(r.n_steps.sum() / dt), n_sample, float(dt), int(r.n_steps.sum())


def parity_vs_oracle(res, idx, o):
    """The GPU batch against the oracle (the reference's arithmetic, libm pow) on photons idx:
    statuses and step counts must agree; states and observables to the last digits."""
    from excalibur_tool_gb300 import _native as N
    from excalibur_tool_gb300.observables.lensing import deflection_angle, redshift_total

    st = res.state.cpu().numpy()[idx]
    ob = res.obs.cpu().numpy()[idx]

    def rel(a, b):
        den = np.maximum(np.abs(a), np.abs(b))
        with np.errstate(invalid="ignore", divide="ignore"):
            return float(np.nanmax(np.where(den > 0, np.abs(a - b) / den, 0.0)))

    cols = ("a_obs", "a_em", "phi_obs", "phi_em", "path", "chord", "min_r", "v1x", "v1y", "v1z")
    ie, ip = N.OBS_COLS.index("excess"), N.OBS_COLS.index("path")
    return {"n_compared": int(len(idx)), "of": int(res.state.shape[0]),
            "status_equal": bool(np.array_equal(res.status.cpu().numpy()[idx], o.status)),
            "n_steps_equal": bool(np.array_equal(res.n_steps.cpu().numpy()[idx], o.n_steps)),
            "bit_identical_states": int((st == o.state).all(axis=1).sum()),
            "max_rel_state": rel(st, o.state),
            "max_rel_obs": {c: rel(ob[:, N.OBS_COLS.index(c)], o.obs[:, N.OBS_COLS.index(c)]) for c in cols},
            "max_abs_dz": float(np.nanmax(np.abs(redshift_total(ob) - redshift_total(o.obs)))),
            "max_excess_diff_over_path": float(np.nanmax(np.abs(ob[:, ie] - o.obs[:, ie]) / o.obs[:, ip])),
            "max_rel_excess": rel(ob[:, ie], o.obs[:, ie]),
            "max_abs_deflection_rad": float(np.nanmax(np.abs(deflection_angle(ob) - deflection_angle(o.obs)))),
            "oracle": "oracle/exc_oracle.c (reference operation order, glibc pow), every photon of the batch"}


def reference_pool(states, n_rays=2048, n_steps=200):
    """The reference's own multiprocessing paths (Integrator(mode="chunked"), then
    PersistentPoolIntegrator, from the package installed under baseline/_ref, one worker per host
    core) on a linspace sample of the batch's initial states, n_steps RK4 steps each, in a process
    of its own (oracle/reference_pool.py). Returns its measurement, or {"unavailable": why}."""
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.core.constants import one_Mpc
    from excalibur_tool_gb300.objects.fields import lens_plus_grf

    if not os.path.isdir(os.path.join(ROOT, "baseline", "_ref", "excalibur")):
        return {"unavailable": "the reference package is not installed under baseline/_ref"}
    phi = lens_plus_grf(128, workloads.BOX, workloads.LENS_MASS, 5 * one_Mpc, workloads.LENS, seed=2)
    idx = np.linspace(0, len(states) - 1, min(n_rays, len(states))).astype(int)
    with tempfile.TemporaryDirectory() as tmp:
        inp, out = os.path.join(tmp, "in.npz"), os.path.join(tmp, "out.json")
        np.savez(inp, phi=phi, box=workloads.BOX, states=np.asarray(states)[idx], dt=workloads.DLAMBDA,
                 n_steps=n_steps)
        r = subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "reference_pool.py"), "--inputs", inp,
                            "--out", out, "--persistent"], capture_output=True, text=True, timeout=900)
        if r.returncode != 0:
            return {"unavailable": "reference pool run failed: " + (r.stderr.strip().splitlines() or ["?"])[-1]}
        with open(out) as f:
            res = json.load(f)
    res["unit"] = UNIT
    res["sample"] = (f"{len(idx)} of {len(states)} initial states of the batch (linspace), {n_steps} RK4 steps "
                     f"each (the reference has no box stop)")
    return res


def cpu_baseline(wl, steps_per_batch, res=None):
    """The oracle on the host cores over the whole batch (~8 s on 16 threads): its rate is the
    CPU baseline, and its states are compared with the GPU's (`res`) photon for photon."""
    spec, states, cfg = _oracle_inputs(wl)
    threads = host_threads()
    traced = {}
    rate, n, dt, steps = time_oracle(spec, states, cfg, threads, full=True, result=traced)
    out = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{n} of {len(states)} photons of the same batch ({steps} photon-steps, {dt:.1f} s), "
                     f"C restatement of integrate_single (oracle/exc_oracle.c), {threads} threads"}
    if res is not None and res.obs is not None:
        out["parity"] = parity_vs_oracle(res, traced["idx"], traced["oracle"])
    out["reference_pool"] = reference_pool(states)
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return
    spec, states, cfg = _oracle_inputs(None)
    threads = host_threads()
    from oracle import oracle as O

    per_step = []
    for k in range(args.warmup + args.steps):
        rate, n, dt, steps = time_oracle(spec, states, cfg, threads, target_s=10.0)
        if k >= args.warmup:
            per_step.append((rate, n, dt, steps))
    total_steps = sum(p[3] for p in per_step)
    total_s = sum(p[2] for p in per_step)
    value = total_steps / total_s
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic (seeded Plummer + Gaussian random field; patch of directions)",
            "config": {"workload": WORKLOAD, "precision": "fp64", "photons": len(states),
                       "parallelism": f"{threads} host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"each step: {per_step[0][1]} of {len(states)} photons "
                                       f"(~10 s of CPU work), C restatement of integrate_single "
                                       f"(oracle/exc_oracle.c), {threads} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    # the reference's own Python path (its multiprocessing pool) beside the C restatement
    line["cpu_baseline"]["reference_pool"] = reference_pool(states)
    print(json.dumps(line), flush=True)


def profile_redshift_map(n: int, n_rows: int = 64, reps: int = 5, host_sample: int = 2000) -> dict:
    """The redshift-map kernels on n synthetic FLRW histories [n, 64, 14] (seeded; the first
    row's quantity columns NaN, as the runners record them): device-resident table, sky
    projection and a 512^2 binned map, timed with CUDA events (the stack is larger than L2 from
    n = 40k on); beside them the host path the reference runs per photon
    (RedshiftCalculator.compute_all_components, scipy's Simpson) on a sample of photons."""
    import torch
    from excalibur_tool_gb300.observables import maps
    from excalibur_tool_gb300.observables.redshift import RedshiftCalculator

    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(21)
    f64 = dict(dtype=torch.float64, device=dev)
    rec = torch.empty((n, n_rows, 14), **f64)
    rec[..., 0] = 4.6e17 - torch.cumsum(torch.rand((n, n_rows), generator=g, **f64) * 1e14 + 5e13, dim=1)
    rec[..., 1:4] = torch.rand((n, n_rows, 3), generator=g, **f64) * 3e24
    rec[..., 4] = -1.0
    rec[..., 5:8] = torch.randn((n, n_rows, 3), generator=g, **f64) * 1e5 + torch.tensor([-3e8, 0.0, 0.0], **f64)
    rec[..., 8] = 1.0 / (1.0 + torch.linspace(0.0, 0.3, n_rows, **f64))
    rec[..., 9] = torch.randn((n, n_rows), generator=g, **f64) * 1e-6
    rec[..., 10:13] = torch.randn((n, n_rows, 3), generator=g, **f64) * 1e-9
    rec[..., 13] = torch.randn((n, n_rows), generator=g, **f64) * 1e-24
    rec[:, 0, 8:] = float("nan")

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for e0, e1 in evs:
            e0.record()
            fn()
            e1.record()
        torch.cuda.synchronize()
        return sum(e0.elapsed_time(e1) for e0, e1 in evs) / reps / 1e3

    t_table = timed(lambda: maps.redshift_table(rec))
    t_sky = timed(lambda: maps.sky_projection(rec))
    table = maps.redshift_table(rec)
    xp, yp, _ = maps.sky_projection(rec)
    ext = maps.square_extent(xp.cpu().numpy(), yp.cpu().numpy())
    t_bin = timed(lambda: maps.bin_sky_map(xp, yp, table[:, 4], grid_resolution=512, extent=ext))
    sample = rec[:host_sample].cpu().numpy()
    t0 = time.perf_counter()
    for tr in sample:
        RedshiftCalculator(tr[~np.isnan(tr).any(axis=1)]).compute_all_components()
    t_host = (time.perf_counter() - t0) / len(sample)
    # the time-delay script's per-photon loop (compute_time_delay_map.py:97-126, 275-297): a
    # norm per recorded segment, then the chord
    t0 = time.perf_counter()
    for tr in sample:
        pos = tr[~np.isnan(tr).any(axis=1)][:, 1:4]
        path = 0.0
        for i in range(len(pos) - 1):
            path += np.linalg.norm(pos[i + 1] - pos[i])
        _ = path / 299792458.0 - np.linalg.norm(pos[-1] - pos[0]) / 299792458.0
    t_host_td = (time.perf_counter() - t0) / len(sample)
    algo_bytes = n * (n_rows * 14 * 8 + len(maps.RS_COLUMNS) * 8)
    return {"redshift_map_photons": n, "rows": n_rows, "table_ms": t_table * 1e3,
            "table_photons_per_s": n / t_table, "table_algo_gbs": algo_bytes / t_table / 1e9,
            "table_columns": len(maps.RS_COLUMNS),
            "sky_projection_ms_incl_host_sync": t_sky * 1e3, "bin_512_ms_incl_host_copy": t_bin * 1e3,
            "host_calculator_photons_per_s": 1.0 / t_host,
            "host_time_delay_photons_per_s": 1.0 / t_host_td, "host_sample": len(sample)}


def profile_batching(scale: int) -> dict:
    """One multi-field RK45 launch of the batching workload at 1/scale (for profiling)."""
    import torch

    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.trace import trace_batch

    dev = torch.device("cuda", 0)
    wl = workloads.multi_field(n_sky=(1 << 20) // scale, n_side=max(8, 256 // int(round(scale ** 0.5))), device=dev)
    t0 = time.perf_counter()
    r = trace_batch(wl.metric, wl.states, wl.cfg, field_index=wl.field_index)
    torch.cuda.synchronize(dev)
    return {"photons": int(wl.states.shape[0]), "seconds": time.perf_counter() - t0,
            "rk45_trials": int(r.n_iter.sum()), "accepted": int(r.n_steps.sum())}


def profile_rk45_mixed(side: int) -> dict:
    """The mixed RK45 tracer once on side x side rays of the slow-Interpolator patch over a 128^3
    float32 grid (for profiling)."""
    import dataclasses
    import torch

    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.trace import trace_batch

    dev = torch.device("cuda", 0)
    wl = workloads.flrw_patch_rk45(128, side, 20.0, seed=4, device=dev)
    t0 = time.perf_counter()
    r = trace_batch(wl.metric, wl.states, dataclasses.replace(wl.cfg, precision="mixed_raw"))
    torch.cuda.synchronize(dev)
    return {"photons": int(wl.states.shape[0]), "seconds": time.perf_counter() - t0,
            "rk45_trials": int(r.n_iter.sum()), "accepted": int(r.n_steps.sum())}


def profile_aux(n: int) -> dict:
    """The auxiliary kernels once each: the device patch generator on n rays, the lens potential
    written on a 128^3 grid, and the surrogate's Born features on n directions of a 20-degree
    patch (for profiling)."""
    import torch

    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.core.constants import one_Mpc
    from excalibur_tool_gb300.objects import spherical_mass as SM
    from excalibur_tool_gb300.photon.photons import Photons
    from excalibur_tool_gb300.surrogate import sky

    dev = torch.device("cuda", 0)
    wl = workloads.flrw_patch(128, 8, device=dev)
    cz = workloads.lcdm()
    side = int(round(n ** 0.5))
    ph = Photons(wl.metric)
    st = ph.device_patch_grid(side, [cz._eta_at_a1, *workloads.OBSERVER], workloads.LENS - workloads.OBSERVER, 10.0)
    lens = SM.spherical_mass(workloads.LENS_MASS, 5 * one_Mpc, workloads.LENS)
    pot = lens.potential_grid((128, 128, 128), (workloads.BOX / 128,) * 3, device=dev)
    patch = sky.Patch(origin=(cz._eta_at_a1, *workloads.OBSERVER),
                      axis=tuple(workloads.LENS - workloads.OBSERVER), patch_deg=20.0)
    uv = torch.rand((n, 2), dtype=torch.float64, device=dev) * 2 - 1
    f = sky.born_features(wl.metric, patch, uv, wl.cfg.stop_box)
    torch.cuda.synchronize(dev)
    return {"generated": int(st.shape[0]), "potential_nodes": int(pot.numel()), "born_rows": int(f.shape[0])}


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args.gpus))
    if args.profile_gemm:
        import torch

        dev = torch.device("cuda", 0)
        tf, sec, fl = gemm_tflops(dev, torch.cuda.current_stream(dev), m=args.profile_gemm)
        print(json.dumps({"gemm_tflops": tf, "ms": sec * 1e3, "flops": fl, "rows": args.profile_gemm}), flush=True)
        return
    if args.profile_infer:
        import torch

        dev = torch.device("cuda", 0)
        print(json.dumps(infer_tflops(dev, torch.cuda.current_stream(dev), m=args.profile_infer)), flush=True)
        return
    if args.profile_training:
        print(json.dumps(profile_training(args.profile_training)), flush=True)
        return
    if args.profile_sweep:
        import torch
        from excalibur_tool_gb300.runners import sweep as S

        with tempfile.TemporaryDirectory() as tmp:
            path = os.path.join(tmp, "manifest.csv")
            S.make_manifest(path, **SWEEP_MANIFEST)
            jobs = S.read_jobs(path)
        t0 = time.perf_counter()
        res = S.run_jobs(jobs)
        torch.cuda.synchronize()
        print(json.dumps({"sweep_rows": len(res), "seconds": time.perf_counter() - t0}), flush=True)
        return
    if args.profile_redshift_map:
        print(json.dumps(profile_redshift_map(args.profile_redshift_map)), flush=True)
        return
    if args.profile_batching:
        print(json.dumps(profile_batching(args.profile_batching)), flush=True)
        return
    if args.profile_aux:
        print(json.dumps(profile_aux(args.profile_aux)), flush=True)
        return
    if args.profile_rk45_mixed:
        print(json.dumps(profile_rk45_mixed(args.profile_rk45_mixed)), flush=True)
        return
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
