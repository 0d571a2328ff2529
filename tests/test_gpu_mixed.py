"""Mixed-precision tracer (FP32 right-hand side, double-float state) against the
FP64 oracle on the 1000 Mpc lens-plus-random-field patch.

The mixed tracer is not bit-faithful to the reference; it is held to error
bounds on the observables that come out of a trace (stated here and in the
assertions):

* redshift:            |dz| <= 1e-9
* time-delay excess:   relative <= 1e-6
* deflection angle:    |d alpha| <= 1e-5 * alpha + 5e-11 rad
* accepted steps and final status: identical (same box-exit step)

Rays whose mixed trajectory comes within its error window of a cell face of
the reference's base-node gradient (or of a stop threshold) are re-traced by
the FP64 parity tracer inside the same `exc_trace` call; `mixed_raw` exposes
the mixed launch alone, with those rays marked EXC_PH_RETRACE.
"""
import dataclasses
import os

import numpy as np
import pytest

from helpers import gpu_trace, rel_err
from test_gpu_parity import _flrw_patch_case
from excalibur_tool_gb300 import _native as N
from excalibur_tool_gb300.observables import lensing as L
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DZ_MAX = 1e-9
TAU_REL_MAX = 1e-6
DEFL_REL, DEFL_ABS = 1e-5, 5e-11


def _check_observables(r, o):
    assert np.array_equal(r["status"], o.status)
    assert np.array_equal(r["n_steps"], o.n_steps)
    z_gpu, z_ref = L.redshift_total(r["obs"]), L.redshift_total(o.obs)
    assert np.abs(z_gpu - z_ref).max() <= DZ_MAX
    t_gpu, t_ref = L.time_delay_excess(r["obs"]), L.time_delay_excess(o.obs)
    assert (np.abs(t_gpu - t_ref) / np.abs(t_ref)).max() <= TAU_REL_MAX
    a_gpu, a_ref = L.deflection_angle(r["obs"]), L.deflection_angle(o.obs)
    assert (np.abs(a_gpu - a_ref) <= DEFL_REL * np.abs(a_ref) + DEFL_ABS).all()
    # trajectory end point and path length: FP32-RHS-limited, far below a grid cell
    assert rel_err(r["state"][:, :4], o.state[:, :4]).max() <= 1e-8
    i = N.OBS_COLS.index("path")
    assert rel_err(r["obs"][:, i], o.obs[:, i]).max() <= 1e-7


@pytest.mark.parametrize("n_grid,side", [(128, 24), (32, 16)])
def test_mixed_matches_fp64_oracle(cuda, n_grid, side):
    spec, st, cfg = _flrw_patch_case(n_grid, side)
    cfg = dataclasses.replace(cfg, precision="mixed")
    r = gpu_trace(spec, st, cfg)
    o = O.trace(spec, st, cfg, threads=8)
    _check_observables(r, o)


@pytest.mark.parametrize("a_stop,max_steps,want", [(0.93, 10000, "A_STOP"), (None, 300, "STEPS")])
def test_mixed_a_stop_and_step_cap(cuda, a_stop, max_steps, want):
    """The a(eta) stop and the step cap end photons where the FP64 tracer does."""
    spec, st, cfg = _flrw_patch_case(32, 8)
    cfg = dataclasses.replace(cfg, precision="mixed", a_stop=a_stop, max_steps=max_steps)
    r = gpu_trace(spec, st, cfg)
    o = O.trace(spec, st, cfg, threads=8)
    assert (o.status == getattr(N, "PH_" + want)).all()
    _check_observables(r, o)


def test_mixed_queue_and_static_schedules_agree(cuda):
    spec, st, cfg = _flrw_patch_case(32, 12)
    cfg = dataclasses.replace(cfg, precision="mixed")
    a = gpu_trace(spec, st, dataclasses.replace(cfg, use_queue=True))
    b = gpu_trace(spec, st, dataclasses.replace(cfg, use_queue=False))
    for k in ("state", "status", "n_steps", "obs"):
        assert np.array_equal(a[k], b[k], equal_nan=True)


def test_mixed_float32_grid(cuda):
    """A float32 grid (one plane) traces against the oracle run on the same rounded grid."""
    import torch
    from helpers import gpu_metric
    from excalibur_tool_gb300.trace import trace_batch

    spec, st, cfg = _flrw_patch_case(32, 8)
    spec.fields[0].data = spec.fields[0].data.astype(np.float32).astype(np.float64)
    cfg = dataclasses.replace(cfg, precision="mixed")
    m = gpu_metric(spec, field_dtype=np.float32)
    res = trace_batch(m, torch.as_tensor(st).cuda(), cfg)
    torch.cuda.synchronize()
    r = {k: getattr(res, a).cpu().numpy() for k, a in
         (("state", "state"), ("status", "status"), ("n_steps", "n_steps"), ("obs", "obs"))}
    o = O.trace(spec, st, cfg, threads=8)
    _check_observables(r, o)


@pytest.fixture(scope="module")
def patch(cuda):
    """The 65,536-ray 1000 Mpc lens patch (128^3 float64 grid) and its oracle trace."""
    from excalibur_tool_gb300 import workloads
    from oracle.oracle import FieldSpec, Spacetime

    wl = workloads.flrw_patch(128, 256, device=cuda)
    cz = workloads.lcdm()
    phi = np.asarray(wl.metric.interp.grid.fields["Phi"])
    spec = Spacetime(kind="flrw", fields=[FieldSpec(phi, (workloads.BOX / 128,) * 3, (0.0, 0.0, 0.0), "periodic")],
                     cosmology="table", a_grid=cz.a_grid, eta_min=cz.eta_min, eta_step=cz.eta_step, H0=cz.H0,
                     omega=(0.3, 0.0, 0.0, 0.7))
    states = wl.states.cpu().numpy()
    o = O.trace(spec, states, wl.cfg, threads=os.cpu_count() or 1)
    return wl, states, o


def _run(wl, precision):
    import torch
    from excalibur_tool_gb300.trace import trace_batch

    res = trace_batch(wl.metric, wl.states, dataclasses.replace(wl.cfg, precision=precision))
    torch.cuda.synchronize()
    return {k: getattr(res, k).cpu().numpy() for k in ("state", "status", "n_steps", "obs")}


def test_mixed_full_patch_every_ray_within_bounds(patch):
    """All 65,536 rays of the lens patch meet the bounds against the FP64 oracle."""
    wl, states, o = patch
    _check_observables(_run(wl, "mixed"), o)


def test_mixed_raw_hands_back_untouched_rays(patch):
    """mixed_raw marks the guarded rays and leaves their state as it came in;
    mixed = mixed_raw elsewhere and = the FP64 parity tracer on those rays."""
    wl, states, o = patch
    raw = _run(wl, "mixed_raw")
    mixed = _run(wl, "mixed")
    back = raw["status"] == N.PH_RETRACE
    assert 0 < back.sum() < 0.05 * len(back)          # a small fraction (about 1.5 % here)
    assert np.array_equal(raw["state"][back], states[back])
    keep = ~back
    for k in ("state", "status", "n_steps", "obs"):
        assert np.array_equal(raw[k][keep], mixed[k][keep], equal_nan=True), k
    assert not (mixed["status"] == N.PH_RETRACE).any()
    assert np.array_equal(mixed["n_steps"][back], o.n_steps[back])
    assert rel_err(mixed["state"][back], o.state[back]).max() <= 1e-12


def test_device_sized_retrace_equals_every_warp(patch):
    """The re-trace pass with the work queue keeps one warp an SM for the ~1,000 rays handed back
    on the lens patch (the rest of the launch leaves at once); without the queue every warp takes
    its static share. The results are the same bits, and for several schedules of the launch."""
    import torch
    from excalibur_tool_gb300.trace import trace_batch

    wl, states, o = patch
    cfg = dataclasses.replace(wl.cfg, precision="mixed")
    ref = trace_batch(wl.metric, wl.states, dataclasses.replace(cfg, use_queue=False))
    for block, per_sm in ((0, 0), (64, 4), (128, 4), (96, 3)):
        got = trace_batch(wl.metric, wl.states, dataclasses.replace(cfg, block_size=block, blocks_per_sm=per_sm))
        torch.cuda.synchronize()
        for k in ("state", "status", "n_steps", "n_iter"):
            assert torch.equal(getattr(got, k), getattr(ref, k)), (k, block, per_sm)
        assert torch.allclose(got.obs, ref.obs, rtol=0, atol=0, equal_nan=True)


def test_pipelined_batches_match_single_launches(patch):
    """Re-traces overlapped on a side stream give the same photons as precision "mixed"."""
    import torch
    from excalibur_tool_gb300.trace import trace_pipelined

    wl, states, o = patch
    parts = [wl.states[i * 16384:(i + 1) * 16384].contiguous() for i in range(4)]
    res = trace_pipelined(wl.metric, parts, dataclasses.replace(wl.cfg, precision="mixed"))
    torch.cuda.synchronize()
    whole = _run(wl, "mixed")
    got = np.concatenate([r.state.cpu().numpy() for r in res])
    assert np.array_equal(got, whole["state"])
    assert np.array_equal(np.concatenate([r.status.cpu().numpy() for r in res]), whole["status"])
    assert np.array_equal(np.concatenate([r.obs.cpu().numpy() for r in res]), whole["obs"], equal_nan=True)


@pytest.mark.parametrize("n_grid,side", [(128, 24), (32, 16)])
def test_mixed_slow_interpolator_matches_fp64_oracle(cuda, n_grid, side):
    """The slow Interpolator's continuous gradient (grad_mode "trilinear"): the same error bounds,
    and no ray needs the FP64 re-trace (a discontinuity of the RHS is what makes one necessary;
    here the formula changes only at the grid's outer cells, which the rays do not reach)."""
    from excalibur_tool_gb300.core.constants import one_Mpc

    spec, st, cfg = _flrw_patch_case(n_grid, side)
    spec.fields[0].boundary = "error"
    spec.fields[0].gradient = "trilinear"
    hi = 990 * one_Mpc if n_grid == 128 else 960 * one_Mpc     # inside the bounds [0, (n-1) spacing)
    cfg = dataclasses.replace(cfg, precision="mixed_raw", stop_box=((0, 0, 0), (hi, hi, hi)))
    raw = gpu_trace(spec, st, cfg)
    assert (raw["status"] != N.PH_RETRACE).all()
    r = gpu_trace(spec, st, dataclasses.replace(cfg, precision="mixed"))
    o = O.trace(spec, st, dataclasses.replace(cfg, precision="fp64"), threads=8)
    assert (o.status == N.PH_LEFT_BOX).all()
    _check_observables(r, o)


def _rk45_face_case(n_grid, side, renormalize_every=0):
    """The patch through the slow Interpolator (continuous gradient) with adaptive RK45
    (Fehlberg, rtol 1e-8, atol 1e-12, dt in [1e10 s, 10 Mpc / c]) and the box stop on the face,
    1.5 cells inside the last node (the slow class's bounds)."""
    from excalibur_tool_gb300.core.constants import one_Mpc

    spec, st, cfg = _flrw_patch_case(n_grid, side)
    spec.fields[0].gradient = "trilinear"
    hi = (n_grid - 1.5) * 1000 * one_Mpc / n_grid
    cfg = dataclasses.replace(cfg, stepper="rk45", tableau="fehlberg", rtol=1e-8, atol=1e-12, dt_min=1e10,
                              dt_max=20 * cfg.dt, max_iter=20000, stop_box=((0, 0, 0), (hi, hi, hi)),
                              stop_face=True, renormalize_every=renormalize_every)
    return spec, st, cfg


def _deviations(r_obs, o_obs, ok):
    z = np.abs(L.redshift_total(r_obs)[ok] - L.redshift_total(o_obs)[ok])
    t0 = L.time_delay_excess(o_obs)[ok]
    t = np.abs(L.time_delay_excess(r_obs)[ok] - t0) / np.abs(t0)
    a = np.abs(L.deflection_angle(r_obs)[ok] - L.deflection_angle(o_obs)[ok])
    return {"dz": z, "tau": t, "alpha": a}


def _check_within_conditioning(r, spec, st, cfg):
    """Adaptive RK45 end points are determined only to the method's truncation error: two step
    sequences that part in their last digits (an error estimate a little above or below 1) end
    with redshifts ~1e-6 apart at rtol 1e-8 on these fields, and the FP64 parity tracer's own
    result moves by as much when its initial speed changes by one part in 1e9 (the FP64 fast
    build, another sum order, moves by as much too). So the mixed tracer is held to that band:
    against the oracle's FP64 RK45 (the parity tracer's arithmetic), its deviation in z, time
    delay and deflection is at most 3x the oracle's own deviation under the 1e-9 speed change
    at the largest ray and 5x at the median (with floors at the RK4 bounds). Both end every ray
    on the box face."""
    o = O.trace(spec, st, cfg, threads=8)
    st2 = st.copy()
    st2[:, 5:8] *= 1.0 + 1e-9
    o2 = O.trace(spec, st2, cfg, threads=8)
    assert (o.status == N.PH_LEFT_BOX).all() and (o2.status == N.PH_LEFT_BOX).all()
    assert np.array_equal(r["status"], o.status)
    ok = np.ones(len(st), bool)
    mix, ref = _deviations(r["obs"], o.obs, ok), _deviations(o2.obs, o.obs, ok)
    floor = {"dz": DZ_MAX, "tau": TAU_REL_MAX, "alpha": DEFL_ABS}
    for k in mix:
        assert mix[k].max() <= 3.0 * ref[k].max() + floor[k], (k, mix[k].max(), ref[k].max())
        assert np.median(mix[k]) <= 5.0 * np.median(ref[k]) + floor[k], (k, np.median(mix[k]), np.median(ref[k]))
    return o


@pytest.mark.parametrize("n_grid,side", [(32, 12), (128, 12)])
def test_mixed_rk45_within_the_fp64_tracers_conditioning(cuda, n_grid, side):
    """Mixed-precision RK45 (FP32 stages, double-float state, FP64 error norm and step control)
    against the oracle's FP64 RK45 on the same face-stopped patch, within the band that the FP64
    tracer's own sensitivity sets (_check_within_conditioning)."""
    spec, st, cfg = _rk45_face_case(n_grid, side)
    r = gpu_trace(spec, st, dataclasses.replace(cfg, precision="mixed"))
    o = _check_within_conditioning(r, spec, st, cfg)
    # the adaptive steps: as many as the FP64 tracer takes, within a few per cent
    assert abs(int(r["n_steps"].sum()) - int(o.n_steps.sum())) <= 0.05 * int(o.n_steps.sum())


def test_mixed_renormalisation_matches_fp64_oracle(cuda):
    """The null-condition renormalisation (integrator.py:298-335), in FP64 inside the mixed
    tracer: every 10 accepted steps with RK4 (base-node field) within the RK4 bounds of the
    oracle's FP64 renormalised trace; every step with RK45 (slow Interpolator) within the FP64
    tracer's conditioning band.

    The reference's FLRW equations do not keep the null condition (u^0 drifts from -1.00 to
    about -1.24 across the patch while |u|/c grows to 1.49), so each renormalisation moves u^0
    by a finite amount, and with RK45 "every N accepted steps" falls where each tracer's step
    sequence puts it."""
    spec, st, cfg = _flrw_patch_case(32, 8)
    cfg = dataclasses.replace(cfg, renormalize_every=10)
    r = gpu_trace(spec, st, dataclasses.replace(cfg, precision="mixed"))
    o = O.trace(spec, st, cfg, threads=8)
    _check_observables(r, o)
    spec, st, cfg = _rk45_face_case(32, 8, renormalize_every=1)
    r = gpu_trace(spec, st, dataclasses.replace(cfg, precision="mixed"))
    _check_within_conditioning(r, spec, st, cfg)


def test_mixed_rk45_retraces_only_near_the_outer_cells(cuda):
    """With the slow Interpolator the mixed RK45 tracer hands back only rays whose stage points
    come within the error window of the grid's outer cells (none on this patch), and those it
    keeps equal what precision "mixed" returns."""
    spec, st, cfg = _rk45_face_case(32, 12)
    raw = gpu_trace(spec, st, dataclasses.replace(cfg, precision="mixed_raw"))
    mixed = gpu_trace(spec, st, dataclasses.replace(cfg, precision="mixed"))
    back = raw["status"] == N.PH_RETRACE
    assert back.mean() < 0.05
    for k in ("state", "status", "n_steps", "obs"):
        assert np.array_equal(raw[k][~back], mixed[k][~back], equal_nan=True), k
