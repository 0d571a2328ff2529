"""Batching: several potential fields of different sizes in one launch (adaptive RK45),
the native launch-schedule autotuner and CUDA-graph replay."""
import dataclasses

import numpy as np
import pytest

from oracle import oracle as O
from oracle.oracle import FieldSpec, Spacetime

pytestmark = pytest.mark.gpu


def _small(cuda):
    from excalibur_tool_gb300 import workloads

    return workloads.multi_field(main_n=32, n_sky=2048, n_side=16, seeds=(1, 2, 3), sizes=(16, 24, 40),
                                 device=cuda)


def _spec(wl):
    from excalibur_tool_gb300 import workloads

    cz = workloads.lcdm()
    ips = [wl.metric.interp] + wl.metric.extra_interpolators
    fields = [FieldSpec(np.asarray(ip.grid.fields["Phi"]), tuple(ip.grid.spacing), tuple(ip.grid.origin), "periodic")
              for ip in ips]
    return Spacetime(kind="flrw", fields=fields, cosmology="table", a_grid=cz.a_grid, eta_min=cz.eta_min,
                     eta_step=cz.eta_step, H0=cz.H0, omega=(0.3, 0.0, 0.0, 0.7))


def test_multi_field_rk45_matches_oracle(cuda):
    """Full-sky rays through the lens grid and patch rays through three random fields, one launch,
    against the C oracle. With the library's correctly rounded cube in the oracle
    (power_mode "dd") every ray has the same accepted/rejected step sequence and bit-identical
    states and observables: the step controller's err**-0.2 / err**-0.25 come from the shared
    IEEE-only routine in csrc/exc_stepctl.h, and nothing else differs. With the reference's libm
    pow the step sequences are still identical, but on the rays where pow misrounds a cube the
    one-ulp difference of adot enters y5 - y4 and the step-size control amplifies it."""
    import torch
    from excalibur_tool_gb300.observables.lensing import deflection_angle
    from excalibur_tool_gb300.trace import trace_batch

    wl = _small(cuda)
    r = trace_batch(wl.metric, wl.states, wl.cfg, field_index=wl.field_index)
    torch.cuda.synchronize()
    states = wl.states.cpu().numpy()
    fidx = wl.field_index.cpu().numpy()
    got = {k: getattr(r, k).cpu().numpy() for k in ("state", "status", "n_steps", "n_iter", "dt", "obs")}
    with O.power_mode("dd"):
        od = O.trace(_spec(wl), states, wl.cfg, field_index=fidx, threads=8)
    for k in ("status", "n_steps", "n_iter", "state", "dt"):
        assert np.array_equal(got[k], getattr(od, k)), k
    assert np.array_equal(got["obs"], od.obs, equal_nan=True)
    o = O.trace(_spec(wl), states, wl.cfg, field_index=fidx, threads=8)
    steps = got["n_steps"]
    assert np.array_equal(got["status"], o.status)
    assert np.array_equal(steps, o.n_steps)
    assert np.array_equal(got["n_iter"], o.n_iter)
    a_gpu, a_ref = deflection_angle(got["obs"]), deflection_angle(o.obs)
    assert (np.abs(a_gpu - a_ref) <= 1e-6 * np.abs(a_ref) + 1e-15).all()
    assert steps.max() > 5 * np.median(steps[steps > 1])       # uneven trajectory lengths in one launch


def test_autotune_and_graph_replay_reproduce_the_launch(cuda):
    import torch
    from excalibur_tool_gb300 import _native as N
    from excalibur_tool_gb300.trace import CapturedTrace, autotune, trace_batch, tune_report

    wl = _small(cuda)
    ref = trace_batch(wl.metric, wl.states, wl.cfg, field_index=wl.field_index)
    tuned = autotune(wl.metric, wl.states, wl.cfg, field_index=wl.field_index, sample=1024, use_cache=False)
    assert tune_report()  # plan recorded
    assert tuned.block_size in (32, 64, 96, 128) and tuned.blocks_per_sm in (0, 2, 3, 4, 5, 6, 7, 8)
    assert tuned.staging in N.STAGING
    rep = next(iter(tune_report().values()))
    assert len(rep["trials"]) == 35 and rep["best_rate"] > 0
    # the three fastest schedules again with the a(eta) table in shared memory
    assert [t[2] for t in rep["trials"]].count("shared") == 3
    cap = CapturedTrace(wl.metric, wl.states, tuned, field_index=wl.field_index)
    for _ in range(2):
        out = cap.run()
    torch.cuda.synchronize()
    for k in ("state", "status", "n_steps", "n_iter"):
        assert torch.equal(getattr(out, k), getattr(ref, k)), k
    assert torch.allclose(out.obs, ref.obs, rtol=0, atol=0, equal_nan=True)
    # other inputs through the same graph: the first half of the batch repeated
    n = wl.states.shape[0]
    other = torch.cat([wl.states[: n // 2], wl.states[: n // 2]])
    out = cap.run(other)
    torch.cuda.synchronize()
    assert torch.equal(out.state[: n // 2], ref.state[: n // 2])


def test_mixed_precision_graph_capture(cuda):
    """The guarded mixed tracer (two launches) replays from a graph with the same results."""
    import torch
    from excalibur_tool_gb300 import workloads
    from excalibur_tool_gb300.trace import CapturedTrace, trace_batch

    wl = workloads.flrw_patch(32, 32, device=cuda)
    cfg = dataclasses.replace(wl.cfg, precision="mixed")
    ref = trace_batch(wl.metric, wl.states, cfg)
    cap = CapturedTrace(wl.metric, wl.states, cfg)
    out = cap.run()
    torch.cuda.synchronize()
    assert torch.equal(out.state, ref.state) and torch.equal(out.status, ref.status)


@pytest.mark.parametrize("precision", ["fp64", "fp64_fast"])
def test_staged_table_gives_the_same_bits(cuda, precision):
    """EXC_STAGING_SHARED (the a(eta) table copied into each block's shared memory) changes where
    the table is read, not what is computed: the multi-field RK45 launch gives the same bits as
    with the table read through the read-only cache, on every schedule tried."""
    import torch
    from excalibur_tool_gb300.trace import trace_batch

    wl = _small(cuda)
    cfg = dataclasses.replace(wl.cfg, precision=precision)
    ref = trace_batch(wl.metric, wl.states, cfg, field_index=wl.field_index)
    for block, per_sm in ((128, 0), (64, 5), (96, 8)):
        got = trace_batch(wl.metric, wl.states, dataclasses.replace(cfg, staging="shared", block_size=block,
                                                                    blocks_per_sm=per_sm),
                          field_index=wl.field_index)
        torch.cuda.synchronize()
        for k in ("state", "status", "n_steps", "n_iter", "dt"):
            assert torch.equal(getattr(got, k), getattr(ref, k)), (k, block, per_sm)
        assert torch.allclose(got.obs, ref.obs, rtol=0, atol=0, equal_nan=True)
