"""On-device records in the runners' trajectory layout, and a time-dependent (4-D) potential
with the in-kernel ISW integral, against the oracle."""
import numpy as np
import pytest

from conftest import golden
from helpers import gpu_trace, rel_err
from excalibur_tool_gb300 import _native as N
from excalibur_tool_gb300.trace import TraceConfig
from oracle import oracle as O
from oracle.oracle import FieldSpec, Spacetime

pytestmark = pytest.mark.gpu


def _spec4d():
    from excalibur_tool_gb300.core.constants import c, one_Mpc, one_Msun
    from excalibur_tool_gb300.objects.fields import lens_plus_grf

    cz = golden("cosmology.npz")
    n, box = 32, 1000 * one_Mpc
    phi3 = lens_plus_grf(n, box, 1e15 * one_Msun, 5 * one_Mpc, np.array([500.0] * 3) * one_Mpc, seed=7)
    eta1 = float(cz["eta_at_a1"])
    span = 1.2 * box / c                      # the photons travel back less than this in eta
    t0, nt = eta1 - span, 3
    dt = span / (nt - 1) * 1.05
    scale = np.array([0.8, 1.0, 1.3])         # Phi grows towards the observer: a non-zero ISW term
    phi4 = np.ascontiguousarray(phi3[..., None] * scale[None, None, None, :])
    f = FieldSpec(phi4, (box / n,) * 3 + (dt,), (0.0, 0.0, 0.0, t0), "periodic")
    return Spacetime(kind="flrw", fields=[f], cosmology="table", a_grid=cz["a_grid"], eta_min=float(cz["eta_min"]),
                     eta_step=float(cz["eta_step"]), H0=float(cz["H0"]), omega=(0.3, 0.0, 0.0, 0.7)), eta1, box


def _states(spec, eta1, n_side=8):
    from excalibur_tool_gb300.core.constants import c, one_Mpc

    half = np.tan(np.deg2rad(5.0))
    t = (np.arange(n_side) + 0.5) / n_side * 2 - 1
    A, B = np.meshgrid(t, t, indexing="ij")
    d = np.stack([np.ones_like(A), A * half, B * half], -1).reshape(-1, 3)
    d /= np.linalg.norm(d, axis=1)[:, None]
    st = np.zeros((len(d), 8))
    st[:, 0] = eta1
    st[:, 1:4] = np.array([0.0, 500.0, 500.0]) * one_Mpc
    st[:, 5:8] = d * c
    st, status = O.null_init(spec, st, -1.0)
    assert (status == 0).all()
    return st


def test_time_dependent_potential_isw_matches_oracle(cuda):
    from excalibur_tool_gb300.core.constants import c, one_Mpc

    spec, eta1, box = _spec4d()
    st = _states(spec, eta1)
    dl = 0.5 * one_Mpc / c
    cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=10000, max_iter=10000,
                      stop_box=((0, 0, 0), (box, box, box)), isw=True)
    r = gpu_trace(spec, st, cfg)
    o = O.trace(spec, st, cfg, threads=8)
    assert np.array_equal(r["status"], o.status) and np.array_equal(r["n_steps"], o.n_steps)
    assert rel_err(r["state"], o.state).max() <= 1e-13
    i = N.OBS_COLS.index("isw_int")
    assert np.abs(o.obs[:, i]).min() > 0                      # the potential does change along the rays
    assert rel_err(r["obs"][:, i], o.obs[:, i]).max() <= 1e-12


def test_records_to_runner_layout(cuda, tmp_path):
    import torch
    from excalibur_tool_gb300.core.constants import c, one_Mpc
    from excalibur_tool_gb300.records import trajectories_from_result, write_trajectories
    from excalibur_tool_gb300.trace import trace_batch
    from helpers import gpu_metric

    spec, eta1, box = _spec4d()
    st = _states(spec, eta1, 4)
    dl = 0.5 * one_Mpc / c
    cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=300, max_iter=300, record_every=7)
    res = trace_batch(gpu_metric(spec), torch.as_tensor(st).cuda(), cfg)
    torch.cuda.synchronize()
    traj = trajectories_from_result(res)
    n = res.n_records.cpu().numpy()
    rec = res.records.cpu().numpy()
    for i in range(len(st)):
        assert np.array_equal(traj[i, :n[i]], rec[i, :n[i]], equal_nan=True) and np.isnan(traj[i, n[i]:]).all()
    o = O.trace(spec, st, cfg, threads=4)
    assert np.array_equal(n, o.n_records)
    for i in range(len(st)):
        assert rel_err(traj[i, :n[i]], o.records[i, :n[i]]).max() <= 1e-12
    p = write_trajectories(str(tmp_path / "t.h5"), traj, {"record_every": 7})
    assert np.array_equal(np.load(p)["trajectories"] if p.endswith(".npz") else traj, traj, equal_nan=True)


def test_staged_table_with_records_and_isw(cuda):
    """The a(eta) table staged in shared memory (TraceConfig.staging = "shared") in the
    record-writing kernel with a time-dependent potential: records, states and the ISW integral
    are the same bits as with the table read through the cache."""
    import dataclasses

    import torch
    from excalibur_tool_gb300.core.constants import c, one_Mpc
    from excalibur_tool_gb300.trace import trace_batch
    from helpers import gpu_metric

    spec, eta1, box = _spec4d()
    st = torch.as_tensor(_states(spec, eta1, 6)).cuda()
    dl = 0.5 * one_Mpc / c
    cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=300, max_iter=300, record_every=3,
                      isw=True)
    m = gpu_metric(spec)
    a = trace_batch(m, st, cfg)
    b = trace_batch(m, st, dataclasses.replace(cfg, staging="shared"))
    torch.cuda.synchronize()
    for k in ("state", "status", "n_steps", "n_records"):
        assert torch.equal(getattr(a, k), getattr(b, k)), k
    n = a.n_records.cpu().numpy()
    ra, rb = a.records.cpu().numpy(), b.records.cpu().numpy()
    assert n.min() > 10
    for i in range(len(n)):   # the recorded rows (the buffer past them is not written)
        assert np.array_equal(ra[i, :n[i]], rb[i, :n[i]], equal_nan=True), i
    assert torch.allclose(a.obs, b.obs, rtol=0, atol=0, equal_nan=True)
