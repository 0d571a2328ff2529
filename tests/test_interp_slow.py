"""The slow Interpolator (grid/interpolator.py of the reference), grad_mode "trilinear".

CPU: the C oracle against tests/golden/interp_slow.npz (made by running the
reference's own class): 3-D float64 and float32 grids, 4-D grids with three
and two snapshots, and 40-step RK4 traces through the fast FLRW metric that
use it. GPU: the CUDA library against the same vectors, through exc_interp
and exc_trace (the parity build must be bit-exact).
"""
import dataclasses

import numpy as np
import pytest

from conftest import golden
from helpers import lcdm_spacetime, rel_err
from excalibur_tool_gb300.trace import TraceConfig
from oracle import oracle as O
from oracle.oracle import FieldSpec


def _pts4(pts3):
    return np.concatenate([pts3, np.zeros((len(pts3), 1))], axis=1)


def _check(out, status, want, ok):
    assert ok.sum() >= 20 and (~ok).sum() >= 20
    assert np.array_equal(status == 0, ok)
    assert np.array_equal(status[~ok], np.full((~ok).sum(), 4))   # EXC_PH_OUTSIDE_GRID
    assert np.array_equal(out[ok], want[ok])


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_oracle_slow_3d_bitexact(dtype):
    g = golden("interp_slow.npz")
    data = g["f3"] if dtype == "f64" else g["f3"].astype(np.float32)
    f = FieldSpec(data, tuple(g["f3_spacing"]), tuple(g["f3_origin"]), "error", "trilinear")
    out, status = O.interp(f, _pts4(g["pts3"]))
    sfx = "" if dtype == "f64" else "_f32"
    _check(out, status, g[f"out3{sfx}"], g[f"ok3{sfx}"].astype(bool))


@pytest.mark.parametrize("nt", [3, 2])
def test_oracle_slow_4d_bitexact(nt):
    g = golden("interp_slow.npz")
    f = FieldSpec(g[f"f4_{nt}"], tuple(g[f"f4_{nt}_spacing"]), tuple(g[f"f4_{nt}_origin"]), "error", "trilinear")
    out, status = O.interp(f, g[f"pts4_{nt}"])
    _check(out, status, g[f"out4_{nt}"], g[f"ok4_{nt}"].astype(bool))


def test_slow_gradient_is_continuous_across_faces():
    """The trilinear-blended gradient has no jump at a cell face (the base-node one does)."""
    g = golden("interp_slow.npz")
    sp, org = g["f3_spacing"], g["f3_origin"]
    x_face = org[0] + 4 * sp[0]
    pts = np.array([[x_face - 1e-6 * sp[0], org[1] + 2.3 * sp[1], org[2] + 3.6 * sp[2], 0.0],
                    [x_face, org[1] + 2.3 * sp[1], org[2] + 3.6 * sp[2], 0.0]])
    slow, _ = O.interp(FieldSpec(g["f3"], tuple(sp), tuple(org), "error", "trilinear"), pts)
    fast, _ = O.interp(FieldSpec(g["f3"], tuple(sp), tuple(org), "error"), pts)
    assert rel_err(slow[0, 1:4], slow[1, 1:4]).max() < 1e-4
    assert rel_err(fast[0, 1:4], fast[1, 1:4]).max() > 1e-2


def _trace_spec(g):
    st = lcdm_spacetime(g["trace_field"], float(g["trace_box"]), boundary="error")
    st.fields[0].gradient = "trilinear"
    dt = float(g["trace_dt"])
    cfg = TraceConfig(stepper="rk4", dt=dt, dt_min=dt, dt_max=dt, max_steps=40, record_every=1, observables=False)
    return st, cfg


def test_oracle_slow_trace_matches_reference():
    g = golden("interp_slow.npz")
    st, cfg = _trace_spec(g)
    res = O.trace(st, g["trace_init"], cfg)
    assert (res.status == 0).all()
    assert np.array_equal(res.state, g["trace_final"])
    want = g["trace_records"]
    assert np.array_equal(res.n_records, np.full(len(want), want.shape[1]))
    assert np.array_equal(res.records[:, :want.shape[1], :8], want)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_oracle_rk45_slow_trace_matches_reference(k):
    """integrate_single with the reference's RK45 (its own tableau and controller, dt clip) through
    the slow Interpolator, from the reference's own run (tests/golden/rk45_slow.npz; 37 iterations
    a photon, 7 of them rejected): the same accepted steps, the states within the ~1e-12 that the
    reference's BLAS-ordered y5 leaves in the step-size control (as for the base-node RK45 case;
    measured: two photons bit for bit, one within 1.0e-13), the quantity columns within 1e-8."""
    g = golden("rk45_slow.npz")
    st = lcdm_spacetime(g["field"], float(g["box"]), boundary="error")
    st.fields[0].gradient = "trilinear"
    rtol, atol, dmin, dmax = (float(v) for v in g["tol"])
    cfg = TraceConfig(stepper="rk45", dt=float(g["dt"]), dt_min=dmin, dt_max=dmax, rtol=rtol, atol=atol,
                      max_steps=30, record_every=1, observables=False)
    res = O.trace(st, g[f"case{k}_init"][None], cfg)
    assert res.status[0] == 0
    want = g[f"case{k}_records"]
    got = res.records[0, :res.n_records[0]]
    assert got.shape == want.shape
    assert np.array_equal(np.isnan(got), np.isnan(want))
    assert rel_err(res.state[0], g[f"case{k}_final"]).max() <= 1e-12
    st8 = ~np.isnan(want[:, :8])
    assert rel_err(got[:, :8][st8], want[:, :8][st8]).max() <= 1e-12
    q = ~np.isnan(want[:, 8:])
    assert rel_err(got[:, 8:][q], want[:, 8:][q]).max() <= 1e-8


def test_slow_descriptor_validation():
    """grad_mode "trilinear" needs the error boundary (the slow class's single bounds rule)."""
    from excalibur_tool_gb300 import _native as N
    from excalibur_tool_gb300.grid.grid import Grid
    from excalibur_tool_gb300.grid.interpolator import Interpolator

    grid = Grid((4, 4, 4), (1.0, 1.0, 1.0))
    ip = Interpolator(grid)
    assert ip.boundary == "error" and ip.gradient_mode == "trilinear"
    assert N.GRAD["trilinear"] == 1


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_gpu_slow_3d_bitexact(dtype):
    from excalibur_tool_gb300.grid.grid import Grid
    from excalibur_tool_gb300.grid.interpolator import Interpolator

    g = golden("interp_slow.npz")
    data = g["f3"] if dtype == "f64" else g["f3"].astype(np.float32)
    grid = Grid(data.shape, tuple(g["f3_spacing"]), tuple(g["f3_origin"]))
    grid.add_field("Phi", data)
    val, grad, dtd, status = Interpolator(grid).evaluate(_pts4(g["pts3"]))
    out = np.column_stack([val.cpu().numpy(), grad.cpu().numpy(), dtd.cpu().numpy()])
    sfx = "" if dtype == "f64" else "_f32"
    _check(out, status.cpu().numpy(), g[f"out3{sfx}"], g[f"ok3{sfx}"].astype(bool))


@pytest.mark.gpu
@pytest.mark.parametrize("nt", [3, 2])
def test_gpu_slow_4d_bitexact(nt):
    from excalibur_tool_gb300.grid.grid import Grid
    from excalibur_tool_gb300.grid.interpolator import Interpolator

    g = golden("interp_slow.npz")
    grid = Grid(g[f"f4_{nt}"].shape, tuple(g[f"f4_{nt}_spacing"]), tuple(g[f"f4_{nt}_origin"]))
    grid.add_field("Phi", g[f"f4_{nt}"])
    ip = Interpolator(grid)
    val, grad, dtd, status = ip.evaluate(g[f"pts4_{nt}"])
    out = np.column_stack([val.cpu().numpy(), grad.cpu().numpy(), dtd.cpu().numpy()])
    _check(out, status.cpu().numpy(), g[f"out4_{nt}"], g[f"ok4_{nt}"].astype(bool))
    # the reference-facing scalar call
    k = int(np.flatnonzero(g[f"ok4_{nt}"])[0])
    p = g[f"pts4_{nt}"][k]
    v, gr, d = ip.value_gradient_and_time_derivative(p[:3], "Phi", p[3])
    assert [v, *gr, d] == list(g[f"out4_{nt}"][k])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp64_fast"])
def test_gpu_slow_trace_matches_reference(precision):
    import torch
    from helpers import gpu_trace

    g = golden("interp_slow.npz")
    st, cfg = _trace_spec(g)
    cfg = dataclasses.replace(cfg, precision=precision)
    r = gpu_trace(st, g["trace_init"], cfg)
    assert (r["status"] == 0).all()
    want = g["trace_records"]
    got = r["records"][:, :want.shape[1], :8]
    if precision == "fp64":
        assert np.array_equal(r["state"], g["trace_final"])
        assert np.array_equal(got, want)
    else:
        assert rel_err(r["state"], g["trace_final"]).max() <= 1e-13
        assert rel_err(got, want).max() <= 1e-13
    torch.cuda.synchronize()
