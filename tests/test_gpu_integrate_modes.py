"""Integrator.integrate against the reference's own runs of it (tests/golden/integrate_modes.npz).

Five photons through a strict ("error") grid, RK4 for 40 steps, the fourth leaving the grid's
interior after three steps (integrator.py:434-476):
* sequential: every photon integrated as integrate_single with record_every = 1 (a history row
  per accepted step, the quantity columns one record late, the final record); the fourth
  raises ValueError with its three steps recorded and its quantities evaluated at the last of
  them; the fifth is never integrated.
* chunked: the photons that succeed are updated, the failed one keeps its input state and an
  empty history; the call returns 4.
Rows agree to 1e-14 (the parity build's correctly rounded cube against libm's pow moves adot by
an ulp where pow misrounds).
"""
import numpy as np
import pytest

from conftest import golden
from helpers import gpu_metric, lcdm_spacetime, rel_err

pytestmark = pytest.mark.gpu


def _setup():
    from excalibur_tool_gb300.integration.integrator import Integrator
    from excalibur_tool_gb300.photon.photon import Photon

    g = golden("integrate_modes.npz")
    spec = lcdm_spacetime(g["field"], float(g["box"]), boundary="error")
    metric = gpu_metric(spec)
    dt = float(g["dt"])
    photons = [Photon(s[:4].copy(), s[4:].copy()) for s in g["inits"]]

    def integ(mode):
        return Integrator(metric, dt=dt, mode=mode, integrator="rk4", dt_min=dt, dt_max=dt, n_workers=2, chunk_size=2)

    return g, photons, integ


def _hist(p):
    return p.history.as_array() if p.history.states else np.zeros((0, 14))


def _assert_rows(got, want):
    got = np.asarray(got)
    assert got.shape == want.shape
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    if ok.any():
        assert rel_err(got[ok], want[ok]).max() <= 1e-14


def test_integrate_sequential_records_and_raises(cuda):
    g, photons, integ = _setup()
    with pytest.raises(ValueError):
        integ("sequential").integrate(photons, "steps", int(g["n_steps"]), verbose=False)
    assert int(g["seq_raised"]) == 1
    for k, p in enumerate(photons):
        _assert_rows(_hist(p), g[f"seq{k}_history"])
        assert rel_err(np.concatenate([p.x, p.u]), g[f"seq{k}_final"]).max() <= 1e-14
        q = g[f"seq{k}_quantities"]
        assert np.shape(p.quantities) == q.shape
        if q.size:
            assert rel_err(p.quantities, q).max() <= 1e-14


def test_integrate_sequential_returns_len(cuda):
    g, photons, integ = _setup()
    ok = [photons[i] for i in (0, 1, 2, 4)]
    assert integ("sequential").integrate(ok, "steps", int(g["n_steps"]), verbose=False) == 4
    for p, k in zip(ok, (0, 1, 2, 4)):
        _assert_rows(_hist(p), g[f"chunked{k}_history"])


@pytest.mark.parametrize("mode", ["chunked", "parallel"])
def test_integrate_pool_modes_count_successes(cuda, mode):
    g, photons, integ = _setup()
    assert integ(mode).integrate(photons, "steps", int(g["n_steps"]), verbose=False) == int(g["chunked_ok"]) == 4
    for k, p in enumerate(photons):
        want = g[f"chunked{k}_history"]
        _assert_rows(_hist(p), want)
        assert rel_err(np.concatenate([p.x, p.u]), g[f"chunked{k}_final"]).max() <= 1e-14
