"""Time delay: the reference's definition and the cancellation-free companion column.

The reference's time delay is (sum_k |x_{k+1} - x_k| - |x_N - x_0|) / c over the recorded
positions (_postprocessing/compute_time_delay_map.py:112-126): the PATH and CHORD columns here,
taken over every accepted state. Their difference cancels catastrophically (both are ~1e25 m,
the excess ~1e15 m), so the EXCESS column also accumulates sum_k (|d_k| - d_k.e) - (|X| - X.e)
with |d| - d.e = |d x e|^2 / (|d| + d.e), which has no cancellation. The CUDA library and the
oracle evaluate it with the same double arithmetic, so the GPU tests hold it to the oracle bit
for bit; here its accuracy is bounded against a 50-digit evaluation of path - chord over the
oracle's own recorded positions.
"""
import mpmath
import numpy as np

from helpers import lcdm_spacetime
from excalibur_tool_gb300 import _native as N
from excalibur_tool_gb300.core.constants import c, one_Mpc, one_Msun
from excalibur_tool_gb300.objects.fields import lens_plus_grf
from excalibur_tool_gb300.trace import TraceConfig
from oracle import oracle as O


def _patch_rays(n_grid=32, n_side=4):
    from conftest import golden

    box = 1000 * one_Mpc
    lens = np.array([500.0, 500.0, 500.0]) * one_Mpc
    phi = lens_plus_grf(n_grid, box, 1e15 * one_Msun, 5 * one_Mpc, lens, seed=2)
    spec = lcdm_spacetime(phi, box)
    half = np.tan(np.deg2rad(5.0))
    t = (np.arange(n_side) + 0.5) / n_side * 2 - 1
    A, B = np.meshgrid(t, t, indexing="ij")
    d = np.stack([np.ones_like(A), A * half, B * half], axis=-1).reshape(-1, 3)
    d /= np.linalg.norm(d, axis=1)[:, None]
    st = np.zeros((len(d), 8))
    st[:, 0] = float(golden("cosmology.npz")["eta_at_a1"])
    st[:, 1:4] = np.array([0.0, 500.0, 500.0]) * one_Mpc
    st[:, 5:8] = d * c
    st, status = O.null_init(spec, st, -1.0)
    assert (status == 0).all()
    dl = 0.5 * one_Mpc / c
    cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=10000, max_iter=10000,
                      stop_box=((0, 0, 0), (box, box, box)), lens_center=tuple(lens), record_every=1,
                      max_records=2200)
    return spec, st, cfg


def test_excess_is_path_minus_chord_to_1e12():
    spec, st, cfg = _patch_rays()
    res = O.trace(spec, st, cfg)
    assert (res.status == N.PH_LEFT_BOX).all()
    i_path, i_chord, i_exc = (N.OBS_COLS.index(k) for k in ("path", "chord", "excess"))
    mpmath.mp.dps = 50
    for p in range(len(st)):
        rows = res.records[p, :res.n_records[p], 1:4]
        # the final record duplicates the last state (integrator.py:403-404): a zero segment
        pts = [[mpmath.mpf(float(v)) for v in row] for row in rows]
        path = mpmath.mpf(0)
        for a, b in zip(pts[:-1], pts[1:]):
            path += mpmath.sqrt(sum((bi - ai) ** 2 for ai, bi in zip(a, b)))
        chord = mpmath.sqrt(sum((bi - ai) ** 2 for ai, bi in zip(pts[0], pts[-1])))
        exact = path - chord
        assert exact > 0
        got = res.obs[p, i_exc]
        assert abs(mpmath.mpf(float(got)) - exact) <= mpmath.mpf("1e-12") * exact, (p, got, exact)
        # the naive columns are the reference's own definition, each to a few ulps of its size
        assert abs(mpmath.mpf(float(res.obs[p, i_path])) - path) <= mpmath.mpf("1e-13") * path
        assert abs(mpmath.mpf(float(res.obs[p, i_chord])) - chord) <= mpmath.mpf("1e-15") * chord
