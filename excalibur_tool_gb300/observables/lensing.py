"""Per-photon observables from the tracer's in-place accumulators.

The kernel accumulates, per photon (trace.TraceResult.obs, columns named in
_native.OBS_COLS): a and Phi at both ends, the trapezoid integral of
dPhi/deta along the path, the path length over accepted states, the chord,
a cancellation-free path-minus-chord, the first and last cartesian spatial
velocities and the closest approach. These functions turn them into the
reference's observables:

* redshift: z_H = a_obs / a_em - 1, z_SW = (Phi_obs - Phi_em) / c^2,
  z_ISW = -int dPhi/deta deta / c^2 (observables/redshift.py:165-273);
* time delay: (sum |dx| - |x_N - x_0|) / c over recorded positions
  (_postprocessing/compute_time_delay_map.py:97-126, :244-310);
* deflection: arccos(clip(v0_hat . v1_hat)) between the first and last
  spatial velocities (_postprocessing/analyze_compare_trajectories.py:165-181),
  and the theory value 4 G M / (c^2 b) (:202-212).

The "_naive" variants reproduce the reference's formulas; the default ones
use the cancellation-free forms (atan2 of cross/dot; path excess summed as
|dx x e|^2 / (|dx| + dx.e)) that stay accurate at 1e25 m.
"""
import numpy as np

from .. import _native as N
from ..core.constants import c, G

_I = {name: i for i, name in enumerate(N.OBS_COLS)}


def col(obs, name):
    return np.asarray(obs)[:, _I[name]]


def redshift_components(obs):
    obs = np.asarray(obs)
    c2 = float(c) ** 2
    z_H = col(obs, "a_obs") / col(obs, "a_em") - 1.0
    z_SW = (col(obs, "phi_obs") - col(obs, "phi_em")) / c2
    z_ISW = -col(obs, "isw_int") / c2
    return {"z_H": z_H, "z_SW": z_SW, "z_ISW": z_ISW, "z_D": np.zeros_like(z_H),
            "z_total": z_H + z_SW + z_ISW,
            "z_total_exact": (1 + z_H) * (1 + z_SW) * (1 + z_ISW) - 1.0}


def redshift_total(obs):
    return redshift_components(obs)["z_total"]


def time_delay_naive(obs):
    return (col(obs, "path") - col(obs, "chord")) / float(c)


def time_delay_excess(obs):
    return col(obs, "excess") / float(c)


def _unit(v):
    n = np.linalg.norm(v, axis=1, keepdims=True)
    return np.where(n < 1e-30, 0.0, v / np.where(n == 0, 1, n))


def deflection_angle_naive(obs):
    v0 = _unit(np.stack([col(obs, "v0x"), col(obs, "v0y"), col(obs, "v0z")], axis=1))
    v1 = _unit(np.stack([col(obs, "v1x"), col(obs, "v1y"), col(obs, "v1z")], axis=1))
    return np.arccos(np.clip(np.sum(v0 * v1, axis=1), -1.0, 1.0))


def deflection_angle(obs):
    v0 = _unit(np.stack([col(obs, "v0x"), col(obs, "v0y"), col(obs, "v0z")], axis=1))
    v1 = _unit(np.stack([col(obs, "v1x"), col(obs, "v1y"), col(obs, "v1z")], axis=1))
    return np.arctan2(np.linalg.norm(np.cross(v0, v1), axis=1), np.sum(v0 * v1, axis=1))


def deflection_theory(min_r, mass_kg):
    b = np.asarray(min_r, dtype=float)
    out = np.full_like(b, np.nan)
    ok = np.isfinite(b) & (b > 0)
    out[ok] = 4.0 * G * float(mass_kg) / (float(c) ** 2 * b[ok])
    return out
