"""Shared builders for the tests: the same spacetime for the oracle and the GPU."""
import numpy as np

from excalibur_tool_gb300.core import constants as K
from oracle.oracle import FieldSpec, Spacetime
from conftest import golden


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.where(den > 0, np.abs(a - b) / den, 0.0)
    return r


def lcdm_spacetime(field, box, boundary="periodic", cosmology="table", analytical=False):
    cz = golden("cosmology.npz")
    n = field.shape[0]
    return Spacetime(kind="flrw", fields=[FieldSpec(field, (box / n,) * 3, (0.0, 0.0, 0.0), boundary)],
                     cosmology=cosmology, a_grid=cz["a_grid"], eta_min=float(cz["eta_min"]),
                     eta_step=float(cz["eta_step"]), H0=float(cz["H0"]), omega=(0.3, 0.0, 0.0, 0.7),
                     analytical=analytical)


def schw_spacetime(mass, radius, center=(0.0, 0.0, 0.0), analytical=True, free_time=True):
    return Spacetime(kind="schwarzschild", mass=mass, radius=radius, center=tuple(center), analytical=analytical,
                     free_time=free_time)


def golden_lcdm():
    """The package's LCDM_Cosmology rebuilt from the reference-generated table."""
    from excalibur_tool_gb300.core.cosmology import LCDM_Cosmology

    cz = golden("cosmology.npz")
    return LCDM_Cosmology.from_table(float(cz["H0"]), 0.3, 0.0, 0.7, 0.0, float(cz["eta_min"]),
                                     float(cz["eta_step"]), cz["a_grid"], float(cz["eta_at_a1"]))


def gpu_metric(spec, field_dtype=None):
    """Package metric object equivalent to an oracle Spacetime spec."""
    from excalibur_tool_gb300.core.cosmology import StaticCosmology
    from excalibur_tool_gb300.grid.grid import Grid
    from excalibur_tool_gb300.grid.interpolator_4d_fast import InterpolatorFast
    from excalibur_tool_gb300.metrics.perturbed_flrw_metric_fast import PerturbedFLRWMetricFast
    from excalibur_tool_gb300.metrics.schwarzschild_metric_fast import SchwarzschildMetricFast

    if spec.kind == "schwarzschild":
        return SchwarzschildMetricFast(spec.mass, spec.radius, center=np.array(spec.center, dtype=float),
                                       analytical_geodesics=spec.analytical, free_time_geodesic=spec.free_time,
                                       coords="spherical")
    from excalibur_tool_gb300.grid.interpolator import Interpolator

    interps = []
    for f in spec.fields:
        g = Grid(f.data.shape, f.spacing, f.origin)
        g.add_field("Phi", f.data)
        if f.gradient == "trilinear":
            interps.append(Interpolator(g, field_dtype=field_dtype))
        else:
            interps.append(InterpolatorFast(g, boundary=f.boundary, field_dtype=field_dtype))
    if spec.cosmology == "static":
        cz = StaticCosmology()
        a_of, adot_of = cz.a_of_eta, cz.adot_of_eta
    else:
        cz = golden_lcdm()
        a_of, adot_of = cz.a_of_eta, (cz.adot_of_eta if spec.cosmology == "table" else None)
    return PerturbedFLRWMetricFast(a_of, interps[0].grid, interps[0], analytical_geodesics=spec.analytical,
                                   adot_of_eta=adot_of, extra_interpolators=interps[1:])


def gpu_trace(spec, states, cfg, field_index=None):
    import torch
    from excalibur_tool_gb300.trace import trace_batch

    m = gpu_metric(spec)
    s = torch.as_tensor(np.ascontiguousarray(states, dtype=np.float64)).cuda()
    fi = None if field_index is None else torch.as_tensor(np.asarray(field_index, dtype=np.int32)).cuda()
    r = trace_batch(m, s, cfg, field_index=fi)
    torch.cuda.synchronize()
    out = {k: (None if v is None else v.cpu().numpy()) for k, v in
           dict(state=r.state, status=r.status, n_steps=r.n_steps, n_iter=r.n_iter, dt=r.dt, obs=r.obs,
                records=r.records, n_records=r.n_records).items()}
    return out
