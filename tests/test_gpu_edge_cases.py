"""Edge cases of the batched tracer on the GPU: empty batches, and results that do not depend
on how a batch is cut (ragged chunks, one photon alone)."""
import numpy as np
import pytest
import torch

from conftest import golden
from helpers import gpu_metric, lcdm_spacetime
from excalibur_tool_gb300.trace import TraceConfig, trace_batch

pytestmark = pytest.mark.gpu


def _setup():
    g = golden("flrw_patch_32.npz")
    box = float(g["box"])
    m = gpu_metric(lcdm_spacetime(g["field"], box))
    dl = float(g["dl"])
    cfg = TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=10000,
                      stop_box=((0, 0, 0), (box, box, box)))
    return g, m, cfg


@pytest.mark.parametrize("precision", ["fp64", "fp64_fast", "mixed"])
def test_empty_batch(cuda, precision):
    import dataclasses

    g, m, cfg = _setup()
    cfg = dataclasses.replace(cfg, precision=precision, record_every=4 if precision != "mixed" else None)
    r = trace_batch(m, torch.zeros((0, 8), dtype=torch.float64, device=cuda), cfg)
    torch.cuda.synchronize()
    assert r.state.shape == (0, 8) and r.status.shape == (0,) and r.n_steps.shape == (0,)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_results_independent_of_batch_cut(cuda, precision):
    import dataclasses

    g, m, cfg = _setup()
    cfg = dataclasses.replace(cfg, precision=precision)
    st = torch.as_tensor(g["states"], device=cuda)
    whole = trace_batch(m, st, cfg)
    parts = [trace_batch(m, st[a:b], cfg) for a, b in ((0, 1), (1, 32), (32, 33), (33, st.shape[0]))]
    torch.cuda.synchronize()
    for name in ("state", "status", "n_steps"):
        cat = torch.cat([getattr(p, name) for p in parts])
        assert torch.equal(cat, getattr(whole, name)), name
    if precision == "fp64":
        assert np.array_equal(whole.n_steps.cpu().numpy(), g["n_steps"])
