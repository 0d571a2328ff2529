"""The tracer as a PyTorch custom operator (torch.ops.excalibur_gb.trace)."""
import numpy as np
import pytest
import torch


def test_operator_registered_and_fake_shapes():
    from torch._subclasses.fake_tensor import FakeTensorMode

    from excalibur_tool_gb300 import ops

    assert hasattr(torch.ops.excalibur_gb, "trace")
    with FakeTensorMode():
        s = torch.empty((37, 8), dtype=torch.float64)
        st, status, steps = torch.ops.excalibur_gb.trace(s, 1, "rk4", "fp64", 1.0, 1.0, 1.0, 10, 100, 1e-9, 1e-13,
                                                       [], [], 0.0)
        assert st.shape == (37, 8) and st.dtype == torch.float64
        assert status.shape == (37,) and status.dtype == torch.int32 and steps.dtype == torch.int32
    with pytest.raises(ValueError):
        ops._metric(10 ** 9)


@pytest.mark.gpu
def test_operator_equals_trace_batch(cuda):
    from helpers import gpu_metric, lcdm_spacetime
    from conftest import golden
    from excalibur_tool_gb300 import ops
    from excalibur_tool_gb300.trace import TraceConfig, trace_batch

    g = golden("flrw_patch_32.npz")
    spec = lcdm_spacetime(g["field"], float(g["box"]))
    m = gpu_metric(spec)
    states = torch.as_tensor(g["states"], device=cuda)
    dl = float(g["dl"])
    box = float(g["box"])
    h = ops.register_metric(m)
    try:
        st, status, steps = torch.ops.excalibur_gb.trace(states, h, "rk4", "fp64", dl, dl, dl, 10000, 10000, 1e-9,
                                                         1e-13, [0.0, 0.0, 0.0], [box, box, box], 0.0)
        ref = trace_batch(m, states, TraceConfig(stepper="rk4", dt=dl, dt_min=dl, dt_max=dl, max_steps=10000,
                                                 stop_box=((0, 0, 0), (box, box, box)), observables=False))
        torch.cuda.synchronize()
        assert torch.equal(st, ref.state) and torch.equal(status, ref.status) and torch.equal(steps, ref.n_steps)
        assert np.array_equal(steps.cpu().numpy(), g["n_steps"])    # and the reference's step counts
    finally:
        ops.release_metric(h)
