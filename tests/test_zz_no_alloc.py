"""exc_trace_noalloc: the work-queue trace for callers that cannot allocate.

Such callers (an application that owns all device memory and forbids
allocating inside its loop, or a latency-bound loop that cannot absorb the
device synchronisation a cudaMalloc/cudaFree implies) hand in only their
inputs and outputs; the queue scratch lives in a fixed array inside the
library. This checks, through the C ABI, that two calls in a row give the
same photons the same results as exc_trace with caller-provided scratch.
Collected last on purpose (file name), and self-contained so it also runs
alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _workload():
    import torch

    from excalibur_tool_gb300.core.constants import c, one_Mpc, one_Msun
    from excalibur_tool_gb300.core.cosmology import LCDM_Cosmology
    from excalibur_tool_gb300.grid.grid import Grid
    from excalibur_tool_gb300.grid.interpolator_4d_fast import InterpolatorFast
    from excalibur_tool_gb300.metrics.perturbed_flrw_metric_fast import PerturbedFLRWMetricFast
    from excalibur_tool_gb300.objects.fields import lens_plus_grf
    from excalibur_tool_gb300.photon.photons import Photons

    n, box = 32, 1000 * one_Mpc
    lens = np.array([500.0, 500.0, 500.0]) * one_Mpc
    phi = lens_plus_grf(n, box, 1e15 * one_Msun, 5 * one_Mpc, lens, seed=7)
    cz = LCDM_Cosmology(70, 0.3, 0.0, 0.7)
    g = Grid((n, n, n), (box / n,) * 3, (0.0, 0.0, 0.0))
    g.add_field("Phi", phi)
    m = PerturbedFLRWMetricFast(cz.a_of_eta, g, InterpolatorFast(g), adot_of_eta=cz.adot_of_eta)
    states = Photons(m).generate_patch_grid(24, [cz._eta_at_a1, 0.0, 500 * one_Mpc, 500 * one_Mpc],
                                            [1.0, 0.0, 0.0], 10.0)
    return m, states.contiguous(), 0.5 * one_Mpc / c, box


def _args(n, states, dt, box, queue, precision="fp64"):
    import torch
    from excalibur_tool_gb300 import _native as N

    st = states.clone()
    status = torch.full((n,), -7, dtype=torch.int32, device=st.device)
    nsteps = torch.zeros(n, dtype=torch.int32, device=st.device)
    a = N.ExcTraceArgs()
    a.n_photons = n
    a.state, a.status, a.n_steps = st.data_ptr(), status.data_ptr(), nsteps.data_ptr()
    a.stepper, a.precision = N.STEPPER["rk4"], N.PRECISION[precision]
    a.dt = a.dt_min = a.dt_max = dt
    a.max_iter, a.max_steps = 100_000, 1 << 40
    a.stop_flags = N.STOP_BOX
    for i in range(3):
        a.box_lo[i], a.box_hi[i] = 0.0, box
    a.queue = queue.data_ptr() if queue is not None else None
    return a, (st, status, nsteps)


def test_noalloc_trace_matches_trace_twice():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from excalibur_tool_gb300 import _native as N

    lib = N.load()
    metric, states, dt, box = _workload()
    dev = states.device
    desc = metric.descriptor(dev)
    n = states.shape[0]
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    queue = torch.zeros(2, dtype=torch.int64, device=dev)
    a, ref = _args(n, states, dt, box, queue)
    N.check(lib.exc_trace(C.byref(desc.struct), C.byref(a), stream), "exc_trace")
    torch.cuda.synchronize()
    ref = [t.cpu().numpy() for t in ref]
    assert (ref[1] == N.PH_LEFT_BOX).all()

    for call in range(2):
        b, out = _args(n, states, dt, box, None)
        rc = lib.exc_trace_noalloc(C.byref(desc.struct), C.byref(b), stream)
        assert rc == 0, lib.exc_last_error()
        torch.cuda.synchronize()
        got = [t.cpu().numpy() for t in out]
        assert np.array_equal(got[1], ref[1]), call
        assert np.array_equal(got[2], ref[2]), call
        assert np.array_equal(got[0], ref[0]), call

    # the guarded mixed-precision trace uses the queue twice (the mixed pass, then the FP64
    # re-trace of the rays it hands back, with the head cleared in between): the same bits as
    # exc_trace with a caller-owned queue, on two calls in a row
    mdesc = metric.descriptor(dev, split=True)
    a, mref = _args(n, states, dt, box, queue, "mixed")
    N.check(lib.exc_trace(C.byref(mdesc.struct), C.byref(a), stream), "exc_trace mixed")
    torch.cuda.synchronize()
    mref = [t.cpu().numpy() for t in mref]
    assert (mref[1] == N.PH_LEFT_BOX).all()
    for call in range(2):
        b, out = _args(n, states, dt, box, None, "mixed")
        rc = lib.exc_trace_noalloc(C.byref(mdesc.struct), C.byref(b), stream)
        assert rc == 0, lib.exc_last_error()
        torch.cuda.synchronize()
        got = [t.cpu().numpy() for t in out]
        for g_, r_ in zip(got, mref):
            assert np.array_equal(g_, r_), call

    # a caller-supplied queue is refused with a message
    b, _ = _args(n, states, dt, box, queue)
    assert lib.exc_trace_noalloc(C.byref(desc.struct), C.byref(b), stream) == N.EXC_ERR_INVALID
    assert b"queue must be NULL" in lib.exc_last_error()
