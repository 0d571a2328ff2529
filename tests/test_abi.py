"""The C ABI: the built library exports every entry point the header declares,
and the ctypes mirrors of the structs have the C layout (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT
from excalibur_tool_gb300 import _native as N

HEADER = os.path.join(ROOT, "include", "excalibur_gb300.h")
HEADERS = [os.path.join(ROOT, "include", h) for h in ("excalibur_gb300.h", "excalibur_mlp.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names.update(re.findall(r"\b(exc_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(N.LIB_PATH):
        from excalibur_tool_gb300 import build

        build.build()
    return C.CDLL(N.LIB_PATH)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name


def test_version_and_errors_without_a_device(lib):
    lib.exc_abi_version.restype = C.c_int
    assert lib.exc_abi_version() == N.EXC_ABI_VERSION
    lib.exc_strerror.restype = C.c_char_p
    assert lib.exc_strerror(N.EXC_ERR_INVALID) == b"invalid argument"


def test_invalid_arguments_rejected_before_any_launch(lib):
    L = N.load()
    m = N.ExcMetric()
    m.kind = 99
    a = N.ExcTraceArgs()
    rc = L.exc_trace(C.byref(m), C.byref(a), None)
    assert rc == N.EXC_ERR_INVALID
    assert b"metric kind" in L.exc_last_error()
    assert L.exc_trace(None, C.byref(a), None) == N.EXC_ERR_INVALID


def _split_flrw_metric():
    m = N.ExcMetric()
    m.kind = N.METRIC_FLRW
    m.c, m.c2, m.c4 = 299792458.0, 299792458.0 ** 2, 299792458.0 ** 4
    m.n_fields = 1
    f = m.fields[0]
    f.data = 4096                      # never dereferenced: every case fails validation first
    f.dtype = N.DTYPE_F32X2
    f.ndim = 3
    for d in range(3):
        f.n[d], f.spacing[d] = 8, 1.0
    return m


def _args(**kw):
    a = N.ExcTraceArgs()
    a.n_photons = 1
    a.state = a.status = 4096
    a.dt = a.dt_min = a.dt_max = 1.0
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def test_split_grids_only_for_the_mixed_tracer(lib):
    """float32x2 planes are rejected by every FP64 entry point before any device work."""
    L = N.load()
    m = _split_flrw_metric()
    for prec in (N.PRECISION["fp64"], N.PRECISION["fp64_fast"]):
        assert L.exc_trace(C.byref(m), C.byref(_args(precision=prec)), None) == N.EXC_ERR_UNSUPPORTED
        assert b"mixed-precision" in L.exc_last_error()
    x = C.c_void_p(4096)
    assert L.exc_geodesic_rhs(C.byref(m), 0, x, x, None, None, 1, None) == N.EXC_ERR_UNSUPPORTED
    assert L.exc_metric_tensor(C.byref(m), x, x, None, None, 1, None) == N.EXC_ERR_UNSUPPORTED
    assert L.exc_null_init(C.byref(m), x, C.c_double(-1.0), None, None, 1, None) == N.EXC_ERR_UNSUPPORTED
    assert L.exc_null_error(C.byref(m), x, x, None, None, 1, None) == N.EXC_ERR_UNSUPPORTED


@pytest.mark.parametrize("kw,msg", [
    (dict(stepper=N.STEPPER["leapfrog4"]), b"RK4 and RK45 steppers only"),
    (dict(records=4096, n_records=4096, max_records=2, record_cols=14), b"record"),
    (dict(obs=4096, obs_flags=N.OBS_ISW), b"ISW"),
])
def test_mixed_rejects_what_it_does_not_implement(lib, kw, msg):
    L = N.load()
    m = _split_flrw_metric()
    a = _args(precision=N.PRECISION["mixed"], **kw)
    assert L.exc_trace(C.byref(m), C.byref(a), None) == N.EXC_ERR_UNSUPPORTED
    assert msg in L.exc_last_error()


def test_struct_layout_matches_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "excalibur_gb300.h"
#include "excalibur_mlp.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(ExcField), sizeof(ExcMetric),
         sizeof(ExcTraceArgs), offsetof(ExcMetric, fields), offsetof(ExcTraceArgs, dt), offsetof(ExcTraceArgs, queue),
         offsetof(ExcTraceArgs, deadline_cycles), sizeof(ExcGemm), offsetof(ExcGemm, bias),
         offsetof(ExcGemm, stride_ct), sizeof(ExcPhotonGen), offsetof(ExcPhotonGen, uv), sizeof(ExcLaunchPlan),
         offsetof(ExcLaunchPlan, trial_rate), offsetof(ExcField, shift), sizeof(ExcAdamTensor),
         offsetof(ExcAdamTensor, rows), offsetof(ExcTraceArgs, staging), offsetof(ExcLaunchPlan, trial_staging));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "sz.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "sz")
        subprocess.run(["gcc", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        got = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    want = [C.sizeof(N.ExcField), C.sizeof(N.ExcMetric), C.sizeof(N.ExcTraceArgs), N.ExcMetric.fields.offset,
            N.ExcTraceArgs.dt.offset, N.ExcTraceArgs.queue.offset, N.ExcTraceArgs.deadline_cycles.offset,
            C.sizeof(N.ExcGemm), N.ExcGemm.bias.offset, N.ExcGemm.stride_ct.offset, C.sizeof(N.ExcPhotonGen),
            N.ExcPhotonGen.uv.offset, C.sizeof(N.ExcLaunchPlan), N.ExcLaunchPlan.trial_rate.offset,
            N.ExcField.shift.offset, C.sizeof(N.ExcAdamTensor), N.ExcAdamTensor.rows.offset,
            N.ExcTraceArgs.staging.offset, N.ExcLaunchPlan.trial_staging.offset]
    assert got == want


def _table_flrw_metric(n_table):
    m = N.ExcMetric()
    m.kind = N.METRIC_FLRW
    m.c, m.c2, m.c4 = 299792458.0, 299792458.0 ** 2, 299792458.0 ** 4
    m.cosmology = 1                    # EXC_COSMO_TABLE
    m.a_table, m.a_table_n = 4096, n_table
    m.eta_min, m.eta_step = 0.0, 1.0
    m.n_fields = 1
    f = m.fields[0]
    f.data = 4096                      # never dereferenced: every case fails validation first
    f.dtype = N.DTYPE_F64
    f.ndim = 3
    for d in range(3):
        f.n[d], f.spacing[d] = 8, 1.0
    return m


def test_staging_is_validated_on_the_host(lib):
    """An unknown staging value, or a table too large for shared memory with EXC_STAGING_SHARED,
    is refused before any device work."""
    L = N.load()
    m = _table_flrw_metric(5000)
    assert L.exc_trace(C.byref(m), C.byref(_args(staging=7)), None) == N.EXC_ERR_INVALID
    assert b"unknown staging" in L.exc_last_error()
    big = _table_flrw_metric(N.STAGING_MAX_TABLE + 1)
    assert L.exc_trace(C.byref(big), C.byref(_args(staging=N.STAGING["shared"])), None) == N.EXC_ERR_INVALID
    assert b"staging" in L.exc_last_error()


def test_new_entry_points_validate_before_any_launch(lib):
    """Argument checks of the lens-grid, multi-tensor Adam and shifted-field paths run on the
    host: the invalid calls below return an error without touching a device."""
    L = N.load()
    n = (C.c_int64 * 3)(0, 4, 4)
    d3 = (C.c_double * 3)(0.0, 0.0, 0.0)
    assert L.exc_spherical_mass_grid(n, d3, d3, d3, 1.0, -1.0, 3.0, 2.0, C.c_void_p(4096), None) == N.EXC_ERR_INVALID
    assert b"n must be" in L.exc_last_error()
    n_ok = (C.c_int64 * 3)(4, 4, 4)
    assert L.exc_spherical_mass_grid(n_ok, d3, d3, d3, 1.0, -1.0, 3.0, 2.0, None, None) == N.EXC_ERR_INVALID
    arr = (N.ExcAdamTensor * 1)()
    assert L.exc_mlp_adam_multi(arr, 0, C.c_void_p(4096), 0.9, 0.999, 1e-8, None) == N.EXC_ERR_INVALID
    assert L.exc_mlp_adam_multi(arr, N.EXC_ADAM_MAX_TENSORS + 1, C.c_void_p(4096), 0.9, 0.999, 1e-8,
                                None) == N.EXC_ERR_INVALID
    assert L.exc_mlp_adam_multi(arr, 1, C.c_void_p(4096), 0.9, 0.999, 1e-8, None) == N.EXC_ERR_INVALID  # p NULL
    # a non-finite query offset is refused by the trace's field validation
    m = N.ExcMetric()
    m.kind = N.METRIC_FLRW
    m.c, m.c2, m.c4 = 299792458.0, 299792458.0 ** 2, 299792458.0 ** 4
    m.n_fields = 1
    f = m.fields[0]
    f.data = 4096
    f.dtype = N.DTYPE_F64
    f.ndim = 3
    for d in range(3):
        f.n[d], f.spacing[d] = 8, 1.0
    f.shift[1] = float("nan")
    assert L.exc_trace(C.byref(m), C.byref(_args()), None) == N.EXC_ERR_INVALID
    assert b"shift" in L.exc_last_error()


def test_map_entry_points_validate_before_any_launch(lib):
    """The redshift-map entry points refuse bad shapes and half-given inputs on the host."""
    L = N.load()
    P = C.c_void_p(4096)
    c = 299792458.0
    # fewer than the 14 FLRW record columns; one velocity array without the other; c <= 0
    assert L.exc_record_redshift(P, 4, 10, 8, c, None, None, P, P, None) == N.EXC_ERR_INVALID
    assert b"n_cols >= 14" in L.exc_last_error()
    assert L.exc_record_redshift(P, 4, 10, 14, c, P, None, P, P, None) == N.EXC_ERR_INVALID
    assert L.exc_record_redshift(P, 4, 10, 14, 0.0, None, None, P, P, None) == N.EXC_ERR_INVALID
    assert L.exc_record_redshift(None, 4, 10, 14, c, None, None, P, P, None) == N.EXC_ERR_INVALID
    assert L.exc_record_redshift(None, 0, 10, 14, c, None, None, None, None, None) == N.EXC_SUCCESS
    assert L.exc_sky_directions(P, 4, 10, 7, P, None) == N.EXC_ERR_INVALID
    d3 = (C.c_double * 3)(1.0, 0.0, 0.0)
    assert L.exc_sky_project(P, -1, d3, d3, d3, P, P, None) == N.EXC_ERR_INVALID
    assert L.exc_sky_project(None, 4, d3, d3, d3, P, P, None) == N.EXC_ERR_INVALID
    ext = (C.c_double * 4)(0.0, 1.0, 0.0, 1.0)
    assert L.exc_sky_bin(P, P, P, 10, 0, 4, ext, P, P, P, None) == N.EXC_ERR_INVALID
    bad = (C.c_double * 4)(1.0, 0.0, 0.0, 1.0)
    assert L.exc_sky_bin(P, P, P, 10, 4, 4, bad, P, P, P, None) == N.EXC_ERR_INVALID
    assert b"x1 > x0" in L.exc_last_error()
    assert L.exc_sky_bin(None, P, P, 10, 4, 4, ext, P, P, P, None) == N.EXC_ERR_INVALID


def test_fused_inference_validates_on_the_host(lib):
    """exc_mlp_infer refuses bad shapes and pointers that its vector loads could not take (a
    misaligned head weight or bias) before any device work."""
    L = N.load()

    def args(**kw):
        a = N.ExcMlpInfer()
        a.x, a.w, a.b, a.w_head, a.b_head, a.y = 4096, 8192, 4096, 4096, 4096, 4096
        a.m, a.width, a.n_members, a.n_out, a.depth = 256, 256, 4, 6, 4
        for k, v in kw.items():
            setattr(a, k, v)
        return a

    for kw, msg in ((dict(m=100), b"multiple of 128"), (dict(width=128), b"width"), (dict(n_out=9), b"n_out"),
                    (dict(depth=0), b"depth"), (dict(w_head=4100), b"aligned"), (dict(b=4100), b"aligned"),
                    (dict(x=4104), b"aligned"), (dict(y=None), b"required")):
        assert L.exc_mlp_infer(C.byref(args(**kw)), None) == N.EXC_ERR_INVALID, kw
        assert msg in L.exc_last_error(), (kw, L.exc_last_error())


@pytest.mark.parametrize("n,sms,occ,want", [
    (65536, 152, 9, 7),        # 2 waves at 9 warps an SM; 7 fills the second (1.92 rays a lane)
    (65536, 152, 8, 7),
    (2097152, 152, 9, 9),      # many waves: the occupancy limit
    (1000, 152, 9, 1),         # fewer rays than an SM's lanes each: one warp an SM
    (43776, 152, 9, 9),        # exactly one full wave
    (43777, 152, 9, 5),        # one ray over: two waves of ~21,900 rays
    (0, 152, 9, 1), (5, 0, 0, 1),
])
def test_balanced_schedule(lib, n, sms, occ, want):
    """The FP64 builds' default launch size: whole warps an SM that make the last wave full."""
    assert N.load().exc_balanced_blocks_per_sm(n, sms, occ) == want
