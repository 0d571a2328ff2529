"""ctypes view of libexcalibur_gb300.so (include/excalibur_gb300.h).

The structs below mirror the header field by field. The library is loaded
from this package directory only (it is built in-tree by build.py); a missing
library or a missing CUDA device raises -- there is no host fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libexcalibur_gb300.so")

EXC_ABI_VERSION = 2
EXC_MAX_FIELDS = 32

# return codes
EXC_SUCCESS, EXC_ERR_INVALID, EXC_ERR_CUDA, EXC_ERR_UNSUPPORTED, EXC_ERR_NO_DEVICE = 0, -1, -2, -3, -4

# per-photon status
PH_STEPS, PH_LEFT_BOX, PH_A_STOP, PH_MAX_ITER, PH_OUTSIDE_GRID, PH_HORIZON, PH_NONFINITE, \
    PH_TIMED_OUT, PH_ABORTED, PH_NOT_RUN, PH_BAD_FIELD, PH_RETRACE = range(12)
STATUS_NAMES = {PH_STEPS: "steps", PH_LEFT_BOX: "left_box", PH_A_STOP: "a_stop",
                PH_MAX_ITER: "max_iter", PH_OUTSIDE_GRID: "outside_grid", PH_HORIZON: "horizon",
                PH_NONFINITE: "nonfinite", PH_TIMED_OUT: "timed_out", PH_ABORTED: "aborted",
                PH_NOT_RUN: "not_run", PH_BAD_FIELD: "bad_field", PH_RETRACE: "retrace"}
FAILED_STATUSES = (PH_OUTSIDE_GRID, PH_HORIZON, PH_NONFINITE, PH_TIMED_OUT, PH_ABORTED, PH_NOT_RUN, PH_BAD_FIELD)

METRIC_FLRW, METRIC_SCHWARZSCHILD = 1, 2
COSMO_STATIC, COSMO_TABLE, COSMO_TABLE_FD = 0, 1, 2
BOUNDARY = {"periodic": 0, "clamp": 1, "error": 2}
GRAD = {"base_node": 0, "trilinear": 1}
PROBE = {"addmul": 0, "div": 1, "sqrt": 2, "fmod": 3}
# exc_record_redshift output columns (EXC_RS_*)
RS_COLUMNS = ("z_H", "z_SW", "z_ISW", "z_D", "z_total", "z_total_exact", "Phi_obs", "Phi_em", "a_obs", "a_em",
              "eta_obs", "eta_em", "x_obs0", "x_obs1", "x_obs2", "x_em0", "x_em1", "x_em2", "n_rows",
              "path", "chord", "time_delay", "td_kept")
DTYPE_F64, DTYPE_F32, DTYPE_F32X2 = 0, 1, 2
STEPPER = {"rk4": 0, "rk45": 1, "leapfrog4": 2}
TABLEAU = {"reference": 0, "fehlberg": 1}
PRECISION = {"fp64": 0, "fp64_fast": 1, "mixed": 2, "mixed_raw": 3, "retrace": 4}
STOP_BOX, STOP_A, STOP_FACE = 1, 2, 4
OBS_ENDPOINTS, OBS_PATH, OBS_ISW = 1, 2, 4
OBS_COLS = ["a_obs", "a_em", "phi_obs", "phi_em", "isw_int", "path", "chord", "excess",
            "v0x", "v0y", "v0z", "v1x", "v1y", "v1z", "min_r", "eta_obs", "eta_em"]
OBS_N = 20


class ExcField(C.Structure):
    _fields_ = [("data", C.c_void_p), ("dtype", C.c_int32), ("ndim", C.c_int32),
                ("boundary", C.c_int32), ("grad_mode", C.c_int32), ("n", C.c_int64 * 4),
                ("origin", C.c_double * 4), ("spacing", C.c_double * 4), ("shift", C.c_double * 3)]


class ExcMetric(C.Structure):
    _fields_ = [("kind", C.c_int32), ("analytical", C.c_int32), ("free_time", C.c_int32),
                ("cosmology", C.c_int32), ("c", C.c_double), ("c2", C.c_double), ("c4", C.c_double),
                ("two_over_c2", C.c_double), ("mass", C.c_double), ("radius", C.c_double),
                ("r_s", C.c_double), ("center", C.c_double * 3), ("a_table", C.c_void_p),
                ("a_table_n", C.c_int64), ("eta_min", C.c_double), ("eta_step", C.c_double),
                ("H0", C.c_double), ("omega_m", C.c_double), ("omega_r", C.c_double),
                ("omega_k", C.c_double), ("omega_lambda", C.c_double), ("n_fields", C.c_int32),
                ("reserved", C.c_int32), ("fields", ExcField * EXC_MAX_FIELDS)]


class ExcTraceArgs(C.Structure):
    _fields_ = [("n_photons", C.c_int64), ("state", C.c_void_p), ("status", C.c_void_p),
                ("n_steps", C.c_void_p), ("n_iter", C.c_void_p), ("dt_state", C.c_void_p),
                ("field_index", C.c_void_p), ("obs", C.c_void_p), ("records", C.c_void_p),
                ("n_records", C.c_void_p), ("record_every", C.c_int32), ("max_records", C.c_int32),
                ("record_cols", C.c_int32), ("stepper", C.c_int32), ("tableau", C.c_int32),
                ("precision", C.c_int32), ("renormalize_every", C.c_int32), ("stop_flags", C.c_int32),
                ("obs_flags", C.c_int32), ("block_size", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("staging", C.c_int32), ("dt", C.c_double), ("dt_min", C.c_double),
                ("dt_max", C.c_double), ("rtol", C.c_double), ("atol", C.c_double),
                ("max_iter", C.c_int64), ("max_steps", C.c_int64), ("box_lo", C.c_double * 3),
                ("box_hi", C.c_double * 3), ("a_stop", C.c_double), ("lens_center", C.c_double * 3),
                ("queue", C.c_void_p), ("abort_flag", C.c_void_p), ("deadline_cycles", C.c_int64)]


GEN_PATCH_GRID, GEN_PATCH_POINTS, GEN_CONE_GRID, GEN_FULL_SKY, GEN_CONE_RANDOM, GEN_IMPACT_BINS = 0, 1, 2, 3, 4, 5


class ExcPhotonGen(C.Structure):
    _fields_ = [("mode", C.c_int32), ("n_side", C.c_int32), ("n_theta", C.c_int32), ("n_phi", C.c_int32),
                ("n", C.c_int64), ("origin", C.c_double * 4), ("axis", C.c_double * 3), ("e1", C.c_double * 3),
                ("e2", C.c_double * 3), ("half", C.c_double), ("rot_axis", C.c_double * 3), ("rot_cos", C.c_double),
                ("rot_sin", C.c_double), ("uv", C.c_void_p), ("seed", C.c_uint64), ("speed", C.c_double),
                ("sign", C.c_double), ("n_bins", C.c_int32), ("random_phi", C.c_int32), ("spherical", C.c_int32),
                ("reserved", C.c_int32), ("b_edges", C.c_void_p), ("bin_offsets", C.c_void_p)]


EXC_TUNE_MAX_TRIALS = 48
# where the FP64 tracers read the a(eta) table (ExcTraceArgs.staging)
STAGING = {"cache": 0, "shared": 1}
STAGING_MAX_TABLE = 12288


class ExcLaunchPlan(C.Structure):
    _fields_ = [("block_size", C.c_int32), ("blocks_per_sm", C.c_int32), ("best_ms", C.c_float),
                ("best_rate", C.c_float), ("n_trials", C.c_int32), ("trial_block", C.c_int32 * EXC_TUNE_MAX_TRIALS),
                ("trial_blocks_per_sm", C.c_int32 * EXC_TUNE_MAX_TRIALS),
                ("trial_ms", C.c_float * EXC_TUNE_MAX_TRIALS), ("trial_rate", C.c_float * EXC_TUNE_MAX_TRIALS),
                ("staging", C.c_int32), ("trial_staging", C.c_int32 * EXC_TUNE_MAX_TRIALS)]


class ExcGemm(C.Structure):
    _fields_ = [("a", C.c_void_p), ("b", C.c_void_p), ("m", C.c_int64), ("n", C.c_int32), ("k", C.c_int32),
                ("stride_a", C.c_int64), ("stride_b", C.c_int64), ("n_batch", C.c_int32),
                ("epilogue", C.c_int32), ("k_splits", C.c_int32), ("reserved", C.c_int32),
                ("bias", C.c_void_p), ("z_in", C.c_void_p), ("c", C.c_void_p), ("c2", C.c_void_p),
                ("ct", C.c_void_p), ("stride_c", C.c_int64), ("ldt", C.c_int64), ("stride_ct", C.c_int64)]


EPI_F32, EPI_BIAS_SILU, EPI_DSILU, EPI_SPLITK = 0, 1, 2, 3


class ExcMlpInfer(C.Structure):
    _fields_ = [("x", C.c_void_p), ("w", C.c_void_p), ("b", C.c_void_p), ("w_head", C.c_void_p),
                ("b_head", C.c_void_p), ("y", C.c_void_p), ("m", C.c_int64), ("width", C.c_int32),
                ("n_members", C.c_int32), ("n_out", C.c_int32), ("depth", C.c_int32)]


class ExcBornArgs(C.Structure):
    _fields_ = [("n", C.c_int64), ("uv", C.c_void_p), ("origin", C.c_double * 3), ("axis", C.c_double * 3),
                ("e1", C.c_double * 3), ("e2", C.c_double * 3), ("half", C.c_double), ("box_lo", C.c_double * 3),
                ("box_hi", C.c_double * 3), ("step", C.c_double), ("c", C.c_double), ("out", C.c_void_p)]

class ExcAdamTensor(C.Structure):
    _fields_ = [("p", C.c_void_p), ("grad", C.c_void_p), ("m1", C.c_void_p), ("m2", C.c_void_p), ("n", C.c_int64),
                ("p_bf16", C.c_void_p), ("pt_bf16", C.c_void_p), ("rows", C.c_int32), ("cols", C.c_int32)]


EXC_ADAM_MAX_TENSORS = 16

_V = C.c_void_p
EXPORTS = {
    "exc_abi_version": (C.c_int, []),
    "exc_strerror": (C.c_char_p, [C.c_int]),
    "exc_last_error": (C.c_char_p, []),
    "exc_trace": (C.c_int, [C.POINTER(ExcMetric), C.POINTER(ExcTraceArgs), C.c_void_p]),
    "exc_geodesic_rhs": (C.c_int, [C.POINTER(ExcMetric), C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_int64, C.c_void_p]),
    "exc_interp": (C.c_int, [C.POINTER(ExcField), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "exc_eval_cosmology": (C.c_int, [C.POINTER(ExcMetric), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                     C.c_void_p]),
    "exc_metric_tensor": (C.c_int, [C.POINTER(ExcMetric), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int64, C.c_void_p]),
    "exc_null_init": (C.c_int, [C.POINTER(ExcMetric), C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                                C.c_int64, C.c_void_p]),
    "exc_null_error": (C.c_int, [C.POINTER(ExcMetric), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_int64, C.c_void_p]),
    "exc_trace_noalloc": (C.c_int, [C.POINTER(ExcMetric), C.POINTER(ExcTraceArgs), C.c_void_p]),
    "exc_gen_count": (C.c_int64, [C.POINTER(ExcPhotonGen)]),
    "exc_spherical_mass_grid": (C.c_int, [C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_void_p, C.c_void_p]),
    "exc_generate_photons": (C.c_int, [C.POINTER(ExcMetric), C.POINTER(ExcPhotonGen), C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "exc_balanced_blocks_per_sm": (C.c_int32, [C.c_int64, C.c_int32, C.c_int32]),
    "exc_autotune": (C.c_int, [C.POINTER(ExcMetric), C.POINTER(ExcTraceArgs), C.c_void_p,
                               C.POINTER(ExcLaunchPlan), C.c_void_p]),
    "exc_probe_scratch_len": (C.c_int64, []),
    "exc_probe_fp64_rates": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.c_void_p]),
    "exc_probe_div_rn": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_void_p, C.c_void_p]),
    # redshift maps from recorded trajectories
    "exc_record_redshift": (C.c_int, [_V, C.c_int64, C.c_int32, C.c_int32, C.c_double, _V, _V, _V, _V, _V]),
    "exc_sky_directions": (C.c_int, [_V, C.c_int64, C.c_int32, C.c_int32, _V, _V]),
    "exc_sky_project": (C.c_int, [_V, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), _V, _V, _V]),
    "exc_sky_bin": (C.c_int, [_V, _V, _V, C.c_int64, C.c_int32, C.c_int32, C.POINTER(C.c_double), _V, _V, _V,
                              _V]),
    # surrogate kernels (include/excalibur_mlp.h)
    "exc_gemm_bf16": (C.c_int, [C.POINTER(ExcGemm), _V]),
    "exc_mlp_infer": (C.c_int, [C.POINTER(ExcMlpInfer), _V]),
    "exc_mlp_features": (C.c_int, [_V, C.c_int64, C.c_int64, C.c_int32, C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), _V, _V]),
    "exc_mlp_head": (C.c_int, [_V, C.c_int64, C.c_int32, C.c_int32, C.c_int32, _V, _V, _V, _V, _V, _V, _V,
                               C.c_int64, _V, _V, _V, _V]),
    "exc_mlp_reduce_splits": (C.c_int, [_V, C.c_int32, C.c_int32, C.c_int64, _V, _V]),
    "exc_mlp_row_sums": (C.c_int, [_V, C.c_int64, C.c_int64, C.c_int64, _V, _V]),
    "exc_mlp_adam": (C.c_int, [_V, _V, _V, _V, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32,
                               _V, _V, C.c_int32, C.c_int32, _V]),
    "exc_mlp_adam_multi": (C.c_int, [C.POINTER(ExcAdamTensor), C.c_int32, _V, C.c_float, C.c_float, C.c_float,
                                     _V]),
    "exc_mlp_error_count": (C.c_int, [C.POINTER(C.c_uint32)]),
    "exc_born_patch": (C.c_int, [C.POINTER(ExcMetric), C.POINTER(ExcBornArgs), _V]),
}

_lib = None
_lock = threading.Lock()


class NativeError(RuntimeError):
    pass


def load(path: str = LIB_PATH):
    """Load the shared library and bind every exported entry point."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise NativeError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(there is no host fallback for the tracer)")
        lib = C.CDLL(path)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.exc_abi_version() != EXC_ABI_VERSION:
            raise NativeError("libexcalibur_gb300.so ABI version mismatch")
        _lib = lib
        return lib


def check(code: int, what: str):
    if code != EXC_SUCCESS:
        lib = load()
        msg = lib.exc_last_error().decode(errors="replace")
        raise NativeError(f"{what} failed: {lib.exc_strerror(code).decode()} ({code}): {msg}")


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_handle(device=None):
    import torch

    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)
