// exc_capi.cu -- the extern "C" boundary (include/excalibur_gb300.h).
//
// Validates arguments, builds the kernel-side metric view (reciprocals for
// the fast path), picks the precision build and enqueues the kernels on the
// caller's stream. No entry point allocates device memory: scratch (the work
// queue counter) is caller-owned.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstdarg>
#include <cstring>
#include <mutex>

#include "exc_dispatch.h"
#include "exc_mixed.h"
#include "exc_sched.h"

namespace {

thread_local char g_err[512] = "";

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(EXC_ERR_CUDA, "%s: %s (%s)", where, cudaGetErrorName(e), cudaGetErrorString(e));
}

int sm_count_current() {
  static std::mutex mu;
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  std::lock_guard<std::mutex> lk(mu);
  if (dev >= 0 && dev < 64 && cache[dev] > 0) return cache[dev];
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  if (dev >= 0 && dev < 64) cache[dev] = n;
  return n;
}

int check_field(const ExcField& f, int idx) {
  if (!f.data) return fail(EXC_ERR_INVALID, "field %d: data is NULL", idx);
  if (f.ndim != 3 && f.ndim != 4) return fail(EXC_ERR_INVALID, "field %d: ndim must be 3 or 4", idx);
  if (f.dtype != EXC_DTYPE_F64 && f.dtype != EXC_DTYPE_F32 && f.dtype != EXC_DTYPE_F32X2)
    return fail(EXC_ERR_INVALID, "field %d: unknown dtype %d", idx, f.dtype);
  if (f.boundary < EXC_BOUNDARY_PERIODIC || f.boundary > EXC_BOUNDARY_ERROR)
    return fail(EXC_ERR_INVALID, "field %d: unknown boundary %d", idx, f.boundary);
  for (int d = 0; d < f.ndim; ++d) {
    if (f.n[d] < 2) return fail(EXC_ERR_INVALID, "field %d: n[%d]=%lld < 2", idx, d, (long long)f.n[d]);
    if (!(f.spacing[d] > 0.0) || !std::isfinite(f.spacing[d]))
      return fail(EXC_ERR_INVALID, "field %d: spacing[%d] must be finite and > 0", idx, d);
    if (!std::isfinite(f.origin[d])) return fail(EXC_ERR_INVALID, "field %d: origin[%d] not finite", idx, d);
  }
  for (int d = 0; d < 3; ++d)
    if (!std::isfinite(f.shift[d])) return fail(EXC_ERR_INVALID, "field %d: shift[%d] not finite", idx, d);
  if (f.grad_mode != EXC_GRAD_BASE_NODE && f.grad_mode != EXC_GRAD_TRILINEAR)
    return fail(EXC_ERR_INVALID, "field %d: unknown grad_mode %d", idx, f.grad_mode);
  if (f.grad_mode == EXC_GRAD_TRILINEAR) {
    if (f.boundary != EXC_BOUNDARY_ERROR)
      return fail(EXC_ERR_INVALID, "field %d: the trilinear gradient needs the error boundary", idx);
    for (int d = 0; d < 3; ++d)
      if (f.n[d] < 3) return fail(EXC_ERR_INVALID, "field %d: the trilinear gradient needs n >= 3 per axis", idx);
  } else if (f.boundary == EXC_BOUNDARY_ERROR) {
    for (int d = 0; d < 3; ++d)
      if (f.n[d] < 4) return fail(EXC_ERR_INVALID, "field %d: error boundary needs n >= 4 per axis", idx);
  }
  return 0;
}

int build_dev_metric(const ExcMetric* m, exc::DevMetric& D) {
  if (!m) return fail(EXC_ERR_INVALID, "metric is NULL");
  if (m->kind != EXC_METRIC_FLRW && m->kind != EXC_METRIC_SCHWARZSCHILD)
    return fail(EXC_ERR_INVALID, "unknown metric kind %d", m->kind);
  if (!(m->c > 0.0) || !(m->c2 > 0.0) || !(m->c4 > 0.0))
    return fail(EXC_ERR_INVALID, "speed-of-light constants must be > 0");
  memset(&D, 0, sizeof(D));
  D.m = *m;
  D.ic2 = 1.0 / m->c2;
  D.ic4 = 1.0 / m->c4;
  if (m->kind == EXC_METRIC_FLRW) {
    if (m->n_fields < 1 || m->n_fields > EXC_MAX_FIELDS)
      return fail(EXC_ERR_INVALID, "n_fields=%d outside [1, %d]", m->n_fields, EXC_MAX_FIELDS);
    for (int i = 0; i < m->n_fields; ++i) {
      int e = check_field(m->fields[i], i);
      if (e) return e;
      if (m->fields[i].dtype != m->fields[0].dtype)
        return fail(EXC_ERR_INVALID, "all fields of one call must share a dtype");
      const ExcField& f = m->fields[i];
      for (int d = 0; d < f.ndim; ++d) D.finv[i][d] = 1.0 / f.spacing[d];
      for (int d = 0; d < 3; ++d) D.finv[i][4 + d] = 1.0 / (2.0 * f.spacing[d]);
      if (f.ndim == 4) D.finv[i][7] = 1.0 / (2.0 * f.spacing[3]);
    }
    if (m->cosmology != EXC_COSMO_STATIC && m->cosmology != EXC_COSMO_TABLE &&
        m->cosmology != EXC_COSMO_TABLE_FD)
      return fail(EXC_ERR_INVALID, "unknown cosmology mode %d", m->cosmology);
    if (m->cosmology != EXC_COSMO_STATIC) {
      if (!m->a_table || m->a_table_n < 2) return fail(EXC_ERR_INVALID, "cosmology table missing (n >= 2)");
      if (!(m->eta_step > 0.0)) return fail(EXC_ERR_INVALID, "eta_step must be > 0");
      D.i_eta_step = 1.0 / m->eta_step;
    }
  } else {
    if (!(m->r_s > 0.0)) return fail(EXC_ERR_INVALID, "Schwarzschild r_s must be > 0");
  }
  return 0;
}

// Split float32x2 grids are read by the mixed-precision tracer alone; every
// FP64 evaluator rejects them (all fields of a call share one dtype).
int reject_split(const ExcMetric* m) {
  if (m->kind == EXC_METRIC_FLRW && m->fields[0].dtype == EXC_DTYPE_F32X2)
    return fail(EXC_ERR_UNSUPPORTED, "split float32x2 grids are read by the mixed-precision tracer only");
  return 0;
}

int check_fidx(const ExcMetric* m, const int32_t* fidx) {
  if (fidx && m->kind != EXC_METRIC_FLRW)
    return fail(EXC_ERR_INVALID, "field_index given for a metric without fields");
  return 0;
}

}  // namespace

namespace exc {
// Lets the other boundary unit (exc_noalloc.cu) report through exc_last_error().
void set_last_error(const char* msg) { snprintf(g_err, sizeof(g_err), "%s", msg); }
}  // namespace exc

extern "C" {

int exc_abi_version(void) { return EXC_ABI_VERSION; }

int32_t exc_balanced_blocks_per_sm(int64_t n_photons, int32_t sm_count, int32_t occupancy) {
  return exc::balanced_warps_per_sm(n_photons, sm_count, occupancy);
}

const char* exc_last_error(void) { return g_err; }

const char* exc_strerror(int code) {
  switch (code) {
    case EXC_SUCCESS: return "success";
    case EXC_ERR_INVALID: return "invalid argument";
    case EXC_ERR_CUDA: return "CUDA runtime error";
    case EXC_ERR_UNSUPPORTED: return "unsupported combination";
    case EXC_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown error";
  }
}

int exc_trace(const ExcMetric* metric, const ExcTraceArgs* a, void* stream) {
  g_err[0] = 0;
  if (!a) return fail(EXC_ERR_INVALID, "args is NULL");
  exc::DevMetric D;
  int e = build_dev_metric(metric, D);
  if (e) return e;
  if (a->n_photons < 0) return fail(EXC_ERR_INVALID, "n_photons < 0");
  if (a->n_photons == 0) return EXC_SUCCESS;
  if (!a->state || !a->status) return fail(EXC_ERR_INVALID, "state and status are required");
  if ((e = check_fidx(metric, a->field_index))) return e;
  if (a->stepper < EXC_STEPPER_RK4 || a->stepper > EXC_STEPPER_LEAPFROG4)
    return fail(EXC_ERR_INVALID, "unknown stepper %d", a->stepper);
  if (a->tableau != EXC_TABLEAU_REFERENCE && a->tableau != EXC_TABLEAU_FEHLBERG)
    return fail(EXC_ERR_INVALID, "unknown tableau %d", a->tableau);
  if (a->precision < EXC_PREC_FP64_EXACT || a->precision > EXC_PREC_RETRACE)
    return fail(EXC_ERR_INVALID, "unknown precision %d", a->precision);
  const bool mixed = a->precision >= EXC_PREC_MIXED;
  if (!mixed && (e = reject_split(metric))) return e;
  if (mixed) {
    const int me = exc_mixed::check(D, *a);
    if (me) return fail(EXC_ERR_UNSUPPORTED, "%s", exc_mixed::why(me));
  }
  if (a->max_iter < 0 || a->max_steps < 0) return fail(EXC_ERR_INVALID, "max_iter/max_steps must be >= 0");
  if (!std::isfinite(a->dt)) return fail(EXC_ERR_INVALID, "dt must be finite");
  if (a->record_every < 0) return fail(EXC_ERR_INVALID, "record_every must be >= 0");
  if (a->renormalize_every < 0) return fail(EXC_ERR_INVALID, "renormalize_every must be >= 0");
  if (a->records) {
    const int want = metric->kind == EXC_METRIC_FLRW ? 14 : 12;
    if (!a->n_records || a->max_records < 1 || a->record_cols != want)
      return fail(EXC_ERR_INVALID, "records need n_records, max_records >= 1 and record_cols == %d", want);
  }
  if (a->obs_flags && !a->obs) return fail(EXC_ERR_INVALID, "obs_flags set but obs is NULL");
  if (a->staging != EXC_STAGING_CACHE && a->staging != EXC_STAGING_SHARED)
    return fail(EXC_ERR_INVALID, "unknown staging %d", a->staging);
  // the FP64 launches read the a(eta) table from shared memory only when the metric has one
  const bool uses_table = metric->kind == EXC_METRIC_FLRW && metric->cosmology != EXC_COSMO_STATIC;
  if (a->staging == EXC_STAGING_SHARED && uses_table && metric->a_table_n > EXC_STAGING_MAX_TABLE)
    return fail(EXC_ERR_INVALID, "staging: the a(eta) table has %lld entries (shared memory holds %d)",
                (long long)metric->a_table_n, EXC_STAGING_MAX_TABLE);
  const int stage_table = a->staging == EXC_STAGING_SHARED && uses_table ? 1 : 0;
  const int block = a->block_size > 0 ? a->block_size : 128;
  if (block % 32 != 0 || block > 128)
    return fail(EXC_ERR_INVALID, "block_size must be a multiple of 32 and <= 128");
  const int sms = sm_count_current();
  if (sms <= 0) return fail(EXC_ERR_NO_DEVICE, "no CUDA device");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t ce;
  if ((a->abort_flag || a->deadline_cycles > 0) && a->precision != EXC_PREC_RETRACE) {
    // photons the launch never reaches keep EXC_PH_NOT_RUN
    ce = exc_fast::fill_status(a->status, a->n_photons, EXC_PH_NOT_RUN, s);
    if (ce != cudaSuccess) return cuda_fail(ce, "fill_status");
  }
  if (a->queue) {
    ce = cudaMemsetAsync(a->queue, 0, 2 * sizeof(uint32_t), s);
    if (ce != cudaSuccess) return cuda_fail(ce, "queue reset");
  }
  if (a->precision == EXC_PREC_FP64_EXACT || a->precision == EXC_PREC_FP64_FAST) {
    D.stage_table = stage_table;
    // no schedule given: the FP64 launchers' balanced default (32-thread blocks, the last wave full)
    const int b64 = (a->block_size > 0 || a->blocks_per_sm > 0) ? block : 0;
    ce = a->precision == EXC_PREC_FP64_EXACT ? exc_exact::trace(D, *a, b64, a->blocks_per_sm, sms, s)
                                              : exc_fast::trace(D, *a, b64, a->blocks_per_sm, sms, s);
  } else {
    if (a->precision != EXC_PREC_RETRACE) {
      ce = exc_mixed::trace(D, *a, block, a->blocks_per_sm, sms, s);
      if (ce != cudaSuccess) return cuda_fail(ce, "mixed trace launch");
    }
    if (a->precision == EXC_PREC_MIXED || a->precision == EXC_PREC_RETRACE) {
      // the FP64 tracer takes the rays the mixed one handed back (status
      // EXC_PH_RETRACE, state and dt untouched); same stream, so in order
      if (a->queue && a->precision == EXC_PREC_MIXED) {
        ce = cudaMemsetAsync(a->queue, 0, 2 * sizeof(uint32_t), s);
        if (ce != cudaSuccess) return cuda_fail(ce, "queue reset");
      }
      D.retrace_only = 1;
      D.retrace_sms = sms;
      D.stage_table = stage_table;
      // with a work queue the re-trace launch fills the SMs and sizes its active blocks on the
      // device from the handed-back share (trace_kernel); the plan's blocks per SM is the mixed
      // pass's
      ce = exc_fast::trace(D, *a, block, a->queue ? 0 : a->blocks_per_sm, sms, s);
      if (ce != cudaSuccess) return cuda_fail(ce, "re-trace launch");
    }
    return EXC_SUCCESS;
  }
  if (ce != cudaSuccess) return cuda_fail(ce, "trace launch");
  return EXC_SUCCESS;
}

int exc_geodesic_rhs(const ExcMetric* metric, int32_t precision, const double* state, double* out,
                     int32_t* status, const int32_t* field_index, int64_t n, void* stream) {
  g_err[0] = 0;
  exc::DevMetric D;
  int e = build_dev_metric(metric, D);
  if (e) return e;
  if (n < 0) return fail(EXC_ERR_INVALID, "n < 0");
  if (n > 0 && (!state || !out)) return fail(EXC_ERR_INVALID, "state/out are required");
  if ((e = check_fidx(metric, field_index))) return e;
  if ((e = reject_split(metric))) return e;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t ce;
  if (precision == EXC_PREC_FP64_EXACT) ce = exc_exact::rhs(D, state, out, status, field_index, n, s);
  else if (precision == EXC_PREC_FP64_FAST) ce = exc_fast::rhs(D, state, out, status, field_index, n, s);
  else return fail(EXC_ERR_UNSUPPORTED, "exc_geodesic_rhs supports the FP64 precisions only");
  if (ce != cudaSuccess) return cuda_fail(ce, "rhs launch");
  return EXC_SUCCESS;
}

int exc_interp(const ExcField* field, const double* points, double* out, int32_t* status, int64_t n,
               void* stream) {
  g_err[0] = 0;
  if (!field) return fail(EXC_ERR_INVALID, "field is NULL");
  int e = check_field(*field, 0);
  if (e) return e;
  if (field->dtype == EXC_DTYPE_F32X2)
    return fail(EXC_ERR_UNSUPPORTED, "exc_interp reads float64 or float32 grids");
  if (n < 0) return fail(EXC_ERR_INVALID, "n < 0");
  if (n > 0 && (!points || !out)) return fail(EXC_ERR_INVALID, "points/out are required");
  cudaError_t ce = exc_exact::interp(*field, points, out, status, n, (cudaStream_t)stream);
  if (ce != cudaSuccess) return cuda_fail(ce, "interp launch");
  return EXC_SUCCESS;
}

int exc_eval_cosmology(const ExcMetric* metric, const double* eta, double* a, double* adot, int64_t n,
                       void* stream) {
  g_err[0] = 0;
  exc::DevMetric D;
  if (!metric) return fail(EXC_ERR_INVALID, "metric is NULL");
  if (metric->cosmology != EXC_COSMO_STATIC && (!metric->a_table || metric->a_table_n < 2))
    return fail(EXC_ERR_INVALID, "cosmology table missing (n >= 2)");
  memset(&D, 0, sizeof(D));
  D.m = *metric;
  D.i_eta_step = metric->eta_step > 0 ? 1.0 / metric->eta_step : 0.0;
  if (n < 0) return fail(EXC_ERR_INVALID, "n < 0");
  if (n > 0 && !eta) return fail(EXC_ERR_INVALID, "eta is required");
  cudaError_t ce = exc_exact::cosmology(D, eta, a, adot, n, (cudaStream_t)stream);
  if (ce != cudaSuccess) return cuda_fail(ce, "cosmology launch");
  return EXC_SUCCESS;
}

int exc_metric_tensor(const ExcMetric* metric, const double* x, double* g_diag, int32_t* status,
                      const int32_t* field_index, int64_t n, void* stream) {
  g_err[0] = 0;
  exc::DevMetric D;
  int e = build_dev_metric(metric, D);
  if (e) return e;
  if (n < 0) return fail(EXC_ERR_INVALID, "n < 0");
  if (n > 0 && (!x || !g_diag)) return fail(EXC_ERR_INVALID, "x/g_diag are required");
  if ((e = check_fidx(metric, field_index))) return e;
  if ((e = reject_split(metric))) return e;
  cudaError_t ce = exc_exact::metric(D, x, g_diag, status, field_index, n, (cudaStream_t)stream);
  if (ce != cudaSuccess) return cuda_fail(ce, "metric launch");
  return EXC_SUCCESS;
}

int exc_null_init(const ExcMetric* metric, double* state, double sign, int32_t* status,
                  const int32_t* field_index, int64_t n, void* stream) {
  g_err[0] = 0;
  exc::DevMetric D;
  int e = build_dev_metric(metric, D);
  if (e) return e;
  if (n < 0) return fail(EXC_ERR_INVALID, "n < 0");
  if (n > 0 && !state) return fail(EXC_ERR_INVALID, "state is required");
  if ((e = check_fidx(metric, field_index))) return e;
  if ((e = reject_split(metric))) return e;
  cudaError_t ce = exc_exact::null_init(D, state, sign, status, field_index, n, (cudaStream_t)stream);
  if (ce != cudaSuccess) return cuda_fail(ce, "null_init launch");
  return EXC_SUCCESS;
}

int exc_null_error(const ExcMetric* metric, const double* state, double* rel_err, int32_t* status,
                   const int32_t* field_index, int64_t n, void* stream) {
  g_err[0] = 0;
  exc::DevMetric D;
  int e = build_dev_metric(metric, D);
  if (e) return e;
  if (n < 0) return fail(EXC_ERR_INVALID, "n < 0");
  if (n > 0 && (!state || !rel_err)) return fail(EXC_ERR_INVALID, "state/rel_err are required");
  if ((e = check_fidx(metric, field_index))) return e;
  if ((e = reject_split(metric))) return e;
  cudaError_t ce = exc_exact::null_error(D, state, rel_err, status, field_index, n, (cudaStream_t)stream);
  if (ce != cudaSuccess) return cuda_fail(ce, "null_error launch");
  return EXC_SUCCESS;
}

}  // extern "C"
