// exc_aux.cuh -- batch evaluators (RHS, interpolation, cosmology, metric,
// null initialisation / error) and their launchers; included once per
// precision build by its *_aux.cu unit.
#pragma once

#include "exc_kernels.cuh"

namespace EXC_NS {

// field index of batch element i, clamped into the descriptor table (the host
// validates indices; this only keeps a bad one from reading past the table)
__device__ __forceinline__ int fidx_ok(const DevMetric& D, const int32_t* fidx, int64_t i) {
  const int f = fidx ? fidx[i] : 0;
  return ((unsigned)f < (unsigned)D.m.n_fields) ? f : 0;
}

__global__ void fill_status_kernel(int32_t* status, int64_t n, int32_t value) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    status[i] = value;
}

// ------------------------------------------------------ batch evaluators
template <class FT>
__global__ void rhs_kernel(const DevMetric D, const double* __restrict__ state, double* __restrict__ out,
                           int32_t* status, const int32_t* field_index, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s[8], o[8];
  for (int k = 0; k < 8; ++k) s[k] = state[i * 8 + k];
  int st;
  if (D.m.kind == EXC_METRIC_SCHWARZSCHILD) st = schw_rhs(D, s, o);
  else st = flrw_rhs<FT>(D, fidx_ok(D, field_index, i), s, o);
  for (int k = 0; k < 8; ++k) out[i * 8 + k] = st ? NAN : o[k];
  if (status) status[i] = st;
}

template <class FT>
__global__ void interp_kernel(const ExcField f, const double fi0, const double fi1, const double fi2,
                              const double fi3, const double* __restrict__ pts, double* __restrict__ out,
                              int32_t* status, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double fi[8] = {fi0, fi1, fi2, fi3, 0.5 * fi0, 0.5 * fi1, 0.5 * fi2, 0.5 * fi3};
  InterpOut o;
  const int st = interp_field<FT>(f, fi, pts[i * 4 + 0], pts[i * 4 + 1], pts[i * 4 + 2], pts[i * 4 + 3], o);
  out[i * 5 + 0] = st ? NAN : o.val;
  out[i * 5 + 1] = st ? NAN : o.gx;
  out[i * 5 + 2] = st ? NAN : o.gy;
  out[i * 5 + 3] = st ? NAN : o.gz;
  out[i * 5 + 4] = st ? NAN : o.dtd;
  if (status) status[i] = st;
}

__global__ void cosmology_kernel(const DevMetric D, const double* __restrict__ eta, double* a_out,
                                 double* adot_out, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a, adot, inv_a;
  const int st = scale_factor(D, eta[i], a, adot, inv_a);
  if (a_out) a_out[i] = st ? NAN : a;
  if (adot_out) adot_out[i] = st ? NAN : adot;
}

template <class FT>
__global__ void metric_kernel(const DevMetric D, const double* __restrict__ x, double* __restrict__ g,
                              int32_t* status, const int32_t* field_index, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xx[4] = {x[i * 4], x[i * 4 + 1], x[i * 4 + 2], x[i * 4 + 3]}, gg[4];
  const int st = metric_diag<FT>(D, fidx_ok(D, field_index, i), xx, gg);
  for (int k = 0; k < 4; ++k) g[i * 4 + k] = st ? NAN : gg[k];
  if (status) status[i] = st;
}

// Photons._solve_u0_from_null_condition, photon/photons.py:540-568.
template <class FT>
__global__ void null_init_kernel(const DevMetric D, double* state, double sign, int32_t* status,
                                 const int32_t* field_index, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double* s = state + i * 8;
  double g[4];
  const int st = metric_diag<FT>(D, fidx_ok(D, field_index, i), s, g);
  if (status) status[i] = st;
  if (st) return;
  const double spatial = g[1] * (s[5] * s[5]) + g[2] * (s[6] * s[6]) + g[3] * (s[7] * s[7]);
  const double u0_sq = (g[0] != 0.0) ? -spatial / g[0] : NAN;
  const double u0 = isfinite(u0_sq) ? sqrt(fabs(u0_sq)) : 1.0;
  s[4] = sign * u0;
}

// Photon.null_condition_relative_error, photon/photon.py:46-68.
template <class FT>
__global__ void null_error_kernel(const DevMetric D, const double* __restrict__ state, double* rel,
                                  int32_t* status, const int32_t* field_index, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* s = state + i * 8;
  double g[4];
  const int st = metric_diag<FT>(D, fidx_ok(D, field_index, i), s, g);
  if (status) status[i] = st;
  if (st) { rel[i] = NAN; return; }
  const double u0 = s[4], u1 = s[5], u2 = s[6], u3 = s[7];
  const double norm = u0 * (g[0] * u0) + u1 * (g[1] * u1) + u2 * (g[2] * u2) + u3 * (g[3] * u3);
  const double den = fabs(g[0] * (u0 * u0)) + fabs(g[1] * (u1 * u1)) + fabs(g[2] * (u2 * u2)) +
                     fabs(g[3] * (u3 * u3));
  rel[i] = den > 0.0 ? fabs(norm) / den : fabs(norm);
}

inline int blocks_for(int64_t n, int b) { return (int)((n + b - 1) / b); }

inline cudaError_t launch_rhs(const DevMetric& D, const double* st, double* out, int32_t* status,
                              const int32_t* fidx, int64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (D.m.kind == EXC_METRIC_FLRW && D.m.fields[0].dtype == EXC_DTYPE_F32)
    rhs_kernel<float><<<blocks_for(n, 128), 128, 0, s>>>(D, st, out, status, fidx, n);
  else
    rhs_kernel<double><<<blocks_for(n, 128), 128, 0, s>>>(D, st, out, status, fidx, n);
  return cudaGetLastError();
}

inline cudaError_t launch_interp(const ExcField& f, const double* pts, double* out, int32_t* status, int64_t n,
                                 cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const double i0 = 1.0 / f.spacing[0], i1 = 1.0 / f.spacing[1], i2 = 1.0 / f.spacing[2];
  const double i3 = f.ndim == 4 ? 1.0 / f.spacing[3] : 0.0;
  if (f.dtype == EXC_DTYPE_F32)
    interp_kernel<float><<<blocks_for(n, 128), 128, 0, s>>>(f, i0, i1, i2, i3, pts, out, status, n);
  else
    interp_kernel<double><<<blocks_for(n, 128), 128, 0, s>>>(f, i0, i1, i2, i3, pts, out, status, n);
  return cudaGetLastError();
}

inline cudaError_t launch_cosmology(const DevMetric& D, const double* eta, double* a, double* adot, int64_t n,
                                    cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cosmology_kernel<<<blocks_for(n, 128), 128, 0, s>>>(D, eta, a, adot, n);
  return cudaGetLastError();
}

inline cudaError_t launch_metric(const DevMetric& D, const double* x, double* g, int32_t* status,
                                 const int32_t* fidx, int64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (D.m.kind == EXC_METRIC_FLRW && D.m.fields[0].dtype == EXC_DTYPE_F32)
    metric_kernel<float><<<blocks_for(n, 128), 128, 0, s>>>(D, x, g, status, fidx, n);
  else
    metric_kernel<double><<<blocks_for(n, 128), 128, 0, s>>>(D, x, g, status, fidx, n);
  return cudaGetLastError();
}

inline cudaError_t launch_null_init(const DevMetric& D, double* st, double sign, int32_t* status,
                                    const int32_t* fidx, int64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (D.m.kind == EXC_METRIC_FLRW && D.m.fields[0].dtype == EXC_DTYPE_F32)
    null_init_kernel<float><<<blocks_for(n, 128), 128, 0, s>>>(D, st, sign, status, fidx, n);
  else
    null_init_kernel<double><<<blocks_for(n, 128), 128, 0, s>>>(D, st, sign, status, fidx, n);
  return cudaGetLastError();
}

inline cudaError_t launch_null_error(const DevMetric& D, const double* st, double* rel, int32_t* status,
                                     const int32_t* fidx, int64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (D.m.kind == EXC_METRIC_FLRW && D.m.fields[0].dtype == EXC_DTYPE_F32)
    null_error_kernel<float><<<blocks_for(n, 128), 128, 0, s>>>(D, st, rel, status, fidx, n);
  else
    null_error_kernel<double><<<blocks_for(n, 128), 128, 0, s>>>(D, st, rel, status, fidx, n);
  return cudaGetLastError();
}

inline cudaError_t launch_fill_status(int32_t* status, int64_t n, int32_t v, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int g = blocks_for(n, 256);
  if (g > 4096) g = 4096;
  fill_status_kernel<<<g, 256, 0, s>>>(status, n, v);
  return cudaGetLastError();
}

}  // namespace EXC_NS
