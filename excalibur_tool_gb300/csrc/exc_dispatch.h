// exc_dispatch.h -- per-build entry points the C ABI calls (one set per
// precision build: exc_exact, exc_fast).
#pragma once
#include <cuda_runtime.h>
#include "exc_devmetric.h"

#define EXC_DECLARE_DISPATCH(NS)                                                                    \
  namespace NS {                                                                                     \
  cudaError_t trace(const exc::DevMetric& D, const ExcTraceArgs& A, int block, int blocks_per_sm,   \
                    int sm_count, cudaStream_t s);                                                   \
  cudaError_t rhs(const exc::DevMetric& D, const double* st, double* out, int32_t* status,          \
                  const int32_t* fidx, int64_t n, cudaStream_t s);                                   \
  cudaError_t interp(const ExcField& f, const double* pts, double* out, int32_t* status, int64_t n,  \
                     cudaStream_t s);                                                                \
  cudaError_t cosmology(const exc::DevMetric& D, const double* eta, double* a, double* adot,        \
                        int64_t n, cudaStream_t s);                                                  \
  cudaError_t metric(const exc::DevMetric& D, const double* x, double* g, int32_t* status,          \
                     const int32_t* fidx, int64_t n, cudaStream_t s);                                \
  cudaError_t null_init(const exc::DevMetric& D, double* st, double sign, int32_t* status,          \
                        const int32_t* fidx, int64_t n, cudaStream_t s);                             \
  cudaError_t null_error(const exc::DevMetric& D, const double* st, double* rel, int32_t* status,   \
                         const int32_t* fidx, int64_t n, cudaStream_t s);                            \
  cudaError_t fill_status(int32_t* status, int64_t n, int32_t v, cudaStream_t s);                   \
  }

EXC_DECLARE_DISPATCH(exc_exact)
EXC_DECLARE_DISPATCH(exc_fast)
