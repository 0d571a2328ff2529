// exc_mixed.h -- entry points of the mixed-precision tracer build.
#pragma once
#include <cuda_runtime.h>
#include "exc_devmetric.h"

namespace exc_mixed {
// 0 when the mixed tracer supports this launch, else a reason code for why().
int check(const exc::DevMetric& D, const ExcTraceArgs& A);
const char* why(int code);
cudaError_t trace(const exc::DevMetric& D, const ExcTraceArgs& A, int block, int blocks_per_sm, int sm_count,
                  cudaStream_t s);
}  // namespace exc_mixed
