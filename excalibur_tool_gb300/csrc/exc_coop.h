// exc_coop.h -- the mixed tracer's FP64 re-trace pass with eight lanes per ray (exc_coop.cu).
#pragma once
#include <cuda_runtime.h>
#include "exc_devmetric.h"

namespace exc_coop {
// Whether the eight-lane re-trace covers this launch (FLRW, RK4, 3-D base-node fields of one
// dtype, no records, renormalisation or ISW); otherwise the one-thread re-trace runs.
bool supports(const exc::DevMetric& D, const ExcTraceArgs& A);
// Traces every photon whose status is EXC_PH_RETRACE, from its initial state.
cudaError_t retrace(const exc::DevMetric& D, const ExcTraceArgs& A, int sm_count, cudaStream_t s);
}  // namespace exc_coop
