// rk45 tracer kernels of the exact FP64 build for launches with a slow-Interpolator
// field (grad_mode EXC_GRAD_TRILINEAR); a unit of their own so that they compile
// in parallel with the base-node kernels.
#define EXC_FAST 0
#define EXC_NS exc_exact
#include "exc_kernels.cuh"

namespace exc_exact {
cudaError_t trace_rk45_slow(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s) {
  return launch_trace_slow<EXC_STEPPER_RK45>(D, A, lc, s);
}
}  // namespace exc_exact
