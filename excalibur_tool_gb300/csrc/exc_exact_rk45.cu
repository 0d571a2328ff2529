// rk45 tracer kernels of the exact FP64 build (one stepper per unit so
// the heavily inlined kernels compile in parallel).
#define EXC_FAST 0
#define EXC_NS exc_exact
#include "exc_kernels.cuh"

namespace exc_exact {
cudaError_t trace_rk45(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s) {
  return launch_trace_stepper<EXC_STEPPER_RK45>(D, A, lc, s);
}
}  // namespace exc_exact
