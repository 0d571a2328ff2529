// lf4 tracer kernels of the fast FP64 build (one stepper per unit so
// the heavily inlined kernels compile in parallel).
#define EXC_FAST 1
#define EXC_NS exc_fast
#include "exc_kernels.cuh"

namespace exc_fast {
cudaError_t trace_lf4(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s) {
  return launch_trace_stepper<EXC_STEPPER_LEAPFROG4>(D, A, lc, s);
}
}  // namespace exc_fast
