// Mixed-precision tracer (FP32 RHS and interpolation, FP64 state).
#include "exc_mixed.h"

namespace exc_mixed {
int check(const exc::DevMetric&, const ExcTraceArgs&) { return 1; }
const char* why(int) { return "mixed precision tracer not built"; }
cudaError_t trace(const exc::DevMetric&, const ExcTraceArgs&, int, int, int, cudaStream_t) {
  return cudaErrorNotSupported;
}
}  // namespace exc_mixed
