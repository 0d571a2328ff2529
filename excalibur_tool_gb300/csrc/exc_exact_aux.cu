// Batch evaluators and the trace dispatcher of the exact FP64 build.
#define EXC_FAST 0
#define EXC_NS exc_exact
#include "exc_aux.cuh"
#include "exc_dispatch.h"

namespace exc_exact {
#include "exc_dispatch_impl.inc"
}  // namespace exc_exact
