// Batch evaluators and the trace dispatcher of the fast FP64 build.
#define EXC_FAST 1
#define EXC_NS exc_fast
#include "exc_aux.cuh"
#include "exc_dispatch.h"

namespace exc_fast {
#include "exc_dispatch_impl.inc"
}  // namespace exc_fast
