// exc_noalloc.cu -- exc_trace_noalloc: the work-queue trace for callers that
// cannot allocate device memory.
//
// exc_trace balances uneven trajectory lengths with a device work-queue
// counter that the caller must supply as scratch (ExcTraceArgs.queue). Some
// callers cannot allocate even that: a host application that owns every
// device buffer and forbids allocation inside its processing loop, or a
// latency-bound loop where a cudaMalloc/cudaFree would stall on an implicit
// device synchronisation. For them this entry point keeps the counter in a
// small array compiled into the library: every GPU that loads the library
// holds EXC_NOALLOC_SCRATCH_BYTES of it until the process exits.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/excalibur_gb300.h"

namespace exc {
void set_last_error(const char* msg);   // exc_capi.cu
}

// The scratch itself. In host code this name is only a handle for
// cudaGetSymbolAddress, never a device address.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[EXC_NOALLOC_SCRATCH_BYTES / 8];

namespace {

// Bytes of scratch one trace launch uses: one 64-bit queue head.
constexpr size_t kQueueBytes = sizeof(unsigned long long);

std::mutex g_mu;

// The array's address, looked up once per device and per CUDA context: a caller that makes
// another context current on the same device (the array then lives at another address in it)
// gets a fresh lookup instead of a stale pointer.
struct Cached {
  void* ctx;
  void* addr;
};
Cached g_addr[EXC_NOALLOC_MAX_DEVICES] = {};

// cuCtxGetCurrent through the runtime's driver entry-point query, so that the library does
// not link the driver library itself (it loads on machines without one). NULL if unavailable:
// the cache is then keyed on the device alone.
typedef int (*CtxGetCurrentFn)(void**);
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

void* current_ctx() {
  void* ctx = nullptr;
  CtxGetCurrentFn fn = ctx_get_current();
  if (!fn || fn(&ctx) != 0) return nullptr;
  return ctx;
}

int reject(int code, const char* msg) {
  char buf[256];
  snprintf(buf, sizeof(buf), "exc_trace_noalloc: %s", msg);
  exc::set_last_error(buf);   // readable through exc_last_error()
  return code;
}

}  // namespace

extern "C" {

int exc_trace_noalloc(const ExcMetric* metric, const ExcTraceArgs* args, void* stream) {
  if (!args) return reject(EXC_ERR_INVALID, "args is NULL");
  if (args->queue)
    return reject(EXC_ERR_INVALID, "args->queue must be NULL: the library supplies the work-queue scratch");
  static_assert(kQueueBytes <= EXC_NOALLOC_SCRATCH_BYTES, "scratch array too small for the queue head");
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return reject(EXC_ERR_NO_DEVICE, "no current CUDA device");
  if (dev >= EXC_NOALLOC_MAX_DEVICES) return reject(EXC_ERR_INVALID, "device ordinal beyond EXC_NOALLOC_MAX_DEVICES");
  void* scratch = nullptr;
  {
    // One-time set-up per device (and per context), with that device current: look up the
    // array's device address (the first call on a device does this).
    std::lock_guard<std::mutex> lk(g_mu);
    void* ctx = current_ctx();
    Cached& c = g_addr[dev];
    if (!c.addr || !ctx || ctx != c.ctx) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) return reject(EXC_ERR_CUDA, cudaGetErrorString(e));
      c.addr = p;
      c.ctx = current_ctx();   // the lookup creates the device's primary context if need be
    }
    scratch = c.addr;
  }
  // exc_trace zeroes the queue head on the stream before the kernel starts,
  // so whatever the previous call left in the array does not matter.
  ExcTraceArgs a = *args;
  a.queue = static_cast<uint32_t*>(scratch);
  return exc_trace(metric, &a, stream);
}

}  // extern "C"
