// exc_probe.cu -- FP64 pipe throughput probe (compiled with --fmad=false, like
// the parity units): multiply/add, IEEE division by a loop-invariant divisor,
// IEEE square root and fmod of an in-range operand, each as four independent
// dependency chains per thread over SMs x 1024 threads, timed with CUDA events.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>

#include "excalibur_gb300.h"

namespace exc {
void set_last_error(const char* msg);
}

namespace {

constexpr int kThreadsPerSm = 1024;
constexpr int kBlock = 256;
constexpr int kIters = 2048;

template <int OP>
__device__ __forceinline__ double op(double x, double b, double y) {
  if (OP == EXC_PROBE_ADDMUL) return x * y + b;          // two FP64 operations
  if (OP == EXC_PROBE_DIV) return x / b + y;             // division + add
  if (OP == EXC_PROBE_SQRT) return sqrt(x) + y;          // square root + add
  return fmod(x, b) + y;                                 // fmod + add (x stays in [0, b))
}

template <int OP>
__global__ void probe_kernel(double* out, double b, double y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double x0 = 0.25 + 1e-9 * (double)(i & 1023), x1 = x0 + 0.125, x2 = x0 + 0.0625, x3 = x0 + 0.03125;
#pragma unroll 4
  for (int k = 0; k < kIters; ++k) {
    x0 = op<OP>(x0, b, y);
    x1 = op<OP>(x1, b, y);
    x2 = op<OP>(x2, b, y);
    x3 = op<OP>(x3, b, y);
  }
  out[i] = x0 + x1 + x2 + x3;
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  return n;
}

template <int OP>
cudaError_t time_op(double* out, int64_t n, double b, double y, cudaStream_t s, double& rate) {
  cudaEvent_t e0, e1;
  cudaError_t err = cudaEventCreate(&e0);
  if (err != cudaSuccess) return err;
  if ((err = cudaEventCreate(&e1)) != cudaSuccess) { cudaEventDestroy(e0); return err; }
  const int grid = (int)(n / kBlock);
  float best = 1e30f;
  for (int rep = 0; rep < 4 && err == cudaSuccess; ++rep) {   // first repetition is the warm-up
    cudaEventRecord(e0, s);
    probe_kernel<OP><<<grid, kBlock, 0, s>>>(out, b, y);
    cudaEventRecord(e1, s);
    if ((err = cudaGetLastError()) != cudaSuccess) break;
    if ((err = cudaEventSynchronize(e1)) != cudaSuccess) break;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // operations of the probed kind per launch (ADDMUL counts both the multiply and the add)
  const double ops = (double)n * kIters * 4 * (OP == EXC_PROBE_ADDMUL ? 2 : 1);
  rate = ops / (best * 1e-3);
  return err;
}

}  // namespace

extern "C" {

int64_t exc_probe_scratch_len(void) {
  const int n = sm_count();
  return n > 0 ? (int64_t)n * kThreadsPerSm : -1;
}

int exc_probe_fp64_rates(double* scratch, int64_t n_scratch, double* rates_out, void* stream) {
  const int64_t need = exc_probe_scratch_len();
  if (need < 0) { exc::set_last_error("no CUDA device"); return EXC_ERR_NO_DEVICE; }
  if (!scratch || !rates_out || n_scratch < need) {
    exc::set_last_error("exc_probe_fp64_rates: scratch of exc_probe_scratch_len() doubles and rates_out[4] required");
    return EXC_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double r[EXC_PROBE_N] = {0, 0, 0, 0};
  // divisor and addend keep every chain finite and in range: x -> x / 3 + 0.5 stays in (0.25, 1)
  cudaError_t err = time_op<EXC_PROBE_ADDMUL>(scratch, need, 0.5, 0.4999999, s, r[EXC_PROBE_ADDMUL]);
  if (err == cudaSuccess) err = time_op<EXC_PROBE_DIV>(scratch, need, 3.0, 0.5, s, r[EXC_PROBE_DIV]);
  if (err == cudaSuccess) err = time_op<EXC_PROBE_SQRT>(scratch, need, 0.0, 0.25, s, r[EXC_PROBE_SQRT]);
  if (err == cudaSuccess) err = time_op<EXC_PROBE_FMOD>(scratch, need, 1.0, 0.3125, s, r[EXC_PROBE_FMOD]);
  if (err != cudaSuccess) {
    exc::set_last_error(cudaGetErrorString(err));
    return EXC_ERR_CUDA;
  }
  for (int k = 0; k < EXC_PROBE_N; ++k) rates_out[k] = r[k];
  return EXC_SUCCESS;
}

}  // extern "C"
