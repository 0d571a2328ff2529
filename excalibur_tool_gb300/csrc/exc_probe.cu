// exc_probe.cu -- FP64 pipe throughput probe (compiled with --fmad=false, like
// the parity units): multiply/add, IEEE division by a loop-invariant divisor,
// IEEE square root and fmod of an in-range operand, each as four independent
// dependency chains per thread over SMs x 1024 threads, timed with CUDA events.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>

#include "excalibur_gb300.h"
#include "exc_divrn.cuh"

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

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// div_rn(x, c, RN(1/c)) against the IEEE quotient x / c, bit for bit. Even samples: x with a
// random sign and significand and an exponent in 2^-200 .. 2^200. Odd samples: x = RN(c m)
// for m = y + ulp(y)/2 a rounding midpoint (one FMA), so that x / c falls next to a midpoint
// -- the quotients hardest to round.
__global__ void div_probe_kernel(const double* divs, int nd, int64_t n, uint64_t seed, unsigned long long* bad) {
  unsigned long long local = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double c = divs[i % nd];
    const double rc = 1.0 / c;
    const uint64_t h = mix64(seed ^ (uint64_t)i), h2 = mix64(h);
    const uint64_t expo = 823 + (h2 % 401);                     // biased exponent: 2^-200 .. 2^200
    double x = __longlong_as_double((long long)((h & 0x800FFFFFFFFFFFFFull) | (expo << 52)));
    if (i & 1) {
      const double y = fabs(x);
      const double half_ulp = __longlong_as_double((long long)((expo - 53) << 52));   // ulp(y) / 2
      x = fma(c, y, c * half_ulp);
    }
    const double a = x / c, b = div_rn(x, c, rc);
    if (__double_as_longlong(a) != __double_as_longlong(b)) ++local;
  }
  if (local) atomicAdd(bad, local);
}

}  // namespace

extern "C" {

int exc_probe_div_rn(const double* divisors, int32_t n_div, int64_t n_samples, uint64_t seed,
                     unsigned long long* mismatches, void* stream) {
  if (!divisors || !mismatches || n_div < 1 || n_samples < 1) {
    exc::set_last_error("exc_probe_div_rn: divisors, mismatches, n_div >= 1 and n_samples >= 1 required");
    return EXC_ERR_INVALID;
  }
  const int n = sm_count();
  if (n < 0) { exc::set_last_error("no CUDA device"); return EXC_ERR_NO_DEVICE; }
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t err = cudaMemsetAsync(mismatches, 0, sizeof(unsigned long long), s);
  if (err == cudaSuccess) {
    div_probe_kernel<<<n * 8, 256, 0, s>>>(divisors, n_div, n_samples, seed, mismatches);
    err = cudaGetLastError();
  }
  if (err != cudaSuccess) {
    exc::set_last_error(cudaGetErrorString(err));
    return EXC_ERR_CUDA;
  }
  return EXC_SUCCESS;
}

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
