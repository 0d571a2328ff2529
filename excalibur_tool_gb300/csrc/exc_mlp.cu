// exc_mlp.cu -- kernels of the sky-map surrogate (include/excalibur_mlp.h).
//
// The GEMM is a Blackwell tensor-core kernel: operand tiles are staged in
// shared memory in the UMMA canonical K-major layout (8-row x 16-byte core
// matrices, no swizzle), one elected thread issues tcgen05.mma (kind::f16,
// BF16 x BF16 -> FP32) into a 128 x N accumulator in tensor memory, the
// completion is signalled through tcgen05.commit on an mbarrier, and the four
// warps read their 32-lane slices back with tcgen05.ld for the fused
// epilogue. Shared-memory stages are double-buffered so that the loads of
// chunk k+1 overlap the MMAs of chunk k. Every wait is bounded; a timeout is
// counted in a device word the host can read (exc_mlp_error_count) and the
// kernel still releases its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/excalibur_gb300.h"
#include "../../include/excalibur_mlp.h"

namespace exc {
void set_last_error(const char* msg);
}

namespace exc_mlp {

__device__ unsigned int g_timeouts;

constexpr int kTileM = 128;
constexpr int kChunkK = 64;                      // K elements per shared-memory stage
constexpr int kStageA = kTileM * kChunkK * 2;    // 16 KB
constexpr int kStageB = 256 * kChunkK * 2;       // 32 KB (N <= 256)
constexpr int kStage = kStageA + kStageB;
constexpr int kStages = 2;
constexpr int kSmem = kStages * kStage;          // 96 KB: at most two CTAs per SM, 2 x 256 TMEM columns
constexpr uint32_t kTmemCols = 256;
constexpr long long kSpinLimit = 1ll << 24;      // try_wait polls before a wait is declared lost

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// UMMA shared-memory descriptor for a K-major operand without swizzle:
// start address, leading byte offset (between K-adjacent core matrices) and
// stride byte offset (between 8-row groups), all in 16-byte units; bits 46-47
// hold the descriptor version of the sm_100 family (1); layout type 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D format F32 (bits 4-5 = 1), A and B
// format BF16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; false when the limit was reached
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + __expf(-z)); }

// Stage one K chunk of A (128 rows from m0) and B (n rows) into the canonical
// K-major layout: element (r, k) at (r / 8) * 1024 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
__device__ __forceinline__ void load_stage(uint8_t* sA, uint8_t* sB, const __nv_bfloat16* A, const __nv_bfloat16* B,
                                           int64_t m0, int64_t m, int n, int k, int k0) {
  const int t = threadIdx.x;
  for (int v = t; v < kTileM * 8; v += blockDim.x) {
    const int r = v >> 3, kv = v & 7;
    uint4 val = make_uint4(0u, 0u, 0u, 0u);
    if (m0 + r < m) val = __ldg(reinterpret_cast<const uint4*>(A + (m0 + r) * (int64_t)k + k0 + kv * 8));
    *reinterpret_cast<uint4*>(sA + (r >> 3) * 1024 + kv * 128 + (r & 7) * 16) = val;
  }
  for (int v = t; v < n * 8; v += blockDim.x) {
    const int r = v >> 3, kv = v & 7;
    const uint4 val = __ldg(reinterpret_cast<const uint4*>(B + (int64_t)r * k + k0 + kv * 8));
    *reinterpret_cast<uint4*>(sB + (r >> 3) * 1024 + kv * 128 + (r & 7) * 16) = val;
  }
}

template <int EPI>
__global__ void __launch_bounds__(128, 1) gemm_kernel(const ExcGemm g) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bars[kStages];
  __shared__ uint32_t tmem_base;
  __shared__ int lost;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t m0 = (int64_t)blockIdx.x * kTileM;
  const int split = blockIdx.y, bidx = blockIdx.z;
  const int n = g.n, k = g.k;
  const __nv_bfloat16* A = reinterpret_cast<const __nv_bfloat16*>(g.a) + bidx * g.stride_a;
  const __nv_bfloat16* B = reinterpret_cast<const __nv_bfloat16*>(g.b) + bidx * g.stride_b;

  if (warp == 0) {
    tmem_alloc(&tmem_base, kTmemCols);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    lost = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  const int nch = k / kChunkK;
  const int splits = EPI == EXC_EPI_SPLITK ? gridDim.y : 1;
  const int c_begin = (int)((int64_t)nch * split / splits), c_end = (int)((int64_t)nch * (split + 1) / splits);
  const uint32_t idesc = idesc_bf16_f32(kTileM, n);
  uint32_t phase[kStages] = {0u, 0u};
  bool ok = true;

  for (int c = c_begin; c < c_end; ++c) {
    const int s = (c - c_begin) & 1;
    uint8_t* sA = smem + s * kStage;
    uint8_t* sB = sA + kStageA;
    // the MMAs that last read this stage (chunk c - 2) must be complete before it is overwritten
    if (c - c_begin >= kStages) {
      if (!mbar_wait(&bars[s], phase[s])) ok = false;
      phase[s] ^= 1u;
    }
    load_stage(sA, sB, A, B, m0, g.m, n, k, c * kChunkK);
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
#pragma unroll
      for (int j = 0; j < kChunkK / 16; ++j)
        umma_bf16(tmem, smem_desc(a0 + j * 256, 128, 1024), smem_desc(b0 + j * 256, 128, 1024), idesc,
                  (c > c_begin || j > 0) ? 1u : 0u);
      umma_commit(&bars[s]);
    }
  }
  // drain: the last commit of each used stage
  const int used = c_end - c_begin;
  for (int s = 0; s < kStages && s < used; ++s) {
    // stage s was last committed by chunk index (used-1) or (used-2) with matching parity
    if (!mbar_wait(&bars[s], phase[s])) ok = false;
  }
  if (!ok) atomicOr(&lost, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (lost) {
    if (threadIdx.x == 0) atomicAdd(&g_timeouts, 1u);
  } else {
    // epilogue: warp w owns TMEM lanes (rows) 32w .. 32w + 31
    const int r = warp * 32 + lane;
    const int64_t row = m0 + r;
    const bool live = row < g.m && used > 0;
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < n; c0 += 16) {
      float v[16];
      tmem_ld16(lane_addr + (uint32_t)c0, v);
      if (!live) continue;
      if (EPI == EXC_EPI_F32) {
        float* C = reinterpret_cast<float*>(g.c) + bidx * g.stride_c + row * n + c0;
#pragma unroll
        for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(C + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
      } else if (EPI == EXC_EPI_SPLITK) {
        float* C = reinterpret_cast<float*>(g.c) + ((int64_t)bidx * splits + split) * g.m * n + row * n + c0;
#pragma unroll
        for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(C + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
      } else if (EPI == EXC_EPI_BIAS_SILU) {
        const float* bias = g.bias + (int64_t)bidx * n + c0;
        __nv_bfloat16 zb[16], hb[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const float z = v[i] + __ldg(bias + i);
          zb[i] = __float2bfloat16_rn(z);
          const float zr = __bfloat162float(zb[i]);   // the value the backward pass will see
          hb[i] = __float2bfloat16_rn(zr * sigmoid(zr));
        }
        const int64_t off = bidx * g.stride_c + row * n + c0;
        if (g.c) {
          uint4* dst = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(g.c) + off);
          dst[0] = *reinterpret_cast<uint4*>(&zb[0]);
          dst[1] = *reinterpret_cast<uint4*>(&zb[8]);
        }
        if (g.c2) {
          uint4* dst = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(g.c2) + off);
          dst[0] = *reinterpret_cast<uint4*>(&hb[0]);
          dst[1] = *reinterpret_cast<uint4*>(&hb[8]);
        }
        if (g.ct) {
          __nv_bfloat16* T = reinterpret_cast<__nv_bfloat16*>(g.ct) + bidx * g.stride_ct + row;
#pragma unroll
          for (int i = 0; i < 16; ++i) T[(int64_t)(c0 + i) * g.ldt] = hb[i];
        }
      } else {  // EXC_EPI_DSILU
        const int64_t off = bidx * g.stride_c + row * n + c0;
        const __nv_bfloat16* Z = reinterpret_cast<const __nv_bfloat16*>(g.z_in) + off;
        __nv_bfloat16 db[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const float z = __bfloat162float(Z[i]);
          const float sg = sigmoid(z);
          db[i] = __float2bfloat16_rn(v[i] * (sg * (1.0f + z * (1.0f - sg))));
        }
        if (g.c) {
          uint4* dst = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(g.c) + off);
          dst[0] = *reinterpret_cast<uint4*>(&db[0]);
          dst[1] = *reinterpret_cast<uint4*>(&db[8]);
        }
        if (g.ct) {
          __nv_bfloat16* T = reinterpret_cast<__nv_bfloat16*>(g.ct) + bidx * g.stride_ct + row;
#pragma unroll
          for (int i = 0; i < 16; ++i) T[(int64_t)(c0 + i) * g.ldt] = db[i];
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

// ------------------------------------------------------------------ features
__global__ void features_kernel(const double* dirs, int64_t n, int64_t n_pad, int nf, double c0, double c1,
                                double s0, double s1, __nv_bfloat16* out) {
  const int64_t total = n_pad * nf;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = i / nf;
    const int kf = (int)(i - p * nf);
    __nv_bfloat16* o = out + p * 4 * nf;
    if (p >= n) {
      const __nv_bfloat16 z = __float2bfloat16_rn(0.0f);
      o[kf] = z; o[nf + kf] = z; o[2 * nf + kf] = z; o[3 * nf + kf] = z;
      continue;
    }
    // the features are stored in BF16 (8-bit significand): FP32 phases are ample
    const float u = (float)((dirs[2 * p] - c0) * s0), v = (float)((dirs[2 * p + 1] - c1) * s1);
    float su, cu, sv, cv;
    sincospif((float)(kf + 1) * u, &su, &cu);
    sincospif((float)(kf + 1) * v, &sv, &cv);
    o[kf] = __float2bfloat16_rn(su);
    o[nf + kf] = __float2bfloat16_rn(cu);
    o[2 * nf + kf] = __float2bfloat16_rn(sv);
    o[3 * nf + kf] = __float2bfloat16_rn(cv);
  }
}

// ---------------------------------------------------------------------- head
// One warp per row; lane l holds columns 8l .. 8l+7 of the 256-wide hidden row.
template <int NOUT>
__global__ void __launch_bounds__(256) head_kernel(const __nv_bfloat16* H, int64_t m, int n_members,
                                                   const float* W, const float* bias, float* Y, const float* T,
                                                   const __nv_bfloat16* Z, __nv_bfloat16* dH, __nv_bfloat16* dHt,
                                                   int64_t ldt, float* dW, float* db, float* loss) {
  constexpr int width = 256;
  __shared__ float sw[NOUT * width];
  __shared__ float sdw[NOUT * width];
  __shared__ float sdb[NOUT], sloss;
  const int e = blockIdx.y;
  const float* We = W + (int64_t)e * NOUT * width;
  for (int i = threadIdx.x; i < NOUT * width; i += blockDim.x) { sw[i] = We[i]; sdw[i] = 0.0f; }
  if (threadIdx.x < NOUT) sdb[threadIdx.x] = 0.0f;
  if (threadIdx.x == 0) sloss = 0.0f;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int64_t wid = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5);
  const int64_t nw = (int64_t)gridDim.x * wpb;
  float gw[NOUT][8];
  float gb[NOUT];
#pragma unroll
  for (int j = 0; j < NOUT; ++j) { gb[j] = 0.0f; for (int q = 0; q < 8; ++q) gw[j][q] = 0.0f; }
  float lsum = 0.0f;
  const float inv = 2.0f / ((float)m * (float)NOUT);
  for (int64_t row = wid; row < m; row += nw) {
    const int64_t off = ((int64_t)e * m + row) * width + lane * 8;
    const uint4 raw = *reinterpret_cast<const uint4*>(H + off);
    const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&raw);
    float h[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) h[q] = __bfloat162float(hb[q]);
    float y[NOUT];
#pragma unroll
    for (int j = 0; j < NOUT; ++j) {
      float acc = 0.0f;
#pragma unroll
      for (int q = 0; q < 8; ++q) acc = fmaf(h[q], sw[j * width + lane * 8 + q], acc);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      y[j] = acc + __ldg(bias + (int64_t)e * NOUT + j);
    }
    if (Y && lane < NOUT) {
#pragma unroll
      for (int j = 0; j < NOUT; ++j)
        if (lane == j) Y[((int64_t)e * m + row) * NOUT + j] = y[j];
    }
    if (!T) continue;
    float dy[NOUT];
#pragma unroll
    for (int j = 0; j < NOUT; ++j) {
      const float d = y[j] - __ldg(T + row * NOUT + j);
      lsum += lane == 0 ? d * d : 0.0f;
      dy[j] = inv * d;
      gb[j] += lane == 0 ? dy[j] : 0.0f;
    }
    float zf[8];
    if (Z) {
      const uint4 zr = *reinterpret_cast<const uint4*>(Z + off);
      const __nv_bfloat16* zb = reinterpret_cast<const __nv_bfloat16*>(&zr);
#pragma unroll
      for (int q = 0; q < 8; ++q) zf[q] = __bfloat162float(zb[q]);
    }
    __nv_bfloat16 out[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float g = 0.0f;
#pragma unroll
      for (int j = 0; j < NOUT; ++j) {
        g = fmaf(dy[j], sw[j * width + lane * 8 + q], g);
        gw[j][q] = fmaf(dy[j], h[q], gw[j][q]);
      }
      if (Z) {
        const float sg = sigmoid(zf[q]);
        g *= sg * (1.0f + zf[q] * (1.0f - sg));
      }
      out[q] = __float2bfloat16_rn(g);
    }
    if (dH) *reinterpret_cast<uint4*>(dH + off) = *reinterpret_cast<uint4*>(out);
    if (dHt) {
      __nv_bfloat16* Tt = dHt + (int64_t)e * width * ldt + row;
#pragma unroll
      for (int q = 0; q < 8; ++q) Tt[(int64_t)(lane * 8 + q) * ldt] = out[q];
    }
  }
  if (T) {
#pragma unroll
    for (int j = 0; j < NOUT; ++j) {
#pragma unroll
      for (int q = 0; q < 8; ++q) atomicAdd(&sdw[j * width + lane * 8 + q], gw[j][q]);
      if (lane == 0) atomicAdd(&sdb[j], gb[j]);
    }
    if (lane == 0) atomicAdd(&sloss, lsum);
    __syncthreads();
    for (int i = threadIdx.x; i < NOUT * width; i += blockDim.x) atomicAdd(dW + (int64_t)e * NOUT * width + i, sdw[i]);
    if (threadIdx.x < NOUT) atomicAdd(db + (int64_t)e * NOUT + threadIdx.x, sdb[threadIdx.x]);
    if (threadIdx.x == 0) atomicAdd(loss + e, sloss);
  }
}

__global__ void reduce_splits_kernel(const float* part, int nb, int splits, int64_t rc, float* out) {
  const int64_t total = (int64_t)nb * rc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / rc, j = i - b * rc;
    float s = 0.0f;
    for (int q = 0; q < splits; ++q) s += part[(b * splits + q) * rc + j];
    out[i] = s;
  }
}

__global__ void row_sums_kernel(const __nv_bfloat16* x, int64_t rows, int64_t m, int64_t ld, float* out) {
  __shared__ float red[32];
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    float s = 0.0f;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) s += __bfloat162float(x[r * ld + i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0) out[r] = s;
    }
    __syncthreads();
  }
}

__global__ void adam_kernel(float* p, const float* g, float* m1, float* m2, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2, __nv_bfloat16* pb, __nv_bfloat16* pt, int rows, int cols) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.0f - b1) * gi;
    const float v = b2 * m2[i] + (1.0f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = v;
    const float pi = p[i] - lr * (a * c1) / (sqrtf(v * c2) + eps);
    p[i] = pi;
    const __nv_bfloat16 bv = __float2bfloat16_rn(pi);
    if (pb) pb[i] = bv;
    if (pt) {
      const int64_t per = (int64_t)rows * cols;
      const int64_t e = i / per, w = i - e * per;
      const int r = (int)(w / cols), c = (int)(w - (int64_t)r * cols);
      pt[e * per + (int64_t)c * rows + r] = bv;
    }
  }
}

int grid_for(int64_t n, int block) {
  int64_t b = (n + block - 1) / block;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace exc_mlp

using namespace exc_mlp;

static int mlp_fail(int code, const char* msg) {
  exc::set_last_error(msg);
  return code;
}
static int mlp_cuda(cudaError_t e) {
  if (e == cudaSuccess) return EXC_SUCCESS;
  exc::set_last_error(cudaGetErrorString(e));
  return EXC_ERR_CUDA;
}
static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <int EPI>
static cudaError_t launch_gemm(const ExcGemm& g, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(gemm_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)((g.m + kTileM - 1) / kTileM), EPI == EXC_EPI_SPLITK ? (unsigned)g.k_splits : 1u,
            (unsigned)g.n_batch);
  gemm_kernel<EPI><<<grid, 128, kSmem, s>>>(g);
  return cudaGetLastError();
}

extern "C" {

int exc_gemm_bf16(const ExcGemm* g, void* stream) {
  if (!g) return mlp_fail(EXC_ERR_INVALID, "gemm: args NULL");
  if (g->m < 1 || g->n_batch < 1) return mlp_fail(EXC_ERR_INVALID, "gemm: m and n_batch must be >= 1");
  if (g->n < 16 || g->n > 256 || g->n % 16) return mlp_fail(EXC_ERR_INVALID, "gemm: n must be a multiple of 16 in [16, 256]");
  if (g->k < kChunkK || g->k % kChunkK) return mlp_fail(EXC_ERR_INVALID, "gemm: k must be a positive multiple of 64");
  if (!g->a || !g->b || !aligned16(g->a) || !aligned16(g->b))
    return mlp_fail(EXC_ERR_INVALID, "gemm: a and b must be 16-byte aligned device pointers");
  if ((g->stride_a % 8) || (g->stride_b % 8)) return mlp_fail(EXC_ERR_INVALID, "gemm: batch strides must keep 16-byte alignment");
  if (g->m > (int64_t)65535 * kTileM) return mlp_fail(EXC_ERR_INVALID, "gemm: m too large for one launch");
  if (g->n_batch > 65535) return mlp_fail(EXC_ERR_INVALID, "gemm: n_batch too large");
  if (g->n_batch > 1 && g->stride_c < g->m * g->n) return mlp_fail(EXC_ERR_INVALID, "gemm: stride_c < m*n");
  if (g->ct && (g->ldt < g->m || (g->n_batch > 1 && g->stride_ct < (int64_t)g->n * g->ldt)))
    return mlp_fail(EXC_ERR_INVALID, "gemm: ct needs ldt >= m and stride_ct >= n*ldt");
  if ((g->c && !aligned16(g->c)) || (g->c2 && !aligned16(g->c2)) || (g->stride_c % 8))
    return mlp_fail(EXC_ERR_INVALID, "gemm: outputs must be 16-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  switch (g->epilogue) {
    case EXC_EPI_F32:
      if (!g->c) return mlp_fail(EXC_ERR_INVALID, "gemm: c is required");
      return mlp_cuda(launch_gemm<EXC_EPI_F32>(*g, s));
    case EXC_EPI_BIAS_SILU:
      if (!g->bias || (!g->c && !g->c2 && !g->ct)) return mlp_fail(EXC_ERR_INVALID, "gemm: bias and an output are required");
      return mlp_cuda(launch_gemm<EXC_EPI_BIAS_SILU>(*g, s));
    case EXC_EPI_DSILU:
      if (!g->z_in || !aligned16(g->z_in) || (!g->c && !g->ct)) return mlp_fail(EXC_ERR_INVALID, "gemm: z_in and an output are required");
      return mlp_cuda(launch_gemm<EXC_EPI_DSILU>(*g, s));
    case EXC_EPI_SPLITK:
      if (!g->c || g->k_splits < 1 || g->k_splits > g->k / kChunkK || g->k_splits > 65535)
        return mlp_fail(EXC_ERR_INVALID, "gemm: split-K needs c and 1 <= k_splits <= k/64");
      return mlp_cuda(launch_gemm<EXC_EPI_SPLITK>(*g, s));
    default:
      return mlp_fail(EXC_ERR_INVALID, "gemm: unknown epilogue");
  }
}

int exc_mlp_features(const double* dirs, int64_t n, int64_t n_pad, int32_t n_freq, const double* center2,
                     const double* scale2, void* out_bf16, void* stream) {
  if (n < 0 || n_pad < n || n_freq < 1) return mlp_fail(EXC_ERR_INVALID, "features: need 0 <= n <= n_pad, n_freq >= 1");
  if (!center2 || !scale2) return mlp_fail(EXC_ERR_INVALID, "features: center and scale are required");
  if (n_pad == 0) return EXC_SUCCESS;
  if ((n && !dirs) || !out_bf16) return mlp_fail(EXC_ERR_INVALID, "features: dirs/out are required");
  const int64_t total = n_pad * n_freq;
  features_kernel<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(
      dirs, n, n_pad, n_freq, center2[0], center2[1], scale2[0], scale2[1], (__nv_bfloat16*)out_bf16);
  return mlp_cuda(cudaGetLastError());
}

int exc_mlp_head(const void* h, int64_t m, int32_t width, int32_t n_out, int32_t n_members, const float* w,
                 const float* b, float* y, const float* targets, const void* z, void* dh, void* dht, int64_t ldt,
                 float* dw, float* db, float* loss, void* stream) {
  if (width != 256) return mlp_fail(EXC_ERR_UNSUPPORTED, "head: width must be 256");
  if (n_out < 1 || n_out > 8) return mlp_fail(EXC_ERR_UNSUPPORTED, "head: n_out must be in [1, 8]");
  if (m < 1 || n_members < 1 || n_members > 65535 || !h || !w || !b || !aligned16(h))
    return mlp_fail(EXC_ERR_INVALID, "head: h, w, b required; m, n_members >= 1");
  if (targets && (!dw || !db || !loss)) return mlp_fail(EXC_ERR_INVALID, "head: training needs dw, db, loss");
  if ((z && !aligned16(z)) || (dh && !aligned16(dh)) || (dht && ldt < m))
    return mlp_fail(EXC_ERR_INVALID, "head: z/dh must be 16-byte aligned, ldt >= m");
  const int block = 256;
  int64_t blocks = (m + 7) / 8;
  if (blocks > 152 * 8) blocks = 152 * 8;
  dim3 grid((unsigned)blocks, (unsigned)n_members);
  cudaStream_t s = (cudaStream_t)stream;
  const __nv_bfloat16* H = (const __nv_bfloat16*)h;
#define EXC_HEAD(NO)                                                                                          \
  head_kernel<NO><<<grid, block, 0, s>>>(H, m, n_members, w, b, y, targets, (const __nv_bfloat16*)z,        \
                                         (__nv_bfloat16*)dh, (__nv_bfloat16*)dht, ldt, dw, db, loss)
  switch (n_out) {
    case 1: EXC_HEAD(1); break;
    case 2: EXC_HEAD(2); break;
    case 3: EXC_HEAD(3); break;
    case 4: EXC_HEAD(4); break;
    case 5: EXC_HEAD(5); break;
    case 6: EXC_HEAD(6); break;
    case 7: EXC_HEAD(7); break;
    default: EXC_HEAD(8); break;
  }
#undef EXC_HEAD
  return mlp_cuda(cudaGetLastError());
}

int exc_mlp_reduce_splits(const float* part, int32_t n_batch, int32_t splits, int64_t rows_x_cols, float* out,
                          void* stream) {
  if (!part || !out || n_batch < 1 || splits < 1 || rows_x_cols < 1) return mlp_fail(EXC_ERR_INVALID, "reduce: bad arguments");
  reduce_splits_kernel<<<grid_for((int64_t)n_batch * rows_x_cols, 256), 256, 0, (cudaStream_t)stream>>>(
      part, n_batch, splits, rows_x_cols, out);
  return mlp_cuda(cudaGetLastError());
}

int exc_mlp_row_sums(const void* x, int64_t rows, int64_t m, int64_t ld, float* out, void* stream) {
  if (!x || !out || rows < 1 || m < 1 || ld < m) return mlp_fail(EXC_ERR_INVALID, "row_sums: bad arguments");
  int64_t blocks = rows < 152 * 8 ? rows : 152 * 8;
  row_sums_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)x, rows, m, ld, out);
  return mlp_cuda(cudaGetLastError());
}

int exc_mlp_adam(float* p, const float* grad, float* m1, float* m2, int64_t n, float lr, float beta1, float beta2,
                 float eps, int32_t t, void* p_bf16, void* pt_bf16, int32_t rows, int32_t cols, void* stream) {
  if (!p || !grad || !m1 || !m2 || n < 1 || t < 1) return mlp_fail(EXC_ERR_INVALID, "adam: bad arguments");
  if (pt_bf16 && (rows < 1 || cols < 1 || n % ((int64_t)rows * cols)))
    return mlp_fail(EXC_ERR_INVALID, "adam: n must be a multiple of rows*cols for the transposed copy");
  const float c1 = 1.0f / (1.0f - powf(beta1, (float)t)), c2 = 1.0f / (1.0f - powf(beta2, (float)t));
  adam_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(p, grad, m1, m2, n, lr, beta1, beta2, eps, c1, c2,
                                                                 (__nv_bfloat16*)p_bf16, (__nv_bfloat16*)pt_bf16,
                                                                 rows, cols);
  return mlp_cuda(cudaGetLastError());
}

int exc_mlp_error_count(uint32_t* out) {
  if (!out) return mlp_fail(EXC_ERR_INVALID, "error_count: out is NULL");
  unsigned int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_timeouts, sizeof(v));
  if (e != cudaSuccess) return mlp_cuda(e);
  *out = v;
  return EXC_SUCCESS;
}

}  // extern "C"
