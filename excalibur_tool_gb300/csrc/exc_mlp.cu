// exc_mlp.cu -- kernels of the sky-map surrogate (include/excalibur_mlp.h).
//
// The GEMM is a Blackwell tensor-core kernel: one thread streams 64-wide K
// chunks of both operands into a ring of shared-memory stages with TMA
// (cp.async.bulk.tensor, 128-byte swizzle, completion counted in bytes on an
// mbarrier), a second thread issues tcgen05.mma (kind::f16, BF16 x BF16 -> FP32)
// into a 128 x N accumulator in tensor memory and frees each stage with
// tcgen05.commit, and the four warps read their 32-lane slices back with
// tcgen05.ld for the fused epilogue. Every wait is bounded; a timeout is
// counted in a device word the host can read (exc_mlp_error_count) and the
// kernel still releases its tensor memory.
#include <cuda.h>
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
constexpr uint32_t kTmemCols = 256;
constexpr long long kSpinLimit = 1ll << 24;      // try_wait polls before a wait is declared lost

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

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

// The sigmoid of the SiLU epilogues: 1 / (1 + 2^(-z log2 e)) from the hardware's approximate
// base-2 exponential and reciprocal (two special-function operations, four instructions; the
// conversions to BF16 around it are packed in pairs so that the special-function pipe keeps
// pace with the FMA pipe). Saturates to 0 and 1 without a branch: 2^(-z log2 e) overflows to
// +inf for z < -88 and the reciprocal of +inf is 0. Within ~1e-6 relative of the exact sigmoid;
// the outputs are rounded to BF16.
__device__ __forceinline__ float sigmoid(float z) {
  float t, r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(t) : "f"(z * -1.4426950408889634f));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + t));
  return r;
}

// Packed FP32 pairs (add/mul/fma .rn.f32x2: two IEEE single-precision operations in one
// instruction, the same values as the scalar ones) for the epilogues, which are bound by the
// number of instructions they issue.
__device__ __forceinline__ uint64_t f2pack(float a, float b) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2unpack(uint64_t r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 h) { return *reinterpret_cast<uint32_t*>(&h); }

// The BIAS_SILU epilogue of a pair of accumulator columns: z = acc + bias rounded to BF16
// (*zbits, the value the backward pass sees), returns SiLU(z) = z sigmoid(z) rounded to BF16 --
// per element exactly the operations of sigmoid() above, two columns an instruction.
__device__ __forceinline__ uint32_t silu_pair(float v0, float v1, float b0, float b1, uint32_t* zbits) {
  float s0, s1;
  f2unpack(add2(f2pack(v0, v1), f2pack(b0, b1)), s0, s1);
  const uint32_t zb = bf16x2_bits(__floats2bfloat162_rn(s0, s1));
  if (zbits) *zbits = zb;
  const uint64_t z = f2pack(__uint_as_float(zb << 16), __uint_as_float(zb & 0xffff0000u));
  float a0, a1, t0, t1, d0, d1, r0, r1, h0, h1;
  f2unpack(mul2(z, f2pack(-1.4426950408889634f, -1.4426950408889634f)), a0, a1);
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(t0) : "f"(a0));
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(t1) : "f"(a1));
  f2unpack(add2(f2pack(t0, t1), f2pack(1.0f, 1.0f)), d0, d1);
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(d0));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(d1));
  f2unpack(mul2(z, f2pack(r0, r1)), h0, h1);
  return bf16x2_bits(__floats2bfloat162_rn(h0, h1));
}

// TMA: one 3-D tile (x = K element, y = row, z = batch member) into shared memory,
// completion counted in bytes on an mbarrier. The tensor map lives in the kernel's
// parameter space (__grid_constant__); its generic address is what the
// instruction takes.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// UMMA shared-memory descriptor for a K-major operand in the 128-byte swizzled
// layout TMA writes (rows of 128 B = 64 BF16, 8-row atoms of 1024 B): stride byte
// offset 1024 B between 8-row groups, leading byte offset unused (16 B), descriptor
// version 1 (bits 46-47), layout type 2 = SWIZZLE_128B (bits 61-63). A K step of 16
// elements inside the 128-byte row advances the start address by 32 B; the stage
// base is 1024-byte aligned so the hardware swizzle lines up with TMA's.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Two K chunks in flight (96 KB of stages) so that two CTAs fit on an SM (and the
// two 256-column accumulators fill its TMEM): one CTA's epilogue overlaps the
// other's loads and MMAs.
constexpr int kTmaStages = 2;
constexpr int kTmaSmem = kTmaStages * kStage + 1024;  // + alignment slack
constexpr int kGemmCtasPerSm = 2;

// Fused epilogue, staged through shared memory, on all kGemmWarps warps, in
// blocks of up to 128 columns (the staging tiles then fit in the operand stages,
// which are free once the last MMA has completed). A warp can read only its
// quarter of the TMEM lanes (warp w: lanes 32 (w % 4) ..), so the four warps of a
// quarter split the 16-column chunks among them (chunk j to warp group j % 4).
// Pass 1: each thread reads its lane (tile row) chunk by chunk, applies the
// epilogue and writes the results into row-major tiles in shared memory. Pass 2:
// the warps copy the tiles out with coalesced stores -- whole output rows per
// warp instruction, and the transposed output one column (up to 128 consecutive
// rows of ct) per pass. Row pitch: 136 BF16 / 132 FP32 elements.
constexpr int kEpiCols = 128;
constexpr int kPitchH = kEpiCols + 8, kPitchF = kEpiCols + 4;
constexpr int kGemmWarps = 16;
static_assert(2 * kTileM * kPitchH * 2 <= kTmaStages * kStage, "BF16 staging tiles must fit the stages");
static_assert(kTileM * kPitchF * 4 <= kTmaStages * kStage, "FP32 staging tile must fit the stages");

template <int EPI>
__device__ __forceinline__ void epilogue(const ExcGemm& g, uint32_t tmem, int64_t m0, int split, int splits, int bidx,
                                         uint8_t* smem, const float* sbias) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = warp & 3, grp = warp >> 2;
  const int n = g.n;
  const int r = q * 32 + lane;
  const int64_t row = m0 + r;
  const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16);
  float* tf = reinterpret_cast<float*>(smem);                                   // FP32 tile
  __nv_bfloat16* t1 = reinterpret_cast<__nv_bfloat16*>(smem);                   // first BF16 tile
  __nv_bfloat16* t2 = t1 + kTileM * kPitchH;                                    // second BF16 tile
  const __nv_bfloat16* Z =
      EPI == EXC_EPI_DSILU ? reinterpret_cast<const __nv_bfloat16*>(g.z_in) + bidx * g.stride_c + row * n : nullptr;
  const int rows = (int)(g.m - m0 < kTileM ? g.m - m0 : kTileM);
  for (int cb = 0; cb < n; cb += kEpiCols) {
    const int cols = n - cb < kEpiCols ? n - cb : kEpiCols;
    if (cb) __syncthreads();   // the previous block's pass 2 has read the tiles
    // pass 1: columns cb + c0 .. cb + c0 + 15 of this thread's row
    for (int c0 = grp * 16; c0 < cols; c0 += 16 * (kGemmWarps / 4)) {
      float v[16];
      tmem_ld16(lane_addr + (uint32_t)(cb + c0), v);
      if (EPI == EXC_EPI_F32 || EPI == EXC_EPI_SPLITK) {
#pragma unroll
        for (int i = 0; i < 16; i += 4)
          *reinterpret_cast<float4*>(tf + r * kPitchF + c0 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
      } else if (EPI == EXC_EPI_BIAS_SILU) {
        const float* bias = sbias + cb + c0;
        // column pairs: one BF16 conversion and one packed FP32 operation per step for both
        __align__(16) uint32_t zb[8], hb[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) hb[i] = silu_pair(v[2 * i], v[2 * i + 1], bias[2 * i], bias[2 * i + 1], &zb[i]);
        if (g.c) {   // the pre-activation is staged only when it is an output (training)
          uint4* d1 = reinterpret_cast<uint4*>(t1 + r * kPitchH + c0);
          d1[0] = *reinterpret_cast<uint4*>(&zb[0]);
          d1[1] = *reinterpret_cast<uint4*>(&zb[4]);
        }
        uint4* d2 = reinterpret_cast<uint4*>(t2 + r * kPitchH + c0);
        d2[0] = *reinterpret_cast<uint4*>(&hb[0]);
        d2[1] = *reinterpret_cast<uint4*>(&hb[4]);
      } else {  // EXC_EPI_DSILU
        __align__(16) __nv_bfloat16 db[16];
        if (row < g.m) {
          __align__(16) __nv_bfloat16 zin[16];
          *reinterpret_cast<uint4*>(&zin[0]) = __ldg(reinterpret_cast<const uint4*>(Z + cb + c0));
          *reinterpret_cast<uint4*>(&zin[8]) = __ldg(reinterpret_cast<const uint4*>(Z + cb + c0 + 8));
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const float z = __bfloat162float(zin[i]);
            const float sg = sigmoid(z);
            db[i] = __float2bfloat16_rn(v[i] * (sg * (1.0f + z * (1.0f - sg))));
          }
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i) db[i] = __float2bfloat16_rn(0.0f);
        }
        uint4* d1 = reinterpret_cast<uint4*>(t1 + r * kPitchH + c0);
        d1[0] = *reinterpret_cast<uint4*>(&db[0]);
        d1[1] = *reinterpret_cast<uint4*>(&db[8]);
      }
    }
    __syncthreads();
    // pass 2: rows (coalesced)
    if (EPI == EXC_EPI_F32 || EPI == EXC_EPI_SPLITK) {
      float* C = reinterpret_cast<float*>(g.c) +
                 (EPI == EXC_EPI_SPLITK ? ((int64_t)bidx * splits + split) * g.m * n : bidx * g.stride_c) + cb;
      // one row (up to 128 FP32 = 512 B) per warp instruction
      for (int rr = warp; rr < rows; rr += kGemmWarps)
        for (int c = lane * 4; c < cols; c += 128)
          *reinterpret_cast<float4*>(C + (m0 + rr) * n + c) = *reinterpret_cast<const float4*>(tf + rr * kPitchF + c);
    } else {
      __nv_bfloat16* outs[2] = {reinterpret_cast<__nv_bfloat16*>(g.c), EPI == EXC_EPI_BIAS_SILU
                                                                          ? reinterpret_cast<__nv_bfloat16*>(g.c2)
                                                                          : nullptr};
      const __nv_bfloat16* tiles[2] = {t1, t2};
      // two rows (up to 128 BF16 = 256 B each) per warp instruction
      const int half = lane >> 4, l16 = lane & 15;
      for (int o = 0; o < 2; ++o) {
        if (!outs[o]) continue;
        __nv_bfloat16* C = outs[o] + bidx * g.stride_c + cb;
        for (int rr = 2 * warp + half; rr < rows; rr += 2 * kGemmWarps)
          for (int c = l16 * 8; c < cols; c += 128)
            *reinterpret_cast<uint4*>(C + (m0 + rr) * n + c) =
                *reinterpret_cast<const uint4*>(tiles[o] + rr * kPitchH + c);
      }
      if (g.ct) {
        // the transposed output: SiLU values (BIAS_SILU) or the masked gradient (DSILU)
        const __nv_bfloat16* src = EPI == EXC_EPI_BIAS_SILU ? t2 : t1;
        __nv_bfloat16* T = reinterpret_cast<__nv_bfloat16*>(g.ct) + bidx * g.stride_ct + (int64_t)cb * g.ldt + m0;
        for (int cc = warp; cc < cols; cc += kGemmWarps)
          for (int rr = lane; rr < rows; rr += 32) T[(int64_t)cc * g.ldt + rr] = src[rr * kPitchH + cc];
      }
    }
  }
}

// C tile [128 x n] of one batch member (blockIdx.z) and K range (blockIdx.y of
// split-K). Thread 0 produces: TMA loads of 64-wide K chunks of A and B into a
// ring of kTmaStages 128-byte-swizzled stages (full[s] counts the bytes); thread 32
// consumes: four tcgen05.mma per chunk into the TMEM accumulator and a commit to
// empty[s] that frees the stage; a final commit to `done` releases the epilogue.
template <int EPI>
__global__ void __launch_bounds__(kGemmWarps * 32, kGemmCtasPerSm) gemm_tma_kernel(const __grid_constant__ CUtensorMap tmA,
                                                                      const __grid_constant__ CUtensorMap tmB,
                                                                      const ExcGemm g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  __shared__ uint64_t full[kTmaStages], empty[kTmaStages], done;
  __shared__ uint32_t tmem_base;
  __shared__ int lost;
  __shared__ float sbias[256];
  const int warp = threadIdx.x >> 5;
  const int64_t m0 = (int64_t)blockIdx.x * kTileM;
  const int split = blockIdx.y, bidx = blockIdx.z;
  const int splits = EPI == EXC_EPI_SPLITK ? gridDim.y : 1;
  const int nch = g.k / kChunkK;
  const int c_begin = (int)((int64_t)nch * split / splits), c_end = (int)((int64_t)nch * (split + 1) / splits);
  const int used = c_end - c_begin;
  const uint32_t stage_bytes = (uint32_t)(kStageA + g.n * kChunkK * 2);
  const int za = g.stride_a ? bidx : 0, zb = g.stride_b ? bidx : 0;

  if (warp == 0) {
    tmem_alloc(&tmem_base, kTmemCols);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kTmaStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    lost = 0;
  }
  if (EPI == EXC_EPI_BIAS_SILU)
    for (int i = threadIdx.x; i < g.n; i += blockDim.x) sbias[i] = __ldg(g.bias + (int64_t)bidx * g.n + i);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (threadIdx.x == 0) {
    // producer
    for (int i = 0; i < used; ++i) {
      const int s = i % kTmaStages;
      if (i >= kTmaStages && !mbar_wait(&empty[s], (uint32_t)((i / kTmaStages - 1) & 1))) {
        atomicOr(&lost, 1);
        break;
      }
      uint8_t* sA = smem + s * kStage;
      uint8_t* sB = sA + kStageA;
      const int k0 = (c_begin + i) * kChunkK;
      mbar_expect_tx(&full[s], stage_bytes);
      tma_load_3d(sA, &tmA, k0, (int)m0, za, &full[s]);
      tma_load_3d(sB, &tmB, k0, 0, zb, &full[s]);
    }
  } else if (threadIdx.x == 32) {
    // MMA issuer
    const uint32_t idesc = idesc_bf16_f32(kTileM, g.n);
    bool ok = true;
    for (int i = 0; i < used && ok; ++i) {
      const int s = i % kTmaStages;
      if (!mbar_wait(&full[s], (uint32_t)((i / kTmaStages) & 1))) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t a0 = smem_u32(smem + s * kStage), b0 = a0 + kStageA;
#pragma unroll
      for (int j = 0; j < kChunkK / 16; ++j)
        umma_bf16(tmem, smem_desc_sw128(a0 + j * 32), smem_desc_sw128(b0 + j * 32), idesc, (i > 0 || j > 0) ? 1u : 0u);
      umma_commit(&empty[s]);
    }
    if (ok) umma_commit(&done);
    else atomicOr(&lost, 1);
  }
  // everyone waits for the accumulator (or for the bail-out flag)
  if (used > 0) {
    bool ready = false;
    for (long long t = 0; t < kSpinLimit && !ready; ++t) {
      ready = mbar_try_wait(&done, 0u);
      if (!ready && *(volatile int*)&lost) break;
    }
    if (!ready) atomicOr(&lost, 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (lost) {
    if (threadIdx.x == 0) atomicAdd(&g_timeouts, 1u);
  } else {
    epilogue<EPI>(g, tmem, m0, split, splits, bidx, smem, sbias);
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

// ------------------------------------------------------------ fused inference
// The ensemble's forward pass for prediction (exc_mlp_infer): one persistent CTA per SM. A
// 128-row tile of Fourier features is loaded once with TMA and stays in shared memory; for
// every member the hidden layers run on it back to back -- tcgen05.mma of the 128 x 256
// activations against the layer's 256 x 256 weights (64-wide K chunks streamed through a
// three-stage TMA ring) into one of two 256-column TMEM accumulators, then an epilogue that adds
// the bias, applies SiLU and rounds to BF16 exactly as the layer-by-layer kernel stores its
// outputs, and writes the result back into shared memory in the 128-byte-swizzled K-major layout
// that TMA would have produced (16-byte unit u of row r of a chunk at unit u ^ (r % 8)), where
// the next layer's MMAs read it. The last layer's epilogue forms the linear head in FP32 (packed
// FMA pairs) from the member's head weights, copied into activation chunk 3 once that layer's
// MMAs have read it. Activations never leave the SM: per row, HBM sees the 512 B of features and
// the outputs.
//
// Sixteen epilogue warps walk the accumulator K chunk by K chunk (warp w reads TMEM lanes
// 32 (w % 4) .. and, in chunk c, columns 64 c + 16 (w / 4) ..) and release each chunk of the next
// layer's A operand as soon as it is written, so that the next layer's MMAs, into the other
// accumulator, follow the epilogue chunk by chunk. Warp 16 lane 0 streams the weight chunks;
// warp 17 lane 0 issues the MMAs and loads each tile's features once the last member's
// first-layer MMAs of the previous tile have completed. Barriers besides the weight ring:
// `fbar` (features landed), `mdone[b]` (a layer's MMAs into accumulator b completed; the last K
// chunk's MMAs run in two column halves, and `mdone_lo[b]` lets the epilogue start on columns
// 0-127 while those of columns 128-255 finish),
// `hready[c]` (chunk c of a layer's activations written), `tfree[b]` (the epilogue is done with
// accumulator b), `wbar` (a member's head weights are in shared memory) and `ybar` (the head's
// partial sums of column quarters 1-3 are in shared memory). A layer's bias reaches the epilogue
// warps spread over their lanes a layer ahead and is shuffled to every lane. Every wait is
// bounded, as in the GEMM.
constexpr int kInferEpiWarps = 16;
constexpr int kInferThreads = (kInferEpiWarps + 2) * 32;
constexpr int kInferStages = 3;
constexpr int kActBytes = 4 * kStageA;                                      // 128 x 256 BF16 in 4 K chunks
constexpr int kInferSmem = 2 * kActBytes + kInferStages * kStageB + 1024;   // features, hidden, weight stages
constexpr uint32_t kInferTmemCols = 512;                                     // two 256-column accumulators
constexpr int kInferMaxOut = 8;
static_assert(kInferSmem + 256 <= 227 * 1024, "fused inference: shared memory per block");
static_assert(kInferMaxOut * 256 * 4 <= kStageA, "a member's head weights fit one activation chunk");

struct InferParams {
  const float* b;        // [depth][E][256]
  const float* w_head;   // [E][n_out][256]
  const float* b_head;   // [E][n_out]
  float* y;              // [E][m][n_out]
  int64_t m;
  int n_members, n_out, depth;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ int ld_shared_volatile(const int* p) {
  int v;
  asm volatile("ld.volatile.shared.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)));
  return v;
}
__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
__device__ __forceinline__ float4 ld_shared_f4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr)
               : "memory");
  return v;
}
// a bounded wait on an mbarrier phase, uniform across the warp (every lane leaves together, so
// the warp-aligned tcgen05.ld that follows runs on all 32 lanes); false when it gave up, or when
// another role gave up (the shared `lost` word, looked at every 16 polls)
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, const int* lost) {
  for (long long w = 0; w < kSpinLimit; ++w) {
    if (__all_sync(0xffffffffu, mbar_try_wait(bar, parity))) return true;
    if ((w & 15) == 15 && __any_sync(0xffffffffu, ld_shared_volatile(lost) != 0)) return false;
  }
  return false;
}
// 16 columns of this thread's TMEM lane: the load is issued, and waited for separately (the
// wait names the registers, so that nothing reads them before it)
__device__ __forceinline__ void tmem_ld16_issue(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}
// the lanes' shared-memory writes (and, with tcgen05.fence before it, their TMEM reads) ordered
// before one arrival for the warp
__device__ __forceinline__ void warp_arrive(uint64_t* bar, int lane) {
  __syncwarp();
  if (lane == 0) mbar_arrive(bar);
}

__global__ void __launch_bounds__(kInferThreads, 1) mlp_infer_kernel(const __grid_constant__ CUtensorMap tmX,
                                                                     const __grid_constant__ CUtensorMap tmW,
                                                                     const InferParams P) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint8_t* sF = smem;                    // features of the tile
  uint8_t* sH = smem + kActBytes;        // hidden activations (overwritten layer after layer)
  uint8_t* sW = smem + 2 * kActBytes;    // weight stages
  __shared__ uint64_t full[kInferStages], empty[kInferStages], fbar, mdone[2], mdone_lo[2], hready[4], tfree[2];
  __shared__ uint64_t ybar, wbar;
  __shared__ uint32_t tmem_base;
  __shared__ int lost;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n_tiles = (P.m + kTileM - 1) / kTileM;
  const int E = P.n_members, depth = P.depth;
  const int my_tiles = (int64_t)blockIdx.x < n_tiles ? (int)((n_tiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  if (warp == 0) {
    tmem_alloc(&tmem_base, kInferTmemCols);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kInferStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&fbar, 1);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&mdone[b], 1);
      mbar_init(&mdone_lo[b], 1);
      mbar_init(&tfree[b], kInferEpiWarps);
    }
    for (int c = 0; c < 4; ++c) mbar_init(&hready[c], kInferEpiWarps);
    mbar_init(&ybar, kInferEpiWarps - 4);
    mbar_init(&wbar, kInferEpiWarps);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    lost = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  volatile int* vlost = &lost;

  if (warp == kInferEpiWarps) {
    // weight producer: chunks in the order the issuer consumes them
    if (lane == 0) {
      int64_t i = 0;   // chunks issued
      for (int t = 0; t < my_tiles && !*vlost; ++t)
        for (int e = 0; e < E && !*vlost; ++e)
          for (int l = 0; l < depth && !*vlost; ++l)
            for (int kc = 0; kc < 4; ++kc) {
              const int s = (int)(i % kInferStages);
              if (i >= kInferStages && !mbar_wait(&empty[s], (uint32_t)((i / kInferStages - 1) & 1))) {
                atomicOr(&lost, 1);
                break;
              }
              mbar_expect_tx(&full[s], (uint32_t)kStageB);
              tma_load_3d(sW + s * kStageB, &tmW, kc * kChunkK, 0, l * E + e, &full[s]);
              ++i;
            }
      // before the CTA can end, the copies it issued have landed (bounded; immediate when the
      // issuer consumed them)
      for (int64_t j = i > kInferStages ? i - kInferStages : 0; j < i; ++j)
        mbar_wait(&full[j % kInferStages], (uint32_t)((j / kInferStages) & 1));
    }
  } else if (warp == kInferEpiWarps + 1) {
    // MMA issuer (and the features of each tile)
    if (lane == 0 && my_tiles > 0) {
      const uint32_t idesc = idesc_bf16_f32(kTileM, 256), idesc_half = idesc_bf16_f32(kTileM, 128);
      int f_issued = 0;
      auto load_features = [&](int t) {
        ++f_issued;
        const int64_t tile = (int64_t)blockIdx.x + (int64_t)t * gridDim.x;
        mbar_expect_tx(&fbar, (uint32_t)kActBytes);
        for (int kc = 0; kc < 4; ++kc) tma_load_3d(sF + kc * kStageA, &tmX, kc * kChunkK, (int)(tile * kTileM), 0, &fbar);
      };
      load_features(0);
      // i: weight chunks consumed; L: layers issued; nh: issued layers whose epilogue writes activations
      int64_t i = 0, L = 0, nh = 0;
      bool ok = true;
      for (int t = 0; t < my_tiles && ok; ++t) {
        if (!mbar_wait(&fbar, (uint32_t)(t & 1))) { ok = false; break; }
        for (int e = 0; e < E && ok; ++e)
          for (int l = 0; l < depth && ok; ++l, ++L) {
            const int b = (int)(L & 1);
            // accumulator b is free once the epilogue of layer L - 2 is done with it; with one layer
            // a member, the epilogue of layer L - 1 (its head) also finishes first, so that at most
            // one head's partial sums are in shared memory
            if (L >= 2 && !mbar_wait(&tfree[b], (uint32_t)(((L >> 1) - 1) & 1))) { ok = false; break; }
            if (depth == 1 && L >= 1 && !mbar_wait(&tfree[b ^ 1], (uint32_t)(((L - 1) >> 1) & 1))) { ok = false; break; }
            const uint8_t* A = l == 0 ? sF : sH;
            const uint32_t d = tmem + (uint32_t)(b * 256);
            for (int kc = 0; kc < 4; ++kc, ++i) {
              // chunk kc of the previous layer's activations is in place
              if (l > 0 && !mbar_wait(&hready[kc], (uint32_t)((nh - 1) & 1))) { ok = false; break; }
              const int s = (int)(i % kInferStages);
              if (!mbar_wait(&full[s], (uint32_t)((i / kInferStages) & 1))) { ok = false; break; }
              tc_fence_after();
              const uint32_t a0 = smem_u32(A + kc * kStageA), b0 = smem_u32(sW + s * kStageB);
              if (kc < 3) {
#pragma unroll
                for (int j = 0; j < kChunkK / 16; ++j)
                  umma_bf16(d, smem_desc_sw128(a0 + j * 32), smem_desc_sw128(b0 + j * 32), idesc,
                            (kc > 0 || j > 0) ? 1u : 0u);
              } else {
                // the last K chunk by column halves (B rows 128-255 start 128 x 128 B into the stage)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
#pragma unroll
                  for (int j = 0; j < kChunkK / 16; ++j)
                    umma_bf16(d + (uint32_t)(h * 128), smem_desc_sw128(a0 + j * 32),
                              smem_desc_sw128(b0 + (uint32_t)(h * 128 * 128) + j * 32), idesc_half, 1u);
                  if (h == 0) umma_commit(&mdone_lo[b]);
                }
              }
              umma_commit(&empty[s]);
            }
            if (!ok) break;
            umma_commit(&mdone[b]);
            if (l < depth - 1) ++nh;
            if (e == E - 1 && l == 0 && t + 1 < my_tiles) {
              // the features buffer is free once these MMAs, its last readers, have completed
              if (!mbar_wait(&mdone[b], (uint32_t)((L >> 1) & 1))) { ok = false; break; }
              load_features(t + 1);
            }
          }
      }
      if (!ok) {
        atomicOr(&lost, 1);
        // a features load still in flight lands before the CTA ends (bounded)
        mbar_wait(&fbar, (uint32_t)(f_issued - 1) & 1u);
      }
    }
  } else {
    // epilogue: lane r of TMEM quarter q is tile row r; this warp's 16 columns of every K chunk
    const int q = warp & 3, sub = warp >> 2;
    const int r = q * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(sub * 16);
    // this warp's two 16-byte units of row r in a K chunk of the activations (swizzled)
    const int u0 = ((2 * sub) ^ (r & 7)) << 4, u1 = ((2 * sub + 1) ^ (r & 7)) << 4;
    // the head's partial sums of column quarter p (1-3) for row r: units 0 and 1 of row r in chunk
    // p - 1 of the activations, which only the quarter-0 thread of row r writes (and reads back)
    const int y0 = (0 ^ (r & 7)) << 4, y1 = (1 ^ (r & 7)) << 4;
    const int n_out = P.n_out;
    const uint32_t sH_u32 = smem_u32(sH);
    const uint32_t sWh_u32 = sH_u32 + 3 * kStageA;   // a member's head weights during its last layer
    int64_t L = 0, heads = 0;
    bool ok = true;
    // The 64 bias values a warp needs in a layer (16 columns of each K chunk) are spread over its
    // lanes, two a lane (lane j: chunk j / 8, columns 2 (j % 8) and 2 (j % 8) + 1 of the warp's
    // 16), loaded a whole layer ahead -- an L2 round trip (the shared-memory carve-out leaves L1
    // small and the line was last read a tile ago) -- and handed to every lane with a shuffle
    // when a chunk needs them.
    const int bofs = (lane >> 3) * 64 + sub * 16 + 2 * (lane & 7);
    float2 bcur = __ldg(reinterpret_cast<const float2*>(P.b + bofs));
    for (int t = 0; t < my_tiles && ok; ++t) {
      const int64_t row = ((int64_t)blockIdx.x + (int64_t)t * gridDim.x) * kTileM + r;
      for (int e = 0; e < E && ok; ++e)
        for (int l = 0; l < depth; ++l, ++L) {
          const int b = (int)(L & 1);
          const int ln = l + 1 < depth ? l + 1 : 0;
          const int en = l + 1 < depth ? e : (e + 1 < E ? e + 1 : 0);
          const float2 bnext = __ldg(reinterpret_cast<const float2*>(P.b + ((int64_t)ln * E + en) * 256 + bofs));
          // columns 0-127 first; the rest (mdone) before chunk 2
          if (!warp_wait(&mdone_lo[b], (uint32_t)((L >> 1) & 1), &lost)) { ok = false; break; }
          tc_fence_after();
          const bool last = l == depth - 1;
          if (last) {
            // the copy below overwrites chunk 3 of the activations, which the second half of the
            // last K chunk's MMAs reads: all of this layer's MMAs complete first
            if (!warp_wait(&mdone[b], (uint32_t)((L >> 1) & 1), &lost)) { ok = false; break; }
            tc_fence_after();
            // the member's head weights go to chunk 3 of the activation buffer, whose last reader
            // (this layer's MMAs) has completed; with one layer a member the previous head, which
            // read them there, is finished first
            if (depth == 1 && L > 0 && !warp_wait(&tfree[b ^ 1], (uint32_t)(((L - 1) >> 1) & 1), &lost)) {
              ok = false;
              break;
            }
            const float4* src = reinterpret_cast<const float4*>(P.w_head + (int64_t)e * n_out * 256);
            for (int i = threadIdx.x; i < n_out * 64; i += kInferEpiWarps * 32) {
              const float4 w4 = __ldg(src + i);
              st_shared_v4(sWh_u32 + (uint32_t)(i * 16), __float_as_uint(w4.x), __float_as_uint(w4.y),
                           __float_as_uint(w4.z), __float_as_uint(w4.w));
            }
            warp_arrive(&wbar, lane);
            if (!warp_wait(&wbar, (uint32_t)(heads & 1), &lost)) { ok = false; break; }
          } else if (l == 0 && L > 0) {
            // chunk 3 still holds the previous member's head weights until every warp has finished
            // that head (the previous layer released its accumulator)
            if (!warp_wait(&tfree[b ^ 1], (uint32_t)(((L - 1) >> 1) & 1), &lost)) { ok = false; break; }
          }
          const uint32_t tl = taddr + (uint32_t)(b * 256);
          uint64_t yacc2[kInferMaxOut];   // the head's sums over this warp's even and odd columns
#pragma unroll
          for (int j = 0; j < kInferMaxOut; ++j) yacc2[j] = 0;
#pragma unroll
          for (int kc = 0; kc < 4; ++kc) {
            if (kc == 2 && !last) {
              if (!warp_wait(&mdone[b], (uint32_t)((L >> 1) & 1), &lost)) { ok = false; break; }
              tc_fence_after();
            }
            float bv[16];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              bv[2 * k] = __shfl_sync(0xffffffffu, bcur.x, kc * 8 + k);
              bv[2 * k + 1] = __shfl_sync(0xffffffffu, bcur.y, kc * 8 + k);
            }
            uint32_t v[16];
            tmem_ld16_issue(tl + (uint32_t)(kc * 64), v);
            tmem_ld_wait(v);
            uint32_t hp[8];
#pragma unroll
            for (int k = 0; k < 8; ++k)
              hp[k] = silu_pair(__uint_as_float(v[2 * k]), __uint_as_float(v[2 * k + 1]), bv[2 * k], bv[2 * k + 1],
                                nullptr);
            if (!last) {
              const uint32_t rowp = sH_u32 + (uint32_t)(kc * kStageA + r * 128);
              st_shared_v4(rowp + u0, hp[0], hp[1], hp[2], hp[3]);
              st_shared_v4(rowp + u1, hp[4], hp[5], hp[6], hp[7]);
              fence_proxy_async_smem();   // the generic stores, visible to the tensor core's reads
              warp_arrive(&hready[kc], lane);
            } else {
              uint64_t h2[8];
#pragma unroll
              for (int k = 0; k < 8; ++k)
                h2[k] = f2pack(__uint_as_float(hp[k] << 16), __uint_as_float(hp[k] & 0xffff0000u));
#pragma unroll
              for (int j = 0; j < kInferMaxOut; ++j) {
                if (j >= n_out) break;
#pragma unroll
                for (int k = 0; k < 8; k += 2) {
                  const float4 w4 = ld_shared_f4(sWh_u32 + (uint32_t)((j * 256 + kc * 64 + sub * 16 + 2 * k) * 4));
                  yacc2[j] = fma2(h2[k], f2pack(w4.x, w4.y), yacc2[j]);
                  yacc2[j] = fma2(h2[k + 1], f2pack(w4.z, w4.w), yacc2[j]);
                }
              }
            }
          }
          if (!ok) break;
          bcur = bnext;
          if (last) {
            float yacc[kInferMaxOut];
#pragma unroll
            for (int j = 0; j < kInferMaxOut; ++j) {
              float lo, hi;
              f2unpack(yacc2[j], lo, hi);
              yacc[j] = lo + hi;
            }
            // column quarters 1-3 hand their partial sums to quarter 0 through shared memory (the
            // activations' units that only quarter 0 writes; the last layer's MMAs, their readers,
            // have completed)
            if (sub > 0) {
              const uint32_t yp = sH_u32 + (uint32_t)((sub - 1) * kStageA + r * 128);
              st_shared_v4(yp + y0, __float_as_uint(yacc[0]), __float_as_uint(yacc[1]), __float_as_uint(yacc[2]),
                           __float_as_uint(yacc[3]));
              st_shared_v4(yp + y1, __float_as_uint(yacc[4]), __float_as_uint(yacc[5]), __float_as_uint(yacc[6]),
                           __float_as_uint(yacc[7]));
              warp_arrive(&ybar, lane);
            } else {
              if (!warp_wait(&ybar, (uint32_t)(heads & 1), &lost)) { ok = false; break; }
              float ys[kInferMaxOut];
#pragma unroll
              for (int j = 0; j < kInferMaxOut; ++j) ys[j] = yacc[j];
#pragma unroll
              for (int p = 0; p < 3; ++p) {
                const uint32_t yp = sH_u32 + (uint32_t)(p * kStageA + r * 128);
                const float4 a4 = ld_shared_f4(yp + y0);
                const float4 c4 = ld_shared_f4(yp + y1);
                ys[0] += a4.x; ys[1] += a4.y; ys[2] += a4.z; ys[3] += a4.w;
                ys[4] += c4.x; ys[5] += c4.y; ys[6] += c4.z; ys[7] += c4.w;
              }
              if (row < P.m) {
#pragma unroll
                for (int j = 0; j < kInferMaxOut; ++j)
                  if (j < n_out) P.y[((int64_t)e * P.m + row) * n_out + j] = ys[j] + __ldg(P.b_head + e * n_out + j);
              }
            }
            ++heads;
          }
          tc_fence_before();
          warp_arrive(&tfree[b], lane);
        }
    }
    if (!ok) atomicOr(&lost, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (lost && threadIdx.x == 0) atomicAdd(&g_timeouts, 1u);
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, kInferTmemCols);
  }
}

// ---------------------------------------------------------------------- head
// A block walks tiles of kHeadRows consecutive rows; in a tile each warp takes kHeadRows / 8
// rows, one at a time, lane l holding columns 8l .. 8l+7 of the 256-wide hidden row. The
// transposed output dHt is staged in shared memory and written column by column, a warp
// storing 64 consecutive rows of one column as bf16 pairs (128 contiguous bytes), instead of
// every lane scattering eight 2-byte stores one matrix row apart.
constexpr int kHeadRows = 64;
constexpr int kHeadStride = 258;   // bf16 per staged row: 129 words, odd, so column reads do not conflict

// Two blocks per SM (at most 128 registers a thread): the grid of a training step is about two
// blocks per SM, and one block a SM would leave eight warps to hide every load.
template <int NOUT>
__global__ void __launch_bounds__(256, 2) head_kernel(const __nv_bfloat16* H, int64_t m, int n_members,
                                                      const float* W, const float* bias, float* Y, const float* T,
                                                      const __nv_bfloat16* Z, __nv_bfloat16* dH, __nv_bfloat16* dHt,
                                                      int64_t ldt, float* dW, float* db, float* loss) {
  constexpr int width = 256;
  static_assert(NOUT * width * 2 <= kHeadRows * kHeadStride, "sdw must fit in the staging tile");
  __shared__ float sw[NOUT * width];
  __shared__ float sdb[NOUT], sloss;
  // the staging tile of dHt during the row loop; afterwards the block's weight-gradient sums
  __shared__ __align__(16) __nv_bfloat16 tile[kHeadRows * kHeadStride];
  float* sdw = reinterpret_cast<float*>(tile);
  const int e = blockIdx.y;
  const float* We = W + (int64_t)e * NOUT * width;
  for (int i = threadIdx.x; i < NOUT * width; i += blockDim.x) sw[i] = We[i];
  if (threadIdx.x < NOUT) sdb[threadIdx.x] = 0.0f;
  if (threadIdx.x == 0) sloss = 0.0f;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int rows_per_warp = kHeadRows / 8;
  float gw[NOUT][8];
  float gb[NOUT];
#pragma unroll
  for (int j = 0; j < NOUT; ++j) { gb[j] = 0.0f; for (int q = 0; q < 8; ++q) gw[j][q] = 0.0f; }
  float lsum = 0.0f;
  const float inv = 2.0f / ((float)m * (float)NOUT);
  const int64_t n_tiles = (m + kHeadRows - 1) / kHeadRows;
  for (int64_t tile_i = blockIdx.x; tile_i < n_tiles; tile_i += gridDim.x) {
    const int64_t r0 = tile_i * kHeadRows;
    for (int k = 0; k < rows_per_warp; ++k) {
      const int jr = warp * rows_per_warp + k;
      const int64_t row = r0 + jr;
      if (row >= m) break;
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
#pragma unroll
        for (int q = 0; q < 8; ++q) tile[jr * kHeadStride + lane * 8 + q] = out[q];
      }
    }
    if (dHt) {
      // tile[jr][c] -> dHt[e][c][r0 + jr]: warp w writes columns w, w + 8, ...; lane l the rows
      // 2l and 2l + 1 as one bf16 pair (ldt is even, r0 a multiple of 64: 4-byte aligned)
      __syncthreads();
      const int64_t rows_here = (m - r0) < kHeadRows ? (m - r0) : kHeadRows;
      const int ja = 2 * lane, jb = 2 * lane + 1;
      for (int c = warp; c < width; c += 8) {
        __nv_bfloat16* dst = dHt + ((int64_t)e * width + c) * ldt + r0;
        if (jb < rows_here) {
          __nv_bfloat162 v;
          v.x = tile[ja * kHeadStride + c];
          v.y = tile[jb * kHeadStride + c];
          *reinterpret_cast<__nv_bfloat162*>(dst + ja) = v;
        } else if (ja < rows_here) {
          dst[ja] = tile[ja * kHeadStride + c];
        }
      }
      __syncthreads();   // the tile is rewritten by the next one
    }
  }
  if (T) {
    __syncthreads();   // every warp is done with the staging tile
    for (int i = threadIdx.x; i < NOUT * width; i += blockDim.x) sdw[i] = 0.0f;
    __syncthreads();
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

struct AdamMulti {
  ExcAdamTensor t[EXC_ADAM_MAX_TENSORS];
};

// blockIdx.y selects the tensor; the schedule {lr, c1, c2} is read once per thread.
__global__ void adam_multi_kernel(const AdamMulti P, const float* sched, float b1, float b2, float eps) {
  const ExcAdamTensor& T = P.t[blockIdx.y];
  const float lr = sched[0], c1 = sched[1], c2 = sched[2];
  __nv_bfloat16* pb = (__nv_bfloat16*)T.p_bf16;
  __nv_bfloat16* pt = (__nv_bfloat16*)T.pt_bf16;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < T.n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = T.grad[i];
    const float a = b1 * T.m1[i] + (1.0f - b1) * gi;
    const float v = b2 * T.m2[i] + (1.0f - b2) * gi * gi;
    T.m1[i] = a;
    T.m2[i] = v;
    const float pi = T.p[i] - lr * (a * c1) / (sqrtf(v * c2) + eps);
    T.p[i] = pi;
    const __nv_bfloat16 bv = __float2bfloat16_rn(pi);
    if (pb) pb[i] = bv;
    if (pt) {
      const int64_t per = (int64_t)T.rows * T.cols;
      const int64_t e = i / per, w = i - e * per;
      const int r = (int)(w / T.cols), c = (int)(w - (int64_t)r * T.cols);
      pt[e * per + (int64_t)c * T.rows + r] = bv;
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

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// [batch][rows][K] BF16 (batch stride 0 = one matrix shared by every member) as a
// 3-D tensor map with 64 x box_rows x 1 boxes, 128-byte swizzle, zero fill.
static bool make_map(CUtensorMap* map, const void* base, int64_t rows, int k, int64_t batch_stride, int batch,
                     int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const int nb = batch_stride ? batch : 1;
  const cuuint64_t dims[3] = {(cuuint64_t)k, (cuuint64_t)rows, (cuuint64_t)nb};
  const cuuint64_t strides[2] = {(cuuint64_t)k * 2, (cuuint64_t)(batch_stride ? batch_stride : rows * (int64_t)k) * 2};
  const cuuint32_t box[3] = {(cuuint32_t)kChunkK, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int EPI>
static cudaError_t launch_gemm(const ExcGemm& g, cudaStream_t s) {
  CUtensorMap ta, tb;
  if (!make_map(&ta, g.a, g.m, g.k, g.stride_a, g.n_batch, kTileM) ||
      !make_map(&tb, g.b, g.n, g.k, g.stride_b, g.n_batch, g.n))
    return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(gemm_tma_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmaSmem);
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)((g.m + kTileM - 1) / kTileM), EPI == EXC_EPI_SPLITK ? (unsigned)g.k_splits : 1u,
            (unsigned)g.n_batch);
  gemm_tma_kernel<EPI><<<grid, kGemmWarps * 32, kTmaSmem, s>>>(ta, tb, g);
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
  if (dht && (ldt & 1)) return mlp_fail(EXC_ERR_INVALID, "head: ldt must be even");
  const int block = 256;
  const int64_t n_tiles = (m + kHeadRows - 1) / kHeadRows;
  int64_t blocks = n_tiles;
  if (targets) {
    // Training: each block adds its partial weight and bias gradients (NOUT x 257 floats) into
    // dw/db with one global atomic per entry, all blocks of a member on the same few addresses,
    // so the block count sets that serialised atomic traffic. About two blocks per SM over all
    // members keep the row loads in flight; the tiles are then shared out evenly.
    const int64_t per_member = (2 * 152 + n_members - 1) / n_members;
    const int64_t cap = per_member < 16 ? 16 : per_member;
    if (blocks > cap) {
      const int64_t tiles_per_block = (n_tiles + cap - 1) / cap;
      blocks = (n_tiles + tiles_per_block - 1) / tiles_per_block;
    }
  }
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

int exc_mlp_adam_multi(const ExcAdamTensor* tensors, int32_t n_tensors, const float* sched, float beta1,
                       float beta2, float eps, void* stream) {
  if (!tensors || !sched || n_tensors < 1 || n_tensors > EXC_ADAM_MAX_TENSORS)
    return mlp_fail(EXC_ERR_INVALID, "adam_multi: 1..EXC_ADAM_MAX_TENSORS tensors and a schedule are required");
  AdamMulti P;
  int64_t nmax = 0;
  for (int k = 0; k < n_tensors; ++k) {
    const ExcAdamTensor& T = tensors[k];
    if (!T.p || !T.grad || !T.m1 || !T.m2 || T.n < 1)
      return mlp_fail(EXC_ERR_INVALID, "adam_multi: every tensor needs p, grad, m1, m2 and n >= 1");
    if (T.pt_bf16 && (T.rows < 1 || T.cols < 1 || T.n % ((int64_t)T.rows * T.cols)))
      return mlp_fail(EXC_ERR_INVALID, "adam_multi: n must be a multiple of rows*cols for a transposed copy");
    P.t[k] = T;
    if (T.n > nmax) nmax = T.n;
  }
  int64_t bx = (nmax + 255) / 256;
  const int64_t cap = (152 * 16 + n_tensors - 1) / n_tensors;
  if (bx > cap) bx = cap;
  dim3 grid((unsigned)(bx < 1 ? 1 : bx), (unsigned)n_tensors);
  adam_multi_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(P, sched, beta1, beta2, eps);
  return mlp_cuda(cudaGetLastError());
}

int exc_mlp_infer(const ExcMlpInfer* a, void* stream) {
  if (!a) return mlp_fail(EXC_ERR_INVALID, "infer: args NULL");
  if (a->m < 1 || a->m % kTileM) return mlp_fail(EXC_ERR_INVALID, "infer: m must be a positive multiple of 128");
  if (a->width != 256) return mlp_fail(EXC_ERR_INVALID, "infer: width must be 256");
  if (a->n_members < 1 || a->depth < 1 || (int64_t)a->depth * a->n_members > 65535)
    return mlp_fail(EXC_ERR_INVALID, "infer: n_members and depth must be >= 1");
  if (a->n_out < 1 || a->n_out > kInferMaxOut) return mlp_fail(EXC_ERR_INVALID, "infer: n_out must be in [1, 8]");
  if (!a->x || !a->w || !a->b || !a->w_head || !a->b_head || !a->y || !aligned16(a->x) || !aligned16(a->w) ||
      !aligned16(a->w_head) || ((uintptr_t)a->b & 7u))
    return mlp_fail(EXC_ERR_INVALID,
                    "infer: x, w, w_head (16-byte aligned), b (8-byte aligned), b_head and y are required");
  if (a->m > (int64_t)INT32_MAX - kTileM) return mlp_fail(EXC_ERR_INVALID, "infer: m too large for one launch");
  CUtensorMap tx, tw;
  if (!make_map(&tx, a->x, a->m, 256, 0, 1, kTileM) ||
      !make_map(&tw, a->w, 256, 256, (int64_t)256 * 256, a->depth * a->n_members, 256))
    return mlp_fail(EXC_ERR_CUDA, "infer: tensor map encoding failed");
  cudaError_t e = cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem);
  if (e != cudaSuccess) return mlp_cuda(e);
  int dev = 0, sms = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return mlp_cuda(e);
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return mlp_cuda(e);
  const int64_t n_tiles = a->m / kTileM;
  const int grid = (int)(n_tiles < sms ? n_tiles : sms);
  InferParams P;
  P.b = a->b;
  P.w_head = a->w_head;
  P.b_head = a->b_head;
  P.y = a->y;
  P.m = a->m;
  P.n_members = a->n_members;
  P.n_out = a->n_out;
  P.depth = a->depth;
  mlp_infer_kernel<<<grid, kInferThreads, kInferSmem, (cudaStream_t)stream>>>(tx, tw, P);
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
