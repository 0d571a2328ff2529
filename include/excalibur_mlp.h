/* excalibur_mlp.h -- C ABI of the sky-map surrogate's kernels (libexcalibur_gb300.so).
 *
 * The reference has no learned part; these entry points are the building
 * blocks of the direction -> (dz, time delay, deflection) MLP: Fourier
 * features of the sky direction, BF16 tensor-core GEMMs (tcgen05, FP32
 * accumulation in tensor memory) with fused bias / SiLU / SiLU-derivative
 * epilogues, the linear head with its MSE loss and gradient, split-K weight
 * gradients and Adam. The host side (excalibur_tool_gb300/surrogate/) owns
 * the buffers and sequences the calls on one stream.
 *
 * Conventions: all pointers are device pointers; matrices are row-major;
 * "bf16" is IEEE bfloat16 stored as uint16; an ensemble of E networks is a
 * batch of E independent problems laid out back to back (strides in
 * elements). Every call returns 0 or a negative ExcError (excalibur_gb300.h)
 * and allocates nothing.
 */
#ifndef EXCALIBUR_MLP_H
#define EXCALIBUR_MLP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* GEMM epilogues: acc = A[m,:] . B[n,:] (FP32) */
enum {
  EXC_EPI_F32 = 0,         /* c (f32) = acc */
  EXC_EPI_BIAS_SILU = 1,   /* z = acc + bias[n]; c (bf16) = z; c2 (bf16) = silu(z); ct (bf16) = silu(z)^T */
  EXC_EPI_DSILU = 2,       /* d = acc * silu'(z_in); c (bf16) = d; ct (bf16) = d^T */
  EXC_EPI_SPLITK = 3       /* c (f32) [batch][split][M][N] = partial acc over the split's K range */
};

/* C = epilogue(A . B^T) for a batch of problems.
 * A: [batch][M][K] bf16, B: [batch][N][K] bf16 (both K contiguous).
 * Limits: N a multiple of 16 in [16, 256]; K a multiple of 64; M >= 1.
 * ct (optional, may be NULL) is [batch][N][ldt] bf16 with ldt >= M. */
typedef struct ExcGemm {
  const void* a;
  const void* b;
  int64_t m;
  int32_t n, k;
  int64_t stride_a, stride_b;   /* elements between batch members */
  int32_t n_batch;
  int32_t epilogue;             /* EXC_EPI_* */
  int32_t k_splits;             /* EXC_EPI_SPLITK: number of K ranges (>= 1) */
  int32_t reserved;
  const float* bias;            /* [batch][N] (EXC_EPI_BIAS_SILU) */
  const void* z_in;             /* [batch][M][N] bf16 (EXC_EPI_DSILU) */
  void* c;
  void* c2;
  void* ct;
  int64_t stride_c;             /* elements between batch members of c, c2, z_in (>= M*N) */
  int64_t ldt;                  /* row length of ct */
  int64_t stride_ct;            /* elements between batch members of ct (>= N*ldt) */
} ExcGemm;

int exc_gemm_bf16(const ExcGemm* g, void* stream);

/* Fourier features of sky directions: for direction (theta, phi) of point i,
 * u = (theta - center[0]) * scale[0], v = (phi - center[1]) * scale[1] and,
 * for k = 1..n_freq, out[i] = [sin(pi k u), cos(pi k u), sin(pi k v), cos(pi k v)]
 * grouped as [sin u (n_freq) | cos u | sin v | cos v] (4 n_freq bf16 values).
 * dirs: [n][2] float64 (theta, phi). Rows n .. n_pad-1 are written as zeros. */
int exc_mlp_features(const double* dirs, int64_t n, int64_t n_pad, int32_t n_freq, const double* center2,
                     const double* scale2, void* out_bf16, void* stream);

/* Linear head y = H . W^T + b (W: [E][n_out][width] f32, b: [E][n_out]) over
 * H: [E][M][width] bf16. With targets (f32 [M][n_out], normalised) it also
 * forms the mean-squared-error gradient dy = 2 (y - t) / (M n_out), writes
 * dH = dy . W (bf16 [E][M][width]) pre-multiplied by silu'(z) when z is given
 * (bf16 [E][M][width], the last hidden pre-activation), its transpose
 * dHt ([E][width][ldt]), the head's gradients dW ([E][n_out][width] f32) and
 * db ([E][n_out] f32) (accumulated: the caller zeroes them), and the per-member
 * loss sum ([E] f32, accumulated). y: [E][M][n_out] f32 (may be NULL when
 * training). Limits: width 256, n_out <= 8. */
int exc_mlp_head(const void* h, int64_t m, int32_t width, int32_t n_out, int32_t n_members, const float* w,
                 const float* b, float* y, const float* targets, const void* z, void* dh, void* dht, int64_t ldt,
                 float* dw, float* db, float* loss, void* stream);

/* The ensemble's forward pass for prediction in one launch, activations kept on chip: per
 * 128-row tile of features x and member e, depth hidden layers h <- bf16(silu(bf16(h W^T + b)))
 * (tcgen05, BF16 x BF16 -> FP32 in tensor memory; the same roundings as exc_gemm_bf16 with
 * EXC_EPI_BIAS_SILU) and the linear head y = h . w_head^T + b_head in FP32. The inference half
 * of exc_gemm_bf16 + exc_mlp_head, without the hidden activations' HBM round trips.
 * x: [m][width] bf16 (m a multiple of 128); w: [depth][n_members][width][width] bf16 (layer l of
 * member e maps its input through w[l][e] (out x in)); b: [depth][n_members][width] f32;
 * w_head: [n_members][n_out][width] f32; b_head: [n_members][n_out] f32; y: [n_members][m][n_out]
 * f32. x, w and w_head 16-byte aligned, b 8-byte aligned (vector loads). Limits: width 256,
 * n_out <= 8. No reference counterpart (the surrogate is new). */
typedef struct ExcMlpInfer {
  const void* x;
  const void* w;
  const float* b;
  const float* w_head;
  const float* b_head;
  float* y;
  int64_t m;
  int32_t width, n_members, n_out, depth;
} ExcMlpInfer;

int exc_mlp_infer(const ExcMlpInfer* a, void* stream);

/* Sum of a [batch][splits][rows][cols] f32 partial-sum array over splits -> out [batch][rows][cols] f32. */
int exc_mlp_reduce_splits(const float* part, int32_t n_batch, int32_t splits, int64_t rows_x_cols, float* out,
                          void* stream);

/* Row sums of a [rows][ld] bf16 matrix over its first m columns -> out [rows] f32 (bias gradients). */
int exc_mlp_row_sums(const void* x, int64_t rows, int64_t m, int64_t ld, float* out, void* stream);

/* One Adam step over n parameters (f32 master copy p, moments m1/m2), with
 * bias corrections for step t; writes the bf16 copy p_bf16 (and its
 * transpose pt_bf16, [cols][rows] per matrix, when not NULL; rows x cols =
 * the matrix shape, n a multiple of rows*cols). */
int exc_mlp_adam(float* p, const float* grad, float* m1, float* m2, int64_t n, float lr, float beta1, float beta2,
                 float eps, int32_t t, void* p_bf16, void* pt_bf16, int32_t rows, int32_t cols, void* stream);

/* One parameter tensor of a multi-tensor Adam step (fields as in exc_mlp_adam). */
typedef struct ExcAdamTensor {
  float* p;
  const float* grad;
  float* m1;
  float* m2;
  int64_t n;
  void* p_bf16;      /* optional bf16 copy */
  void* pt_bf16;     /* optional transposed bf16 copy ([cols][rows] per matrix) */
  int32_t rows, cols;
} ExcAdamTensor;
#define EXC_ADAM_MAX_TENSORS 16

/* exc_mlp_adam over up to EXC_ADAM_MAX_TENSORS tensors in one launch (the network's weights,
 * biases and head of every ensemble member in a training step), with the step's learning rate
 * and bias corrections read on the device from sched = {lr, 1 / (1 - beta1^t),
 * 1 / (1 - beta2^t)} (float32): a training step captured once in a CUDA graph can then be
 * replayed with a schedule that changes every step. */
int exc_mlp_adam_multi(const ExcAdamTensor* tensors, int32_t n_tensors, const float* sched, float beta1,
                       float beta2, float eps, void* stream);

/* First-order (Born) line integrals along the straight rays of a tangent-plane
 * patch, the baseline features of the sky-map surrogate. For ray i, d = unit(axis
 * + uv[i][0] half e1 + uv[i][1] half e2) from origin (x, y, z) to the first face of
 * [box_lo, box_hi) at distance L, sampled at the midpoints of n = ceil(L / step)
 * equal segments with the field's trilinear Phi and base-node gradient (FP32):
 *   out[i][0] = -(2 / c^3) sum Phi dl                        (Shapiro delay, s)
 *   out[i][1..2] = D . e1, D . e2,  D = -(2 / c^2) sum (L - l) grad_perp Phi dl  (m)
 *   out[i][3] = tau_B = (S2 - |S1|^2 / L) / (2 c),  theta(l) = -(2 / c^2) int_0^l grad_perp Phi,
 *               S1 = sum theta dl, S2 = sum |theta|^2 dl       (geometric delay, s)
 *   out[i][4..5] = theta(L) . e1, theta(L) . e2              (deflection, rad)
 *   out[i][6..7] = -(2 / c^3) sum Phi (l / L)^k dl, k = 1, 2   (moments of the delay integrand)
 * grad_perp = the gradient minus its component along d. Field 0 of the metric
 * (float64, float32 or float32x2; periodic, clamp or error boundary: samples
 * outside an error-mode interior are skipped). out: [n][8] float64, device. */
typedef struct ExcBornArgs {
  int64_t n;
  const double* uv;
  double origin[3];
  double axis[3], e1[3], e2[3];
  double half;
  double box_lo[3], box_hi[3];
  double step;          /* segment length (m) */
  double c;
  double* out;
} ExcBornArgs;

struct ExcMetric;
int exc_born_patch(const struct ExcMetric* metric, const ExcBornArgs* args, void* stream);

/* Number of GEMM launches whose bounded tensor-core waits ran out since the
 * library was loaded (0 in a healthy run; such a launch leaves its outputs
 * unwritten). Synchronous: copies one word from the device. */
int exc_mlp_error_count(uint32_t* out);

#ifdef __cplusplus
}
#endif

#endif /* EXCALIBUR_MLP_H */
