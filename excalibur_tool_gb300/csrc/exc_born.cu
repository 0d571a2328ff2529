// exc_born.cu -- first-order line integrals along straight patch rays (ExcBornArgs in
// include/excalibur_mlp.h): the sky-map surrogate's baseline features.
//
// One thread per ray marches the straight line from the observer to the box face
// in equal segments, gathering Phi (trilinear) and the base-node gradient from
// the grid at each midpoint in FP32, and accumulates the Shapiro delay, the
// deflection, the transverse displacement at the face and the geometric delay.
// The work is L1/L2 gathers (the grid stays on chip); there is no tensor or FP64
// arithmetic in the loop.
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/excalibur_gb300.h"
#include "../../include/excalibur_mlp.h"

namespace exc {
void set_last_error(const char* msg);
}

namespace {

struct BornField {
  const void* data;
  int dtype, boundary;
  int n[3];
  float inv_s[3], s[3], o[3];
};

__device__ __forceinline__ float node(const BornField& F, int64_t i) {
  if (F.dtype == EXC_DTYPE_F32X2) return __ldg((const float*)F.data + 2 * i);
  if (F.dtype == EXC_DTYPE_F32) return __ldg((const float*)F.data + i);
  return (float)__ldg((const double*)F.data + i);
}

// wrap / clamp a cell index; false when the error-mode interior is left
__device__ __forceinline__ bool cell(const BornField& F, int d, float x, int& i, float& f, int& im, int& ip) {
  const float fl = floorf(x);
  i = (int)fl;
  f = x - fl;
  const int n = F.n[d];
  if (F.boundary == EXC_BOUNDARY_PERIODIC) {
    i %= n;
    if (i < 0) i += n;
    ip = i + 1 == n ? 0 : i + 1;
    im = i == 0 ? n - 1 : i - 1;
    return true;
  }
  if (F.boundary == EXC_BOUNDARY_CLAMP) {
    if (i < 0) { i = 0; f = 0.0f; }
    if (i > n - 2) { i = n - 2; f = 1.0f; }
    ip = i + 1;
    im = i > 0 ? i - 1 : i;
    return true;
  }
  if (i < 1 || i >= n - 2) return false;
  ip = i + 1;
  im = i - 1;
  return true;
}

__global__ void born_kernel(const BornField F, const ExcBornArgs A) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= A.n) return;
  // direction and straight exit (in double: once per ray)
  const double u = A.uv[2 * r], v = A.uv[2 * r + 1];
  double d[3];
  for (int k = 0; k < 3; ++k) d[k] = A.axis[k] + u * A.half * A.e1[k] + v * A.half * A.e2[k];
  const double nd = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  for (int k = 0; k < 3; ++k) d[k] /= nd;
  double L = 1e300;
  for (int k = 0; k < 3; ++k) {
    if (d[k] > 0) L = fmin(L, (A.box_hi[k] - A.origin[k]) / d[k]);
    else if (d[k] < 0) L = fmin(L, (A.box_lo[k] - A.origin[k]) / d[k]);
  }
  double* out = A.out + r * 8;
  if (!(L > 0.0 && L < 1e299)) {
    for (int k = 0; k < 8; ++k) out[k] = NAN;
    return;
  }
  const int ns = (int)ceil(L / A.step);
  const float dl = (float)(L / ns);
  // march in cell units (FP32 is ample for a first-order baseline)
  float p0[3], dc[3], df[3];
  for (int k = 0; k < 3; ++k) {
    p0[k] = (float)((A.origin[k] - F.o[k]) * F.inv_s[k]);
    dc[k] = (float)(d[k] * F.inv_s[k]);      // cells per metre along the ray
    df[k] = (float)d[k];
  }
  const int sy = F.n[2], sx = F.n[1] * F.n[2];
  float sphi = 0.0f, sphi1 = 0.0f, sphi2 = 0.0f, th[3] = {0.0f, 0.0f, 0.0f}, D[3] = {0.0f, 0.0f, 0.0f}, S1[3] = {0.0f, 0.0f, 0.0f}, S2 = 0.0f;
  const float c2 = (float)(A.c * A.c);
  const float kg = -2.0f / c2;
  const float Lf = (float)L;
  for (int s = 0; s < ns; ++s) {
    const float l = ((float)s + 0.5f) * dl;
    int ix, iy, iz, ixm, iym, izm, ixp, iyp, izp;
    float fx, fy, fz;
    if (!cell(F, 0, p0[0] + l * dc[0], ix, fx, ixm, ixp) || !cell(F, 1, p0[1] + l * dc[1], iy, fy, iym, iyp) ||
        !cell(F, 2, p0[2] + l * dc[2], iz, fz, izm, izp))
      continue;
    const int64_t b = (int64_t)ix * sx + (int64_t)iy * sy + iz;
    const float c000 = node(F, b), c100 = node(F, (int64_t)ixp * sx + (int64_t)iy * sy + iz);
    const float c010 = node(F, (int64_t)ix * sx + (int64_t)iyp * sy + iz), c001 = node(F, b - iz + izp);
    const float c110 = node(F, (int64_t)ixp * sx + (int64_t)iyp * sy + iz);
    const float c101 = node(F, (int64_t)ixp * sx + (int64_t)iy * sy + izp);
    const float c011 = node(F, (int64_t)ix * sx + (int64_t)iyp * sy + izp);
    const float c111 = node(F, (int64_t)ixp * sx + (int64_t)iyp * sy + izp);
    const float c00 = fmaf(fx, c100 - c000, c000), c10 = fmaf(fx, c110 - c010, c010);
    const float c01 = fmaf(fx, c101 - c001, c001), c11 = fmaf(fx, c111 - c011, c011);
    const float c0 = fmaf(fy, c10 - c00, c00), c1 = fmaf(fy, c11 - c01, c01);
    const float phi = fmaf(fz, c1 - c0, c0);
    float g[3];
    g[0] = (c100 - node(F, (int64_t)ixm * sx + (int64_t)iy * sy + iz)) * (0.5f * F.inv_s[0]);
    g[1] = (c010 - node(F, (int64_t)ix * sx + (int64_t)iym * sy + iz)) * (0.5f * F.inv_s[1]);
    g[2] = (c001 - node(F, b - iz + izm)) * (0.5f * F.inv_s[2]);
    const float gd = g[0] * df[0] + g[1] * df[1] + g[2] * df[2];
    const float w = l / Lf;
    sphi += phi * dl;
    sphi1 += phi * w * dl;
    sphi2 += phi * w * w * dl;
    float t2 = 0.0f;
    for (int k = 0; k < 3; ++k) {
      const float gp = kg * (g[k] - gd * df[k]);          // d theta / dl
      th[k] += gp * dl;
      D[k] += (Lf - l) * gp * dl;
      S1[k] += th[k] * dl;
      t2 += th[k] * th[k];
    }
    S2 += t2 * dl;
  }
  const double c = A.c;
  out[0] = -2.0 * (double)sphi / (c * c * c);
  out[1] = D[0] * A.e1[0] + D[1] * A.e1[1] + D[2] * A.e1[2];
  out[2] = D[0] * A.e2[0] + D[1] * A.e2[1] + D[2] * A.e2[2];
  const double s1 = (double)S1[0] * S1[0] + (double)S1[1] * S1[1] + (double)S1[2] * S1[2];
  out[3] = ((double)S2 - s1 / L) / (2.0 * c);
  out[4] = th[0] * A.e1[0] + th[1] * A.e1[1] + th[2] * A.e1[2];
  out[5] = th[0] * A.e2[0] + th[1] * A.e2[1] + th[2] * A.e2[2];
  out[6] = -2.0 * (double)sphi1 / (c * c * c);
  out[7] = -2.0 * (double)sphi2 / (c * c * c);
}

}  // namespace

extern "C" int exc_born_patch(const ExcMetric* metric, const ExcBornArgs* a, void* stream) {
  if (!metric || !a || (a->n > 0 && (!a->uv || !a->out)) || a->n < 0) {
    exc::set_last_error("born: metric, args, uv and out are required");
    return EXC_ERR_INVALID;
  }
  if (metric->kind != EXC_METRIC_FLRW || metric->n_fields < 1 || metric->fields[0].ndim != 3 || !metric->fields[0].data) {
    exc::set_last_error("born: needs an FLRW metric with a 3-D field 0");
    return EXC_ERR_INVALID;
  }
  if (!(a->step > 0.0) || !(a->c > 0.0)) {
    exc::set_last_error("born: step and c must be > 0");
    return EXC_ERR_INVALID;
  }
  if (a->n == 0) return EXC_SUCCESS;
  const ExcField& f = metric->fields[0];
  BornField F;
  F.data = f.data;
  F.dtype = f.dtype;
  F.boundary = f.boundary;
  for (int d = 0; d < 3; ++d) {
    F.n[d] = (int)f.n[d];
    F.s[d] = (float)f.spacing[d];
    F.inv_s[d] = (float)(1.0 / f.spacing[d]);
    F.o[d] = (float)(f.origin[d] - f.shift[d]);   // a shifted grid is queried at x + shift
  }
  const int64_t blocks = (a->n + 127) / 128;
  born_kernel<<<(unsigned)blocks, 128, 0, (cudaStream_t)stream>>>(F, *a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    exc::set_last_error(cudaGetErrorString(e));
    return EXC_ERR_CUDA;
  }
  return EXC_SUCCESS;
}
