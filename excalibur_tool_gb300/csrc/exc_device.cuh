// exc_device.cuh -- device-side physics of the photon-geodesic hot path (FP64).
//
// Every function restates one reference routine in the reference's own
// operation order (C and Python share left-to-right associativity for
// + - * /), so the translation unit compiled without FMA contraction
// (EXC_FAST == 0) reproduces the reference's IEEE double arithmetic; its divisions by
// launch constants (c^2, c^4, grid spacings, table step) take the correctly rounded
// quotient from a host reciprocal (div_rn), identical to the IEEE division at a third of
// its FP64 pipe cost. The unit compiled with contraction (EXC_FAST == 1) replaces those
// divisions, and 1/a, with plain multiplications by reciprocals: GB300's FP64 pipe is
// narrow and each IEEE division costs about eight FP64 pipe slots.
//
// Reference quirks kept on purpose (parity):
//  * gradient = central difference at the base node, piecewise constant per
//    cell (grid/interpolator_4d_fast.py:86-89, :243-253);
//  * Phi/c^2 fed into a term that divides by c^4 again, Gamma^i_00 = dPhi/a^2
//    in SI (metrics/perturbed_flrw_metric_fast.py:36, :46, :57, :67);
//  * Python's floor-mod for periodic wrap (interpolator_4d_fast.py:10-17);
//  * exact-integer c**2 / c**4 converted to float64 at the point of use.
#pragma once

#include <cstdint>
#include <cmath>
#include "exc_devmetric.h"
#include "exc_divrn.cuh"

#ifndef EXC_FAST
#error "EXC_FAST must be defined (0 = exact reference order, 1 = fast)"
#endif

#ifndef EXC_NS
#error "EXC_NS must name the precision build's namespace"
#endif

namespace EXC_NS {

using exc::DevMetric;

// ---------------------------------------------------------------- helpers
// Python float modulo: result carries the sign of the divisor
// (CPython float_rem / numpy npy_remainder semantics).
__device__ __forceinline__ double py_fmod(double a, double b) {
  double m = fmod(a, b);
  if (m != 0.0) {
    if ((b < 0.0) != (m < 0.0)) m += b;
  } else {
    m = copysign(0.0, b);
  }
  return m;
}

// py_fmod(d, L) for the periodic wrap, L > 0: a d already in (0, L) is its own remainder (fmod is
// exact), so the division-free test returns it unchanged and only the rare wrap pays for fmod.
// The same bits as py_fmod for every d (0 and -0 take the fmod path, which gives +0).
__device__ __forceinline__ double py_wrap(double d, double L) {
  return (d > 0.0 && d < L) ? d : py_fmod(d, L);
}

// Python integer modulo (non-negative for n > 0).
__device__ __forceinline__ int64_t py_imod(int64_t i, int64_t n) {
  int64_t r = i % n;
  if (r != 0 && ((r < 0) != (n < 0))) r += n;
  return r;
}

// x**3 and x**4 rounded once. The reference evaluates them with libm pow()
// (Python float ** int, numpy float64 ** int), which rounds the exact power
// correctly except in rare near-halfway cases; a double-double product
// (Dekker's exact square via FMA) gives the same rounding.
__device__ __forceinline__ double pow3_cr(double x) {
  double p = x * x;
  double e = fma(x, x, -p);
  double hi = p * x;
  double lo = fma(p, x, -hi) + e * x;
  return hi + lo;
}
__device__ __forceinline__ double pow4_cr(double x) {
  double p = x * x;
  double e = fma(x, x, -p);
  double hi = p * p;
  double lo = fma(p, p, -hi) + 2.0 * p * e;
  return hi + lo;
}

template <class FT>
__device__ __forceinline__ double ldf(const FT* p, int64_t i) {
  return (double)__ldg(p + i);
}
// split grid (EXC_DTYPE_F32X2): interleaved (hi, lo) pairs; hi + lo is exact in FP64
template <>
__device__ __forceinline__ double ldf<float2>(const float2* p, int64_t i) {
  const float2 v = __ldg(p + i);
  return (double)v.x + (double)v.y;
}

struct InterpOut {
  double val, gx, gy, gz, dtd;
};

// x / c by a launch constant: the correctly rounded quotient on the parity path (div_rn,
// bit-identical to an IEEE division), x * (1/c) on the fast path.
__device__ __forceinline__ double div_c(double x, double c, double inv_c) {
#if EXC_FAST
  (void)c;
  return x * inv_c;
#else
  return ::div_rn(x, c, inv_c);
#endif
}

__device__ __forceinline__ double trilinear(double c000, double c100, double c010, double c001,
                                            double c110, double c101, double c011, double c111,
                                            double dx, double dy, double dz) {
  // _interp_trilinear_from_corners, interpolator_4d_fast.py:29-43
  return c000 * (1.0 - dx) * (1.0 - dy) * (1.0 - dz) +
         c100 * dx * (1.0 - dy) * (1.0 - dz) +
         c010 * (1.0 - dx) * dy * (1.0 - dz) +
         c001 * (1.0 - dx) * (1.0 - dy) * dz +
         c110 * dx * dy * (1.0 - dz) +
         c101 * dx * (1.0 - dy) * dz +
         c011 * (1.0 - dx) * dy * dz +
         c111 * dx * dy * dz;
}

// True when the field carries a query offset (any non-zero bit in ExcField.shift).
__device__ __forceinline__ bool has_shift(const ExcField& f) {
  return (__double_as_longlong(f.shift[0]) | __double_as_longlong(f.shift[1]) |
          __double_as_longlong(f.shift[2])) != 0;
}

// One spatial snapshot `it` (of nt, innermost index) of a 3-D/4-D field.
// Returns an EXC_PH_* failure code, or 0 with `o` filled (o.dtd = 0).
// The cell coordinate rel = (x - origin) / spacing is the correctly rounded quotient in
// every build (div_rn): the base-node gradient is discontinuous across cell faces, and
// positions that sit exactly on a node plane (an observer placed on a grid
// node, as the reference runner does) must select the reference's cell.
template <class FT>
__device__ __forceinline__ int interp_snapshot(const ExcField& f, const double* fi, const FT* __restrict__ d,
                                               int64_t nt, int64_t it, double x, double y, double z,
                                               InterpOut& o) {
  const int64_t nx = f.n[0], ny = f.n[1], nz = f.n[2];
  const double ox = f.origin[0], oy = f.origin[1], oz = f.origin[2];
  const double sx = f.spacing[0], sy = f.spacing[1], sz = f.spacing[2];
#define EXC_IDX(i, j, k) ((((int64_t)(i) * ny + (j)) * nz + (k)) * nt + it)
  if (f.boundary == EXC_BOUNDARY_PERIODIC) {
    // fused_interpolation_gradient_3d_periodic, interpolator_4d_fast.py:195-255
    const double Lx = (double)nx * sx, Ly = (double)ny * sy, Lz = (double)nz * sz;
    x = ox + py_wrap(x - ox, Lx);
    y = oy + py_wrap(y - oy, Ly);
    z = oz + py_wrap(z - oz, Lz);
    const double rx = div_rn(x - ox, sx, fi[0]), ry = div_rn(y - oy, sy, fi[1]), rz = div_rn(z - oz, sz, fi[2]);
    if (!isfinite(rx) || !isfinite(ry) || !isfinite(rz)) return EXC_PH_NONFINITE;
    int64_t i0 = (int64_t)floor(rx), j0 = (int64_t)floor(ry), k0 = (int64_t)floor(rz);
    const double dx = rx - (double)i0, dy = ry - (double)j0, dz = rz - (double)k0;
    i0 = py_imod(i0, nx); j0 = py_imod(j0, ny); k0 = py_imod(k0, nz);
    const int64_t i1 = py_imod(i0 + 1, nx), j1 = py_imod(j0 + 1, ny), k1 = py_imod(k0 + 1, nz);
    const int64_t im = py_imod(i0 - 1, nx), jm = py_imod(j0 - 1, ny), km = py_imod(k0 - 1, nz);
    const double c000 = ldf(d, EXC_IDX(i0, j0, k0)), c100 = ldf(d, EXC_IDX(i1, j0, k0));
    const double c010 = ldf(d, EXC_IDX(i0, j1, k0)), c001 = ldf(d, EXC_IDX(i0, j0, k1));
    const double c110 = ldf(d, EXC_IDX(i1, j1, k0)), c101 = ldf(d, EXC_IDX(i1, j0, k1));
    const double c011 = ldf(d, EXC_IDX(i0, j1, k1)), c111 = ldf(d, EXC_IDX(i1, j1, k1));
    o.val = trilinear(c000, c100, c010, c001, c110, c101, c011, c111, dx, dy, dz);
    o.gx = div_c(c100 - ldf(d, EXC_IDX(im, j0, k0)), 2.0 * sx, fi[4]);
    o.gy = div_c(c010 - ldf(d, EXC_IDX(i0, jm, k0)), 2.0 * sy, fi[5]);
    o.gz = div_c(c001 - ldf(d, EXC_IDX(i0, j0, km)), 2.0 * sz, fi[6]);
    o.dtd = 0.0;
    return 0;
  }
  if (f.boundary == EXC_BOUNDARY_CLAMP) {
    // fused_interpolation_gradient_3d_clamp, interpolator_4d_fast.py:101-188
    const double ex = 1e-12 * sx, ey = 1e-12 * sy, ez = 1e-12 * sz;
    const double hx = ox + (double)(nx - 1) * sx - ex;
    const double hy = oy + (double)(ny - 1) * sy - ey;
    const double hz = oz + (double)(nz - 1) * sz - ez;
    if (x < ox) x = ox; else if (x > hx) x = hx;
    if (y < oy) y = oy; else if (y > hy) y = hy;
    if (z < oz) z = oz; else if (z > hz) z = hz;
    const double rx = div_rn(x - ox, sx, fi[0]), ry = div_rn(y - oy, sy, fi[1]), rz = div_rn(z - oz, sz, fi[2]);
    if (!isfinite(rx) || !isfinite(ry) || !isfinite(rz)) return EXC_PH_NONFINITE;
    int64_t i0 = (int64_t)floor(rx), j0 = (int64_t)floor(ry), k0 = (int64_t)floor(rz);
    if (i0 < 0) i0 = 0;
    if (j0 < 0) j0 = 0;
    if (k0 < 0) k0 = 0;
    if (i0 > nx - 2) i0 = nx - 2;
    if (j0 > ny - 2) j0 = ny - 2;
    if (k0 > nz - 2) k0 = nz - 2;
    const double dx = rx - (double)i0, dy = ry - (double)j0, dz = rz - (double)k0;
    const double c000 = ldf(d, EXC_IDX(i0, j0, k0)), c100 = ldf(d, EXC_IDX(i0 + 1, j0, k0));
    const double c010 = ldf(d, EXC_IDX(i0, j0 + 1, k0)), c001 = ldf(d, EXC_IDX(i0, j0, k0 + 1));
    const double c110 = ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0)), c101 = ldf(d, EXC_IDX(i0 + 1, j0, k0 + 1));
    const double c011 = ldf(d, EXC_IDX(i0, j0 + 1, k0 + 1)), c111 = ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0 + 1));
    o.val = trilinear(c000, c100, c010, c001, c110, c101, c011, c111, dx, dy, dz);
    // one-sided at the low edge, central otherwise (the centre index is <= n-2)
    o.gx = (i0 <= 0) ? div_c(c100 - c000, sx, fi[0]) : div_c(c100 - ldf(d, EXC_IDX(i0 - 1, j0, k0)), 2.0 * sx, fi[4]);
    o.gy = (j0 <= 0) ? div_c(c010 - c000, sy, fi[1]) : div_c(c010 - ldf(d, EXC_IDX(i0, j0 - 1, k0)), 2.0 * sy, fi[5]);
    o.gz = (k0 <= 0) ? div_c(c001 - c000, sz, fi[2]) : div_c(c001 - ldf(d, EXC_IDX(i0, j0, k0 - 1)), 2.0 * sz, fi[6]);
    o.dtd = 0.0;
    return 0;
  }
  // EXC_BOUNDARY_ERROR: fused_interpolation_gradient_3d_error,
  // interpolator_4d_fast.py:50-91 (same arithmetic as the legacy strict
  // interpolator, grid/interpolator_fast.py:119-192)
  const double rx = div_rn(x - ox, sx, fi[0]), ry = div_rn(y - oy, sy, fi[1]), rz = div_rn(z - oz, sz, fi[2]);
  if (rx < 1.0 || rx >= (double)nx - 2.0 || ry < 1.0 || ry >= (double)ny - 2.0 ||
      rz < 1.0 || rz >= (double)nz - 2.0)
    return EXC_PH_OUTSIDE_GRID;
  if (!isfinite(rx) || !isfinite(ry) || !isfinite(rz)) return EXC_PH_NONFINITE;
  const int64_t i0 = (int64_t)floor(rx), j0 = (int64_t)floor(ry), k0 = (int64_t)floor(rz);
  const double dx = rx - (double)i0, dy = ry - (double)j0, dz = rz - (double)k0;
  const double c000 = ldf(d, EXC_IDX(i0, j0, k0)), c100 = ldf(d, EXC_IDX(i0 + 1, j0, k0));
  const double c010 = ldf(d, EXC_IDX(i0, j0 + 1, k0)), c001 = ldf(d, EXC_IDX(i0, j0, k0 + 1));
  const double c110 = ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0)), c101 = ldf(d, EXC_IDX(i0 + 1, j0, k0 + 1));
  const double c011 = ldf(d, EXC_IDX(i0, j0 + 1, k0 + 1)), c111 = ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0 + 1));
  o.val = trilinear(c000, c100, c010, c001, c110, c101, c011, c111, dx, dy, dz);
  o.gx = div_c(c100 - ldf(d, EXC_IDX(i0 - 1, j0, k0)), 2.0 * sx, fi[4]);
  o.gy = div_c(c010 - ldf(d, EXC_IDX(i0, j0 - 1, k0)), 2.0 * sy, fi[5]);
  o.gz = div_c(c001 - ldf(d, EXC_IDX(i0, j0, k0 - 1)), 2.0 * sz, fi[6]);
  o.dtd = 0.0;
  return 0;
#undef EXC_IDX
}

// ---- the slow Interpolator (grid/interpolator.py), grad_mode EXC_GRAD_TRILINEAR

// Difference of two grid nodes. numpy subtracts two float32 elements in
// float32 (grid/interpolator.py:147-152 on a float32 field); every other grid
// type differences in FP64.
template <class FT>
__device__ __forceinline__ double node_diff(const FT* __restrict__ d, int64_t a, int64_t b) {
  return ldf(d, a) - ldf(d, b);
}
template <>
__device__ __forceinline__ double node_diff<float>(const float* __restrict__ d, int64_t a, int64_t b) {
  return (double)(__ldg(d + a) - __ldg(d + b));
}

// numpy's sum of eight float64 terms (its pairwise summation with eight
// partial sums, as np.sum applies it to a length-8 array).
__device__ __forceinline__ double sum8(const double p[8]) {
  return ((p[0] + p[1]) + (p[2] + p[3])) + ((p[4] + p[5]) + (p[6] + p[7]));
}

// Integer index of an already-floored coordinate, clipped to [lo, hi] in the
// double domain first so that no out-of-range value is converted.
__device__ __forceinline__ int64_t clip_index(double v, int64_t lo, int64_t hi) {
  if (!(v > (double)lo)) return lo;
  if (v >= (double)hi) return hi;
  return (int64_t)v;
}

// Interpolator.gradient (grid/interpolator.py:88-158) on snapshot `it`: the
// central differences at the eight corners of the cell whose base index is
// floor(rel) clipped to [1, n-2] (each corner clipped again), blended with
// the trilinear weights of the unclipped fraction rel - floor(rel). Corner
// order (:117-126) and weight expressions (:129-138) as listed there.
template <class FT>
__device__ __forceinline__ void slow_gradient(const ExcField& f, const double* fi, const FT* __restrict__ d,
                                              int64_t nt, int64_t it, double rx, double ry, double rz,
                                              InterpOut& o) {
  const int64_t nx = f.n[0], ny = f.n[1], nz = f.n[2];
#define EXC_IDX(i, j, k) ((((int64_t)(i) * ny + (j)) * nz + (k)) * nt + it)
  const double flx = floor(rx), fly = floor(ry), flz = floor(rz);
  const double wx = rx - flx, wy = ry - fly, wz = rz - flz;
  const int64_t bi = clip_index(flx, 1, nx - 2), bj = clip_index(fly, 1, ny - 2), bk = clip_index(flz, 1, nz - 2);
  const double w[8] = {(1.0 - wx) * (1.0 - wy) * (1.0 - wz), wx * (1.0 - wy) * (1.0 - wz),
                       (1.0 - wx) * wy * (1.0 - wz),         (1.0 - wx) * (1.0 - wy) * wz,
                       wx * wy * (1.0 - wz),                 wx * (1.0 - wy) * wz,
                       (1.0 - wx) * wy * wz,                 wx * wy * wz};
  // corner c's offsets: x for c in {1,4,5,7}, y for {2,4,6,7}, z for {3,5,6,7}
  constexpr unsigned kOx = 0xB2u, kOy = 0xD4u, kOz = 0xE8u;
  double px[8], py[8], pz[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int64_t i = min(bi + (int64_t)((kOx >> c) & 1u), nx - 2);
    const int64_t j = min(bj + (int64_t)((kOy >> c) & 1u), ny - 2);
    const int64_t k = min(bk + (int64_t)((kOz >> c) & 1u), nz - 2);
    px[c] = div_c(node_diff(d, EXC_IDX(i + 1, j, k), EXC_IDX(i - 1, j, k)), 2.0 * f.spacing[0], fi[4]) * w[c];
    py[c] = div_c(node_diff(d, EXC_IDX(i, j + 1, k), EXC_IDX(i, j - 1, k)), 2.0 * f.spacing[1], fi[5]) * w[c];
    pz[c] = div_c(node_diff(d, EXC_IDX(i, j, k + 1), EXC_IDX(i, j, k - 1)), 2.0 * f.spacing[2], fi[6]) * w[c];
  }
  o.gx = sum8(px);
  o.gy = sum8(py);
  o.gz = sum8(pz);
#undef EXC_IDX
}

// Interpolator.interpolate on a 3-D field (grid/interpolator.py:13-69): the value
// alone, for callers that need Phi but not its gradient (the mixed tracer's
// FP64 endpoint quantities). Same arithmetic as interp_slow's 3-D value.
template <class FT>
__device__ __forceinline__ int slow_value3(const ExcField& f, double x, double y, double z, double& val) {
  const FT* d = (const FT*)f.data;
  if (has_shift(f)) {
    x += f.shift[0];
    y += f.shift[1];
    z += f.shift[2];
  }
  const int64_t nx = f.n[0], ny = f.n[1], nz = f.n[2];
  const double rx = (x - f.origin[0]) / f.spacing[0];
  const double ry = (y - f.origin[1]) / f.spacing[1];
  const double rz = (z - f.origin[2]) / f.spacing[2];
  if (rx < 0.0 || rx >= (double)(nx - 1) || ry < 0.0 || ry >= (double)(ny - 1) || rz < 0.0 ||
      rz >= (double)(nz - 1))
    return EXC_PH_OUTSIDE_GRID;
  if (!isfinite(rx) || !isfinite(ry) || !isfinite(rz)) return EXC_PH_NONFINITE;
  const double flx = floor(rx), fly = floor(ry), flz = floor(rz);
  const int64_t i0 = (int64_t)flx, j0 = (int64_t)fly, k0 = (int64_t)flz;
#define EXC_IDX(i, j, k) (((int64_t)(i) * ny + (j)) * nz + (k))
  val = trilinear(ldf(d, EXC_IDX(i0, j0, k0)), ldf(d, EXC_IDX(i0 + 1, j0, k0)), ldf(d, EXC_IDX(i0, j0 + 1, k0)),
                  ldf(d, EXC_IDX(i0, j0, k0 + 1)), ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0)),
                  ldf(d, EXC_IDX(i0 + 1, j0, k0 + 1)), ldf(d, EXC_IDX(i0, j0 + 1, k0 + 1)),
                  ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0 + 1)), rx - flx, ry - fly, rz - flz);
#undef EXC_IDX
  return 0;
}

// Interpolator.value_gradient_and_time_derivative (grid/interpolator.py:198-206)
// for an ExcField with grad_mode EXC_GRAD_TRILINEAR. Unlike the fast classes,
// the slow one raises only for a position outside the bounds: a NaN grid value
// passes through (and ends a traced photon as non-finite).
template <class FT>
__device__ __forceinline__ int interp_slow(const ExcField& f, const double* fi, const FT* __restrict__ d,
                                           double x, double y, double z, double t, InterpOut& o) {
  const int64_t nx = f.n[0], ny = f.n[1], nz = f.n[2];
  // _index_and_weights (:13-44): bounds rel in [0, n-1), no clipping needed after it
  const double rx = div_rn(x - f.origin[0], f.spacing[0], fi[0]);
  const double ry = div_rn(y - f.origin[1], f.spacing[1], fi[1]);
  const double rz = div_rn(z - f.origin[2], f.spacing[2], fi[2]);
  if (rx < 0.0 || rx >= (double)(nx - 1) || ry < 0.0 || ry >= (double)(ny - 1) || rz < 0.0 ||
      rz >= (double)(nz - 1))
    return EXC_PH_OUTSIDE_GRID;
  if (!isfinite(rx) || !isfinite(ry) || !isfinite(rz)) return EXC_PH_NONFINITE;
  const double flx = floor(rx), fly = floor(ry), flz = floor(rz);
  const int64_t i0 = (int64_t)flx, j0 = (int64_t)fly, k0 = (int64_t)flz;
  const double wx = rx - flx, wy = ry - fly, wz = rz - flz;
  if (f.ndim != 4) {
#define EXC_IDX(i, j, k) (((int64_t)(i) * ny + (j)) * nz + (k))
    // _interpolate_3d (:52-69)
    o.val = trilinear(ldf(d, EXC_IDX(i0, j0, k0)), ldf(d, EXC_IDX(i0 + 1, j0, k0)), ldf(d, EXC_IDX(i0, j0 + 1, k0)),
                      ldf(d, EXC_IDX(i0, j0, k0 + 1)), ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0)),
                      ldf(d, EXC_IDX(i0 + 1, j0, k0 + 1)), ldf(d, EXC_IDX(i0, j0 + 1, k0 + 1)),
                      ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0 + 1)), wx, wy, wz);
#undef EXC_IDX
    slow_gradient<FT>(f, fi, d, 1, 0, rx, ry, rz, o);
    o.dtd = 0.0;
    return 0;
  }
  const int64_t nt = f.n[3];
#define EXC_IDX(i, j, k, l) ((((int64_t)(i) * ny + (j)) * nz + (k)) * nt + (l))
  const double rt = div_rn(t - f.origin[3], f.spacing[3], fi[3]);
  if (!isfinite(rt)) return EXC_PH_NONFINITE;
  const double flt = floor(rt);
  const double wt = rt - flt;
  // _interpolate_4d (:71-86): w[a][b][c][e] = ((wx_a * wy_b) * wz_c) * wt_e summed
  // as numpy sums the sixteen products in C order (eight partial sums)
  const int64_t l0 = clip_index(flt, 0, nt - 2);
  const double Wx[2] = {1.0 - wx, wx}, Wy[2] = {1.0 - wy, wy}, Wz[2] = {1.0 - wz, wz}, Wt[2] = {1.0 - wt, wt};
  double r[8];
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int a = q >> 3, b = (q >> 2) & 1, c = (q >> 1) & 1, e = q & 1;
    const double p = ldf(d, EXC_IDX(i0 + a, j0 + b, k0 + c, l0 + e)) * (((Wx[a] * Wy[b]) * Wz[c]) * Wt[e]);
    if (q < 8) r[q] = p;
    else r[q - 8] += p;
  }
  o.val = sum8(r);
  // gradient on the nearest snapshot (:92-96): round half to even, clipped to [0, nt-1]
  slow_gradient<FT>(f, fi, d, nt, clip_index(rint(rt), 0, nt - 1), rx, ry, rz, o);
  // time_derivative (:160-174): snapshots lt -/+ 1 around lt = clip(floor(rel_t), 1, nt-2);
  // numpy's clip gives nt-2 when that bound is below 1, and index -1 is the last snapshot
  const double lv = fmin(fmax(flt, 1.0), (double)(nt - 2));
  const int64_t lt = (int64_t)lv;
  const int64_t lp = lt - 1 < 0 ? lt - 1 + nt : lt - 1, ln = lt + 1;
  double v[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int64_t l = s ? ln : lp;
    v[s] = trilinear(ldf(d, EXC_IDX(i0, j0, k0, l)), ldf(d, EXC_IDX(i0 + 1, j0, k0, l)),
                     ldf(d, EXC_IDX(i0, j0 + 1, k0, l)), ldf(d, EXC_IDX(i0, j0, k0 + 1, l)),
                     ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0, l)), ldf(d, EXC_IDX(i0 + 1, j0, k0 + 1, l)),
                     ldf(d, EXC_IDX(i0, j0 + 1, k0 + 1, l)), ldf(d, EXC_IDX(i0 + 1, j0 + 1, k0 + 1, l)), wx, wy, wz);
  }
#undef EXC_IDX
  o.dtd = div_c(v[1] - v[0], 2.0 * f.spacing[3], fi[7]);
  return 0;
}

// InterpolatorFast.value_gradient_and_time_derivative (interpolator_4d_fast.py:443-502),
// including the 4-D snapshot blend (:265-402). A NaN value maps to
// EXC_PH_OUTSIDE_GRID, like the reference's ValueError at :500-501.
// grad_mode EXC_GRAD_TRILINEAR selects the slow Interpolator instead. SLOW =
// false compiles that path out (callers whose host side has ruled such fields
// out: the tracer kernels of base-node launches, the mixed tracer), so that it
// does not weigh on their register allocation.
template <class FT, bool SLOW = true>
__device__ __forceinline__ int interp_field(const ExcField& f, const double* fi, double x, double y, double z,
                                            double t, InterpOut& o) {
  const FT* d = (const FT*)f.data;
  // a shifted interpolator queries x + shift (ExcField.shift; zero = none). The test is on the
  // bit patterns (integer pipe, uniform per launch): an unshifted grid costs no FP64 operation.
  if (has_shift(f)) {
    x += f.shift[0];
    y += f.shift[1];
    z += f.shift[2];
  }
  if constexpr (SLOW) {
    if (f.grad_mode == EXC_GRAD_TRILINEAR) return interp_slow<FT>(f, fi, d, x, y, z, t, o);
  }
  if (f.ndim != 4) {
    int st = interp_snapshot<FT>(f, fi, d, 1, 0, x, y, z, o);
    if (st) return st;
    if (isnan(o.val)) return EXC_PH_OUTSIDE_GRID;
    return 0;
  }
  const int64_t nt = f.n[3];
  const double ot = f.origin[3], stp = f.spacing[3];
  double rt;
  if (f.boundary == EXC_BOUNDARY_CLAMP) {
    const double et = 1e-12 * stp;
    const double ht = ot + (double)(nt - 1) * stp - et;
    if (t < ot) t = ot; else if (t > ht) t = ht;
    rt = div_rn(t - ot, stp, fi[3]);
  } else {
    rt = div_rn(t - ot, stp, fi[3]);
    if (rt < 0.0 || rt >= (double)nt - 1.0) return EXC_PH_OUTSIDE_GRID;
  }
  if (!isfinite(rt)) return EXC_PH_NONFINITE;
  int64_t it0 = (int64_t)floor(rt);
  if (it0 < 0) it0 = 0;
  if (it0 > nt - 2) it0 = nt - 2;
  const double wt = rt - (double)it0;
  InterpOut a, b;
  int s0 = interp_snapshot<FT>(f, fi, d, nt, it0, x, y, z, a);
  if (s0) return s0;
  int s1 = interp_snapshot<FT>(f, fi, d, nt, it0 + 1, x, y, z, b);
  if (s1) return s1;
  if (isnan(a.val) || isnan(b.val)) return EXC_PH_OUTSIDE_GRID;
  o.val = (1.0 - wt) * a.val + wt * b.val;
  o.gx = (1.0 - wt) * a.gx + wt * b.gx;
  o.gy = (1.0 - wt) * a.gy + wt * b.gy;
  o.gz = (1.0 - wt) * a.gz + wt * b.gz;
  o.dtd = div_c(b.val - a.val, stp, fi[3]);
  return 0;
}

// ------------------------------------------------------------ cosmology
// The block's copy of the a(eta) table under EXC_STAGING_SHARED (dynamic shared memory, filled by
// the trace kernel's prologue).
extern __shared__ double stage_tab_s[];

__device__ __forceinline__ double a_table_at(const DevMetric& D, int64_t i) {
  return D.stage_table ? stage_tab_s[i] : __ldg(D.m.a_table + i);
}

// a_interp_numba, core/cosmology.py:8-25 (clamped linear interpolation).
__device__ __forceinline__ double a_interp(const DevMetric& D, double eta, int& st) {
  const ExcMetric& m = D.m;
  const int64_t n = m.a_table_n;
  if (eta <= m.eta_min) return a_table_at(D, 0);
  const double max_eta = m.eta_min + m.eta_step * (double)(n - 1);
  if (eta >= max_eta) return a_table_at(D, n - 1);
  if (isnan(eta)) { st = EXC_PH_NONFINITE; return NAN; }
  int64_t i = (int64_t)div_c(eta - m.eta_min, m.eta_step, D.i_eta_step);
  // the quotient can round up to n-1 within an ulp of the table end (the
  // reference would index past its table there); stay on the last cell
  if (i > n - 2) i = n - 2;
  const double t = div_c(eta - (m.eta_min + (double)i * m.eta_step), m.eta_step, D.i_eta_step);
  return (1.0 - t) * a_table_at(D, i) + t * a_table_at(D, i + 1);
}

// LCDM_Cosmology.adot_of_eta given a = a_of_eta(eta), inv_a = 1/a (core/cosmology.py:69-93).
__device__ __forceinline__ double adot_analytic(const ExcMetric& m, double a, double inv_a) {
#if EXC_FAST
  const double z = inv_a - 1.0;
#else
  (void)inv_a;
  const double z = 1.0 / a - 1.0;
#endif
  const double zp = 1.0 + z;
  const double E = sqrt(m.omega_m * pow3_cr(zp) + m.omega_r * pow4_cr(zp) +
                        m.omega_k * (zp * zp) + m.omega_lambda);
  const double H = m.H0 * E;
  return a * a * H;
}

// PerturbedFLRWMetricFast._get_scale_factor_and_derivative
// (perturbed_flrw_metric_fast.py:190-225), incl. its finite/zero guards.
// inv_a = 1/a is returned for the fast path (1.0 on the parity path).
__device__ __forceinline__ int scale_factor(const DevMetric& D, double eta, double& a, double& adot,
                                            double& inv_a) {
  const ExcMetric& m = D.m;
  int st = 0;
  inv_a = 1.0;
  if (m.cosmology == EXC_COSMO_STATIC) {
    a = 1.0;
    adot = 0.0;
    return 0;
  }
  a = a_interp(D, eta, st);
  if (m.cosmology == EXC_COSMO_TABLE) {
#if EXC_FAST
    inv_a = 1.0 / a;
#endif
    adot = adot_analytic(m, a, inv_a);
  } else {
    const double ae = fabs(eta);
    const double h = (1e-6 * ae > 1e-6) ? 1e-6 * ae : 1e-6;
    const double ap = a_interp(D, eta + h, st);
    const double am = a_interp(D, eta - h, st);
    adot = (ap - am) / (2.0 * h);
  }
  if (st) return st;
  if (!isfinite(a) || fabs(a) < 1e-30) a = 1e-30;
  if (!isfinite(adot)) adot = 0.0;
#if EXC_FAST
  inv_a = 1.0 / a;
#endif
  return 0;
}

// ------------------------------------------------------------ FLRW RHS
// compute_tensorial_acceleration, perturbed_flrw_metric_fast.py:7-76.
__device__ __forceinline__ void flrw_accel_tensorial(const DevMetric& D, double u0, double u1, double u2,
                                                     double u3, double a, double adot, double inv_a,
                                                     double phi, double gx, double gy, double gz,
                                                     double phi_dot, double du[4]) {
  const double c2 = D.m.c2, c4 = D.m.c4, ic2 = D.ic2, ic4 = D.ic4;
  const double a2 = a * a;
#if EXC_FAST
  const double adot_a = adot * inv_a;
  const double ia2 = inv_a * inv_a;
#else
  // a and a^2 divide several terms: one IEEE reciprocal each, then correctly rounded
  // quotients from it (div_rn), identical to the reference's divisions
  (void)inv_a;
  const double ra = 1.0 / a, ra2 = 1.0 / a2;
  const double adot_a = ::div_rn(adot, a, ra);
#endif
  const double usq = u1 * u1 + u2 * u2 + u3 * u3;
  const double psi = phi;
  const double gxc = div_c(gx, c2, ic2), gyc = div_c(gy, c2, ic2), gzc = div_c(gz, c2, ic2);
  const double pdc = div_c(phi_dot, c2, ic2);
  const double G000 = pdc * u0 * u0;
  const double G0ij = (div_c(a * adot, c2, ic2) + div_c(2.0 * a * adot, c4, ic4) * (phi + psi) -
                       div_c(a2, c4, ic4) * phi_dot) * usq;
  const double G00i = 2.0 * (gxc * u0 * u1 + gyc * u0 * u2 + gzc * u0 * u3);
  du[0] = -(G000 + G0ij + G00i);
  const double hub = 2.0 * (adot_a - pdc);
#if EXC_FAST
  const double G100 = gx * ia2 * u0 * u0;
  const double G200 = gy * ia2 * u0 * u0;
  const double G300 = gz * ia2 * u0 * u0;
#else
  const double G100 = ::div_rn(gx, a2, ra2) * u0 * u0;
  const double G200 = ::div_rn(gy, a2, ra2) * u0 * u0;
  const double G300 = ::div_rn(gz, a2, ra2) * u0 * u0;
#endif
  const double G1ii = -gxc * u1 * u1 + gxc * (u2 * u2 + u3 * u3) + (-gyc) * u1 * u2 + (-gzc) * u1 * u3;
  du[1] = -(G100 + hub * u0 * u1 + G1ii);
  const double G2ii = -gyc * u2 * u2 + gyc * (u1 * u1 + u3 * u3) + (-gxc) * u2 * u1 + (-gzc) * u2 * u3;
  du[2] = -(G200 + hub * u0 * u2 + G2ii);
  const double G3ii = -gzc * u3 * u3 + gzc * (u1 * u1 + u2 * u2) + (-gxc) * u3 * u1 + (-gyc) * u3 * u2;
  du[3] = -(G300 + hub * u0 * u3 + G3ii);
}

// compute_analytical_acceleration, perturbed_flrw_metric_fast.py:78-99.
__device__ __forceinline__ void flrw_accel_analytical(const DevMetric& D, double u0, double u1, double u2,
                                                      double u3, double a, double adot, double inv_a,
                                                      double phi, double gx, double gy, double gz,
                                                      double phi_dot, double du[4]) {
  const double c2 = D.m.c2, c4 = D.m.c4, tc2 = D.m.two_over_c2, ic2 = D.ic2, ic4 = D.ic4;
  const double vsq = u1 * u1 + u2 * u2 + u3 * u3;
  const double dphidl = gx * u1 + gy * u2 + gz * u3;
  const double psi = phi;
#if EXC_FAST
  const double aa = adot * inv_a;
  const double aa2 = 2.0 * adot * inv_a;
#else
  (void)inv_a;
  const double ra = 1.0 / a;
  const double aa = ::div_rn(adot, a, ra);
  const double aa2 = ::div_rn(2.0 * adot, a, ra);
#endif
  const double pdc2 = div_c(phi_dot, c2, ic2);
  du[0] = -(aa + pdc2) * (u0 * u0) - tc2 * u0 * dphidl -
          (div_c(aa, c2, ic2) - div_c(aa2, c4, ic4) * (phi + psi) - div_c(phi_dot, c4, ic4)) * vsq;
  const double hub = 2.0 * (aa - pdc2);
  du[1] = -gx * (u0 * u0) - hub * u0 * u1 + tc2 * u1 * (gy * u2 + gz * u3) +
          div_c(gx, c2, ic2) * (2.0 * (u1 * u1) - vsq);
  du[2] = -gy * (u0 * u0) - hub * u0 * u2 + tc2 * u2 * (gx * u1 + gz * u3) +
          div_c(gy, c2, ic2) * (2.0 * (u2 * u2) - vsq);
  du[3] = -gz * (u0 * u0) - hub * u0 * u3 + tc2 * u3 * (gy * u2 + gx * u1) +
          div_c(gz, c2, ic2) * (2.0 * (u3 * u3) - vsq);
}

// PerturbedFLRWMetricFast.geodesic_equations, perturbed_flrw_metric_fast.py:227-273.
template <class FT, bool SLOW = true>
__device__ __forceinline__ int flrw_rhs(const DevMetric& D, int fi, const double s[8], double out[8]) {
  double a, adot, inv_a;
  int st = scale_factor(D, s[0], a, adot, inv_a);
  if (st) return st;
  InterpOut ip;
  st = interp_field<FT, SLOW>(D.m.fields[fi], D.finv[fi], s[1], s[2], s[3], s[0], ip);
  if (st) return st;
  const double phi_n = div_c(ip.val, D.m.c2, D.ic2);
  const double phid_n = div_c(ip.dtd, D.m.c2, D.ic2);
  double du[4];
  if (D.m.analytical)
    flrw_accel_analytical(D, s[4], s[5], s[6], s[7], a, adot, inv_a, phi_n, ip.gx, ip.gy, ip.gz, phid_n, du);
  else
    flrw_accel_tensorial(D, s[4], s[5], s[6], s[7], a, adot, inv_a, phi_n, ip.gx, ip.gy, ip.gz, phid_n, du);
  out[0] = s[4]; out[1] = s[5]; out[2] = s[6]; out[3] = s[7];
  out[4] = du[0]; out[5] = du[1]; out[6] = du[2]; out[7] = du[3];
  return 0;
}

// ----------------------------------------------------- Schwarzschild RHS
// SchwarzschildMetricFast.geodesic_equations (schwarzschild_metric_fast.py:253-303)
// with _schw_accel_analytical (:104-157) / _schw_accel_tensorial (:12-101),
// spherical (t, r, theta, phi) state.
__device__ __forceinline__ int schw_rhs(const DevMetric& D, const double s[8], double out[8]) {
  const ExcMetric& m = D.m;
  double r = s[1];
  const double th = s[2], ph = s[3];
  if (!isfinite(r) || !isfinite(th) || !isfinite(ph)) return EXC_PH_NONFINITE;
  if (r <= m.radius) r = m.radius;
  if (r <= m.r_s) return EXC_PH_HORIZON;
  const double rs = m.r_s;
  const double u0 = s[4], u1 = s[5], u2 = s[6], u3 = s[7];
  double sn, cs;
  sincos(th, &sn, &cs);
  double u0_out, du0, du1, du2, du3;
  if (m.analytical) {
    double dtdl_eff;
    if (m.free_time) {
      du0 = -(rs / (r * (r - rs))) * u0 * u1;
      dtdl_eff = u0;
    } else {
      const double f = 1.0 - rs / r;
      const double inv_f = 1.0 / f;
      const double inv_f2 = inv_f * inv_f;
      const double v = inv_f2 * (u1 * u1) + (r * r) * inv_f * (u2 * u2) +
                       (r * r) * (sn * sn) * inv_f * (u3 * u3);
      dtdl_eff = -(1.0 / m.c) * sqrt(v);
      du0 = 0.0;
    }
    const double r3 = pow3_cr(r);   // Python `r**3` raises OverflowError on overflow
    if (isinf(r3)) return EXC_PH_NONFINITE;
    du1 = rs / (2.0 * r * (r - rs)) * u1 * u1 -
          (r - rs) / (2.0 * r3) * (m.c2 * rs * dtdl_eff * dtdl_eff - 2.0 * r3 * (u2 * u2 + (sn * sn) * u3 * u3));
    du2 = -2.0 / r * u1 * u2 + sn * cs * u3 * u3;
    du3 = -2.0 / r * u1 * u3 - 2.0 * (cs / sn) * u2 * u3;
    u0_out = dtdl_eff;
  } else {
    const double inv_r = 1.0 / r;
    const double rmrs = r - rs;
    const double inv_rmrs = 1.0 / rmrs;
    const double u0u1 = u0 * u1, u2u2 = u2 * u2, u3u3 = u3 * u3;
    const double G010 = 0.5 * rs * inv_r * inv_rmrs;
    const double G100 = 0.5 * m.c2 * rs * rmrs / (r * r * r);
    const double G111 = -G010;
    const double G122 = -rmrs;
    const double G133 = -rmrs * (sn * sn);
    const double G212 = inv_r;
    const double G233 = -sn * cs;
    const double G313 = inv_r;
    const double G323 = cs / sn;
    du0 = -(2.0 * G010 * u0u1);
    du1 = -(G100 * (u0 * u0) + G111 * (u1 * u1) + G122 * u2u2 + G133 * u3u3);
    du2 = -(2.0 * G212 * u1 * u2 + G233 * u3u3);
    du3 = -(2.0 * G313 * u1 * u3 + 2.0 * G323 * u2 * u3);
    u0_out = u0;
  }
  if (!isfinite(du0)) return EXC_PH_NONFINITE;
  out[0] = u0_out; out[1] = u1; out[2] = u2; out[3] = u3;
  out[4] = du0; out[5] = du1; out[6] = du2; out[7] = du3;
  return 0;
}

// ------------------------------------------------ metric tensor (diagonal)
// PerturbedFLRWMetricFast.metric_tensor (perturbed_flrw_metric_fast.py:126-141) /
// SchwarzschildMetricFast.metric_tensor (schwarzschild_metric_fast.py:190-201).
// Both metrics are diagonal; every off-diagonal entry is 0.
template <class FT, bool SLOW = true>
__device__ __forceinline__ int metric_diag(const DevMetric& D, int fi, const double x[4], double g[4]) {
  const ExcMetric& m = D.m;
  if (m.kind == EXC_METRIC_SCHWARZSCHILD) {
    const double r = x[1];
    const double fr = 1.0 - m.r_s / r;
    const double sn = sin(x[2]);
    g[0] = -fr * m.c2;
    g[1] = 1.0 / fr;
    g[2] = r * r;
    g[3] = (r * r) * (sn * sn);
    return 0;
  }
  double a, adot, inv_a;
  int st = scale_factor(D, x[0], a, adot, inv_a);
  if (st) return st;
  InterpOut ip;
  st = interp_field<FT, SLOW>(m.fields[fi], D.finv[fi], x[1], x[2], x[3], x[0], ip);
  if (st) return st;
  const double phi = ip.val / m.c2;
  const double psi = phi;
  const double a2 = a * a;
  g[0] = -a2 * (1.0 + 2.0 * psi) * m.c2;
  g[1] = a2 * (1.0 - 2.0 * phi);
  g[2] = g[1];
  g[3] = g[1];
  return 0;
}

}  // namespace EXC_NS
