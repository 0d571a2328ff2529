/*
 * exc_oracle.c -- CPU restatement of the reference's photon-geodesic hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker the CUDA tracer is compared against
 * (tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg). Nothing
 * in the shipped package links or calls it.
 *
 * Each function restates one routine of lmagristella/excalibur-tool in the
 * reference's own operation order, in plain C double arithmetic compiled with
 * -ffp-contract=off (no FMA contraction) and glibc libm (the same sin/cos/pow
 * numpy uses on Linux), so it reproduces the reference executed as plain
 * Python. Its outputs are pinned against vectors produced by running the
 * reference itself (tests/golden/make_golden.py).
 *
 * It reads the same ExcMetric / ExcTraceArgs structs as the GPU library
 * (include/excalibur_gb300.h) with HOST pointers.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/excalibur_gb300.h"
#include "../excalibur_tool_gb300/csrc/exc_stepctl.h"

/* ------------------------------------------------------------ helpers */
/* How x**3 and x**4 are evaluated (oracle_set_power_mode):
 *   0 (default) glibc pow(), as the reference's Python/numpy `**` does;
 *   1 the double-double power the CUDA library uses (csrc/exc_device.cuh pow3_cr /
 *     pow4_cr): Dekker's exact square by FMA, the product's error term carried, one final
 *     rounding. The two differ only where pow() misrounds a near-halfway case (by one ulp);
 *     mode 1 lets a test show that such ulps are the only difference between the GPU and the
 *     reference's arithmetic. */
static int g_power_mode = 0;

void oracle_set_power_mode(int mode) { g_power_mode = mode; }
int oracle_power_mode(void) { return g_power_mode; }

static double pow3_dd(double x) {
  const double p = x * x;
  const double e = fma(x, x, -p);
  const double hi = p * x;
  const double lo = fma(p, x, -hi) + e * x;
  return hi + lo;
}

static double pow4_dd(double x) {
  const double p = x * x;
  const double e = fma(x, x, -p);
  const double hi = p * p;
  const double lo = fma(p, p, -hi) + 2.0 * p * e;
  return hi + lo;
}

static double cube(double x) { return g_power_mode ? pow3_dd(x) : pow(x, 3.0); }
static double fourth(double x) { return g_power_mode ? pow4_dd(x) : pow(x, 4.0); }

/* x**3 (p == 3) or x**4 (p == 4) of n values under the current power mode. */
void oracle_power(const double* x, double* out, int64_t n, int p) {
  for (int64_t i = 0; i < n; ++i) out[i] = (p == 4) ? fourth(x[i]) : cube(x[i]);
}

static double py_fmod(double a, double b) { /* CPython float_rem */
  double m = fmod(a, b);
  if (m != 0.0) {
    if ((b < 0.0) != (m < 0.0)) m += b;
  } else {
    m = copysign(0.0, b);
  }
  return m;
}

static int64_t py_imod(int64_t i, int64_t n) {
  int64_t r = i % n;
  if (r != 0 && ((r < 0) != (n < 0))) r += n;
  return r;
}

static double fld(const ExcField* f, int64_t idx) {
  if (f->dtype == EXC_DTYPE_F32) return (double)((const float*)f->data)[idx];
  return ((const double*)f->data)[idx];
}

typedef struct {
  double val, gx, gy, gz, dtd;
} Interp;

/* interpolator_4d_fast.py:29-43 */
static double trilinear(double c000, double c100, double c010, double c001, double c110, double c101,
                        double c011, double c111, double dx, double dy, double dz) {
  return c000 * (1 - dx) * (1 - dy) * (1 - dz) + c100 * dx * (1 - dy) * (1 - dz) +
         c010 * (1 - dx) * dy * (1 - dz) + c001 * (1 - dx) * (1 - dy) * dz + c110 * dx * dy * (1 - dz) +
         c101 * dx * (1 - dy) * dz + c011 * (1 - dx) * dy * dz + c111 * dx * dy * dz;
}

/* One snapshot of fused_interpolation_gradient_3d_{periodic,clamp,error}
 * (interpolator_4d_fast.py:50-255). Returns 0 or an EXC_PH_* code. */
static int snapshot(const ExcField* f, int64_t nt, int64_t it, double x, double y, double z, Interp* o) {
  const int64_t nx = f->n[0], ny = f->n[1], nz = f->n[2];
  const double ox = f->origin[0], oy = f->origin[1], oz = f->origin[2];
  const double sx = f->spacing[0], sy = f->spacing[1], sz = f->spacing[2];
#define IX(i, j, k) (((((int64_t)(i)) * ny + (j)) * nz + (k)) * nt + it)
  double rx, ry, rz, dx, dy, dz;
  int64_t i0, j0, k0;
  if (f->boundary == EXC_BOUNDARY_PERIODIC) {
    const double Lx = (double)nx * sx, Ly = (double)ny * sy, Lz = (double)nz * sz;
    x = ox + py_fmod(x - ox, Lx);
    y = oy + py_fmod(y - oy, Ly);
    z = oz + py_fmod(z - oz, Lz);
    rx = (x - ox) / sx; ry = (y - oy) / sy; rz = (z - oz) / sz;
    if (!isfinite(rx) || !isfinite(ry) || !isfinite(rz)) return EXC_PH_NONFINITE; /* int(nan) raises */
    i0 = (int64_t)floor(rx); j0 = (int64_t)floor(ry); k0 = (int64_t)floor(rz);
    dx = rx - (double)i0; dy = ry - (double)j0; dz = rz - (double)k0;
    i0 = py_imod(i0, nx); j0 = py_imod(j0, ny); k0 = py_imod(k0, nz);
    const int64_t i1 = py_imod(i0 + 1, nx), j1 = py_imod(j0 + 1, ny), k1 = py_imod(k0 + 1, nz);
    o->val = trilinear(fld(f, IX(i0, j0, k0)), fld(f, IX(i1, j0, k0)), fld(f, IX(i0, j1, k0)),
                       fld(f, IX(i0, j0, k1)), fld(f, IX(i1, j1, k0)), fld(f, IX(i1, j0, k1)),
                       fld(f, IX(i0, j1, k1)), fld(f, IX(i1, j1, k1)), dx, dy, dz);
    const int64_t ip = py_imod(i0 + 1, nx), im = py_imod(i0 - 1, nx);
    const int64_t jp = py_imod(j0 + 1, ny), jm = py_imod(j0 - 1, ny);
    const int64_t kp = py_imod(k0 + 1, nz), km = py_imod(k0 - 1, nz);
    o->gx = (fld(f, IX(ip, j0, k0)) - fld(f, IX(im, j0, k0))) / (2.0 * sx);
    o->gy = (fld(f, IX(i0, jp, k0)) - fld(f, IX(i0, jm, k0))) / (2.0 * sy);
    o->gz = (fld(f, IX(i0, j0, kp)) - fld(f, IX(i0, j0, km))) / (2.0 * sz);
    o->dtd = 0.0;
    return 0;
  }
  if (f->boundary == EXC_BOUNDARY_CLAMP) {
    const double ex = 1e-12 * sx, ey = 1e-12 * sy, ez = 1e-12 * sz;
    double hi;
    hi = ox + (nx - 1) * sx - ex; if (x < ox) x = ox; else if (x > hi) x = hi;
    hi = oy + (ny - 1) * sy - ey; if (y < oy) y = oy; else if (y > hi) y = hi;
    hi = oz + (nz - 1) * sz - ez; if (z < oz) z = oz; else if (z > hi) z = hi;
    rx = (x - ox) / sx; ry = (y - oy) / sy; rz = (z - oz) / sz;
    if (!isfinite(rx) || !isfinite(ry) || !isfinite(rz)) return EXC_PH_NONFINITE;
    i0 = (int64_t)floor(rx); j0 = (int64_t)floor(ry); k0 = (int64_t)floor(rz);
    if (i0 < 0) i0 = 0;
    if (j0 < 0) j0 = 0;
    if (k0 < 0) k0 = 0;
    if (i0 > nx - 2) i0 = nx - 2;
    if (j0 > ny - 2) j0 = ny - 2;
    if (k0 > nz - 2) k0 = nz - 2;
    dx = rx - (double)i0; dy = ry - (double)j0; dz = rz - (double)k0;
    o->val = trilinear(fld(f, IX(i0, j0, k0)), fld(f, IX(i0 + 1, j0, k0)), fld(f, IX(i0, j0 + 1, k0)),
                       fld(f, IX(i0, j0, k0 + 1)), fld(f, IX(i0 + 1, j0 + 1, k0)), fld(f, IX(i0 + 1, j0, k0 + 1)),
                       fld(f, IX(i0, j0 + 1, k0 + 1)), fld(f, IX(i0 + 1, j0 + 1, k0 + 1)), dx, dy, dz);
    /* interpolator_4d_fast.py:152-186: one-sided at the low edge, central otherwise */
    if (i0 <= 0) o->gx = (fld(f, IX(1, j0, k0)) - fld(f, IX(0, j0, k0))) / sx;
    else o->gx = (fld(f, IX(i0 + 1, j0, k0)) - fld(f, IX(i0 - 1, j0, k0))) / (2.0 * sx);
    if (j0 <= 0) o->gy = (fld(f, IX(i0, 1, k0)) - fld(f, IX(i0, 0, k0))) / sy;
    else o->gy = (fld(f, IX(i0, j0 + 1, k0)) - fld(f, IX(i0, j0 - 1, k0))) / (2.0 * sy);
    if (k0 <= 0) o->gz = (fld(f, IX(i0, j0, 1)) - fld(f, IX(i0, j0, 0))) / sz;
    else o->gz = (fld(f, IX(i0, j0, k0 + 1)) - fld(f, IX(i0, j0, k0 - 1))) / (2.0 * sz);
    o->dtd = 0.0;
    return 0;
  }
  rx = (x - ox) / sx; ry = (y - oy) / sy; rz = (z - oz) / sz;
  if (rx < 1.0 || rx >= (nx - 2.0) || ry < 1.0 || ry >= (ny - 2.0) || rz < 1.0 || rz >= (nz - 2.0))
    return EXC_PH_OUTSIDE_GRID;
  if (!isfinite(rx) || !isfinite(ry) || !isfinite(rz)) return EXC_PH_NONFINITE;
  i0 = (int64_t)floor(rx); j0 = (int64_t)floor(ry); k0 = (int64_t)floor(rz);
  dx = rx - (double)i0; dy = ry - (double)j0; dz = rz - (double)k0;
  o->val = trilinear(fld(f, IX(i0, j0, k0)), fld(f, IX(i0 + 1, j0, k0)), fld(f, IX(i0, j0 + 1, k0)),
                     fld(f, IX(i0, j0, k0 + 1)), fld(f, IX(i0 + 1, j0 + 1, k0)), fld(f, IX(i0 + 1, j0, k0 + 1)),
                     fld(f, IX(i0, j0 + 1, k0 + 1)), fld(f, IX(i0 + 1, j0 + 1, k0 + 1)), dx, dy, dz);
  o->gx = (fld(f, IX(i0 + 1, j0, k0)) - fld(f, IX(i0 - 1, j0, k0))) / (2.0 * sx);
  o->gy = (fld(f, IX(i0, j0 + 1, k0)) - fld(f, IX(i0, j0 - 1, k0))) / (2.0 * sy);
  o->gz = (fld(f, IX(i0, j0, k0 + 1)) - fld(f, IX(i0, j0, k0 - 1))) / (2.0 * sz);
  o->dtd = 0.0;
  return 0;
#undef IX
}

/* ---- the slow Interpolator (grid/interpolator.py), grad_mode EXC_GRAD_TRILINEAR */

/* f[a] - f[b]: numpy subtracts two float32 elements in float32 (:147-152). */
static double node_diff(const ExcField* f, int64_t a, int64_t b) {
  if (f->dtype == EXC_DTYPE_F32) {
    const float* p = (const float*)f->data;
    const float d = p[a] - p[b];
    return (double)d;
  }
  return fld(f, a) - fld(f, b);
}

/* np.sum of eight float64 terms: numpy's pairwise sum keeps eight partial sums
 * r[j] (here one term each) and adds them as ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)). */
static double np_sum8(const double p[8]) {
  return ((p[0] + p[1]) + (p[2] + p[3])) + ((p[4] + p[5]) + (p[6] + p[7]));
}

/* np.clip of a floored coordinate to [lo, hi] (lo <= hi). */
static int64_t clip_floor(double v, int64_t lo, int64_t hi) {
  if (!(v > (double)lo)) return lo;
  if (v >= (double)hi) return hi;
  return (int64_t)v;
}

/* Interpolator.gradient (:88-158) on snapshot `it` of nt. */
static void slow_gradient(const ExcField* f, int64_t nt, int64_t it, double rx, double ry, double rz, Interp* o) {
  const int64_t nx = f->n[0], ny = f->n[1], nz = f->n[2];
#define IX(i, j, k) (((((int64_t)(i)) * ny + (j)) * nz + (k)) * nt + it)
  const double flx = floor(rx), fly = floor(ry), flz = floor(rz);
  const double wx = rx - flx, wy = ry - fly, wz = rz - flz;
  /* :102-106, base index clipped to [1, n-2]; the fraction is not */
  const int64_t bi = clip_floor(flx, 1, nx - 2), bj = clip_floor(fly, 1, ny - 2), bk = clip_floor(flz, 1, nz - 2);
  /* corners and weights in the order of :117-138 */
  static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  const double w[8] = {(1 - wx) * (1 - wy) * (1 - wz), wx * (1 - wy) * (1 - wz), (1 - wx) * wy * (1 - wz),
                       (1 - wx) * (1 - wy) * wz,       wx * wy * (1 - wz),       wx * (1 - wy) * wz,
                       (1 - wx) * wy * wz,             wx * wy * wz};
  double px[8], py[8], pz[8];
  for (int c = 0; c < 8; ++c) {
    int64_t i = bi + off[c][0], j = bj + off[c][1], k = bk + off[c][2];
    if (i > nx - 2) i = nx - 2; /* :144-146 (the lower clip cannot bind: base >= 1) */
    if (j > ny - 2) j = ny - 2;
    if (k > nz - 2) k = nz - 2;
    px[c] = node_diff(f, IX(i + 1, j, k), IX(i - 1, j, k)) / (2 * f->spacing[0]) * w[c];
    py[c] = node_diff(f, IX(i, j + 1, k), IX(i, j - 1, k)) / (2 * f->spacing[1]) * w[c];
    pz[c] = node_diff(f, IX(i, j, k + 1), IX(i, j, k - 1)) / (2 * f->spacing[2]) * w[c];
  }
  o->gx = np_sum8(px);
  o->gy = np_sum8(py);
  o->gz = np_sum8(pz);
#undef IX
}

/* Interpolator.value_gradient_and_time_derivative (:198-206). Only the bounds
 * check raises there: NaN grid values pass through. */
static int slow_interp(const ExcField* f, double x, double y, double z, double t, Interp* o) {
  const int64_t nx = f->n[0], ny = f->n[1], nz = f->n[2];
  /* _index_and_weights (:13-44) */
  const double rx = (x - f->origin[0]) / f->spacing[0];
  const double ry = (y - f->origin[1]) / f->spacing[1];
  const double rz = (z - f->origin[2]) / f->spacing[2];
  if (rx < 0 || rx >= (double)(nx - 1) || ry < 0 || ry >= (double)(ny - 1) || rz < 0 || rz >= (double)(nz - 1))
    return EXC_PH_OUTSIDE_GRID;
  if (!isfinite(rx) || !isfinite(ry) || !isfinite(rz)) return EXC_PH_NONFINITE;
  const double flx = floor(rx), fly = floor(ry), flz = floor(rz);
  const int64_t i0 = (int64_t)flx, j0 = (int64_t)fly, k0 = (int64_t)flz;
  const double wx = rx - flx, wy = ry - fly, wz = rz - flz;
  if (f->ndim != 4) {
#define IX(i, j, k) ((((int64_t)(i)) * ny + (j)) * nz + (k))
    /* _interpolate_3d (:52-69) */
    o->val = trilinear(fld(f, IX(i0, j0, k0)), fld(f, IX(i0 + 1, j0, k0)), fld(f, IX(i0, j0 + 1, k0)),
                       fld(f, IX(i0, j0, k0 + 1)), fld(f, IX(i0 + 1, j0 + 1, k0)), fld(f, IX(i0 + 1, j0, k0 + 1)),
                       fld(f, IX(i0, j0 + 1, k0 + 1)), fld(f, IX(i0 + 1, j0 + 1, k0 + 1)), wx, wy, wz);
#undef IX
    slow_gradient(f, 1, 0, rx, ry, rz, o);
    o->dtd = 0.0;
    return 0;
  }
  const int64_t nt = f->n[3];
#define IX(i, j, k, l) (((((int64_t)(i)) * ny + (j)) * nz + (k)) * nt + (l))
  const double rt = (t - f->origin[3]) / f->spacing[3];
  if (!isfinite(rt)) return EXC_PH_NONFINITE;
  const double flt = floor(rt);
  const double wt = rt - flt;
  /* _interpolate_4d (:71-86): weights ((wx_a * wy_b) * wz_c) * wt_e, the sixteen
   * products summed in C order by numpy's pairwise sum (eight partial sums) */
  const int64_t l0 = clip_floor(flt, 0, nt - 2);
  const double Wx[2] = {1 - wx, wx}, Wy[2] = {1 - wy, wy}, Wz[2] = {1 - wz, wz}, Wt[2] = {1 - wt, wt};
  double r[8];
  for (int q = 0; q < 16; ++q) {
    const int a = q >> 3, b = (q >> 2) & 1, c = (q >> 1) & 1, e = q & 1;
    const double p = fld(f, IX(i0 + a, j0 + b, k0 + c, l0 + e)) * (((Wx[a] * Wy[b]) * Wz[c]) * Wt[e]);
    if (q < 8) r[q] = p;
    else r[q - 8] += p;
  }
  o->val = np_sum8(r);
  /* gradient on the nearest snapshot (:92-96): np.round is round-half-even */
  slow_gradient(f, nt, clip_floor(nearbyint(rt), 0, nt - 1), rx, ry, rz, o);
  /* time_derivative (:160-174): np.clip(floor, 1, nt-2) is nt-2 when nt-2 < 1,
   * and Python index -1 is the last snapshot */
  double lv = flt > 1.0 ? flt : 1.0;
  if (lv > (double)(nt - 2)) lv = (double)(nt - 2);
  const int64_t lt = (int64_t)lv;
  const int64_t lp = lt - 1 < 0 ? lt - 1 + nt : lt - 1, ln = lt + 1;
  double v[2];
  for (int s = 0; s < 2; ++s) {
    const int64_t l = s ? ln : lp;
    v[s] = trilinear(fld(f, IX(i0, j0, k0, l)), fld(f, IX(i0 + 1, j0, k0, l)), fld(f, IX(i0, j0 + 1, k0, l)),
                     fld(f, IX(i0, j0, k0 + 1, l)), fld(f, IX(i0 + 1, j0 + 1, k0, l)),
                     fld(f, IX(i0 + 1, j0, k0 + 1, l)), fld(f, IX(i0, j0 + 1, k0 + 1, l)),
                     fld(f, IX(i0 + 1, j0 + 1, k0 + 1, l)), wx, wy, wz);
  }
#undef IX
  o->dtd = (v[1] - v[0]) / (2 * f->spacing[3]);
  return 0;
}

/* InterpolatorFast.value_gradient_and_time_derivative (interpolator_4d_fast.py:443-502);
 * grad_mode EXC_GRAD_TRILINEAR selects the slow Interpolator. */
int oracle_interp_one(const ExcField* f, double x, double y, double z, double t, double out[5]) {
  Interp o;
  int st;
  /* _ShiftedInterpolator (excalibur_run_compare_schwarzschild_vs_flrw.py:50-52):
   * the query point is x + shift, one float64 addition per component */
  x = x + f->shift[0];
  y = y + f->shift[1];
  z = z + f->shift[2];
  if (f->grad_mode == EXC_GRAD_TRILINEAR) {
    st = slow_interp(f, x, y, z, t, &o);
  } else if (f->ndim != 4) {
    st = snapshot(f, 1, 0, x, y, z, &o);
    if (!st && isnan(o.val)) st = EXC_PH_OUTSIDE_GRID;
  } else {
    const int64_t nt = f->n[3];
    const double ot = f->origin[3], stp = f->spacing[3];
    double rt;
    if (f->boundary == EXC_BOUNDARY_CLAMP) {
      const double hi = ot + (nt - 1) * stp - 1e-12 * stp;
      if (t < ot) t = ot; else if (t > hi) t = hi;
      rt = (t - ot) / stp;
    } else {
      rt = (t - ot) / stp;
      if (rt < 0.0 || rt >= (nt - 1.0)) { st = EXC_PH_OUTSIDE_GRID; goto done; }
    }
    if (!isfinite(rt)) { st = EXC_PH_NONFINITE; goto done; }
    int64_t it0 = (int64_t)floor(rt);
    if (it0 < 0) it0 = 0;
    if (it0 > nt - 2) it0 = nt - 2;
    const double wt = rt - (double)it0;
    Interp a, b;
    st = snapshot(f, nt, it0, x, y, z, &a);
    if (!st) st = snapshot(f, nt, it0 + 1, x, y, z, &b);
    if (!st && (isnan(a.val) || isnan(b.val))) st = EXC_PH_OUTSIDE_GRID;
    if (!st) {
      o.val = (1.0 - wt) * a.val + wt * b.val;
      o.gx = (1.0 - wt) * a.gx + wt * b.gx;
      o.gy = (1.0 - wt) * a.gy + wt * b.gy;
      o.gz = (1.0 - wt) * a.gz + wt * b.gz;
      o.dtd = (b.val - a.val) / stp;
    }
  }
done:
  if (st) {
    for (int i = 0; i < 5; ++i) out[i] = NAN;
    return st;
  }
  out[0] = o.val; out[1] = o.gx; out[2] = o.gy; out[3] = o.gz; out[4] = o.dtd;
  return 0;
}

/* ---------------------------------------------------------- cosmology */
/* a_interp_numba, cosmology.py:8-25 */
static double a_interp(const ExcMetric* m, double eta, int* st) {
  const double* tab = m->a_table;
  const int64_t n = m->a_table_n;
  if (eta <= m->eta_min) return tab[0];
  const double max_eta = m->eta_min + m->eta_step * (n - 1);
  if (eta >= max_eta) return tab[n - 1];
  if (isnan(eta)) { *st = EXC_PH_NONFINITE; return NAN; }
  int64_t i = (int64_t)((eta - m->eta_min) / m->eta_step);
  if (i > n - 2) i = n - 2; /* within an ulp of the table end */
  const double t = (eta - (m->eta_min + i * m->eta_step)) / m->eta_step;
  return (1 - t) * tab[i] + t * tab[i + 1];
}

/* perturbed_flrw_metric_fast.py:190-225 with LCDM_Cosmology.adot_of_eta (cosmology.py:69-93) */
static int scale_factor(const ExcMetric* m, double eta, double* a_out, double* adot_out) {
  int st = 0;
  double a, adot;
  if (m->cosmology == EXC_COSMO_STATIC) {
    a = 1.0;
    adot = 0.0;
  } else if (m->cosmology == EXC_COSMO_TABLE) {
    a = a_interp(m, eta, &st);
    const double z = 1.0 / a - 1.0;
    const double E = sqrt(m->omega_m * cube(1 + z) + m->omega_r * fourth(1 + z) +
                          m->omega_k * pow(1 + z, 2.0) + m->omega_lambda);
    adot = a * a * (m->H0 * E);
  } else {
    a = a_interp(m, eta, &st);
    const double h = fmax(1e-6 * fabs(eta), 1e-6);
    adot = (a_interp(m, eta + h, &st) - a_interp(m, eta - h, &st)) / (2 * h);
  }
  if (st) return st;
  if (!isfinite(a) || fabs(a) < 1e-30) a = 1e-30;
  if (!isfinite(adot)) adot = 0.0;
  *a_out = a;
  *adot_out = adot;
  return 0;
}

int oracle_cosmology(const ExcMetric* m, const double* eta, double* a, double* adot, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    double aa = NAN, ad = NAN;
    int st = scale_factor(m, eta[i], &aa, &ad);
    if (a) a[i] = st ? NAN : aa;
    if (adot) adot[i] = st ? NAN : ad;
  }
  return 0;
}

/* --------------------------------------------------------------- RHS */
static int flrw_rhs(const ExcMetric* m, int fi, const double* s, double* out) {
  double a, adot, ip[5];
  int st = scale_factor(m, s[0], &a, &adot);
  if (st) return st;
  st = oracle_interp_one(&m->fields[fi], s[1], s[2], s[3], s[0], ip);
  if (st) return st;
  const double c2 = m->c2, c4 = m->c4;
  const double phi = ip[0] / c2, phi_dot = ip[4] / c2;
  const double gx = ip[1], gy = ip[2], gz = ip[3];
  const double u0 = s[4], u1 = s[5], u2 = s[6], u3 = s[7];
  double du0, du1, du2, du3;
  if (!m->analytical) {
    /* compute_tensorial_acceleration, perturbed_flrw_metric_fast.py:7-76 */
    const double a2 = a * a, adot_a = adot / a;
    const double usq = u1 * u1 + u2 * u2 + u3 * u3;
    const double psi = phi;
    const double G000 = (phi_dot / c2) * u0 * u0;
    const double G0ij = (a * adot / c2 + 2 * a * adot / c4 * (phi + psi) - a2 / c4 * phi_dot) * usq;
    const double G00i = 2 * ((gx / c2) * u0 * u1 + (gy / c2) * u0 * u2 + (gz / c2) * u0 * u3);
    du0 = -(G000 + G0ij + G00i);
    du1 = -((gx) / a2 * u0 * u0 + 2 * (adot_a - phi_dot / c2) * u0 * u1 +
            (-(gx / c2) * u1 * u1 + (gx / c2) * (u2 * u2 + u3 * u3) + (-(gy / c2)) * u1 * u2 +
             (-(gz / c2)) * u1 * u3));
    du2 = -((gy) / a2 * u0 * u0 + 2 * (adot_a - phi_dot / c2) * u0 * u2 +
            (-(gy / c2) * u2 * u2 + (gy / c2) * (u1 * u1 + u3 * u3) + (-(gx / c2)) * u2 * u1 +
             (-(gz / c2)) * u2 * u3));
    du3 = -((gz) / a2 * u0 * u0 + 2 * (adot_a - phi_dot / c2) * u0 * u3 +
            (-(gz / c2) * u3 * u3 + (gz / c2) * (u1 * u1 + u2 * u2) + (-(gx / c2)) * u3 * u1 +
             (-(gy / c2)) * u3 * u2));
  } else {
    /* compute_analytical_acceleration, perturbed_flrw_metric_fast.py:78-99 */
    const double tc2 = m->two_over_c2;
    const double vsq = u1 * u1 + u2 * u2 + u3 * u3;
    const double dpl = gx * u1 + gy * u2 + gz * u3;
    const double psi = phi;
    du0 = -(adot / a + phi_dot / c2) * (u0 * u0) - tc2 * u0 * dpl -
          (adot / a / c2 - 2 * adot / a / c4 * (phi + psi) - phi_dot / c4) * vsq;
    du1 = -gx * (u0 * u0) - 2 * (adot / a - phi_dot / c2) * u0 * u1 + tc2 * u1 * (gy * u2 + gz * u3) +
          gx / c2 * (2 * (u1 * u1) - vsq);
    du2 = -gy * (u0 * u0) - 2 * (adot / a - phi_dot / c2) * u0 * u2 + tc2 * u2 * (gx * u1 + gz * u3) +
          gy / c2 * (2 * (u2 * u2) - vsq);
    du3 = -gz * (u0 * u0) - 2 * (adot / a - phi_dot / c2) * u0 * u3 + tc2 * u3 * (gy * u2 + gx * u1) +
          gz / c2 * (2 * (u3 * u3) - vsq);
  }
  out[0] = u0; out[1] = u1; out[2] = u2; out[3] = u3;
  out[4] = du0; out[5] = du1; out[6] = du2; out[7] = du3;
  return 0;
}

/* schwarzschild_metric_fast.py:253-303 with :12-157 */
static int schw_rhs(const ExcMetric* m, const double* s, double* out) {
  double r = s[1];
  const double th = s[2], ph = s[3];
  if (!isfinite(r) || !isfinite(th) || !isfinite(ph)) return EXC_PH_NONFINITE;
  if (r <= m->radius) r = m->radius;
  if (r <= m->r_s) return EXC_PH_HORIZON;
  const double rs = m->r_s;
  const double u0 = s[4], u1 = s[5], u2 = s[6], u3 = s[7];
  const double sn = sin(th), cs = cos(th);
  double u0_out, du0, du1, du2, du3;
  if (m->analytical) {
    double dte;
    if (m->free_time) {
      du0 = -(rs / (r * (r - rs))) * u0 * u1;
      dte = u0;
    } else {
      const double f = 1.0 - rs / r, inv_f = 1.0 / f, inv_f2 = inv_f * inv_f;
      const double v = inv_f2 * (u1 * u1) + (r * r) * inv_f * (u2 * u2) + (r * r) * (sn * sn) * inv_f * (u3 * u3);
      dte = -(1.0 / m->c) * sqrt(v);
      du0 = 0.0;
    }
    const double r3 = cube(r);
    if (isinf(r3)) return EXC_PH_NONFINITE; /* Python float ** int raises OverflowError */
    du1 = rs / (2.0 * r * (r - rs)) * u1 * u1 -
          (r - rs) / (2.0 * r3) * (m->c2 * rs * dte * dte - 2.0 * r3 * (u2 * u2 + (sn * sn) * u3 * u3));
    du2 = -2.0 / r * u1 * u2 + sn * cs * u3 * u3;
    du3 = -2.0 / r * u1 * u3 - 2.0 * (cs / sn) * u2 * u3;
    u0_out = dte;
  } else {
    const double inv_r = 1.0 / r, rmrs = r - rs, inv_rmrs = 1.0 / rmrs;
    const double G010 = 0.5 * rs * inv_r * inv_rmrs;
    const double G100 = 0.5 * m->c2 * rs * (rmrs) / (r * r * r);
    du0 = -(2.0 * G010 * (u0 * u1));
    du1 = -(G100 * (u0 * u0) + (-G010) * (u1 * u1) + (-(rmrs)) * (u2 * u2) + (-(rmrs) * (sn * sn)) * (u3 * u3));
    du2 = -(2.0 * inv_r * u1 * u2 + (-sn * cs) * (u3 * u3));
    du3 = -(2.0 * inv_r * u1 * u3 + 2.0 * (cs / sn) * u2 * u3);
    u0_out = u0;
  }
  if (!isfinite(du0)) return EXC_PH_NONFINITE;
  out[0] = u0_out; out[1] = u1; out[2] = u2; out[3] = u3;
  out[4] = du0; out[5] = du1; out[6] = du2; out[7] = du3;
  return 0;
}

static int rhs(const ExcMetric* m, int fi, const double* s, double* out) {
  return m->kind == EXC_METRIC_SCHWARZSCHILD ? schw_rhs(m, s, out) : flrw_rhs(m, fi, s, out);
}

int oracle_rhs(const ExcMetric* m, const double* states, double* out, int32_t* status, const int32_t* fidx,
               int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    double o[8];
    int st = rhs(m, fidx ? fidx[i] : 0, states + 8 * i, o);
    for (int k = 0; k < 8; ++k) out[8 * i + k] = st ? NAN : o[k];
    if (status) status[i] = st;
  }
  return 0;
}

/* metric_tensor diagonal (perturbed_flrw_metric_fast.py:126-141; schwarzschild_metric_fast.py:190-201) */
static int metric_diag(const ExcMetric* m, int fi, const double* x, double* g) {
  if (m->kind == EXC_METRIC_SCHWARZSCHILD) {
    const double r = x[1], f = 1.0 - m->r_s / r, sn = sin(x[2]);
    g[0] = -f * m->c2;
    g[1] = 1.0 / f;
    g[2] = r * r;
    g[3] = (r * r) * (sn * sn);
    return 0;
  }
  double a, adot, ip[5];
  int st = scale_factor(m, x[0], &a, &adot);
  if (st) return st;
  st = oracle_interp_one(&m->fields[fi], x[1], x[2], x[3], x[0], ip);
  if (st) return st;
  const double phi = ip[0] / m->c2, psi = phi;
  g[0] = -(a * a) * (1 + 2 * psi) * m->c2;
  g[1] = g[2] = g[3] = (a * a) * (1 - 2 * phi);
  return 0;
}

int oracle_metric_tensor(const ExcMetric* m, const double* x, double* g, int32_t* status, const int32_t* fidx,
                         int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    double gg[4];
    int st = metric_diag(m, fidx ? fidx[i] : 0, x + 4 * i, gg);
    for (int k = 0; k < 4; ++k) g[4 * i + k] = st ? NAN : gg[k];
    if (status) status[i] = st;
  }
  return 0;
}

/* Photons._solve_u0_from_null_condition, photons.py:540-568 */
int oracle_null_init(const ExcMetric* m, double* states, double sign, int32_t* status, const int32_t* fidx,
                     int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    double* s = states + 8 * i, g[4];
    int st = metric_diag(m, fidx ? fidx[i] : 0, s, g);
    if (status) status[i] = st;
    if (st) continue;
    const double sp = g[1] * (s[5] * s[5]) + g[2] * (s[6] * s[6]) + g[3] * (s[7] * s[7]);
    const double u0_sq = g[0] != 0 ? -sp / g[0] : NAN;
    s[4] = sign * (isfinite(u0_sq) ? sqrt(fabs(u0_sq)) : 1.0);
  }
  return 0;
}

/* Photon.null_condition_relative_error, photon.py:46-68 */
int oracle_null_error(const ExcMetric* m, const double* states, double* rel, int32_t* status, const int32_t* fidx,
                      int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    const double* s = states + 8 * i;
    double g[4];
    int st = metric_diag(m, fidx ? fidx[i] : 0, s, g);
    if (status) status[i] = st;
    if (st) { rel[i] = NAN; continue; }
    const double norm = s[4] * (g[0] * s[4]) + s[5] * (g[1] * s[5]) + s[6] * (g[2] * s[6]) + s[7] * (g[3] * s[7]);
    const double den = fabs(g[0] * (s[4] * s[4])) + fabs(g[1] * (s[5] * s[5])) + fabs(g[2] * (s[6] * s[6])) +
                       fabs(g[3] * (s[7] * s[7]));
    rel[i] = den > 0 ? fabs(norm) / den : fabs(norm);
  }
  return 0;
}

/* ----------------------------------------------------------- steppers */
/* RK4.step, integrator.py:10-22 */
static int step_rk4(const ExcMetric* m, int fi, const double* s, double dt, double* out) {
  double k1[8], k2[8], k3[8], k4[8], t[8];
  int st;
  if ((st = rhs(m, fi, s, k1))) return st;
  for (int i = 0; i < 8; ++i) t[i] = s[i] + 0.5 * dt * k1[i];
  if ((st = rhs(m, fi, t, k2))) return st;
  for (int i = 0; i < 8; ++i) t[i] = s[i] + 0.5 * dt * k2[i];
  if ((st = rhs(m, fi, t, k3))) return st;
  for (int i = 0; i < 8; ++i) t[i] = s[i] + dt * k3[i];
  if ((st = rhs(m, fi, t, k4))) return st;
  for (int i = 0; i < 8; ++i) out[i] = s[i] + (dt / 6) * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]);
  return 0;
}

/* Leapfrog4.step, integrator.py:24-90 (class constants as float64) */
static int step_lf4(const ExcMetric* m, int fi, const double* s, double dt, double* out) {
  const double w0 = -0x1.b3d16dd72c671p+0, w1 = 0x1.59e8b6eb96339p+0;
  const double c1 = 0x1.59e8b6eb96339p-1, c2 = -0x1.67a2dbae58ce0p-3;
  const double cs[4] = {c1, c2, c2, c1}, ds[3] = {w1, w0, w1};
  double y[8], k[8];
  memcpy(y, s, sizeof(y));
  for (int stage = 0; stage < 3; ++stage) {
    for (int i = 0; i < 4; ++i) y[i] += cs[stage] * dt * y[4 + i];
    int st = rhs(m, fi, y, k);
    if (st) return st;
    for (int i = 0; i < 4; ++i) y[4 + i] += ds[stage] * dt * k[4 + i];
  }
  for (int i = 0; i < 4; ++i) y[i] += cs[3] * dt * y[4 + i];
  memcpy(out, y, sizeof(y));
  return 0;
}

/* RK45Adaptive.step, integrator.py:93-152 */
static int step_rk45(const ExcMetric* m, int fi, int tableau, const double* s, double dt, double rtol, double atol,
                     double* out, double* dt_new, int* accepted) {
  static const double B[6][6] = {
      {0, 0, 0, 0, 0, 0},
      {1.0 / 4, 0, 0, 0, 0, 0},
      {3.0 / 32, 9.0 / 32, 0, 0, 0, 0},
      {1932.0 / 2197, -7200.0 / 2197, 7296.0 / 2197, 0, 0, 0},
      {439.0 / 216, -8, 3680.0 / 513, -845.0 / 4104, 0, 0},
      {-8.0 / 27, 2, -3544.0 / 2565, 1859.0 / 4104, -11.0 / 40, 0}};
  double C5[6] = {16.0 / 135, 0, 665.0 / 1287, 28561.0 / 56430, -9.0 / 50, 2.0 / 55};
  static const double C4[6] = {25.0 / 216, 0, 1408.0 / 2565, 2197.0 / 4104, -1.0 / 5, 0};
  if (tableau == EXC_TABLEAU_FEHLBERG) C5[2] = 6656.0 / 12825;
  double K[6][8];
  memset(K, 0, sizeof(K));
  int st;
  if ((st = rhs(m, fi, s, K[0]))) return st;
  for (int i = 1; i < 6; ++i) {
    double y[8];
    for (int q = 0; q < 8; ++q) {
      const double incr = B[i][0] * K[0][q] + B[i][1] * K[1][q] + B[i][2] * K[2][q] + B[i][3] * K[3][q] +
                          B[i][4] * K[4][q] + B[i][5] * K[5][q];
      y[q] = s[q] + dt * incr;
    }
    if ((st = rhs(m, fi, y, K[i]))) return st;
  }
  double r2[8];
  for (int q = 0; q < 8; ++q) {
    double d5 = 0.0, d4 = 0.0;
    for (int j = 0; j < 6; ++j) { d5 += C5[j] * K[j][q]; d4 += C4[j] * K[j][q]; }
    const double y5 = s[q] + dt * d5, y4 = s[q] + dt * d4;
    const double a0 = fabs(s[q]), a1 = fabs(y5);
    const double mx = (isnan(a0) || isnan(a1)) ? NAN : (a0 > a1 ? a0 : a1);
    const double r = (y5 - y4) / (atol + rtol * mx);
    r2[q] = r * r;
    out[q] = y5;
  }
  const double err = sqrt((((r2[0] + r2[1]) + (r2[2] + r2[3])) + ((r2[4] + r2[5]) + (r2[6] + r2[7]))) / 8);
  if (err <= 1.0) {
    const double g = err > 0 ? 0.9 * exc_ctl_pow_m1_5(err) : 5.0;
    *dt_new = dt * (g < 5.0 ? g : 5.0);
    *accepted = 1;
  } else {
    const double g = 0.9 * exc_ctl_pow_m1_4(err);
    *dt_new = dt * (g > 0.1 ? g : 0.1);
    *accepted = 0;
    memcpy(out, s, 8 * sizeof(double)); /* a rejected trial returns the input state */
  }
  return 0;
}

/* Integrator._renormalize_state_to_null, integrator.py:298-335 */
static int renormalize(const ExcMetric* m, int fi, double* s) {
  double g[4];
  int st = metric_diag(m, fi, s, g);
  if (st) return st;
  const double A = g[0], Bc = 2.0 * (0.0 * s[5] + 0.0 * s[6] + 0.0 * s[7]);
  const double Cc = s[5] * (g[1] * s[5]) + s[6] * (g[2] * s[6]) + s[7] * (g[3] * s[7]);
  if (fabs(A) < 1e-300) return 0;
  const double disc = Bc * Bc - 4.0 * A * Cc;
  if (disc < 0) return 0;
  const double sq = sqrt(disc), ua = (-Bc + sq) / (2.0 * A), ub = (-Bc - sq) / (2.0 * A);
  s[4] = fabs(ua - s[4]) <= fabs(ub - s[4]) ? ua : ub;
  return 0;
}

/* ------------------------------------------------------ observables */
static void cart_pos(const ExcMetric* m, const double* s, double* p) {
  if (m->kind == EXC_METRIC_SCHWARZSCHILD) {
    p[0] = s[1] * sin(s[2]) * cos(s[3]);
    p[1] = s[1] * sin(s[2]) * sin(s[3]);
    p[2] = s[1] * cos(s[2]);
  } else {
    p[0] = s[1]; p[1] = s[2]; p[2] = s[3];
  }
}

static void cart_vel(const ExcMetric* m, const double* s, double* v) {
  if (m->kind == EXC_METRIC_SCHWARZSCHILD) { /* analyze_compare_trajectories.py:99-112 */
    const double st = sin(s[2]), ct = cos(s[2]), sp = sin(s[3]), cp = cos(s[3]);
    const double r = s[1], dr = s[5], dth = s[6], dph = s[7];
    v[0] = dr * (st * cp) + (r * dth) * (ct * cp) + (r * st * dph) * (-sp);
    v[1] = dr * (st * sp) + (r * dth) * (ct * sp) + (r * st * dph) * (cp);
    v[2] = dr * (ct) + (r * dth) * (-st);
  } else {
    v[0] = s[5]; v[1] = s[6]; v[2] = s[7];
  }
}

static double norm3(const double* v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

/* |d| - d.e (e a unit vector) without cancellation: |d x e|^2 / (|d| + d.e), in double in
 * this order, as the CUDA library evaluates the time-delay excess (csrc/exc_kernels.cuh). The
 * reference itself has no such column: its time delay is path - chord over the recorded
 * positions (_postprocessing/compute_time_delay_map.py:112-126), the PATH and CHORD columns. */
static double excess_term(const double* d, const double* e) {
  const double nd = norm3(d);
  const double de = d[0] * e[0] + d[1] * e[1] + d[2] * e[2];
  if (de <= 0.0) return nd - de;
  const double cx = d[1] * e[2] - d[2] * e[1];
  const double cy = d[2] * e[0] - d[0] * e[2];
  const double cz = d[0] * e[1] - d[1] * e[0];
  const double den = nd + de;
  return den > 0.0 ? (cx * cx + cy * cy + cz * cz) / den : 0.0;
}

static int quantities(const ExcMetric* m, int fi, const double* s, double* q) {
  if (m->kind == EXC_METRIC_SCHWARZSCHILD) {
    q[0] = s[1]; q[1] = m->mass; q[2] = m->radius; q[3] = m->r_s; q[4] = NAN; q[5] = NAN;
    return 0;
  }
  double a, adot, ip[5];
  int st = scale_factor(m, s[0], &a, &adot);
  if (st) return st;
  st = oracle_interp_one(&m->fields[fi], s[1], s[2], s[3], s[0], ip);
  if (st) return st;
  q[0] = a; q[1] = ip[0]; q[2] = ip[1]; q[3] = ip[2]; q[4] = ip[3]; q[5] = ip[4];
  return 0;
}

static void write_record(const ExcTraceArgs* A, int64_t p, int* nrec, const double* s, const double* q) {
  if (*nrec < A->max_records) {
    double* row = A->records + (p * A->max_records + *nrec) * A->record_cols;
    for (int i = 0; i < 8; ++i) row[i] = s[i];
    for (int i = 8; i < A->record_cols; ++i) row[i] = q ? q[i - 8] : NAN;
  }
  (*nrec)++;
}

static double clip(double x, double lo, double hi) {
  if (isnan(x) || isnan(lo) || isnan(hi)) return NAN;
  return fmin(fmax(x, lo), hi);
}

/* EXC_STOP_FACE (FLRW): lambda >= 0 at which x + lambda * sign(dt) * u first reaches a face of
 * the stop box; a step that would come within EXC_FACE_MARGIN of it ends there instead. */
static double face_clip(const double* s, double dt, const double* lo, const double* hi, int* clipped) {
  const double sg = dt < 0.0 ? -1.0 : 1.0;
  double tmin = INFINITY;
  for (int d = 0; d < 3; ++d) {
    const double v = sg * s[5 + d];
    if (v > 0.0) tmin = fmin(tmin, (hi[d] - s[1 + d]) / v);
    else if (v < 0.0) tmin = fmin(tmin, (lo[d] - s[1 + d]) / v);
  }
  *clipped = tmin < EXC_FACE_MARGIN * fabs(dt);
  return *clipped ? sg * fmax(tmin, 0.0) : dt;
}

/* Integrator.integrate_single, integrator.py:218-409, plus the box / a stops
 * and the in-place observables the GPU kernel accumulates. */
static void trace_one(const ExcMetric* m, const ExcTraceArgs* A, int64_t p) {
  const int fi = A->field_index ? A->field_index[p] : 0;
  double s[8], ns[8], q[6], qprev[6];
  memcpy(s, A->state + 8 * p, sizeof(s));
  double dt = A->dt_state ? A->dt_state[p] : A->dt;
  int64_t steps = 0, it = 0;
  int status = -1, nrec = 0, qvalid = 0;
  const int rec = A->records != NULL;
  if (rec) write_record(A, p, &nrec, s, NULL);
  double p0[3], pprev[3], e0[3], v0[3], path = 0, excess = 0, isw = 0, pdot_prev = 0, min_r, a_obs = NAN,
         phi_obs = NAN, eta_obs = s[0];
  cart_pos(m, s, p0);
  memcpy(pprev, p0, sizeof(p0));
  cart_vel(m, s, v0);
  const double nv = norm3(v0);
  for (int i = 0; i < 3; ++i) e0[i] = nv > 0 ? v0[i] / nv : 0.0;
  {
    double rel[3];
    for (int i = 0; i < 3; ++i) rel[i] = m->kind == EXC_METRIC_SCHWARZSCHILD ? p0[i] : p0[i] - A->lens_center[i];
    min_r = norm3(rel);
  }
  if (m->kind == EXC_METRIC_FLRW && A->obs_flags && quantities(m, fi, s, q) == 0) {
    a_obs = q[0]; phi_obs = q[1]; pdot_prev = q[5];
  }
  for (;;) {
    if (it >= A->max_iter) { status = EXC_PH_MAX_ITER; break; }
    if (steps >= A->max_steps) { status = EXC_PH_STEPS; break; }
    dt = dt < 0 ? -clip(-dt, A->dt_min, A->dt_max) : clip(dt, A->dt_min, A->dt_max);
    int face = 0;
    const int face_mode = m->kind == EXC_METRIC_FLRW && (A->stop_flags & EXC_STOP_FACE);
    if (face_mode) dt = face_clip(s, dt, A->box_lo, A->box_hi, &face);
    double dt_new = dt;
    int accepted = 1, st;
    if (A->stepper == EXC_STEPPER_RK4) st = step_rk4(m, fi, s, dt, ns);
    else if (A->stepper == EXC_STEPPER_LEAPFROG4) st = step_lf4(m, fi, s, dt, ns);
    else st = step_rk45(m, fi, A->tableau, s, dt, A->rtol, A->atol, ns, &dt_new, &accepted);
    if (st) { status = st; break; }
    int stop = 0;
    if (accepted) {
      if (A->renormalize_every && (steps % A->renormalize_every) == 0) {
        st = renormalize(m, fi, ns);
        if (st) { status = st; break; }
      }
      const double eta_old = s[0];
      memcpy(s, ns, sizeof(s));
      if (rec && (A->record_every == 1 || (A->record_every > 1 && (steps % A->record_every) == 0))) {
        write_record(A, p, &nrec, s, qvalid ? qprev : NULL);
        st = quantities(m, fi, s, qprev);
        if (st) { status = st; steps++; it++; dt = dt_new; break; }
        qvalid = 1;
      }
      if (A->obs_flags) {
        double pc[3], d[3], rel[3];
        cart_pos(m, s, pc);
        for (int i = 0; i < 3; ++i) d[i] = pc[i] - pprev[i];
        path += norm3(d);
        excess += excess_term(d, e0);
        for (int i = 0; i < 3; ++i) rel[i] = m->kind == EXC_METRIC_SCHWARZSCHILD ? pc[i] : pc[i] - A->lens_center[i];
        const double r = norm3(rel);
        if (r < min_r) min_r = r;
        if (m->kind == EXC_METRIC_FLRW && (A->obs_flags & EXC_OBS_ISW) && quantities(m, fi, s, q) == 0) {
          isw += 0.5 * (pdot_prev + q[5]) * (s[0] - eta_old);
          pdot_prev = q[5];
        }
        memcpy(pprev, pc, sizeof(pc));
      }
      steps++;
      if (face_mode) {
        if (face) {
          status = EXC_PH_LEFT_BOX;
          stop = 1;
        }
      } else if (A->stop_flags & EXC_STOP_BOX) {
        double pc[3];
        cart_pos(m, s, pc);
        if (m->kind == EXC_METRIC_SCHWARZSCHILD)
          for (int i = 0; i < 3; ++i) pc[i] += m->center[i];
        if (!(pc[0] >= A->box_lo[0] && pc[0] < A->box_hi[0] && pc[1] >= A->box_lo[1] && pc[1] < A->box_hi[1] &&
              pc[2] >= A->box_lo[2] && pc[2] < A->box_hi[2])) {
          status = EXC_PH_LEFT_BOX;
          stop = 1;
        }
      }
      if (!stop && m->kind == EXC_METRIC_FLRW && (A->stop_flags & EXC_STOP_A)) {
        double a, adot;
        if (scale_factor(m, s[0], &a, &adot) == 0 && a <= A->a_stop) {
          status = EXC_PH_A_STOP;
          stop = 1;
        }
      }
    }
    dt = dt_new;
    it++;
    if (stop) break;
  }
  const int failed = status >= EXC_PH_OUTSIDE_GRID;
  double qf[6];
  int qst = failed ? 1 : quantities(m, fi, s, qf);
  if (rec) {
    if (!failed && qst == 0) write_record(A, p, &nrec, s, qf);
    A->n_records[p] = nrec;
  }
  if (!failed && qst) status = qst;
  memcpy(A->state + 8 * p, s, sizeof(s));
  A->status[p] = status;
  if (A->n_steps) A->n_steps[p] = (int32_t)steps;
  if (A->n_iter) A->n_iter[p] = (int32_t)it;
  if (A->dt_state) A->dt_state[p] = dt;
  if (A->obs && A->obs_flags) {
    double* o = A->obs + p * EXC_OBSCOL_N;
    for (int i = 0; i < EXC_OBSCOL_N; ++i) o[i] = NAN;
    o[EXC_OBSCOL_ETA_OBS] = eta_obs;
    o[EXC_OBSCOL_ETA_EM] = s[0];
    o[EXC_OBSCOL_A_OBS] = a_obs;
    o[EXC_OBSCOL_PHI_OBS] = phi_obs;
    if (m->kind == EXC_METRIC_FLRW && !failed && qst == 0) { o[EXC_OBSCOL_A_EM] = qf[0]; o[EXC_OBSCOL_PHI_EM] = qf[1]; }
    o[EXC_OBSCOL_ISW_INT] = isw;
    if (A->obs_flags & EXC_OBS_PATH) {
      double pc[3], X[3];
      cart_pos(m, s, pc);
      for (int i = 0; i < 3; ++i) X[i] = pc[i] - p0[i];
      o[EXC_OBSCOL_PATH] = path;
      o[EXC_OBSCOL_CHORD] = norm3(X);
      o[EXC_OBSCOL_EXCESS] = excess - excess_term(X, e0);
    }
    double v1[3];
    cart_vel(m, s, v1);
    o[EXC_OBSCOL_V0X] = v0[0]; o[EXC_OBSCOL_V0Y] = v0[1]; o[EXC_OBSCOL_V0Z] = v0[2];
    o[EXC_OBSCOL_V1X] = v1[0]; o[EXC_OBSCOL_V1Y] = v1[1]; o[EXC_OBSCOL_V1Z] = v1[2];
    o[EXC_OBSCOL_MIN_R] = min_r;
  }
}

typedef struct {
  const ExcMetric* m;
  const ExcTraceArgs* A;
  int64_t* next;
  pthread_mutex_t* mu;
} Work;

static void* worker(void* arg) {
  Work* w = (Work*)arg;
  for (;;) {
    pthread_mutex_lock(w->mu);
    const int64_t p0 = *w->next;
    *w->next += 16;
    pthread_mutex_unlock(w->mu);
    if (p0 >= w->A->n_photons) break;
    const int64_t p1 = p0 + 16 < w->A->n_photons ? p0 + 16 : w->A->n_photons;
    for (int64_t p = p0; p < p1; ++p) trace_one(w->m, w->A, p);
  }
  return NULL;
}

/* Trace every photon with `n_threads` host threads (0 or 1 = calling thread). */
int oracle_trace(const ExcMetric* m, const ExcTraceArgs* A, int n_threads) {
  if (n_threads <= 1) {
    for (int64_t p = 0; p < A->n_photons; ++p) trace_one(m, A, p);
    return 0;
  }
  pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
  pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
  int64_t next = 0;
  Work w = {m, A, &next, &mu};
  for (int i = 0; i < n_threads; ++i) pthread_create(&th[i], NULL, worker, &w);
  for (int i = 0; i < n_threads; ++i) pthread_join(th[i], NULL);
  free(th);
  return 0;
}

int oracle_interp(const ExcField* f, const double* pts, double* out, int32_t* status, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    int st = oracle_interp_one(f, pts[4 * i], pts[4 * i + 1], pts[4 * i + 2], pts[4 * i + 3], out + 5 * i);
    if (status) status[i] = st;
  }
  return 0;
}

int oracle_step(const ExcMetric* m, int stepper, int tableau, const double* s, double dt, double rtol, double atol,
                double* out, double* dt_new, int* accepted) {
  *dt_new = dt;
  *accepted = 1;
  if (stepper == EXC_STEPPER_RK4) return step_rk4(m, 0, s, dt, out);
  if (stepper == EXC_STEPPER_LEAPFROG4) return step_lf4(m, 0, s, dt, out);
  return step_rk45(m, 0, tableau, s, dt, rtol, atol, out, dt_new, accepted);
}
