// exc_mixed.cu -- mixed-precision FLRW tracer (EXC_PREC_MIXED).
//
// GB300 executes FP64 at 1/64 of its FP32 rate, so this build keeps the FP64
// pipe out of the step loop altogether:
//  * the RHS (a(eta), adot, trilinear Phi, base-node gradient, tensorial or
//    analytical Christoffel contraction) is evaluated in FP32;
//  * the accumulated state -- position in grid-cell units, conformal time and
//    the four velocity components -- is carried as double-float pairs
//    (hi + lo FP32, ~48-bit significand; Dekker / Knuth error-free sums and
//    FMA-based products), because per-step increments are 1e-4..1e-9 of the
//    values they are added to;
//  * RK4's position increment is formed exactly as dt u + dt^2/6 (a1+a2+a3)
//    (the same algebra as the reference's (dt/6)(k1+2k2+2k3+k4) for x' = u),
//    so the large dt u term is a double-float product and only the small
//    curvature correction comes from FP32 stages;
//  * endpoint observables (a, Phi at both ends) are evaluated once per photon
//    in FP64 with the parity code; the time-delay excess is accumulated in the
//    cancellation-free form from the velocity component perpendicular to the
//    initial direction, which the kernel integrates in FP32 alongside u.
// The cell a stage point falls in is taken from the double-float position, so
// photons starting on a grid node plane (the runner's observer placement)
// select the same cell as the reference.
//
// The reference's RHS is discontinuous: the base-node gradient jumps at every
// cell face (and, with the finite-difference adot, a(eta)'s slope at every
// table node), and the box / a(eta) stops are thresholds. A mixed trajectory
// differs from the FP64 one by a small drift (measured <= 2e-9 of the distance
// travelled along the ray, far less across it), so a ray whose stage point
// falls within that distance of a face can take the other cell there and end
// up to ~1e-7 rad / 3e-8 in z away from the FP64 result -- the FP64 tracer
// moves the same way under the same shift of its input. Every such decision
// is guarded: a stage point or stop test within the error window
//   W = W0 (stage arithmetic) + KAPPA * (distance travelled) * (|e_d| + ET)
// of a discontinuity ends the ray with EXC_PH_RETRACE, its state untouched,
// and the host layer re-traces it with the FP64 parity tracer.
#define EXC_FAST 1
#define EXC_NS exc_mixed_f64
#include "exc_device.cuh"

#include <cooperative_groups.h>

#include "exc_mixed.h"

namespace exc_mixed {

namespace cg = cooperative_groups;
using exc::DevMetric;

// ----------------------------------------------------------- double-float
struct df {
  float hi, lo;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const df t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_of(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}
__device__ __forceinline__ double dbl(df a) { return (double)a.hi + (double)a.lo; }
// --------------------------------------------------------------- params
struct MixField {
  const void* data;
  int dtype, boundary;
  int nodes;         // n0 n1 n2
  int n[3];
  float s[3];        // spacing (m)
  df inv_s[3];       // 1 / spacing as double-float
  float inv_2s[3];   // 1 / (2 spacing)
  int slow;          // grad_mode EXC_GRAD_TRILINEAR (the slow Interpolator)
  df box[6];         // stop-box faces in cells of this field (lo xyz, hi xyz), for EXC_STOP_FACE
};

// Fehlberg 4(5) for the mixed tracer (integrator.py:93-152). With k_j the velocity stage
// derivatives (K for u^mu) and S_j = sum_l B_jl k_l, stage j's velocity is u + dt S_j and, as
// x' = u, its point is x + dt c_j u + dt^2 sum_m BB_jm k_m (BB = B.B, c_j = sum_l B_jl). The
// 5th-order update is x + dt W5 u + dt^2 sum_m CB5_m k_m, u + dt sum_j C5_j k_j (CB5 = C5.B,
// W5 = sum C5), and y5 - y4 the same with the weight differences dC = C5 - C4 (dW = W5 - 1,
// the 4th-order weights summing to 1). So the large dt u term is one double-float product and
// the FP32 stage values enter only the small corrections.
// Sums of stage values weighted by FP32-rounded coefficients would carry the coefficients'
// rounding as the same relative bias on every step (the Hubble drag, ~1e-3 of u per step, is
// nearly the same at every stage), so they are formed about stage 0: sum_j w_j v_j =
// W v_0 + sum_j w_j (v_j - v_0), W = sum_j w_j kept as hi + lo (W5, and WCB5 = sum CB5).
struct RKF {
  float b[6][6], bb[6][6], c[6];
  float c5[6], dc[6], cb5[6], cbe[6];
  df w5, wcb5;
  float dw;
};

// Constants that multiply every step's background (Hubble) terms are kept as
// hi + lo pairs: a constant rounded once to FP32 would bias every step the
// same way and the bias would accumulate along the trajectory, while the
// rounding of the varying operands averages out.
struct MixParams {
  DevMetric D;
  MixField mf[EXC_MAX_FIELDS];
  float ic2, ic4, two_over_c2, c2f_over_c4;
  df ic2d, H0, om, orad, ok, ol;
  df eta_min, inv_eta_step;
  int table_n, table_in_smem;
  float a_stop_f;     // a_stop rounded once on the host (no FP64 conversion in the step loop)
  RKF rk;
};

// c * x with c = c.hi + c.lo, rounded once: the FMA adds the small c.lo * x to
// the exact product c.hi * x, so the constant's own rounding does not bias the
// result (rounding c.hi * x first would drop the correction every time).
__device__ __forceinline__ float cmul(df c, float x) { return fmaf(c.hi, x, c.lo * x); }

// Error window of the mixed trajectory against the FP64 one, in cells of each
// axis: kWin0 covers one stage point's FP32 offset arithmetic, kWinRate the
// drift per unit distance travelled along the ray (5x the largest drift seen
// on the 1000 Mpc lens patch), kWinTrans the share of that drift across the
// ray (the measured transverse drift is ~1e-2 of the along-ray one).
constexpr float kWin0 = 5e-8f, kWinRate = 1e-8f, kWinTrans = 0.02f;

// ----------------------------------------------------- FP32 cosmology
__device__ __forceinline__ float table_at(const MixParams& Pm, const float* tab_s, int i) {
  if (Pm.table_in_smem) return tab_s[i];
  return (float)__ldg(Pm.D.m.a_table + i);
}

// Background at table coordinate (cell ie + fraction fe): a(eta) as the
// reference's a_interp_numba (cosmology.py:8-25), and the two combinations the
// geodesic equation uses, aa = adot / a and r2 = a adot / c^2, with
// adot = a^2 H0 E(z) (cosmology.py:84-93), evaluated in FP32.
__device__ __forceinline__ void cosmo_f32(const MixParams& Pm, const float* tab_s, int ie, float fe, float& a,
                                          float& aa, float& r2) {
  const int cosmo = Pm.D.m.cosmology;
  if (cosmo == EXC_COSMO_STATIC) {
    a = 1.0f;
    aa = 0.0f;
    r2 = 0.0f;
    return;
  }
  const int n = Pm.table_n;
  float slope_cell;
  if (ie < 0) {
    a = table_at(Pm, tab_s, 0);
    slope_cell = 0.0f;
  } else if (ie >= n - 1) {
    a = table_at(Pm, tab_s, n - 1);
    slope_cell = 0.0f;
  } else {
    const float a0 = table_at(Pm, tab_s, ie), a1 = table_at(Pm, tab_s, ie + 1);
    a = fmaf(fe, a1 - a0, a0);
    slope_cell = a1 - a0;
  }
  if (cosmo == EXC_COSMO_TABLE) {
    const float x = 1.0f / a;                       // 1 + z
    const float x2 = x * x, x3 = x2 * x, x4 = x2 * x2;
    // E^2 summed with its rounding errors carried (two-sum / exact product
    // error) and rounded once: the constants' lo parts sit below half an ulp of
    // E^2 and would otherwise be dropped the same way on every call.
    const float p3 = Pm.om.hi * x3;
    const float e3 = fmaf(Pm.om.hi, x3, -p3);
    const float rest = fmaf(Pm.orad.hi, x4, Pm.ok.hi * x2);
    const df s1 = two_sum(p3, Pm.ol.hi);
    const df s2 = two_sum(s1.hi, rest);
    float lo = fmaf(Pm.om.lo, x3, Pm.ol.lo);
    lo = fmaf(Pm.orad.lo, x4, fmaf(Pm.ok.lo, x2, lo));
    lo += (e3 + s1.lo) + s2.lo;
    const float E2 = s2.hi + lo;
    const float aE = a * sqrtf(E2);
    aa = cmul(Pm.H0, aE);                           // adot / a = a H0 E
    r2 = cmul(Pm.ic2d, (a * a) * aa);               // a adot / c^2 = a^2 (adot / a) / c^2
  } else {
    // finite-difference adot of a piecewise-linear table = the cell's slope
    const float adot = cmul(Pm.inv_eta_step, slope_cell);
    aa = adot / a;
    r2 = cmul(Pm.ic2d, a * adot);
  }
}

// --------------------------------------------------------- FP32 RHS
struct Stage {
  int cx, cy, cz;    // cell of the base point
  float fx, fy, fz;  // base fraction in the cell (hi part)
  float lx, ly, lz;  // ... and its lo part: the fraction is fx + lx exactly
  int ce;            // table cell of the base eta
  float fe, le;
  float wx, wy, wz, we;   // error windows of this step's base point (cells, table cells)
};

// Cell and in-cell fraction of base fraction (f + l) + offset o, with the
// floor taken on the exact sum; `near` is set when the point lies within `w`
// of a cell face (where the FP64 trajectory might take the other cell).
__device__ __forceinline__ int stage_cell(float f, float l, float o, float w, float& frac, bool& near) {
  df t = two_sum(f, o);
  t.lo += l;
  float fl = floorf(t.hi);
  if (t.hi == fl && t.lo < 0.0f) fl -= 1.0f;
  const float r = (t.hi - fl) + t.lo;
  frac = r;
  near = near || r < w || r > 1.0f - w;
  return (int)fl;
}

__device__ __forceinline__ float ld32(const MixField& F, int idx) {
  if (F.dtype == EXC_DTYPE_F64) return (float)__ldg((const double*)F.data + idx);
  if (F.dtype == EXC_DTYPE_F32X2) return __ldg((const float*)F.data + 2 * (int64_t)idx);   // hi of the pair
  return __ldg((const float*)F.data + idx);
}
// hi and lo of a node (lo = 0 unless the grid is split)
__device__ __forceinline__ float2 ld32x2(const MixField& F, int idx) {
  if (F.dtype == EXC_DTYPE_F32X2) return __ldg((const float2*)F.data + idx);
  return make_float2(ld32(F, idx), 0.0f);
}

// Interpolation (value + base-node gradient) at base cell + offset (cells).
// Returns 0 or an EXC_PH_* code.
__device__ __forceinline__ int interp_f32(const MixField& F, const Stage& B, float ox, float oy, float oz, float w0,
                                          float& val, float& gx, float& gy, float& gz) {
  float fx, fy, fz;
  bool near = false;
  int ix = B.cx + stage_cell(B.fx, B.lx, ox, B.wx + w0, fx, near);
  int iy = B.cy + stage_cell(B.fy, B.ly, oy, B.wy + w0, fy, near);
  int iz = B.cz + stage_cell(B.fz, B.lz, oz, B.wz + w0, fz, near);
  if (near) return EXC_PH_RETRACE;
  const int nx = F.n[0], ny = F.n[1], nz = F.n[2];
  int ixm, iym, izm, ixp, iyp, izp;
  bool one_x = false, one_y = false, one_z = false;
  if (F.boundary == EXC_BOUNDARY_PERIODIC) {
    ix %= nx; if (ix < 0) ix += nx;
    iy %= ny; if (iy < 0) iy += ny;
    iz %= nz; if (iz < 0) iz += nz;
    ixp = ix + 1 == nx ? 0 : ix + 1; ixm = ix == 0 ? nx - 1 : ix - 1;
    iyp = iy + 1 == ny ? 0 : iy + 1; iym = iy == 0 ? ny - 1 : iy - 1;
    izp = iz + 1 == nz ? 0 : iz + 1; izm = iz == 0 ? nz - 1 : iz - 1;
  } else if (F.boundary == EXC_BOUNDARY_CLAMP) {
    // position clamped to [0, n-1) then cell clamped to [0, n-2]
    if (ix < 0) { ix = 0; fx = 0.0f; }
    if (iy < 0) { iy = 0; fy = 0.0f; }
    if (iz < 0) { iz = 0; fz = 0.0f; }
    if (ix > nx - 2) { fx = ix > nx - 2 ? 1.0f : fx; ix = nx - 2; }
    if (iy > ny - 2) { fy = 1.0f; iy = ny - 2; }
    if (iz > nz - 2) { fz = 1.0f; iz = nz - 2; }
    ixp = ix + 1; iyp = iy + 1; izp = iz + 1;
    one_x = ix <= 0; one_y = iy <= 0; one_z = iz <= 0;
    ixm = one_x ? ix : ix - 1; iym = one_y ? iy : iy - 1; izm = one_z ? iz : iz - 1;
  } else {
    // strict interior: rel in [1, n-2)
    if (ix < 1 || ix >= nx - 2 || iy < 1 || iy >= ny - 2 || iz < 1 || iz >= nz - 2) return EXC_PH_OUTSIDE_GRID;
    ixp = ix + 1; iyp = iy + 1; izp = iz + 1;
    ixm = ix - 1; iym = iy - 1; izm = iz - 1;
  }
  const int sy = nz, sx = ny * nz;
  const int b = ix * sx + iy * sy + iz;
  const float c000 = ld32(F, b);
  const float2 p100 = ld32x2(F, ixp * sx + iy * sy + iz);
  const float2 p010 = ld32x2(F, ix * sx + iyp * sy + iz);
  const float2 p001 = ld32x2(F, b - iz + izp);
  const float c100 = p100.x, c010 = p010.x, c001 = p001.x;
  const float c110 = ld32(F, ixp * sx + iyp * sy + iz);
  const float c101 = ld32(F, ixp * sx + iy * sy + izp);
  const float c011 = ld32(F, ix * sx + iyp * sy + izp);
  const float c111 = ld32(F, ixp * sx + iyp * sy + izp);
  const float2 pxm = ld32x2(F, ixm * sx + iy * sy + iz);
  const float2 pym = ld32x2(F, ix * sx + iym * sy + iz);
  const float2 pzm = ld32x2(F, b - iz + izm);
  // trilinear as nested lerps (the reference's eight-product sum, regrouped)
  const float c00 = fmaf(fx, c100 - c000, c000), c10 = fmaf(fx, c110 - c010, c010);
  const float c01 = fmaf(fx, c101 - c001, c001), c11 = fmaf(fx, c111 - c011, c011);
  const float c0 = fmaf(fy, c10 - c00, c00), c1 = fmaf(fy, c11 - c01, c01);
  val = fmaf(fz, c1 - c0, c0);
  // central differences: hi-plane differences of neighbouring nodes are exact
  // (Sterbenz); a split grid adds the lo-plane difference
  const float dgx = (c100 - pxm.x) + (p100.y - pxm.y);
  const float dgy = (c010 - pym.x) + (p010.y - pym.y);
  const float dgz = (c001 - pzm.x) + (p001.y - pzm.y);
  gx = dgx * (one_x ? 2.0f * F.inv_2s[0] : F.inv_2s[0]);
  gy = dgy * (one_y ? 2.0f * F.inv_2s[1] : F.inv_2s[1]);
  gz = dgz * (one_z ? 2.0f * F.inv_2s[2] : F.inv_2s[2]);
  return 0;
}

// The slow Interpolator (grid/interpolator.py:13-158, grad_mode EXC_GRAD_TRILINEAR)
// at base cell + offset: trilinear value, and the gradient as the trilinear blend
// of central differences at the cell's eight corners (base index clipped to
// [1, n-2], each corner clipped again, weights from the unclipped fraction).
// Value and gradient are continuous across interior cell faces, so no window
// check is needed there; the formula changes only at the bounds rel = 0, n-1
// and at the clip faces rel = 1, n-2, and a stage point within the error
// window of one of those (cells 0, 1, n-3, n-2 of an axis) is handed back.
__device__ __forceinline__ int interp_f32_slow(const MixField& F, const Stage& B, float ox, float oy, float oz,
                                               float w0, float& val, float& gx, float& gy, float& gz) {
  float fx, fy, fz;
  bool nearx = false, neary = false, nearz = false;
  const int ix = B.cx + stage_cell(B.fx, B.lx, ox, B.wx + w0, fx, nearx);
  const int iy = B.cy + stage_cell(B.fy, B.ly, oy, B.wy + w0, fy, neary);
  const int iz = B.cz + stage_cell(B.fz, B.lz, oz, B.wz + w0, fz, nearz);
  const int nx = F.n[0], ny = F.n[1], nz = F.n[2];
  if ((nearx && (ix <= 1 || ix >= nx - 3)) || (neary && (iy <= 1 || iy >= ny - 3)) ||
      (nearz && (iz <= 1 || iz >= nz - 3)))
    return EXC_PH_RETRACE;
  if (ix < 0 || ix > nx - 2 || iy < 0 || iy > ny - 2 || iz < 0 || iz > nz - 2) return EXC_PH_OUTSIDE_GRID;
  const int sy = nz, sx = ny * nz;
  const int b = ix * sx + iy * sy + iz;
  const float c000 = ld32(F, b), c100 = ld32(F, b + sx), c010 = ld32(F, b + sy), c001 = ld32(F, b + 1);
  const float c110 = ld32(F, b + sx + sy), c101 = ld32(F, b + sx + 1), c011 = ld32(F, b + sy + 1);
  const float c111 = ld32(F, b + sx + sy + 1);
  const float c00 = fmaf(fx, c100 - c000, c000), c10 = fmaf(fx, c110 - c010, c010);
  const float c01 = fmaf(fx, c101 - c001, c001), c11 = fmaf(fx, c111 - c011, c011);
  const float c0 = fmaf(fy, c10 - c00, c00), c1 = fmaf(fy, c11 - c01, c01);
  val = fmaf(fz, c1 - c0, c0);
  // corner indices (clipped) and weights
  const int bx = min(max(ix, 1), nx - 2), by = min(max(iy, 1), ny - 2), bz = min(max(iz, 1), nz - 2);
  const int X[2] = {bx, min(bx + 1, nx - 2)}, Y[2] = {by, min(by + 1, ny - 2)}, Z[2] = {bz, min(bz + 1, nz - 2)};
  const float WX[2] = {1.0f - fx, fx}, WY[2] = {1.0f - fy, fy}, WZ[2] = {1.0f - fz, fz};
  float sgx = 0.0f, sgy = 0.0f, sgz = 0.0f;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const float w = WX[a] * WY[e] * WZ[c];
        const int q = X[a] * sx + Y[e] * sy + Z[c];
        // central differences: hi-plane difference plus (split grids) the lo-plane one
        const float2 xp = ld32x2(F, q + sx), xm = ld32x2(F, q - sx);
        const float2 yp = ld32x2(F, q + sy), ym = ld32x2(F, q - sy);
        const float2 zp = ld32x2(F, q + 1), zm = ld32x2(F, q - 1);
        sgx = fmaf(w, (xp.x - xm.x) + (xp.y - xm.y), sgx);
        sgy = fmaf(w, (yp.x - ym.x) + (yp.y - ym.y), sgy);
        sgz = fmaf(w, (zp.x - zm.x) + (zp.y - zm.y), sgz);
      }
  gx = sgx * F.inv_2s[0];
  gy = sgy * F.inv_2s[1];
  gz = sgz * F.inv_2s[2];
  return 0;
}

// du^mu/dlambda in FP32 (perturbed_flrw_metric_fast.py:7-99); u in SI.
// The spatial part is returned split as du_i = -(hub * u_i + L_i): `hub` is
// the Hubble drag coefficient 2 (adot/a) u^0 and L the gradient (lensing)
// terms, so the caller can integrate the velocity component perpendicular to
// the initial direction without losing it under the much larger drag term.
template <bool SLOW>
__device__ __forceinline__ int rhs_f32(const MixParams& Pm, const MixField& F, const float* tab_s, const Stage& B,
                                       float ox, float oy, float oz, float oe, float w0, const float u[4],
                                       float du[4], float L[3], float& hub) {
  float fe;
  bool near = false;
  const int ie = B.ce + stage_cell(B.fe, B.le, oe, B.we + w0, fe, near);
  // a(eta) is continuous; only the finite-difference adot jumps at table nodes
  if (near && Pm.D.m.cosmology == EXC_COSMO_TABLE_FD) return EXC_PH_RETRACE;
  float a, aa, r2;
  cosmo_f32(Pm, tab_s, ie, fe, a, aa, r2);
  float phi_si, gx, gy, gz;
  const int st = (SLOW && F.slow) ? interp_f32_slow(F, B, ox, oy, oz, w0, phi_si, gx, gy, gz)
                                    : interp_f32(F, B, ox, oy, oz, w0, phi_si, gx, gy, gz);
  if (st) return st;
  const float ic2 = Pm.ic2;
  const float phi = phi_si * ic2;
  const float u0 = u[0], u1 = u[1], u2 = u[2], u3 = u[3];
  const float inv_a = 1.0f / a;
  const float usq = fmaf(u1, u1, fmaf(u2, u2, u3 * u3));
  hub = 2.0f * aa * u0;
  if (!Pm.D.m.analytical) {
    const float gxc = gx * ic2, gyc = gy * ic2, gzc = gz * ic2;
    // Gamma^0_ij = a adot / c^2 + 2 a adot / c^4 (phi + psi); the dPhi/deta terms vanish on a static grid
    const float G0ij = fmaf(r2 * usq, 2.0f * Pm.c2f_over_c4 * (phi + phi), r2 * usq);
    const float G00i = 2.0f * u0 * fmaf(gxc, u1, fmaf(gyc, u2, gzc * u3));
    du[0] = -(G0ij + G00i);
    const float ia2u0 = inv_a * inv_a * u0 * u0;
    L[0] = fmaf(gx, ia2u0, gxc * (fmaf(u2, u2, u3 * u3) - u1 * u1) - u1 * fmaf(gyc, u2, gzc * u3));
    L[1] = fmaf(gy, ia2u0, gyc * (fmaf(u1, u1, u3 * u3) - u2 * u2) - u2 * fmaf(gxc, u1, gzc * u3));
    L[2] = fmaf(gz, ia2u0, gzc * (fmaf(u1, u1, u2 * u2) - u3 * u3) - u3 * fmaf(gxc, u1, gyc * u2));
  } else {
    const float tc2 = Pm.two_over_c2;
    const float dpl = fmaf(gx, u1, fmaf(gy, u2, gz * u3));
    du[0] = -aa * (u0 * u0) - tc2 * u0 * dpl - (cmul(Pm.ic2d, aa) - 2.0f * aa * Pm.ic4 * (phi + phi)) * usq;
    const float u02 = u0 * u0;
    L[0] = gx * u02 - tc2 * u1 * fmaf(gy, u2, gz * u3) - gx * ic2 * (2.0f * u1 * u1 - usq);
    L[1] = gy * u02 - tc2 * u2 * fmaf(gx, u1, gz * u3) - gy * ic2 * (2.0f * u2 * u2 - usq);
    L[2] = gz * u02 - tc2 * u3 * fmaf(gy, u2, gx * u1) - gz * ic2 * (2.0f * u3 * u3 - usq);
  }
  du[1] = -fmaf(hub, u1, L[0]);
  du[2] = -fmaf(hub, u2, L[1]);
  du[3] = -fmaf(hub, u3, L[2]);
  return 0;
}

// ------------------------------------------------------------ photon
struct MPhoton {
  df P[3];       // position, grid-cell units relative to the field origin
  df eta;        // conformal time (s)
  df U[4];       // u^0 (dimensionless), u^i (m/s)
  df dt, d6, c6;  // dt, dt/6, dt^2/6 (hi + lo; formed in FP64 once per photon)
  float dtf;
  int64_t idx;
  int fi, steps, it, status;
  // observables
  df e[3];       // unit initial direction (hi + lo): the axis of the excess

  float lc[3];   // lens centre, cell units
  float box[6];  // stop box, cell units (lo xyz, hi xyz)
  float box_tol; // largest FP32 rounding of the box faces (cells)
  float wrate[4];  // error-window growth: cells of x, y, z and table cells of eta per step
                   // (RK4), or per unit lambda travelled (RK45)
  float lam;       // RK45: |lambda| travelled over accepted steps
  df excess;     // sum |dx x e|^2 / (|dx| + dx.e), in x-spacing units
  df path;       // sum |dx|, in x-spacing units
  float min_r2;  // min |x - lens|^2, in x-spacing units squared
};

__device__ __forceinline__ const MixField& field_of(const MixParams& Pm, int fi) { return Pm.mf[fi]; }

__device__ __forceinline__ int64_t next_photon(const ExcTraceArgs& A, int64_t& static_next, int64_t stride) {
  if (A.queue == nullptr) {
    const int64_t p = static_next;
    static_next += stride;
    return p;
  }
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned long long base = 0;
  if (g.thread_rank() == 0)
    base = atomicAdd(reinterpret_cast<unsigned long long*>(A.queue), (unsigned long long)g.size());
  base = g.shfl(base, 0);
  return (int64_t)(base + g.thread_rank());
}

// FP64 endpoint quantities a(eta) and Phi(x) with the parity code (once per photon).
template <bool SLOW>
__device__ __forceinline__ int endpoint(const MixParams& Pm, int fi, const double s[4], double& a, double& phi) {
  const ExcField& f = Pm.D.m.fields[fi];
  double adot, inv_a;
  int st = exc_mixed_f64::scale_factor(Pm.D, s[0], a, adot, inv_a);
  if (st) return st;
  if (SLOW && f.grad_mode == EXC_GRAD_TRILINEAR) {
    if (f.dtype == EXC_DTYPE_F32) return exc_mixed_f64::slow_value3<float>(f, s[1], s[2], s[3], phi);
    if (f.dtype == EXC_DTYPE_F32X2) return exc_mixed_f64::slow_value3<float2>(f, s[1], s[2], s[3], phi);
    return exc_mixed_f64::slow_value3<double>(f, s[1], s[2], s[3], phi);
  }
  exc_mixed_f64::InterpOut ip;
  if (f.dtype == EXC_DTYPE_F32)
    st = exc_mixed_f64::interp_field<float, false>(f, Pm.D.finv[fi], s[1], s[2], s[3], s[0], ip);
  else if (f.dtype == EXC_DTYPE_F32X2)
    st = exc_mixed_f64::interp_field<float2, false>(f, Pm.D.finv[fi], s[1], s[2], s[3], s[0], ip);
  else
    st = exc_mixed_f64::interp_field<double, false>(f, Pm.D.finv[fi], s[1], s[2], s[3], s[0], ip);
  phi = ip.val;
  return st;
}

__device__ __forceinline__ void photon_begin(const MixParams& Pm, const ExcTraceArgs& A, MPhoton& P, int64_t p) {
  const ExcMetric& m = Pm.D.m;
  P.idx = p;
  int fi = A.field_index ? A.field_index[p] : 0;
  P.status = -1;
  if ((unsigned)fi >= (unsigned)m.n_fields) { fi = 0; P.status = EXC_PH_BAD_FIELD; }
  P.fi = fi;
  const ExcField& f = m.fields[fi];
  const double* s = A.state + p * 8;
  double btol = 0.0;
  for (int d = 0; d < 3; ++d) {
    // the reference's cell coordinate of the (shifted) query point; the lens and box are
    // given in the state's coordinates and take the same shift
    const double o = f.origin[d], sh = f.shift[d];
    P.P[d] = df_of(((s[1 + d] + sh) - o) / f.spacing[d]);
    P.lc[d] = (float)(((A.lens_center[d] + sh) - o) / f.spacing[d]);
    const double blo = ((A.box_lo[d] + sh) - o) / f.spacing[d], bhi = ((A.box_hi[d] + sh) - o) / f.spacing[d];
    P.box[d] = (float)blo;
    P.box[3 + d] = (float)bhi;
    btol = fmax(btol, fmax(fabs((double)P.box[d] - blo), fabs((double)P.box[3 + d] - bhi)));
  }
  P.box_tol = (float)btol;
  P.eta = df_of(s[0]);
  for (int d = 0; d < 4; ++d) P.U[d] = df_of(s[4 + d]);
  double dt = A.dt_state ? A.dt_state[p] : A.dt;
  // the reference clips |dt| into [dt_min, dt_max] every iteration; for RK4 it is fixed after the first clip
  const double adt = fmin(fmax(fabs(dt), A.dt_min), A.dt_max);
  dt = dt < 0.0 ? -adt : adt;
  P.dt = df_of(dt);
  P.d6 = df_of(dt / 6.0);
  P.c6 = df_of(dt * dt / 6.0);
  P.dtf = (float)dt;
  P.steps = 0;
  P.it = 0;
  // axis of the time-delay excess: the unit initial direction, kept as hi + lo
  const double vn = sqrt(s[5] * s[5] + s[6] * s[6] + s[7] * s[7]);
  for (int d = 0; d < 3; ++d) P.e[d] = df_of(vn > 0.0 ? s[5 + d] / vn : 0.0);
  // error windows grow with the distance travelled: |dt u| per step (RK4), |u| per unit
  // lambda (RK45, whose steps vary), in cells of each axis
  const double per = A.stepper == EXC_STEPPER_RK45 ? 1.0 : fabs(dt);
  for (int d = 0; d < 3; ++d)
    P.wrate[d] = (float)(kWinRate * per * vn / f.spacing[d] * (fabs(vn > 0.0 ? s[5 + d] / vn : 0.0) + kWinTrans));
  P.wrate[3] = m.cosmology != EXC_COSMO_STATIC ? (float)(kWinRate * per * fabs(s[4]) * Pm.D.i_eta_step) : 0.0f;
  P.lam = 0.0f;
  P.excess = {0.0f, 0.0f};
  P.path = {0.0f, 0.0f};
  float r2 = 0.0f;
  for (int d = 0; d < 3; ++d) {
    const float r = ((P.P[d].hi - P.lc[d]) + P.P[d].lo) * (float)(f.spacing[d] / f.spacing[0]);
    r2 = fmaf(r, r, r2);
  }
  P.min_r2 = r2;
}

// Base decomposition of the current state for the stage evaluations.
// floor of a double-float and the exact remainder as an unnormalised pair (f, l)
__device__ __forceinline__ int df_floor2(df a, float& f, float& l) {
  float fl = floorf(a.hi);
  if (a.hi == fl && a.lo < 0.0f) fl -= 1.0f;
  const df r = two_sum(a.hi, -fl);
  f = r.hi;
  l = r.lo + a.lo;
  return (int)fl;
}

// `n`: the window's growth variable -- accepted steps (RK4) or lambda travelled (RK45).
__device__ __forceinline__ void base_stage(const MixParams& Pm, const MPhoton& P, Stage& B, float n) {
  B.cx = df_floor2(P.P[0], B.fx, B.lx);
  B.cy = df_floor2(P.P[1], B.fy, B.ly);
  B.cz = df_floor2(P.P[2], B.fz, B.lz);
  if (Pm.D.m.cosmology != EXC_COSMO_STATIC) {
    const df rel = df_mul(df_add(P.eta, {-Pm.eta_min.hi, -Pm.eta_min.lo}), Pm.inv_eta_step);
    B.ce = df_floor2(rel, B.fe, B.le);
  } else {
    B.ce = 0;
    B.fe = 0.0f;
    B.le = 0.0f;
  }
  // the base point of step 0 is the initial position itself (no drift yet)
  const float w0 = P.steps > 0 ? kWin0 : 0.0f;
  B.wx = fmaf(n, P.wrate[0], w0);
  B.wy = fmaf(n, P.wrate[1], w0);
  B.wz = fmaf(n, P.wrate[2], w0);
  B.we = fmaf(n, P.wrate[3], w0);
}

// v - (v.e) e in FP32 with the axis' lo parts folded in: the axis is fixed
// per photon, so its FP32 rounding would leak the same fraction of the
// parallel component into every step.
__device__ __forceinline__ void perp(const float v[3], const df e[3], float out[3]) {
  float pr = v[0] * e[0].lo;
  pr = fmaf(v[1], e[1].lo, pr);
  pr = fmaf(v[2], e[2].lo, pr);
  pr = fmaf(v[0], e[0].hi, fmaf(v[1], e[1].hi, fmaf(v[2], e[2].hi, pr)));
  for (int d = 0; d < 3; ++d) out[d] = fmaf(-pr, e[d].hi, fmaf(-pr, e[d].lo, v[d]));
}

// Component of the double-float velocity perpendicular to the unit axis e,
// u - (u.e) e, in double-float arithmetic (the result is ~1e-4 of |u|, so
// FP32 would lose it), returned as FP32.
__device__ __forceinline__ void perp_df(const df U[3], const df e[3], float out[3]) {
  df ue = df_mul(U[0], e[0]);
  ue = df_add(ue, df_mul(U[1], e[1]));
  ue = df_add(ue, df_mul(U[2], e[2]));
  for (int d = 0; d < 3; ++d) {
    const df pe = df_mul(ue, e[d]);
    out[d] = df_add(U[d], {-pe.hi, -pe.lo}).hi;
  }
}

// Step sizes of one step: dt, and for RK4 dt/6 and dt^2/6, as hi + lo pairs.
struct StepDt {
  float f;
  df dt, d6, c6;
};

// One RK4 step (integrator.py:10-22) in mixed precision. Returns 0 or EXC_PH_*.
template <bool SLOW>
__device__ __forceinline__ int step_rk4_mixed(const MixParams& Pm, const float* tab_s, MPhoton& P, const bool obs,
                                              const StepDt& sd) {
  const MixField& F = field_of(Pm, P.fi);
  Stage B;
  base_stage(Pm, P, B, (float)P.steps);
  const float dt = sd.f, h = 0.5f * dt;
  const float isx = F.inv_s[0].hi, isy = F.inv_s[1].hi, isz = F.inv_s[2].hi;
  const float ie = Pm.inv_eta_step.hi;
  const float u[4] = {P.U[0].hi, P.U[1].hi, P.U[2].hi, P.U[3].hi};
  float k1[4], k2[4], k3[4], k4[4], L1[3], L2[3], L3[3], L4[3], hb1, hb2, hb3, hb4, us2[4], us3[4], us4[4];
  int st = rhs_f32<SLOW>(Pm, F, tab_s, B, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, u, k1, L1, hb1);
  if (st) return st;
  for (int i = 0; i < 4; ++i) us2[i] = fmaf(h, k1[i], u[i]);
  st = rhs_f32<SLOW>(Pm, F, tab_s, B, h * u[1] * isx, h * u[2] * isy, h * u[3] * isz, h * u[0] * ie, kWin0, us2, k2, L2,
               hb2);
  if (st) return st;
  for (int i = 0; i < 4; ++i) us3[i] = fmaf(h, k2[i], u[i]);
  st = rhs_f32<SLOW>(Pm, F, tab_s, B, h * us2[1] * isx, h * us2[2] * isy, h * us2[3] * isz, h * us2[0] * ie, kWin0, us3,
               k3, L3, hb3);
  if (st) return st;
  for (int i = 0; i < 4; ++i) us4[i] = fmaf(dt, k3[i], u[i]);
  st = rhs_f32<SLOW>(Pm, F, tab_s, B, dt * us3[1] * isx, dt * us3[2] * isy, dt * us3[3] * isz, dt * us3[0] * ie, kWin0,
               us4, k4, L4, hb4);
  if (st) return st;
  float up[3];
  if (obs) perp_df(&P.U[1], P.e, up);    // perpendicular velocity at the start of the step
  // x' = u: RK4 gives dx = dt u + dt^2/6 (k1 + k2 + k3); u' = k: du = dt/6 (k1 + 2 k2 + 2 k3 + k4)
  // dt/6 and dt^2/6 as hi + lo pairs: they scale every increment (see MixParams)
  const df d6 = sd.d6, c6 = sd.c6;
  // lengths below in units of the x spacing, scaled by the hi + lo reciprocal
  // (cmul): per-photon constants rounded to FP32 would bias every step alike
  const df lunit = F.inv_s[0];
  float dxf[3];
  for (int d = 0; d < 3; ++d) {
    const float corr = cmul(c6, k1[1 + d] + k2[1 + d] + k3[1 + d]);
    const df inc = df_add_f(df_mul(P.U[1 + d], sd.dt), corr);     // metres
    dxf[d] = cmul(lunit, inc.hi);
    P.P[d] = df_add(P.P[d], df_mul(inc, F.inv_s[d]));
  }
  P.eta = df_add(P.eta, df_add_f(df_mul(P.U[0], sd.dt), cmul(c6, k1[0] + k2[0] + k3[0])));
  P.U[0] = df_add_f(P.U[0], cmul(d6, (k1[0] + k4[0]) + 2.0f * (k2[0] + k3[0])));
  // Spatial velocity: k_s = -(hub_s us_s + L_s) is linear in the stage velocity
  // us_s = u + c_s dt k_(s-1), so the RK4 sum (k1 + 2k2 + 2k3 + k4) equals
  //   -[(hub1 + 2 hub2 + 2 hub3 + hub4) u + h (2 hub2 k1 + 2 hub3 k2) + dt hub4 k3 + (L1 + 2 L2 + 2 L3 + L4)].
  // The first term is a scalar times the double-float velocity, so the drag,
  // ~1e3 times the lensing terms, cannot tilt u through independent FP32
  // roundings of its components.
  {
    const float Hs = (hb1 + hb4) + 2.0f * (hb2 + hb3);
    const float g2 = 2.0f * h * hb2, g3 = 2.0f * h * hb3, g4 = dt * hb4;
    for (int d = 0; d < 3; ++d) {
      const float rest = fmaf(g2, k1[1 + d], fmaf(g3, k2[1 + d], fmaf(g4, k3[1 + d],
                                  (L1[d] + L4[d]) + 2.0f * (L2[d] + L3[d]))));
      const df tot = df_add_f(df_mul_f(P.U[1 + d], Hs), rest);
      const df inc = df_mul(tot, d6);
      P.U[1 + d] = df_add(P.U[1 + d], {-inc.hi, -inc.lo});
    }
  }
  if (obs) {
    // perpendicular displacement of this step, dx_perp = dt u_perp + dt^2/6 (q1 + q2 + q3), where
    // q_k = -(hub_k w_k + L_perp_k) are the stage derivatives of u_perp (the drag term is
    // parallel to u, so only u_perp and the lensing terms survive the projection).
    float Lp[3], q1[3], q2[3], q3[3], w[3];
    perp(L1, P.e, Lp);
    for (int d = 0; d < 3; ++d) q1[d] = -fmaf(hb1, up[d], Lp[d]);
    perp(L2, P.e, Lp);
    for (int d = 0; d < 3; ++d) { w[d] = fmaf(h, q1[d], up[d]); q2[d] = -fmaf(hb2, w[d], Lp[d]); }
    perp(L3, P.e, Lp);
    for (int d = 0; d < 3; ++d) { w[d] = fmaf(h, q2[d], up[d]); q3[d] = -fmaf(hb3, w[d], Lp[d]); }
    float dperp2 = 0.0f;
    for (int d = 0; d < 3; ++d) {
      const float dp = cmul(lunit, cmul(sd.dt, up[d]) + cmul(c6, q1[d] + q2[d] + q3[d]));
      dperp2 = fmaf(dp, dp, dperp2);
    }
    const float len = sqrtf(fmaf(dxf[0], dxf[0], fmaf(dxf[1], dxf[1], dxf[2] * dxf[2])));
    const float par = fmaf(dxf[0], P.e[0].hi, fmaf(dxf[1], P.e[1].hi, dxf[2] * P.e[2].hi));
    P.excess = df_add_f(P.excess, par > 0.0f ? dperp2 / (len + par) : len - par);
    P.path = df_add_f(P.path, len);
    float r2 = 0.0f;
    for (int d = 0; d < 3; ++d) {
      const float r = ((P.P[d].hi - P.lc[d]) + P.P[d].lo) * (F.s[d] * lunit.hi);
      r2 = fmaf(r, r, r2);
    }
    P.min_r2 = fminf(P.min_r2, r2);
  }
  return 0;
}

// One RK45Adaptive trial step (integrator.py:93-152) in mixed precision: six FP32 RHS
// evaluations at the stage points, the 5th-order update on the double-float state, and the
// error control in FP64 -- the weighted RMS norm of y5 - y4 (tol = atol + rtol max(|y|, |y5|)
// per component, np.mean over the eight) and the step-size factor 0.9 err^-1/5 (accepted,
// at most 5) or 0.9 err^-1/4 (rejected, at least 0.1). The components of y5 - y4 are formed
// from the stage values (the common dt u term cancels exactly), each ratio to its tolerance in
// FP32. On acceptance the state (and the observables) move; `dt_new` is the next trial step.
// Returns 0 or EXC_PH_*.
template <bool SLOW>
__device__ __forceinline__ int step_rk45_mixed(const MixParams& Pm, const float* tab_s, MPhoton& P, const bool obs,
                                               const StepDt& sd, const ExcTraceArgs& A, bool& accepted,
                                               double& dt_new) {
  const MixField& F = field_of(Pm, P.fi);
  const RKF& R = Pm.rk;
  Stage B;
  base_stage(Pm, P, B, P.lam);
  const float dt = sd.f, dt2 = dt * dt;
  const float isx = F.inv_s[0].hi, isy = F.inv_s[1].hi, isz = F.inv_s[2].hi;
  const float ie = Pm.inv_eta_step.hi;
  const float u[4] = {P.U[0].hi, P.U[1].hi, P.U[2].hi, P.U[3].hi};
  float K[6][4];
  float kE[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  // C5-weighted sums about stage 0 (RKF): the deviations here, the stage-0 terms added below
  float k5_0 = 0.0f, Hs = 0.0f, rest[3] = {0.0f, 0.0f, 0.0f};
  float hb0 = 0.0f, dr0[3] = {0.0f, 0.0f, 0.0f};
  float up[3] = {0.0f, 0.0f, 0.0f}, Q[6][3], q5[3] = {0.0f, 0.0f, 0.0f}, Lp[3];
  if (obs) perp_df(&P.U[1], P.e, up);
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    float S[4] = {0.0f, 0.0f, 0.0f, 0.0f}, O[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int l = 0; l < j; ++l)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        S[i] = fmaf(R.b[j][l], K[l][i], S[i]);
        O[i] = fmaf(R.bb[j][l], K[l][i], O[i]);
      }
    float us[4], off[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      us[i] = fmaf(dt, S[i], u[i]);
      off[i] = fmaf(dt * R.c[j], u[i], dt2 * O[i]);
    }
    float L[3], hb;
    const int st = rhs_f32<SLOW>(Pm, F, tab_s, B, off[1] * isx, off[2] * isy, off[3] * isz, off[0] * ie,
                                 j ? kWin0 : 0.0f, us, K[j], L, hb);
    if (st) return st;
#pragma unroll
    for (int i = 0; i < 4; ++i) kE[i] = fmaf(R.dc[j], K[j][i], kE[i]);
    // spatial k_j = -(hb_j us_j + L_j) with us_j = u + dt S_j: sum_j C5_j k_j =
    // -[(sum C5_j hb_j) u + sum_j C5_j (dt hb_j S_j + L_j)], the drag on u a scalar multiple
    float dr[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) dr[d] = fmaf(dt * hb, S[1 + d], L[d]);
    if (j == 0) {
      hb0 = hb;
#pragma unroll
      for (int d = 0; d < 3; ++d) dr0[d] = dr[d];
    } else {
      k5_0 = fmaf(R.c5[j], K[j][0] - K[0][0], k5_0);
      Hs = fmaf(R.c5[j], hb - hb0, Hs);
#pragma unroll
      for (int d = 0; d < 3; ++d) rest[d] = fmaf(R.c5[j], dr[d] - dr0[d], rest[d]);
    }
    if (obs) {
      // the perpendicular velocity's stage derivatives q_j = -(hb_j w_j + L_perp_j),
      // w_j = u_perp + dt sum_l B_jl q_l (see step_rk4_mixed)
      perp(L, P.e, Lp);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        float w = up[d];
#pragma unroll
        for (int l = 0; l < j; ++l) w = fmaf(dt * R.b[j][l], Q[l][d], w);
        Q[j][d] = -fmaf(hb, w, Lp[d]);
        q5[d] = fmaf(R.cb5[j], Q[j][d] - Q[0][d], q5[d]);
      }
    }
  }
  k5_0 += cmul(R.w5, K[0][0]);
  Hs += cmul(R.w5, hb0);
#pragma unroll
  for (int d = 0; d < 3; ++d) rest[d] += cmul(R.w5, dr0[d]);
  // y5 - y4 per component (SI), and the position / eta corrections of y5
  float c5x[4], e[8];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float cb5 = 0.0f, cbe = 0.0f;
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      cb5 = fmaf(R.cb5[m], K[m][i] - K[0][i], cb5);
      cbe = fmaf(R.cbe[m], K[m][i], cbe);
    }
    c5x[i] = cb5 + cmul(R.wcb5, K[0][i]);
    e[i] = dt * fmaf(R.dw, u[i], dt * cbe);    // x^mu: dt dW u + dt^2 CBE.k
    e[4 + i] = dt * kE[i];                     // u^mu: dt dC.k
  }
  // tolerances atol + rtol max(|s|, |y5|): the state's coordinates in SI (FP32 is ample for a
  // tolerance), y5 = s + increment
  const ExcField& f = Pm.D.m.fields[P.fi];
  double q[8];
  {
    const float rt = (float)A.rtol, at = (float)A.atol;
    float sv[8], yv[8];
    sv[0] = P.eta.hi;
    yv[0] = fmaf(dt * R.w5.hi, u[0], dt2 * c5x[0]) + sv[0];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      sv[1 + d] = fmaf(P.P[d].hi, F.s[d], (float)(f.origin[d] - f.shift[d]));
      yv[1 + d] = fmaf(dt * R.w5.hi, u[1 + d], dt2 * c5x[1 + d]) + sv[1 + d];
    }
    sv[4] = u[0];
    yv[4] = fmaf(dt, k5_0, u[0]);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      sv[5 + d] = u[1 + d];
      yv[5 + d] = u[1 + d] - dt * fmaf(Hs, u[1 + d], rest[d]);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float tol = fmaf(rt, fmaxf(fabsf(sv[i]), fabsf(yv[i])), at);
      const double r = (double)(e[i] / tol);
      q[i] = r * r;
    }
  }
  // FP64: np.mean of the eight squared ratios (pairwise order), its square root, the factor
  const double err = sqrt((((q[0] + q[1]) + (q[2] + q[3])) + ((q[4] + q[5]) + (q[6] + q[7]))) * 0.125);
  const double dtd = dbl(sd.dt);
  if (!(err <= 1.0)) {
    accepted = false;
    // err^-1/4 = 1 / sqrt(sqrt(err)); NaN (a non-finite stage) keeps the step at the 0.1 floor
    const double g = 0.9 / sqrt(sqrt(err));
    dt_new = dtd * ((g > 0.1) ? g : 0.1);
    return 0;
  }
  accepted = true;
  if (err > 0.0) {
    // err^-1/5: an FP32 estimate finished by one Newton step for g^-5 = err in FP64
    double g = (double)exp2f(-0.2f * log2f((float)err));
    const double g2 = g * g;
    g = g * (1.2 - 0.2 * err * (g2 * g2 * g));
    g *= 0.9;
    dt_new = dtd * ((g < 5.0) ? g : 5.0);
  } else {
    dt_new = dtd * 5.0;
  }
  // the 5th-order update
  const df dtw5 = df_mul(sd.dt, R.w5), dt2d = df_mul(sd.dt, sd.dt);
  const df lunit = F.inv_s[0];
  float dxf[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const df inc = df_add_f(df_mul(P.U[1 + d], dtw5), cmul(dt2d, c5x[1 + d]));   // metres
    dxf[d] = cmul(lunit, inc.hi);
    P.P[d] = df_add(P.P[d], df_mul(inc, F.inv_s[d]));
  }
  P.eta = df_add(P.eta, df_add_f(df_mul(P.U[0], dtw5), cmul(dt2d, c5x[0])));
  P.U[0] = df_add_f(P.U[0], cmul(sd.dt, k5_0));
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const df tot = df_add_f(df_mul_f(P.U[1 + d], Hs), rest[d]);
    const df inc = df_mul(tot, sd.dt);
    P.U[1 + d] = df_add(P.U[1 + d], {-inc.hi, -inc.lo});
  }
  P.lam += fabsf(dt);
  if (obs) {
    // perpendicular displacement dt W5 u_perp + dt^2 sum_m CB5_m q_m; then as in step_rk4_mixed
#pragma unroll
    for (int d = 0; d < 3; ++d) q5[d] += cmul(R.wcb5, Q[0][d]);
    float dperp2 = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float dp = cmul(lunit, cmul(dtw5, up[d]) + cmul(dt2d, q5[d]));
      dperp2 = fmaf(dp, dp, dperp2);
    }
    const float len = sqrtf(fmaf(dxf[0], dxf[0], fmaf(dxf[1], dxf[1], dxf[2] * dxf[2])));
    const float par = fmaf(dxf[0], P.e[0].hi, fmaf(dxf[1], P.e[1].hi, dxf[2] * P.e[2].hi));
    P.excess = df_add_f(P.excess, par > 0.0f ? dperp2 / (len + par) : len - par);
    P.path = df_add_f(P.path, len);
    float r2 = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float r = ((P.P[d].hi - P.lc[d]) + P.P[d].lo) * (F.s[d] * lunit.hi);
      r2 = fmaf(r, r, r2);
    }
    P.min_r2 = fminf(P.min_r2, r2);
  }
  return 0;
}

// Integrator._renormalize_state_to_null (integrator.py:298-335) in FP64 at the double-float
// state: u^0 from g00 u0^2 + g_ij u^i u^j = 0 (the metric is diagonal), the root nearer the
// current u^0; left alone when |g00| < 1e-300 or the discriminant is negative.
template <bool SLOW>
__device__ __forceinline__ int renormalize_f64(const MixParams& Pm, MPhoton& P) {
  const ExcField& f = Pm.D.m.fields[P.fi];
  double x[4], g[4];
  x[0] = dbl(P.eta);
  for (int d = 0; d < 3; ++d) x[1 + d] = (f.origin[d] + dbl(P.P[d]) * f.spacing[d]) - f.shift[d];
  int st;
  if (f.dtype == EXC_DTYPE_F32) st = exc_mixed_f64::metric_diag<float, SLOW>(Pm.D, P.fi, x, g);
  else if (f.dtype == EXC_DTYPE_F32X2) st = exc_mixed_f64::metric_diag<float2, SLOW>(Pm.D, P.fi, x, g);
  else st = exc_mixed_f64::metric_diag<double, SLOW>(Pm.D, P.fi, x, g);
  if (st) return st;
  const double u1 = dbl(P.U[1]), u2 = dbl(P.U[2]), u3 = dbl(P.U[3]);
  const double Acoef = g[0];
  const double Ccoef = u1 * (g[1] * u1) + u2 * (g[2] * u2) + u3 * (g[3] * u3);
  if (fabs(Acoef) < 1e-300) return 0;
  const double disc = -4.0 * Acoef * Ccoef;
  if (disc < 0.0) return 0;
  const double sq = sqrt(disc);
  const double ua = sq / (2.0 * Acoef), ub = -sq / (2.0 * Acoef);
  const double cur = dbl(P.U[0]);
  P.U[0] = df_of((fabs(ua - cur) <= fabs(ub - cur)) ? ua : ub);
  return 0;
}

template <bool SLOW>
__device__ __forceinline__ void photon_finish(const MixParams& Pm, const ExcTraceArgs& A, MPhoton& P) {
  const int64_t p = P.idx;
  if (P.status == EXC_PH_RETRACE) {   // everything else stays as it came in, for the FP64 tracer
    A.status[p] = EXC_PH_RETRACE;
    return;
  }
  double* s = A.state + p * 8;
  const ExcField& f = Pm.D.m.fields[P.fi];
  double s0[8];
  for (int i = 0; i < 8; ++i) s0[i] = s[i];         // the photon's initial state (not yet overwritten)
  double x[4];
  x[0] = dbl(P.eta);
  for (int d = 0; d < 3; ++d) x[1 + d] = (f.origin[d] + dbl(P.P[d]) * f.spacing[d]) - f.shift[d];
  const bool failed = P.status >= EXC_PH_OUTSIDE_GRID;
  double a_em = NAN, phi_em = NAN;
  if (!failed) {
    const int qst = endpoint<SLOW>(Pm, P.fi, x, a_em, phi_em);   // integrator.py:403 evaluates these unconditionally
    if (qst) P.status = qst;
  }
  for (int d = 0; d < 4; ++d) s[d] = x[d];
  for (int d = 0; d < 4; ++d) s[4 + d] = dbl(P.U[d]);
  A.status[p] = P.status;
  if (A.n_steps) A.n_steps[p] = P.steps;
  if (A.n_iter) A.n_iter[p] = P.it;
  if (A.dt_state) A.dt_state[p] = dbl(P.dt);
  if (A.obs && A.obs_flags) {
    double* o = A.obs + p * EXC_OBSCOL_N;
    for (int i = 0; i < EXC_OBSCOL_N; ++i) o[i] = NAN;
    double a_obs = NAN, phi_obs = NAN;
    if (endpoint<SLOW>(Pm, P.fi, s0, a_obs, phi_obs)) { a_obs = NAN; phi_obs = NAN; }
    o[EXC_OBSCOL_ETA_OBS] = s0[0];
    o[EXC_OBSCOL_ETA_EM] = x[0];
    o[EXC_OBSCOL_A_OBS] = a_obs;
    o[EXC_OBSCOL_PHI_OBS] = phi_obs;
    if (P.status < EXC_PH_OUTSIDE_GRID) { o[EXC_OBSCOL_A_EM] = a_em; o[EXC_OBSCOL_PHI_EM] = phi_em; }
    o[EXC_OBSCOL_ISW_INT] = 0.0;
    const double X[3] = {x[1] - s0[1], x[2] - s0[2], x[3] - s0[3]};
    const double chord = sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
    const double su = f.spacing[0];
    o[EXC_OBSCOL_PATH] = dbl(P.path) * su;
    o[EXC_OBSCOL_CHORD] = chord;
    // chord correction |X x e|^2 / (|X| + X.e) with the same unit axis e
    const double e[3] = {dbl(P.e[0]), dbl(P.e[1]), dbl(P.e[2])};
    const double cx = X[1] * e[2] - X[2] * e[1], cy = X[2] * e[0] - X[0] * e[2], cz = X[0] * e[1] - X[1] * e[0];
    const double par = X[0] * e[0] + X[1] * e[1] + X[2] * e[2];
    const double corr = par > 0.0 ? (cx * cx + cy * cy + cz * cz) / (chord + par) : chord - par;
    o[EXC_OBSCOL_EXCESS] = dbl(P.excess) * su - corr;
    o[EXC_OBSCOL_V0X] = s0[5]; o[EXC_OBSCOL_V0Y] = s0[6]; o[EXC_OBSCOL_V0Z] = s0[7];
    o[EXC_OBSCOL_V1X] = s[5]; o[EXC_OBSCOL_V1Y] = s[6]; o[EXC_OBSCOL_V1Z] = s[7];
    const double r0x = (s0[1] - A.lens_center[0]), r0y = (s0[2] - A.lens_center[1]), r0z = (s0[3] - A.lens_center[2]);
    const double r0 = sqrt(r0x * r0x + r0y * r0y + r0z * r0z);
    const double rmin = sqrt((double)P.min_r2) * su;
    o[EXC_OBSCOL_MIN_R] = fmin(r0, rmin);
  }
}

__device__ __forceinline__ bool df_ge(df a, float b) { return a.hi > b || (a.hi == b && a.lo >= 0.0f); }
__device__ __forceinline__ bool df_lt(df a, float b) { return a.hi < b || (a.hi == b && a.lo < 0.0f); }

// EXC_STOP_FACE: the parameter at which the position reaches a face of the stop box along the
// current velocity (cells of the field, faces as hi + lo pairs); a step that would come within
// EXC_FACE_MARGIN of it is shortened to end there. Returns whether it was.
__device__ __forceinline__ bool face_step(const MixParams& Pm, const MPhoton& P, StepDt& sd) {
  const MixField& F = field_of(Pm, P.fi);
  const float sg = sd.f < 0.0f ? -1.0f : 1.0f;
  float tmin = INFINITY;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float v = sg * P.U[1 + d].hi * F.inv_s[d].hi;   // cells per unit lambda
    if (v > 0.0f) tmin = fminf(tmin, ((F.box[3 + d].hi - P.P[d].hi) + (F.box[3 + d].lo - P.P[d].lo)) / v);
    else if (v < 0.0f) tmin = fminf(tmin, ((F.box[d].hi - P.P[d].hi) + (F.box[d].lo - P.P[d].lo)) / v);
  }
  if (!(tmin < (float)EXC_FACE_MARGIN * fabsf(sd.f))) return false;
  const double t = (double)(sg * fmaxf(tmin, 0.0f));
  sd.f = (float)t;
  sd.dt = df_of(t);
  sd.d6 = df_of(t / 6.0);
  sd.c6 = df_of(t * t / 6.0);
  return true;
}

// One iteration of the integrate_single loop (integrator.py:347-400) + stops.
template <bool SLOW, bool RK45>
__device__ __forceinline__ bool photon_iterate(const MixParams& Pm, const float* tab_s, const ExcTraceArgs& A,
                                               MPhoton& P) {
  if (P.status >= 0) return true;    // set at begin (bad field index)
  if (P.it >= A.max_iter) { P.status = EXC_PH_MAX_ITER; return true; }
  if (P.steps >= A.max_steps) { P.status = EXC_PH_STEPS; return true; }
  if (RK45) {
    // the reference clips |dt| into [dt_min, dt_max] every iteration (integrator.py:358-364)
    double dt = dbl(P.dt);
    const double adt = fmin(fmax(fabs(dt), A.dt_min), A.dt_max);
    dt = dt < 0.0 ? -adt : adt;
    P.dt = df_of(dt);
    P.dtf = (float)dt;
  }
  StepDt sd{P.dtf, P.dt, P.d6, P.c6};
  const bool face_mode = (A.stop_flags & EXC_STOP_FACE) != 0;
  const bool face = face_mode && face_step(Pm, P, sd);
  bool accepted = true;
  double dt_new = 0.0;
  const int st = RK45 ? step_rk45_mixed<SLOW>(Pm, tab_s, P, A.obs_flags != 0, sd, A, accepted, dt_new)
                      : step_rk4_mixed<SLOW>(Pm, tab_s, P, A.obs_flags != 0, sd);
  if (st) { P.status = st; return true; }
  if (RK45) {
    P.dt = df_of(dt_new);
    P.dtf = (float)dt_new;
  }
  if (!accepted) { P.it++; return false; }
  if (A.renormalize_every && (P.steps % A.renormalize_every) == 0) {
    const int rs = renormalize_f64<SLOW>(Pm, P);
    if (rs) { P.status = rs; return true; }
  }
  if (!isfinite(P.U[0].hi) || !isfinite(P.P[0].hi) || !isfinite(P.P[1].hi) || !isfinite(P.P[2].hi)) {
    P.status = EXC_PH_NONFINITE;
    return true;
  }
  P.steps++;
  P.it++;
  if (face_mode) {
    // the box stop lands on the face: no other box test, so no window about the faces
    if (face) { P.status = EXC_PH_LEFT_BOX; return true; }
  } else if (A.stop_flags & EXC_STOP_BOX) {
    bool in = true, near = false;
    const float n = (float)P.steps;
    for (int d = 0; d < 3; ++d) {
      in = in && df_ge(P.P[d], P.box[d]) && df_lt(P.P[d], P.box[3 + d]);
      const float w = P.box_tol + fmaf(n, P.wrate[d], kWin0);
      near = near || fabsf((P.P[d].hi - P.box[d]) + P.P[d].lo) < w ||
             fabsf((P.P[d].hi - P.box[3 + d]) + P.P[d].lo) < w;
    }
    if (near) { P.status = EXC_PH_RETRACE; return true; }
    if (!in) { P.status = EXC_PH_LEFT_BOX; return true; }
  }
  if (A.stop_flags & EXC_STOP_A) {
    Stage B;
    base_stage(Pm, P, B, RK45 ? P.lam : (float)P.steps);
    float a, aa, r2;
    cosmo_f32(Pm, tab_s, B.ce, B.fe, a, aa, r2);
    // FP32 a(eta) carries ~3e-7 relative error; within a guard band of a_stop the
    // decision is taken on the FP64 table interpolation the reference performs.
    const float as = Pm.a_stop_f;
    if (a <= as * (1.0f - 1e-5f)) { P.status = EXC_PH_A_STOP; return true; }
    if (a <= as * (1.0f + 1e-5f)) {
      double a64, adot64, inv_a64;
      const double eta = dbl(P.eta);
      if (exc_mixed_f64::scale_factor(Pm.D, eta, a64, adot64, inv_a64) == 0) {
        // the conformal time drifts like the position: the window is the drift over the time travelled
        const double eta_win = (double)kWinRate * fabs(eta - A.state[P.idx * 8]) + 1e-15 * fabs(eta);
        if (fabs(a64 - A.a_stop) <= fabs(adot64) * eta_win) { P.status = EXC_PH_RETRACE; return true; }
        if (a64 <= A.a_stop) { P.status = EXC_PH_A_STOP; return true; }
      }
    }
  }
  return false;
}

// MINB = 1: registers as the compiler likes (144, three 128-thread blocks per SM);
// MINB = 4: capped at 128 registers (a few spills to L1) for four blocks per SM.
// SLOW: the launch has a slow-Interpolator field (a separate instantiation, so
// the base-node kernels keep their register allocation).
template <int MINB, bool SLOW, bool RK45>
__global__ void __launch_bounds__(128, MINB) trace_mixed_kernel(const MixParams Pm, const ExcTraceArgs A) {
  extern __shared__ float tab_s[];
  if (Pm.table_in_smem) {
    for (int i = threadIdx.x; i < Pm.table_n; i += blockDim.x) tab_s[i] = (float)__ldg(Pm.D.m.a_table + i);
    __syncthreads();
  }
  MPhoton P;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t static_next = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const long long t0 = clock64();
  int64_t p = next_photon(A, static_next, stride);
  bool active = p < A.n_photons;
  if (active) photon_begin(Pm, A, P, p);
  while (active) {
    bool done = photon_iterate<SLOW, RK45>(Pm, tab_s, A, P);
    if (!done && (P.it & 63) == 0) {
      if (A.abort_flag && *(volatile const int32_t*)A.abort_flag) { P.status = EXC_PH_ABORTED; done = true; }
      else if (A.deadline_cycles > 0 && clock64() - t0 > A.deadline_cycles) { P.status = EXC_PH_TIMED_OUT; done = true; }
    }
    if (done) {
      photon_finish<SLOW>(Pm, A, P);
      if (P.status == EXC_PH_ABORTED || P.status == EXC_PH_TIMED_OUT) break;
      p = next_photon(A, static_next, stride);
      active = p < A.n_photons;
      if (active) photon_begin(Pm, A, P, p);
    }
  }
}

// ------------------------------------------------------------- host side
int check(const DevMetric& D, const ExcTraceArgs& A) {
  if (D.m.kind != EXC_METRIC_FLRW) return 1;
  if (A.stepper != EXC_STEPPER_RK4 && A.stepper != EXC_STEPPER_RK45) return 2;
  if (A.records) return 3;
  for (int i = 0; i < D.m.n_fields; ++i) {
    if (D.m.fields[i].ndim != 3) return 5;
    if (D.m.fields[i].grad_mode != EXC_GRAD_BASE_NODE && D.m.fields[i].grad_mode != EXC_GRAD_TRILINEAR) return 8;
    const int64_t* n = D.m.fields[i].n;
    if (n[0] * n[1] * n[2] >= (int64_t)1 << 31) return 6;
  }
  if (A.obs_flags & EXC_OBS_ISW) return 7;
  return 0;
}

const char* why(int code) {
  switch (code) {
    case 1: return "mixed precision supports the FLRW metric only";
    case 2: return "mixed precision supports the RK4 and RK45 steppers only";
    case 3: return "mixed precision does not record trajectories";
    case 5: return "mixed precision supports 3-D (static) potential grids only";
    case 6: return "mixed precision needs grids below 2^31 nodes";
    case 7: return "mixed precision has no ISW accumulator (static grids only)";
    case 8: return "mixed precision: unknown gradient mode";
    default: return "mixed precision: unsupported";
  }
}

static df df_host(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}

cudaError_t trace(const DevMetric& D, const ExcTraceArgs& A, int block, int blocks_per_sm, int sm_count,
                  cudaStream_t s) {
  MixParams* P = new MixParams();   // ~9 KB host-side parameter block (not device memory)
  P->D = D;
  const ExcMetric& m = D.m;
  for (int i = 0; i < m.n_fields; ++i) {
    const ExcField& f = m.fields[i];
    MixField& F = P->mf[i];
    F.data = f.data;
    F.dtype = f.dtype;
    F.boundary = f.boundary;
    F.slow = f.grad_mode == EXC_GRAD_TRILINEAR;
    F.nodes = (int)(f.n[0] * f.n[1] * f.n[2]);
    for (int d = 0; d < 3; ++d) {
      F.n[d] = (int)f.n[d];
      F.s[d] = (float)f.spacing[d];
      F.inv_s[d] = df_host(1.0 / f.spacing[d]);
      F.inv_2s[d] = (float)(1.0 / (2.0 * f.spacing[d]));
    }
  }
  P->ic2 = (float)(1.0 / m.c2);
  P->ic4 = (float)(1.0 / m.c4);
  P->c2f_over_c4 = (float)(m.c2 / m.c4);
  P->two_over_c2 = (float)m.two_over_c2;
  P->ic2d = df_host(1.0 / m.c2);
  if (m.cosmology != EXC_COSMO_STATIC) {
    P->eta_min = df_host(m.eta_min);
    P->inv_eta_step = df_host(1.0 / m.eta_step);
    P->table_n = (int)m.a_table_n;
  }
  P->H0 = df_host(m.H0);
  P->om = df_host(m.omega_m);
  P->orad = df_host(m.omega_r);
  P->ok = df_host(m.omega_k);
  P->ol = df_host(m.omega_lambda);
  size_t smem = 0;
  if (m.cosmology != EXC_COSMO_STATIC && m.a_table_n <= 12288) {
    P->table_in_smem = 1;
    smem = (size_t)m.a_table_n * sizeof(float);
  }
  P->a_stop_f = (float)A.a_stop;
  // stop-box faces in each field's cells, as the photons' positions are kept
  for (int i = 0; i < m.n_fields; ++i) {
    const ExcField& f = m.fields[i];
    for (int d = 0; d < 3; ++d) {
      P->mf[i].box[d] = df_host(((A.box_lo[d] + f.shift[d]) - f.origin[d]) / f.spacing[d]);
      P->mf[i].box[3 + d] = df_host(((A.box_hi[d] + f.shift[d]) - f.origin[d]) / f.spacing[d]);
    }
  }
  if (A.stepper == EXC_STEPPER_RK45) {
    // Fehlberg's nodes and 4th-order weights; the 5th-order weights of the reference (665/1287
    // for the third) or Fehlberg's (6656/12825), integrator.py:106-115
    const double b[6][6] = {{0, 0, 0, 0, 0, 0},
                            {1.0 / 4.0, 0, 0, 0, 0, 0},
                            {3.0 / 32.0, 9.0 / 32.0, 0, 0, 0, 0},
                            {1932.0 / 2197.0, -7200.0 / 2197.0, 7296.0 / 2197.0, 0, 0, 0},
                            {439.0 / 216.0, -8.0, 3680.0 / 513.0, -845.0 / 4104.0, 0, 0},
                            {-8.0 / 27.0, 2.0, -3544.0 / 2565.0, 1859.0 / 4104.0, -11.0 / 40.0, 0}};
    const double c5[6] = {16.0 / 135.0, 0.0,
                          A.tableau == EXC_TABLEAU_FEHLBERG ? 6656.0 / 12825.0 : 665.0 / 1287.0,
                          28561.0 / 56430.0, -9.0 / 50.0, 2.0 / 55.0};
    const double c4[6] = {25.0 / 216.0, 0.0, 1408.0 / 2565.0, 2197.0 / 4104.0, -1.0 / 5.0, 0.0};
    RKF& R = P->rk;
    double w5 = 0.0;
    for (int j = 0; j < 6; ++j) {
      double cj = 0.0, cb5 = 0.0, cbe = 0.0;
      for (int l = 0; l < 6; ++l) {
        R.b[j][l] = (float)b[j][l];
        double bb = 0.0;
        for (int q = 0; q < 6; ++q) bb += b[j][q] * b[q][l];
        R.bb[j][l] = (float)bb;
        cj += b[j][l];
        cb5 += c5[l] * b[l][j];
        cbe += (c5[l] - c4[l]) * b[l][j];
      }
      R.c[j] = (float)cj;
      R.c5[j] = (float)c5[j];
      R.dc[j] = (float)(c5[j] - c4[j]);
      R.cb5[j] = (float)cb5;
      R.cbe[j] = (float)cbe;
      w5 += c5[j];
    }
    R.w5 = df_host(w5);
    double wcb5 = 0.0;
    for (int m = 0; m < 6; ++m)
      for (int l = 0; l < 6; ++l) wcb5 += c5[l] * b[l][m];
    R.wcb5 = df_host(wcb5);
    // the 4th-order weights sum to 1: dW is the 5th-order sum's departure from it
    R.dw = (float)(A.tableau == EXC_TABLEAU_FEHLBERG ? 0.0 : 665.0 / 1287.0 - 6656.0 / 12825.0);
  }
  int per_sm = blocks_per_sm;
  // a plan with four or more resident blocks per SM takes the 128-register build
  bool slow = false;
  for (int i = 0; i < m.n_fields; ++i) slow = slow || P->mf[i].slow;
  const bool rk45 = A.stepper == EXC_STEPPER_RK45;
  void (*kern)(const MixParams, const ExcTraceArgs) =
      rk45 ? (slow ? (per_sm >= 4 ? trace_mixed_kernel<4, true, true> : trace_mixed_kernel<1, true, true>)
                   : (per_sm >= 4 ? trace_mixed_kernel<4, false, true> : trace_mixed_kernel<1, false, true>))
           : (slow ? (per_sm >= 4 ? trace_mixed_kernel<4, true, false> : trace_mixed_kernel<1, true, false>)
                   : (per_sm >= 4 ? trace_mixed_kernel<4, false, false> : trace_mixed_kernel<1, false, false>));
  cudaError_t e = cudaSuccess;
  if (per_sm <= 0) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
    if (e != cudaSuccess) { delete P; return e; }
    if (per_sm < 1) per_sm = 1;
  }
  int64_t grid = (int64_t)sm_count * per_sm;
  const int64_t need = (A.n_photons + block - 1) / block;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  kern<<<(int)grid, block, smem, s>>>(*P, A);
  e = cudaGetLastError();
  delete P;
  return e;
}

}  // namespace exc_mixed
