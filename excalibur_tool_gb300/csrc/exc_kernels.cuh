// exc_kernels.cuh -- FP64 tracer kernels and their launchers.
//
// Included by exc_exact.cu (EXC_FAST=0, built without FMA contraction) and
// exc_fast.cu (EXC_FAST=1) inside namespace EXC_NS, so one source yields the
// parity path and the fast FP64 path.
//
// Execution model: one thread owns one photon; its 8-component state, RK
// stages and running observables stay in registers for the whole trajectory.
// The kernel is persistent (grid = SMs x blocks_per_sm) and lanes refill:
// a lane whose photon terminates takes the next photon index from a device
// counter (warp-aggregated atomicAdd) and keeps stepping in lock-step with
// the lanes still on their old photons, so uneven trajectory lengths do not
// idle the warp.
#pragma once

#include <cooperative_groups.h>
#include "exc_device.cuh"
#include "exc_sched.h"
#include "exc_stepctl.h"

namespace EXC_NS {

namespace cg = cooperative_groups;

// Template tag of the FLRW kernels that can read slow-Interpolator fields
// (ExcField.grad_mode EXC_GRAD_TRILINEAR): a separate instantiation, so that the
// base-node kernels are compiled without that path.
constexpr int kFlrwSlowInterp = 0x100 | EXC_METRIC_FLRW;
constexpr bool is_flrw(int mk) { return (mk & 0xff) == EXC_METRIC_FLRW; }
constexpr bool slow_interp(int mk) { return mk == kFlrwSlowInterp; }

// ------------------------------------------------------- photon context
struct Photon {
  double s[8];
  double dt;
  int64_t idx;
  int32_t steps, it, status;
  // observables
  double a_obs, phi_obs, eta_obs;
  double path, excess, min_r;
  double p0[3], pprev[3], e0[3], v0[3];
  double isw, pdot_prev;
  // records
  int32_t nrec;
  double q[6];   // quantities attached to the next record (reference lags them by one record)
  bool qvalid;
  bool bad_field;
};

template <int MK>
__device__ __forceinline__ void cart_pos(const ExcMetric& m, const double s[8], double out[3]) {
  if (MK == EXC_METRIC_SCHWARZSCHILD) {
    // _sph_to_xyz_rel, _postprocessing/analyze_compare_trajectories.py:86-96 (lens-centred)
    double st, ct, sp, cp;
    sincos(s[2], &st, &ct);
    sincos(s[3], &sp, &cp);
    out[0] = s[1] * st * cp;
    out[1] = s[1] * st * sp;
    out[2] = s[1] * ct;
  } else {
    out[0] = s[1]; out[1] = s[2]; out[2] = s[3];
  }
}

template <int MK>
__device__ __forceinline__ void cart_vel(const double s[8], double v[3]) {
  if (MK == EXC_METRIC_SCHWARZSCHILD) {
    // _sph_vel_to_cart, analyze_compare_trajectories.py:99-112
    double st, ct, sp, cp;
    sincos(s[2], &st, &ct);
    sincos(s[3], &sp, &cp);
    const double r = s[1], dr = s[5], dth = s[6], dph = s[7];
    v[0] = dr * (st * cp) + (r * dth) * (ct * cp) + (r * st * dph) * (-sp);
    v[1] = dr * (st * sp) + (r * dth) * (ct * sp) + (r * st * dph) * (cp);
    v[2] = dr * (ct) + (r * dth) * (-st);
  } else {
    v[0] = s[5]; v[1] = s[6]; v[2] = s[7];
  }
}

__device__ __forceinline__ double norm3(const double v[3]) {
  return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

// |d| - d.e without cancellation (e a unit vector): |d x e|^2 / (|d| + d.e).
__device__ __forceinline__ double excess_term(const double d[3], const double e[3]) {
  const double nd = norm3(d);
  const double de = d[0] * e[0] + d[1] * e[1] + d[2] * e[2];
  if (de <= 0.0) return nd - de;
  const double cx = d[1] * e[2] - d[2] * e[1];
  const double cy = d[2] * e[0] - d[0] * e[2];
  const double cz = d[0] * e[1] - d[1] * e[0];
  const double den = nd + de;
  return den > 0.0 ? (cx * cx + cy * cy + cz * cz) / den : 0.0;
}

template <int MK, class FT>
struct Tracer {
  const DevMetric& D;
  const ExcTraceArgs& A;
  int fi;

  __device__ __forceinline__ Tracer(const DevMetric& d, const ExcTraceArgs& a) : D(d), A(a), fi(0) {}

  __device__ __forceinline__ int rhs(const double s[8], double out[8]) const {
    if (MK == EXC_METRIC_SCHWARZSCHILD) return schw_rhs(D, s, out);
    return flrw_rhs<FT, slow_interp(MK)>(D, fi, s, out);
  }

  // Metric.metric_physical_quantities (perturbed_flrw_metric_fast.py:275-282;
  // schwarzschild_metric_fast.py:305-308).
  __device__ __forceinline__ int quantities(const double s[8], double q[6]) const {
    if (MK == EXC_METRIC_SCHWARZSCHILD) {
      q[0] = s[1]; q[1] = D.m.mass; q[2] = D.m.radius; q[3] = D.m.r_s; q[4] = NAN; q[5] = NAN;
      return 0;
    }
    double a, adot, inv_a;
    int st = scale_factor(D, s[0], a, adot, inv_a);
    if (st) return st;
    InterpOut ip;
    st = interp_field<FT, slow_interp(MK)>(D.m.fields[fi], D.finv[fi], s[1], s[2], s[3], s[0], ip);
    if (st) return st;
    q[0] = a; q[1] = ip.val; q[2] = ip.gx; q[3] = ip.gy; q[4] = ip.gz; q[5] = ip.dtd;
    return 0;
  }

  // ---- steppers (integrator.py:9-152) --------------------------------
  // RK4.step, integrator.py:10-22
  __device__ __forceinline__ int step_rk4(const double s[8], double dt, double out[8]) const {
    // k1..k4 in a loop over the stages: one inlined copy of the RHS instead of four, with the
    // unrolled form's operations in its order -- acc = k1 + 2 k2 + 2 k3, the stage points
    // s + (dt/2) k1, s + (dt/2) k2, s + dt k3, then s + (dt/6)(acc + k4). (Measured on GB300:
    // 2 % faster than the unrolled form, and a quarter of its code to compile.)
    double k[8], acc[8], tmp[8];
    const double h = 0.5 * dt;
#pragma unroll
    for (int i = 0; i < 8; ++i) tmp[i] = s[i];
#pragma unroll 1
    for (int stage = 0; stage < 4; ++stage) {
      const int st = rhs(tmp, k);
      if (st) return st;
      if (stage == 3) break;
      const double c = stage < 2 ? h : dt;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        acc[i] = stage == 0 ? k[i] : acc[i] + 2.0 * k[i];
        tmp[i] = s[i] + c * k[i];
      }
    }
    const double d6 = ::div_rn(dt, 6.0, 1.0 / 6.0);   // dt / 6, correctly rounded (1/6 folded at compile time)
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = s[i] + d6 * (acc[i] + k[i]);
    return 0;
  }

  // Leapfrog4.step (Forest-Ruth), integrator.py:24-90. Coefficients are the
  // float64 values of the reference's class constants.
  __device__ __forceinline__ int step_lf4(const double s[8], double dt, double out[8]) const {
    const double w0 = -0x1.b3d16dd72c671p+0, w1 = 0x1.59e8b6eb96339p+0;
    const double c1 = 0x1.59e8b6eb96339p-1, c2 = -0x1.67a2dbae58ce0p-3;
    const double cs[4] = {c1, c2, c2, c1};
    const double ds[3] = {w1, w0, w1};
    double y[8], k[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = s[i];
#pragma unroll
    for (int stage = 0; stage < 3; ++stage) {
      const double cd = cs[stage] * dt;
#pragma unroll
      for (int i = 0; i < 4; ++i) y[i] = y[i] + cd * y[4 + i];
      int st = rhs(y, k);
      if (st) return st;
      const double dd = ds[stage] * dt;
#pragma unroll
      for (int i = 0; i < 4; ++i) y[4 + i] = y[4 + i] + dd * k[4 + i];
    }
    const double cd = cs[3] * dt;
#pragma unroll
    for (int i = 0; i < 4; ++i) y[i] = y[i] + cd * y[4 + i];
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = y[i];
    return 0;
  }

  // RK45Adaptive.step, integrator.py:93-152 (Fehlberg 4(5) nodes; weights of
  // the reference, or Fehlberg's 6656/12825 when tableau == FEHLBERG).
  __device__ __forceinline__ int step_rk45(const double s[8], double dt, double out[8], double& dt_new,
                                           bool& accepted) const {
    const double B1_0 = 1.0 / 4.0;
    const double B2_0 = 3.0 / 32.0, B2_1 = 9.0 / 32.0;
    const double B3_0 = 1932.0 / 2197.0, B3_1 = -7200.0 / 2197.0, B3_2 = 7296.0 / 2197.0;
    const double B4_0 = 439.0 / 216.0, B4_1 = -8.0, B4_2 = 3680.0 / 513.0, B4_3 = -845.0 / 4104.0;
    const double B5_0 = -8.0 / 27.0, B5_1 = 2.0, B5_2 = -3544.0 / 2565.0, B5_3 = 1859.0 / 4104.0,
                 B5_4 = -11.0 / 40.0;
    const double C5_0 = 16.0 / 135.0, C5_3 = 28561.0 / 56430.0, C5_4 = -9.0 / 50.0, C5_5 = 2.0 / 55.0;
    const double C5_2 = (A.tableau == EXC_TABLEAU_FEHLBERG) ? 6656.0 / 12825.0 : 665.0 / 1287.0;
    const double C4_0 = 25.0 / 216.0, C4_2 = 1408.0 / 2565.0, C4_3 = 2197.0 / 4104.0, C4_4 = -1.0 / 5.0;
    double K0[8], K1[8], K2[8], K3[8], K4[8], K5[8], y[8];
    int st = rhs(s, K0);
    if (st) return st;
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = s[i] + dt * (B1_0 * K0[i]);
    if ((st = rhs(y, K1))) return st;
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = s[i] + dt * (B2_0 * K0[i] + B2_1 * K1[i]);
    if ((st = rhs(y, K2))) return st;
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = s[i] + dt * (B3_0 * K0[i] + B3_1 * K1[i] + B3_2 * K2[i]);
    if ((st = rhs(y, K3))) return st;
#pragma unroll
    for (int i = 0; i < 8; ++i)
      y[i] = s[i] + dt * (B4_0 * K0[i] + B4_1 * K1[i] + B4_2 * K2[i] + B4_3 * K3[i]);
    if ((st = rhs(y, K4))) return st;
#pragma unroll
    for (int i = 0; i < 8; ++i)
      y[i] = s[i] + dt * (B5_0 * K0[i] + B5_1 * K1[i] + B5_2 * K2[i] + B5_3 * K3[i] + B5_4 * K4[i]);
    if ((st = rhs(y, K5))) return st;
    // y5, y4 and the weighted RMS error (np.mean of 8 terms = pairwise sum / 8)
    double q[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const double y5 = s[i] + dt * (C5_0 * K0[i] + 0.0 * K1[i] + C5_2 * K2[i] + C5_3 * K3[i] +
                                     C5_4 * K4[i] + C5_5 * K5[i]);
      const double y4 = s[i] + dt * (C4_0 * K0[i] + 0.0 * K1[i] + C4_2 * K2[i] + C4_3 * K3[i] +
                                     C4_4 * K4[i] + 0.0 * K5[i]);
      const double err = y5 - y4;
      const double m0 = fabs(s[i]), m1 = fabs(y5);
      const double mx = (isnan(m0) || isnan(m1)) ? NAN : fmax(m0, m1);   // np.maximum
      const double tol = A.atol + A.rtol * mx;
      const double r = err / tol;
      q[i] = r * r;
      out[i] = y5;
    }
    const double mean = (((q[0] + q[1]) + (q[2] + q[3])) + ((q[4] + q[5]) + (q[6] + q[7]))) / 8.0;
    const double err_ratio = sqrt(mean);
    if (err_ratio <= 1.0) {
      const double g = (err_ratio > 0.0) ? 0.9 * exc_ctl_pow_m1_5(err_ratio) : 5.0;
      dt_new = dt * ((g < 5.0) ? g : 5.0);
      accepted = true;
    } else {
      const double g = 0.9 * exc_ctl_pow_m1_4(err_ratio);
      dt_new = dt * ((g > 0.1) ? g : 0.1);
      accepted = false;
    }
    return 0;
  }

  // Integrator._renormalize_state_to_null, integrator.py:298-335.
  __device__ __forceinline__ int renormalize(double s[8]) const {
    double g[4];
    int st = metric_diag<FT, slow_interp(MK)>(D, fi, s, g);
    if (st) return st;
    const double u1 = s[5], u2 = s[6], u3 = s[7];
    const double Acoef = g[0];
    const double Bcoef = 2.0 * (0.0 * u1 + 0.0 * u2 + 0.0 * u3);
    const double Ccoef = u1 * (g[1] * u1) + u2 * (g[2] * u2) + u3 * (g[3] * u3);
    if (fabs(Acoef) < 1e-300) return 0;
    const double disc = Bcoef * Bcoef - 4.0 * Acoef * Ccoef;
    if (disc < 0.0) return 0;
    const double sq = sqrt(disc);
    const double ua = (-Bcoef + sq) / (2.0 * Acoef);
    const double ub = (-Bcoef - sq) / (2.0 * Acoef);
    const double cur = s[4];
    s[4] = (fabs(ua - cur) <= fabs(ub - cur)) ? ua : ub;
    return 0;
  }
};

// np.clip(x, lo, hi) == minimum(maximum(x, lo), hi), NaN-propagating
__device__ __forceinline__ double np_clip(double x, double lo, double hi) {
  if (isnan(x) || isnan(lo) || isnan(hi)) return NAN;
  return fmin(fmax(x, lo), hi);
}

// EXC_STOP_FACE (FLRW): the parameter lambda >= 0 at which x + lambda * sign(dt) * u first
// reaches a face of the stop box; a step that would come within EXC_FACE_MARGIN of it is
// shortened to end there (`clipped`).
__device__ __forceinline__ double face_clip(const double s[8], double dt, const double lo[3], const double hi[3],
                                            bool& clipped) {
  const double sg = dt < 0.0 ? -1.0 : 1.0;
  double tmin = INFINITY;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double v = sg * s[5 + d];
    if (v > 0.0) tmin = fmin(tmin, (hi[d] - s[1 + d]) / v);
    else if (v < 0.0) tmin = fmin(tmin, (lo[d] - s[1 + d]) / v);
  }
  clipped = tmin < EXC_FACE_MARGIN * fabs(dt);
  return clipped ? sg * fmax(tmin, 0.0) : dt;
}

// ------------------------------------------------------------- queue
__device__ __forceinline__ int64_t next_photon(const ExcTraceArgs& A, int64_t& static_next, int64_t stride) {
  if (A.queue == nullptr) {
    const int64_t p = static_next;
    static_next += stride;
    return p;
  }
  // warp-aggregated fetch: one atomic per group of lanes arriving together
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned long long base = 0;
  if (g.thread_rank() == 0)
    base = atomicAdd(reinterpret_cast<unsigned long long*>(A.queue), (unsigned long long)g.size());
  base = g.shfl(base, 0);
  return (int64_t)(base + g.thread_rank());
}

template <int MK, class FT, bool REC>
__device__ __forceinline__ void write_record(const Tracer<MK, FT>& T, const ExcTraceArgs& A, Photon& P,
                                             const double* q) {
  if (!REC) return;
  if (P.nrec < A.max_records) {
    double* row = A.records + ((int64_t)P.idx * A.max_records + P.nrec) * A.record_cols;
#pragma unroll
    for (int i = 0; i < 8; ++i) row[i] = P.s[i];
    for (int i = 8; i < A.record_cols; ++i) row[i] = q ? q[i - 8] : NAN;
  }
  P.nrec++;
}

// Start a photon: load state, record the initial row, initialise observables.
template <int MK, class FT, bool REC>
__device__ __forceinline__ void photon_begin(Tracer<MK, FT>& T, const ExcTraceArgs& A, Photon& P, int64_t p) {
  P.idx = p;
  T.fi = A.field_index ? A.field_index[p] : 0;
  P.bad_field = (unsigned)T.fi >= (unsigned)T.D.m.n_fields && is_flrw(MK);
  if (P.bad_field) T.fi = 0;   // never index past the descriptor table
  const double* src = A.state + p * 8;
#pragma unroll
  for (int i = 0; i < 8; ++i) P.s[i] = src[i];
  P.dt = A.dt_state ? A.dt_state[p] : A.dt;
  P.steps = 0; P.it = 0; P.status = -1;
  P.nrec = 0; P.qvalid = false;
  write_record<MK, FT, REC>(T, A, P, nullptr);   // integrator.py:339-342 (no quantities yet)
  if (A.obs_flags) {
    cart_pos<MK>(T.D.m, P.s, P.p0);
#pragma unroll
    for (int i = 0; i < 3; ++i) P.pprev[i] = P.p0[i];
    cart_vel<MK>(P.s, P.v0);
    const double nv = norm3(P.v0);
#pragma unroll
    for (int i = 0; i < 3; ++i) P.e0[i] = nv > 0.0 ? P.v0[i] / nv : 0.0;
    P.path = 0.0; P.excess = 0.0; P.isw = 0.0; P.pdot_prev = 0.0;
    P.eta_obs = P.s[0];
    double rel[3];
    if (MK == EXC_METRIC_SCHWARZSCHILD) { rel[0] = P.p0[0]; rel[1] = P.p0[1]; rel[2] = P.p0[2]; }
    else { for (int i = 0; i < 3; ++i) rel[i] = P.p0[i] - A.lens_center[i]; }
    P.min_r = norm3(rel);
    P.a_obs = NAN; P.phi_obs = NAN;
    if (is_flrw(MK)) {
      double q[6];
      if (T.quantities(P.s, q) == 0) { P.a_obs = q[0]; P.phi_obs = q[1]; P.pdot_prev = q[5]; }
    }
  }
}

// Per accepted step: path, stable excess, min_r, ISW.
template <int MK, class FT>
__device__ __forceinline__ void photon_accumulate(const Tracer<MK, FT>& T, const ExcTraceArgs& A, Photon& P,
                                                  const double* s_old) {
  double pc[3];
  cart_pos<MK>(T.D.m, P.s, pc);
  if (A.obs_flags & EXC_OBS_PATH) {
    double d[3] = {pc[0] - P.pprev[0], pc[1] - P.pprev[1], pc[2] - P.pprev[2]};
    P.path += norm3(d);
    P.excess += excess_term(d, P.e0);
  }
  if (A.obs_flags & EXC_OBS_ENDPOINTS) {
    double rel[3];
    if (MK == EXC_METRIC_SCHWARZSCHILD) { rel[0] = pc[0]; rel[1] = pc[1]; rel[2] = pc[2]; }
    else { for (int i = 0; i < 3; ++i) rel[i] = pc[i] - A.lens_center[i]; }
    const double r = norm3(rel);
    if (r < P.min_r) P.min_r = r;
  }
  if (is_flrw(MK) && (A.obs_flags & EXC_OBS_ISW)) {
    double q[6];
    if (T.quantities(P.s, q) == 0) {
      P.isw += 0.5 * (P.pdot_prev + q[5]) * (P.s[0] - s_old[0]);
      P.pdot_prev = q[5];
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) P.pprev[i] = pc[i];
}

template <int MK, class FT, bool REC>
__device__ __forceinline__ void photon_finish(const Tracer<MK, FT>& T, const ExcTraceArgs& A, Photon& P) {
  const int64_t p = P.idx;
  const bool failed = P.status >= EXC_PH_OUTSIDE_GRID;
  double qf[6];
  int qst = 0;
  // integrator.py:403 evaluates the quantities at the final state unconditionally;
  // a failure there (e.g. outside the strict grid interior) fails the photon.
  if (!failed) qst = T.quantities(P.s, qf);
  if (REC) {
    // integrator.py:403-404: quantities at the final state, then the final record
    if (!failed && qst == 0) write_record<MK, FT, REC>(T, A, P, qf);
    A.n_records[p] = P.nrec;
  }
  if (!failed && qst) P.status = qst;   // the reference raises inside state_quantities
#pragma unroll
  for (int i = 0; i < 8; ++i) A.state[p * 8 + i] = P.s[i];
  A.status[p] = P.status;
  if (A.n_steps) A.n_steps[p] = P.steps;
  if (A.n_iter) A.n_iter[p] = P.it;
  if (A.dt_state) A.dt_state[p] = P.dt;
  if (A.obs && A.obs_flags) {
    double* o = A.obs + p * EXC_OBSCOL_N;
    for (int i = 0; i < EXC_OBSCOL_N; ++i) o[i] = NAN;
    o[EXC_OBSCOL_ETA_OBS] = P.eta_obs;
    o[EXC_OBSCOL_ETA_EM] = P.s[0];
    o[EXC_OBSCOL_A_OBS] = P.a_obs;
    o[EXC_OBSCOL_PHI_OBS] = P.phi_obs;
    if (is_flrw(MK) && !failed && qst == 0) { o[EXC_OBSCOL_A_EM] = qf[0]; o[EXC_OBSCOL_PHI_EM] = qf[1]; }
    o[EXC_OBSCOL_ISW_INT] = P.isw;
    if (A.obs_flags & EXC_OBS_PATH) {
      double pc[3];
      cart_pos<MK>(T.D.m, P.s, pc);
      double X[3] = {pc[0] - P.p0[0], pc[1] - P.p0[1], pc[2] - P.p0[2]};
      const double chord = norm3(X);
      o[EXC_OBSCOL_PATH] = P.path;
      o[EXC_OBSCOL_CHORD] = chord;
      o[EXC_OBSCOL_EXCESS] = P.excess - excess_term(X, P.e0);
    }
    double v1[3];
    cart_vel<MK>(P.s, v1);
    o[EXC_OBSCOL_V0X] = P.v0[0]; o[EXC_OBSCOL_V0Y] = P.v0[1]; o[EXC_OBSCOL_V0Z] = P.v0[2];
    o[EXC_OBSCOL_V1X] = v1[0]; o[EXC_OBSCOL_V1Y] = v1[1]; o[EXC_OBSCOL_V1Z] = v1[2];
    o[EXC_OBSCOL_MIN_R] = P.min_r;
  }
}

// One iteration of Integrator.integrate_single's loop (integrator.py:347-400)
// plus the added box / scale-factor stops. Returns true when the photon ends.
template <int MK, class FT, int STEPPER, bool REC>
__device__ __forceinline__ bool photon_iterate(Tracer<MK, FT>& T, const ExcTraceArgs& A, Photon& P) {
  if (P.bad_field) { P.status = EXC_PH_BAD_FIELD; return true; }
  if (P.it >= A.max_iter) { P.status = EXC_PH_MAX_ITER; return true; }
  if (P.steps >= A.max_steps) { P.status = EXC_PH_STEPS; return true; }
  double dt = P.dt;
  if (dt < 0.0) dt = -np_clip(-dt, A.dt_min, A.dt_max);   // integrator.py:358-364
  else dt = np_clip(dt, A.dt_min, A.dt_max);
  bool face = false;
  if (is_flrw(MK) && (A.stop_flags & EXC_STOP_FACE)) dt = face_clip(P.s, dt, A.box_lo, A.box_hi, face);
  double ns[8];
  double dt_new = dt;
  bool accepted = true;
  int st;
  if (STEPPER == EXC_STEPPER_RK4) st = T.step_rk4(P.s, dt, ns);
  else if (STEPPER == EXC_STEPPER_LEAPFROG4) st = T.step_lf4(P.s, dt, ns);
  else st = T.step_rk45(P.s, dt, ns, dt_new, accepted);
  if (st) { P.status = st; P.dt = dt; return true; }
  bool stop = false;
  if (accepted) {
    if (A.renormalize_every && (P.steps % A.renormalize_every) == 0) {
      st = T.renormalize(ns);
      if (st) { P.status = st; P.dt = dt; return true; }
    }
    double s_old0[1] = {P.s[0]};
#pragma unroll
    for (int i = 0; i < 8; ++i) P.s[i] = ns[i];
    if (REC && (A.record_every == 1 || (A.record_every > 1 && (P.steps % A.record_every) == 0))) {
      write_record<MK, FT, REC>(T, A, P, P.qvalid ? P.q : nullptr);
      st = T.quantities(P.s, P.q);
      if (st) { P.status = st; P.dt = dt_new; P.steps++; P.it++; return true; }
      P.qvalid = true;
    }
    if (A.obs_flags) photon_accumulate<MK, FT>(T, A, P, s_old0);
    P.steps++;
    if (is_flrw(MK) && (A.stop_flags & EXC_STOP_FACE)) {
      if (face) {
        P.status = EXC_PH_LEFT_BOX;
        stop = true;
      }
    } else if (A.stop_flags & EXC_STOP_BOX) {
      double pc[3];
      cart_pos<MK>(T.D.m, P.s, pc);
      if (MK == EXC_METRIC_SCHWARZSCHILD) for (int i = 0; i < 3; ++i) pc[i] += T.D.m.center[i];
      if (!(pc[0] >= A.box_lo[0] && pc[0] < A.box_hi[0] && pc[1] >= A.box_lo[1] && pc[1] < A.box_hi[1] &&
            pc[2] >= A.box_lo[2] && pc[2] < A.box_hi[2])) {
        P.status = EXC_PH_LEFT_BOX;
        stop = true;
      }
    }
    if (!stop && is_flrw(MK) && (A.stop_flags & EXC_STOP_A)) {
      double a, adot, inv_a;
      if (scale_factor(T.D, P.s[0], a, adot, inv_a) == 0 && a <= A.a_stop) {
        P.status = EXC_PH_A_STOP;
        stop = true;
      }
    }
  }
  P.dt = dt_new;
  P.it++;
  return stop;
}

// Next photon to trace; in a re-trace pass only those the mixed tracer handed back.
__device__ __forceinline__ int64_t next_work(const DevMetric& D, const ExcTraceArgs& A, int64_t& static_next,
                                             int64_t stride) {
  int64_t p = next_photon(A, static_next, stride);
  if (D.retrace_only)
    while (p < A.n_photons && A.status[p] != EXC_PH_RETRACE) p = next_photon(A, static_next, stride);
  return p;
}

template <int MK, class FT, int STEPPER, bool REC>
__global__ void __launch_bounds__(128) trace_kernel(const DevMetric D, const ExcTraceArgs A) {
  // Re-tracing the rays the mixed tracer handed back. A few of them (a guard's share of one
  // batch) run fastest in as few warps an SM as hold them: the warps of an SM share its FP64
  // throughput, and a lone warp's dependent FP64 chain waits least. Many run fastest with every
  // resident warp. The share is estimated from the same 1,024 statuses in every block; the warps
  // an SM needs at 32 rays a warp stay (blocks 0 .. SMs-1 first, one on each SM as the launch
  // hands them out), the rest leave at once -- the work queue hands every ray to the warps that
  // stay (the static assignment, without a queue, keeps every warp).
  bool retrace_idle = false;
  if (D.retrace_only && A.queue) {
    __shared__ int s_hits;
    if (threadIdx.x == 0) s_hits = 0;
    __syncthreads();
    int hits = 0;
    for (int k = threadIdx.x; k < 1024; k += blockDim.x)
      hits += A.status[(int64_t)k * A.n_photons / 1024] == EXC_PH_RETRACE;
    if (hits) atomicAdd(&s_hits, hits);
    __syncthreads();
    const double rays = (double)s_hits * (double)A.n_photons * (1.0 / 1024.0);
    const int sms = D.retrace_sms > 0 ? D.retrace_sms : 1;
    const double need = ceil(rays / ((double)sms * 32.0));   // warps an SM
    const int warps = blockDim.x >> 5;
    const double rank = (double)(blockIdx.x / sms) * warps + (threadIdx.x >> 5);   // the warp's rank on its SM
    retrace_idle = rank >= (need < 1.0 ? 1.0 : need);
  }
  if (D.stage_table) {
    for (int64_t i = threadIdx.x; i < D.m.a_table_n; i += blockDim.x) stage_tab_s[i] = __ldg(D.m.a_table + i);
    __syncthreads();
  }
  if (retrace_idle) return;   // warp-uniform, and no block barrier follows
  Tracer<MK, FT> T(D, A);
  Photon P;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t static_next = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const long long t0 = clock64();
  int64_t p = next_work(D, A, static_next, stride);
  bool active = p < A.n_photons;
  if (active) photon_begin<MK, FT, REC>(T, A, P, p);
  while (active) {
    bool done = photon_iterate<MK, FT, STEPPER, REC>(T, A, P);
    if (!done && (P.it & 63) == 0) {
      if (A.abort_flag && *(volatile const int32_t*)A.abort_flag) { P.status = EXC_PH_ABORTED; done = true; }
      else if (A.deadline_cycles > 0 && clock64() - t0 > A.deadline_cycles) { P.status = EXC_PH_TIMED_OUT; done = true; }
    }
    if (done) {
      photon_finish<MK, FT, REC>(T, A, P);
      const bool stop_all = (P.status == EXC_PH_ABORTED || P.status == EXC_PH_TIMED_OUT);
      if (stop_all) break;
      p = next_work(D, A, static_next, stride);
      active = p < A.n_photons;
      if (active) photon_begin<MK, FT, REC>(T, A, P, p);
    }
  }
}

// ------------------------------------------------------------ launchers
struct LaunchCfg {
  int block;          // threads per block
  int blocks_per_sm;  // 0 = as many as fit (occupancy query)
  int sm_count;
};

template <int MK, class FT, int STEPPER, bool REC>
cudaError_t launch_trace_t(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s) {
  auto kern = trace_kernel<MK, FT, STEPPER, REC>;
  const size_t smem = D.stage_table ? (size_t)D.m.a_table_n * sizeof(double) : 0;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int block = lc.block, per_sm = lc.blocks_per_sm;
  if (block <= 0) {
    // The library's default for a batch: 32-thread blocks, and as many of them an SM as make the
    // last wave of similar trajectories full -- the batch over the waves it needs at the occupancy
    // limit, rounded up to whole warps an SM (65,536 rays: 7 warps an SM, 1.92 rays a lane,
    // where 128-thread blocks at the limit put 1.68 and ran the second wave two thirds full).
    block = 32;
    if (per_sm <= 0) {
      int occ = 0;
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, block, smem);
      if (e != cudaSuccess) return e;
      per_sm = exc::balanced_warps_per_sm(A.n_photons, lc.sm_count, occ);
    }
  }
  if (per_sm <= 0) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
  }
  int64_t grid = (int64_t)lc.sm_count * per_sm;
  const int64_t need = (A.n_photons + block - 1) / block;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  kern<<<(int)grid, block, smem, s>>>(D, A);
  return cudaGetLastError();
}

template <int MK, class FT, int STEPPER>
cudaError_t launch_trace_r(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s) {
  if (A.records) return launch_trace_t<MK, FT, STEPPER, true>(D, A, lc, s);
  return launch_trace_t<MK, FT, STEPPER, false>(D, A, lc, s);
}

// Slow-Interpolator launches (defined in the *_slow translation units, which
// compile in parallel with the base-node ones).
cudaError_t trace_rk4_slow(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s);
cudaError_t trace_rk45_slow(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s);
cudaError_t trace_lf4_slow(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s);

template <int STEPPER>
cudaError_t launch_trace_slow(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s) {
  if (D.m.fields[0].dtype == EXC_DTYPE_F32) return launch_trace_r<kFlrwSlowInterp, float, STEPPER>(D, A, lc, s);
  if (D.m.fields[0].dtype == EXC_DTYPE_F64) return launch_trace_r<kFlrwSlowInterp, double, STEPPER>(D, A, lc, s);
  if (D.m.fields[0].dtype == EXC_DTYPE_F32X2) {
    // split grids reach the FP64 tracer only as the mixed tracer's re-trace pass (fast build)
    if constexpr ((STEPPER == EXC_STEPPER_RK4 || STEPPER == EXC_STEPPER_RK45) && EXC_FAST) {
      if (!A.records) return launch_trace_t<kFlrwSlowInterp, float2, STEPPER, false>(D, A, lc, s);
    }
  }
  return cudaErrorInvalidValue;
}

// The dtype of field 0 selects the instantiation (all fields of a launch share it);
// a slow-Interpolator field anywhere in the launch selects the kernels that read it.
template <int STEPPER>
cudaError_t launch_trace_stepper(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s) {
  if (D.m.kind == EXC_METRIC_SCHWARZSCHILD)
    return launch_trace_r<EXC_METRIC_SCHWARZSCHILD, double, STEPPER>(D, A, lc, s);
  bool slow = false;
  for (int i = 0; i < D.m.n_fields; ++i) slow = slow || D.m.fields[i].grad_mode == EXC_GRAD_TRILINEAR;
  if (slow) {
    if constexpr (STEPPER == EXC_STEPPER_RK4) return trace_rk4_slow(D, A, lc, s);
    else if constexpr (STEPPER == EXC_STEPPER_RK45) return trace_rk45_slow(D, A, lc, s);
    else return trace_lf4_slow(D, A, lc, s);
  }
  if (D.m.fields[0].dtype == EXC_DTYPE_F32) return launch_trace_r<EXC_METRIC_FLRW, float, STEPPER>(D, A, lc, s);
  if (D.m.fields[0].dtype == EXC_DTYPE_F32X2) {
    // split grids reach the FP64 tracer only as the mixed tracer's re-trace pass (fast build)
    if constexpr ((STEPPER == EXC_STEPPER_RK4 || STEPPER == EXC_STEPPER_RK45) && EXC_FAST) {
      if (!A.records) return launch_trace_t<EXC_METRIC_FLRW, float2, STEPPER, false>(D, A, lc, s);
    }
    return cudaErrorInvalidValue;
  }
  return launch_trace_r<EXC_METRIC_FLRW, double, STEPPER>(D, A, lc, s);
}

// Defined in the per-stepper translation units (each compiles one stepper's kernels).
cudaError_t trace_rk4(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s);
cudaError_t trace_rk45(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s);
cudaError_t trace_lf4(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s);

inline cudaError_t launch_trace(const DevMetric& D, const ExcTraceArgs& A, LaunchCfg lc, cudaStream_t s) {
  switch (A.stepper) {
    case EXC_STEPPER_RK4: return trace_rk4(D, A, lc, s);
    case EXC_STEPPER_RK45: return trace_rk45(D, A, lc, s);
    default: return trace_lf4(D, A, lc, s);
  }
}

}  // namespace EXC_NS
