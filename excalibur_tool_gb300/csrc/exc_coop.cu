// exc_coop.cu -- the FP64 re-trace pass of the mixed tracer, eight lanes per ray.
//
// The rays the mixed tracer hands back (status EXC_PH_RETRACE, state untouched) are traced
// again in FP64 from their initial state. There are few of them (1-2 % of a patch), so the
// pass lasts as long as one FP64 trajectory: on GB300 the FP64 pipe of an SM sub-partition
// spends many cycles on every warp instruction whatever the number of active lanes, and a
// one-thread ray is a chain of ~1,000 such instructions per RK4 step. Here a ray is a group of
// eight lanes of a warp (four rays per warp, in lock step): lane l holds state component l, and
// the right-hand side is split across the group -- three lanes take the three cell coordinates
// and gradient differences, each lane loads one corner of the interpolation cell and forms its
// weighted value (an eight-lane sum gives Phi), and each lane evaluates the right-hand side of
// its own component (dx^mu = u^mu; du^mu with one formula for the three spatial components).
// Fewer instructions per step, each serving four rays, shorten the pass.
//
// Same physics and stops as the fast FP64 tracer (exc_kernels.cuh: the reference's formulas
// with FMA contraction and reciprocals of launch constants); the results differ from that
// tracer's by the order of a few sums. Launches it does not cover (RK45, Leapfrog, the slow
// Interpolator, 4-D fields, renormalisation, records, ISW) keep the one-thread re-trace.
//
// Every lane of a warp executes every shuffle: the groups run one instruction stream, a group
// without a ray traces a copy of photon 0 whose results are dropped, and failures are taken
// after all of a step's shuffles.
#define EXC_FAST 1
#define EXC_NS exc_coop_f64
#include "exc_device.cuh"

#include "exc_coop.h"

namespace exc_coop {

using exc::DevMetric;
using namespace exc_coop_f64;

constexpr unsigned kFull = 0xffffffffu;
constexpr int kG = 8;   // lanes per ray

__device__ __forceinline__ double gshfl(double v, int src) { return __shfl_sync(kFull, v, src, kG); }
__device__ __forceinline__ int gshfl_i(int v, int src) { return __shfl_sync(kFull, v, src, kG); }
__device__ __forceinline__ long long gshfl_ll(long long v, int src) { return __shfl_sync(kFull, v, src, kG); }
__device__ __forceinline__ double gsum(double v) {
  v += __shfl_xor_sync(kFull, v, 4, kG);
  v += __shfl_xor_sync(kFull, v, 2, kG);
  v += __shfl_xor_sync(kFull, v, 1, kG);
  return v;
}
// true in every lane of the group when the flag is set in any lane of it
__device__ __forceinline__ bool gany(bool f, int gbase) {
  return ((__ballot_sync(kFull, f) >> gbase) & 0xffu) != 0u;
}
__device__ __forceinline__ void bcast8(double v, double y[8]) {
#pragma unroll
  for (int q = 0; q < 8; ++q) y[q] = gshfl(v, q);
}

struct Ray {
  double s;                  // this lane's state component
  double dt;
  int64_t idx;
  int steps, it, status;     // status < 0: running
  // observables (the same value in every lane of the group)
  double a_obs, phi_obs, eta_obs, path, excess, min_r;
  double p0[3], pprev[3], e0[3], v0[3];
};

// Phi, its base-node gradient and the scale factor at the broadcast state y
// (PerturbedFLRWMetricFast.geodesic_equations' inputs, perturbed_flrw_metric_fast.py:227-251;
// fused_interpolation_gradient_3d_{periodic,clamp,error}, grid/interpolator_4d_fast.py:50-255).
// Returns 0 or an EXC_PH_* code, the same in every lane of the group.
template <class FT>
__device__ __forceinline__ int fields_at(const DevMetric& D, int fi, const double y[8], int l, double& a,
                                         double& adot, double& inv_a, double& phi, double g[3]) {
  int st = scale_factor(D, y[0], a, adot, inv_a);   // the same in every lane
  const ExcField& f = D.m.fields[fi];
  const FT* d = (const FT*)f.data;
  const double* fiv = D.finv[fi];
  // lanes 0-2: the cell of axis l (the others repeat axis 0)
  const int ax = l < 3 ? l : 0;
  const int64_t n = f.n[ax];
  const double o = f.origin[ax], sp = f.spacing[ax];
  double x = ax == 0 ? y[1] : (ax == 1 ? y[2] : y[3]);
  if (has_shift(f)) x += f.shift[ax];
  double frac = 0.0;
  long long i0 = 0, i1 = 1, im = 0;
  int ast = 0;
  bool lowedge = false;
  if (f.boundary == EXC_BOUNDARY_PERIODIC) {
    x = o + py_fmod(x - o, (double)n * sp);
    const double r = div_rn(x - o, sp, fiv[ax]);
    if (!isfinite(r)) ast = EXC_PH_NONFINITE;
    const long long k = ast ? 0 : (long long)floor(r);
    frac = r - (double)k;
    i0 = py_imod(k, n);
    i1 = py_imod(i0 + 1, n);
    im = py_imod(i0 - 1, n);
  } else if (f.boundary == EXC_BOUNDARY_CLAMP) {
    const double hx = o + (double)(n - 1) * sp - 1e-12 * sp;
    if (x < o) x = o; else if (x > hx) x = hx;
    const double r = div_rn(x - o, sp, fiv[ax]);
    if (!isfinite(r)) ast = EXC_PH_NONFINITE;
    long long k = ast ? 0 : (long long)floor(r);
    if (k < 0) k = 0;
    if (k > n - 2) k = n - 2;
    frac = r - (double)k;
    i0 = k;
    i1 = k + 1;
    lowedge = k <= 0;
    im = lowedge ? k : k - 1;
  } else {
    // strict interior rel in [1, n-2); outside it the indices stay at a valid cell
    const double r = div_rn(x - o, sp, fiv[ax]);
    if (r < 1.0 || r >= (double)n - 2.0) ast = EXC_PH_OUTSIDE_GRID;
    else if (!isfinite(r)) ast = EXC_PH_NONFINITE;   // NaN (an infinity is outside first)
    const long long k = ast ? 1 : (long long)floor(r);
    frac = r - (double)k;
    i0 = k;
    i1 = k + 1;
    im = k - 1;
  }
  if (l >= 3) ast = 0;
  // the first failure among the scale factor and the three axes, in every lane
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int sq = gshfl_i(ast, q);
    st = st ? st : sq;
  }
  double fr[3];
  long long a0[3], a1[3], am[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    fr[q] = gshfl(frac, q);
    a0[q] = gshfl_ll(i0, q);
    a1[q] = gshfl_ll(i1, q);
    am[q] = gshfl_ll(im, q);
  }
  const int64_t ny = f.n[1], nz = f.n[2];
  // corner l of the cell: bit 0 = +x, bit 1 = +y, bit 2 = +z (node 0 of the grid after a failure)
  const int bx = l & 1, by = (l >> 1) & 1, bz = (l >> 2) & 1;
  const int64_t ci = bx ? a1[0] : a0[0], cj = by ? a1[1] : a0[1], ck = bz ? a1[2] : a0[2];
  const double v = ldf(d, st ? 0 : (ci * ny + cj) * nz + ck);
  const double w = (bx ? fr[0] : 1.0 - fr[0]) * (by ? fr[1] : 1.0 - fr[1]) * (bz ? fr[2] : 1.0 - fr[2]);
  phi = gsum(w * v);
  // gradient: lane q < 3 differences the +q corner (lanes 1, 2, 4) and the -q node
  const double cplus = gshfl(v, l == 0 ? 1 : (l == 1 ? 2 : 4));
  const double c000 = gshfl(v, 0);
  double gq = 0.0;
  if (l < 3) {
    // lanes 0-2: ax == l, so sp and fiv[ax] are this axis' spacing and reciprocal
    if (f.boundary == EXC_BOUNDARY_CLAMP && lowedge) {
      gq = div_c(cplus - c000, sp, fiv[ax]);
    } else {
      const int64_t mi = l == 0 ? am[0] : a0[0], mj = l == 1 ? am[1] : a0[1], mk = l == 2 ? am[2] : a0[2];
      const double cm = ldf(d, st ? 0 : (mi * ny + mj) * nz + mk);
      gq = div_c(cplus - cm, 2.0 * sp, fiv[4 + ax]);
    }
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) g[q] = gshfl(gq, q);
  if (!st && isnan(phi)) st = EXC_PH_OUTSIDE_GRID;
  return st;
}

// The right-hand side of this lane's component: dx^l = u^l (l < 4), du^(l-4) (l >= 4), from
// compute_tensorial_acceleration / compute_analytical_acceleration
// (perturbed_flrw_metric_fast.py:7-99), the spatial components in one shared formula.
template <class FT>
__device__ __forceinline__ int rhs(const DevMetric& D, int fi, double yl, int l, double& out) {
  double y[8];
  bcast8(yl, y);
  double a, adot, inv_a, phi_si, g[3];
  const int st = fields_at<FT>(D, fi, y, l, a, adot, inv_a, phi_si, g);
  const double ic2 = D.ic2, ic4 = D.ic4;
  const double phi = phi_si * ic2;
  const double u0 = y[4];
  const double usq = y[5] * y[5] + y[6] * y[6] + y[7] * y[7];
  // the spatial component of lanes 5-7 (selected, not indexed: the arrays stay in registers)
  const double ui = l == 6 ? y[6] : (l == 7 ? y[7] : y[5]);
  const double gi = l == 6 ? g[1] : (l == 7 ? g[2] : g[0]);
  double du0, dui;
  if (!D.m.analytical) {
    const double gdotc = (g[0] * y[5] + g[1] * y[6] + g[2] * y[7]) * ic2;
    const double adot_a = adot * inv_a;
    du0 = -((a * adot * ic2 + 2.0 * a * adot * ic4 * (phi + phi)) * usq + 2.0 * u0 * gdotc);
    const double gic = gi * ic2;
    const double Gii = gic * (usq - 2.0 * ui * ui) - ui * (gdotc - gic * ui);
    dui = -(gi * (inv_a * inv_a) * u0 * u0 + 2.0 * adot_a * u0 * ui + Gii);
  } else {
    const double tc2 = D.m.two_over_c2;
    const double dphidl = g[0] * y[5] + g[1] * y[6] + g[2] * y[7];
    const double aa = adot * inv_a;
    du0 = -aa * (u0 * u0) - tc2 * u0 * dphidl - (aa * ic2 - 2.0 * aa * ic4 * (phi + phi)) * usq;
    dui = -gi * (u0 * u0) - 2.0 * aa * u0 * ui + tc2 * ui * (dphidl - gi * ui) + gi * ic2 * (2.0 * (ui * ui) - usq);
  }
  const double ul = l == 0 ? y[4] : (l == 1 ? y[5] : (l == 2 ? y[6] : y[7]));
  out = l < 4 ? ul : (l == 4 ? du0 : dui);
  return st;
}

// a(eta) and Phi at the state (Metric.metric_physical_quantities' first two columns).
template <class FT>
__device__ __forceinline__ int quantities(const DevMetric& D, int fi, double yl, int l, double& a, double& phi) {
  double y[8];
  bcast8(yl, y);
  double adot, inv_a, g[3];
  return fields_at<FT>(D, fi, y, l, a, adot, inv_a, phi, g);
}

__device__ __forceinline__ double norm3(const double v[3]) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

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

// Load photon p into the group and take the observer-end quantities.
template <class FT>
__device__ __forceinline__ void ray_begin(const DevMetric& D, const ExcTraceArgs& A, Ray& R, int64_t p, int fi,
                                          int l) {
  R.idx = p;
  R.s = A.state[p * 8 + l];
  R.dt = A.dt_state ? A.dt_state[p] : A.dt;
  R.steps = 0;
  R.it = 0;
  R.status = -1;
  double y[8];
  bcast8(R.s, y);
  double rel[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    R.p0[q] = y[1 + q];
    R.pprev[q] = y[1 + q];
    R.v0[q] = y[5 + q];
  }
  const double nv = norm3(R.v0);
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    R.e0[q] = nv > 0.0 ? R.v0[q] / nv : 0.0;
    rel[q] = R.p0[q] - A.lens_center[q];
  }
  R.path = 0.0;
  R.excess = 0.0;
  R.eta_obs = y[0];
  R.min_r = norm3(rel);
  double a, phi;
  const int st = quantities<FT>(D, fi, R.s, l, a, phi);
  R.a_obs = st ? NAN : a;
  R.phi_obs = st ? NAN : phi;
}

// One RK4 step (integrator.py:10-22) and the loop's bookkeeping and stops
// (integrator.py:347-400 plus the box / a stops). Returns true when the ray ends.
template <class FT>
__device__ __forceinline__ bool ray_iterate(const DevMetric& D, const ExcTraceArgs& A, Ray& R, int fi, int l,
                                            int gbase) {
  const bool cap = R.it >= A.max_iter || R.steps >= A.max_steps;
  double dt = R.dt;
  {
    // integrator.py:358-364
    const double adt = fmin(fmax(fabs(dt), A.dt_min), A.dt_max);
    dt = dt < 0.0 ? -adt : adt;
  }
  double y[8];
  bcast8(R.s, y);
  bool face = false;
  if (A.stop_flags & EXC_STOP_FACE) {
    // the step that would come within EXC_FACE_MARGIN of a face of the stop box ends on it
    const double sg = dt < 0.0 ? -1.0 : 1.0;
    double tmin = INFINITY;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double v = sg * y[5 + q];
      if (v > 0.0) tmin = fmin(tmin, (A.box_hi[q] - y[1 + q]) / v);
      else if (v < 0.0) tmin = fmin(tmin, (A.box_lo[q] - y[1 + q]) / v);
    }
    face = tmin < EXC_FACE_MARGIN * fabs(dt);
    if (face) dt = sg * fmax(tmin, 0.0);
  }
  const double h = 0.5 * dt;
  double k1, k2, k3, k4;
  const int s1 = rhs<FT>(D, fi, R.s, l, k1);
  const int s2 = rhs<FT>(D, fi, R.s + h * k1, l, k2);
  const int s3 = rhs<FT>(D, fi, R.s + h * k2, l, k3);
  const int s4 = rhs<FT>(D, fi, R.s + dt * k3, l, k4);
  const double ns = R.s + (dt / 6.0) * (k1 + 2.0 * k2 + 2.0 * k3 + k4);
  const bool nonfinite = gany(!isfinite(ns), gbase);
  double z[8];
  bcast8(ns, z);
  // decisions (no shuffle below)
  if (cap) {
    R.status = R.it >= A.max_iter ? EXC_PH_MAX_ITER : EXC_PH_STEPS;
    return true;
  }
  const int st = s1 ? s1 : (s2 ? s2 : (s3 ? s3 : s4));
  if (st) { R.status = st; R.dt = dt; return true; }
  if (nonfinite) { R.status = EXC_PH_NONFINITE; R.dt = dt; return true; }
  R.s = ns;
  if (A.obs_flags) {
    double d[3], rel[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      d[q] = z[1 + q] - R.pprev[q];
      rel[q] = z[1 + q] - A.lens_center[q];
      R.pprev[q] = z[1 + q];
    }
    if (A.obs_flags & EXC_OBS_PATH) {
      R.path += norm3(d);
      R.excess += excess_term(d, R.e0);
    }
    if (A.obs_flags & EXC_OBS_ENDPOINTS) R.min_r = fmin(R.min_r, norm3(rel));
  }
  R.steps++;
  R.dt = dt;
  R.it++;
  if (A.stop_flags & EXC_STOP_FACE) {
    if (face) { R.status = EXC_PH_LEFT_BOX; return true; }
  } else if (A.stop_flags & EXC_STOP_BOX) {
    if (!(z[1] >= A.box_lo[0] && z[1] < A.box_hi[0] && z[2] >= A.box_lo[1] && z[2] < A.box_hi[1] &&
          z[3] >= A.box_lo[2] && z[3] < A.box_hi[2])) {
      R.status = EXC_PH_LEFT_BOX;
      return true;
    }
  }
  if (A.stop_flags & EXC_STOP_A) {
    double a, adot, inv_a;
    if (scale_factor(D, z[0], a, adot, inv_a) == 0 && a <= A.a_stop) { R.status = EXC_PH_A_STOP; return true; }
  }
  return false;
}

// The end of a ray: the emitter-end quantities, then (write) the state, status and observables.
template <class FT>
__device__ __forceinline__ void ray_finish(const DevMetric& D, const ExcTraceArgs& A, Ray& R, int fi, int l,
                                           bool write) {
  double a_em, phi_em;
  const int qst = quantities<FT>(D, fi, R.s, l, a_em, phi_em);   // integrator.py:403
  double y[8];
  bcast8(R.s, y);
  if (!write) return;
  const int64_t p = R.idx;
  const bool failed = R.status >= EXC_PH_OUTSIDE_GRID;
  if (!failed && qst) R.status = qst;
  A.state[p * 8 + l] = R.s;
  if (l != 0) return;
  A.status[p] = R.status;
  if (A.n_steps) A.n_steps[p] = R.steps;
  if (A.n_iter) A.n_iter[p] = R.it;
  if (A.dt_state) A.dt_state[p] = R.dt;
  if (A.obs && A.obs_flags) {
    double* o = A.obs + p * EXC_OBSCOL_N;
    for (int i = 0; i < EXC_OBSCOL_N; ++i) o[i] = NAN;
    o[EXC_OBSCOL_ETA_OBS] = R.eta_obs;
    o[EXC_OBSCOL_ETA_EM] = y[0];
    o[EXC_OBSCOL_A_OBS] = R.a_obs;
    o[EXC_OBSCOL_PHI_OBS] = R.phi_obs;
    if (!failed && qst == 0) {
      o[EXC_OBSCOL_A_EM] = a_em;
      o[EXC_OBSCOL_PHI_EM] = phi_em;
    }
    o[EXC_OBSCOL_ISW_INT] = 0.0;
    if (A.obs_flags & EXC_OBS_PATH) {
      double X[3] = {y[1] - R.p0[0], y[2] - R.p0[1], y[3] - R.p0[2]};
      o[EXC_OBSCOL_PATH] = R.path;
      o[EXC_OBSCOL_CHORD] = norm3(X);
      o[EXC_OBSCOL_EXCESS] = R.excess - excess_term(X, R.e0);
    }
    o[EXC_OBSCOL_V0X] = R.v0[0];
    o[EXC_OBSCOL_V0Y] = R.v0[1];
    o[EXC_OBSCOL_V0Z] = R.v0[2];
    o[EXC_OBSCOL_V1X] = y[5];
    o[EXC_OBSCOL_V1Y] = y[6];
    o[EXC_OBSCOL_V1Z] = y[7];
    o[EXC_OBSCOL_MIN_R] = R.min_r;
  }
}

// Persistent: each group takes the next photon still marked EXC_PH_RETRACE (its leader fetches
// eight indices at a time, the group tests them together), traces it, and fetches again; the
// warp runs until its four groups are out of work. Stage evaluations of a group without a ray
// run on photon 0's state and are dropped.
template <class FT>
__global__ void __launch_bounds__(128) coop_retrace_kernel(const DevMetric D, const ExcTraceArgs A) {
  const int lane = threadIdx.x & 31;
  const int l = lane & (kG - 1), gbase = lane & ~(kG - 1);
  const unsigned gmask = 0xffu << gbase;
  const int64_t groups = (int64_t)gridDim.x * (blockDim.x / kG);
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kG;
  int64_t static_next = gid * kG;
  const long long t0 = clock64();
  const double dummy = A.state[l];
  Ray R;
  R.s = dummy;
  R.dt = A.dt;
  R.idx = 0;
  R.steps = R.it = 0;
  R.status = -1;
  int fi = 0;
  unsigned pending = 0u;
  long long cand0 = 0;
  bool active = false, exhausted = false;
  for (;;) {
    bool fresh = false;
    if (!active && !exhausted) {
      // group-uniform control flow: the eight lanes of a group stay together here
      for (;;) {
        if (pending == 0u) {
          long long base = 0;
          if (A.queue) {
            if (l == 0) base = (long long)atomicAdd(reinterpret_cast<unsigned long long*>(A.queue), (unsigned long long)kG);
            base = __shfl_sync(gmask, base, gbase);
          } else {
            base = static_next;
            static_next += groups * kG;
          }
          if (base >= A.n_photons) { exhausted = true; break; }
          cand0 = base;
          const int64_t q = base + l;
          const bool hit = q < A.n_photons && A.status[q] == EXC_PH_RETRACE;
          pending = (__ballot_sync(gmask, hit) >> gbase) & 0xffu;
          continue;
        }
        const int k = __ffs(pending) - 1;
        pending &= pending - 1u;
        const int64_t p = cand0 + k;
        const int f = A.field_index ? A.field_index[p] : 0;
        if ((unsigned)f >= (unsigned)D.m.n_fields) {   // the mixed pass never hands such a photon back
          if (l == 0) A.status[p] = EXC_PH_BAD_FIELD;
          continue;
        }
        fi = f;
        R.idx = p;
        active = true;
        fresh = true;
        break;
      }
    }
    __syncwarp();
    if (__all_sync(kFull, !active)) break;
    if (__any_sync(kFull, fresh)) {
      Ray tmp;
      ray_begin<FT>(D, A, tmp, fresh ? R.idx : 0, fresh ? fi : 0, l);
      if (fresh) R = tmp;
    }
    if (!active) {
      R.s = dummy;
      R.dt = A.dt;
      R.steps = R.it = 0;
      R.status = -1;
    }
    bool ended = ray_iterate<FT>(D, A, R, active ? fi : 0, l, gbase);
    if (active && !ended && (R.it & 63) == 0) {
      if (A.abort_flag && *(volatile const int32_t*)A.abort_flag) { R.status = EXC_PH_ABORTED; ended = true; }
      else if (A.deadline_cycles > 0 && clock64() - t0 > A.deadline_cycles) { R.status = EXC_PH_TIMED_OUT; ended = true; }
    }
    const bool fin = active && ended;
    if (__any_sync(kFull, fin)) ray_finish<FT>(D, A, R, active ? fi : 0, l, fin);
    if (fin) {
      active = false;
      if (R.status == EXC_PH_ABORTED || R.status == EXC_PH_TIMED_OUT) exhausted = true;
    }
  }
}

bool supports(const DevMetric& D, const ExcTraceArgs& A) {
  if (D.m.kind != EXC_METRIC_FLRW || A.stepper != EXC_STEPPER_RK4) return false;
  if (A.records || A.renormalize_every || (A.obs_flags & EXC_OBS_ISW)) return false;
  if (A.n_photons < 1) return false;
  for (int i = 0; i < D.m.n_fields; ++i) {
    const ExcField& f = D.m.fields[i];
    if (f.ndim != 3 || f.grad_mode != EXC_GRAD_BASE_NODE) return false;
    if (f.dtype != D.m.fields[0].dtype) return false;
  }
  return true;
}

cudaError_t retrace(const DevMetric& D, const ExcTraceArgs& A, int sm_count, cudaStream_t s) {
  // four warps per SM (one per sub-partition), four rays per warp
  const int block = 128;
  const int grid = sm_count > 0 ? sm_count : 1;
  const int dtype = D.m.fields[0].dtype;
  if (dtype == EXC_DTYPE_F32X2) coop_retrace_kernel<float2><<<grid, block, 0, s>>>(D, A);
  else if (dtype == EXC_DTYPE_F32) coop_retrace_kernel<float><<<grid, block, 0, s>>>(D, A);
  else coop_retrace_kernel<double><<<grid, block, 0, s>>>(D, A);
  return cudaGetLastError();
}

}  // namespace exc_coop
