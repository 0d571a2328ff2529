// exc_maps.cu -- redshift maps from recorded trajectories (include/excalibur_gb300.h,
// exc_record_redshift / exc_sky_directions / exc_sky_project / exc_sky_bin).
//
// The reference turns a file of recorded photon histories into sky maps on the host, one
// photon at a time (_postprocessing/compute_redshift_map.py:30-171: rows holding a NaN are
// dropped, then RedshiftCalculator(...).compute_all_components() per photon, with
// scipy.integrate.simpson for the ISW integral; :54-95 for the sky positions) and grids them
// with scipy's griddata. Here the NaN-padded record stack the tracer leaves in HBM
// ([n_photons][n_rows][n_cols] float64, the runners' trajectory-file layout) is read in place:
// one thread per photon scans its rows once and evaluates every component in the reference's
// operation order (compiled with --fmad=false, so no product is contracted): the ISW Simpson sum
// follows scipy's irregular-spacing rule and numpy's pairwise summation term for term, and the
// time delay of _postprocessing/compute_time_delay_map.py:97-126,244-310 (path over the recorded
// rows minus the chord) is summed in the same scan. numpy sums up to 128 terms as one block,
// which a single scan can follow; longer histories (more than 257 rows, where the block split
// depends on the clean-row count) compact their clean rows into a scratch index list first and
// sum from it in a second pass. Sky positions are a per-photon projection; maps are pixel means by
// atomics (binning in place of griddata's interpolation).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/excalibur_gb300.h"
#include "exc_divrn.cuh"

namespace exc {
void set_last_error(const char* msg);
}

namespace {

constexpr int kThreads = 128;
// the most rows a history can have for its pair terms (at most (n - 1) / 2) to fit one numpy block
constexpr int kOnePassRows = 257;

// |v| as an integer: for non-NaN doubles its order is that of the magnitudes. The tests below
// run on the integer pipe; this kernel is bound by the FP64 pipe (its divisions and square
// roots), and a floating-point NaN test or maximum per value would take a quarter of it.
__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

__device__ __forceinline__ bool row_clean(const double* row, int n_cols) {
  for (int c = 0; c < n_cols; ++c)
    if (abs_bits(row[c]) > 0x7ff0000000000000ull) return false;   // NaN
  return true;
}

// x**3: the exact square (Dekker's split by an FMA) times x in double-double, rounded once at
// the end -- the correctly rounded cube but for rare near-halfway cases, which is what libm's
// pow gives for numpy's float64 power.
__device__ __forceinline__ double cube_dd(double x) {
  const double p = x * x;
  const double e = fma(x, x, -p);
  const double hi = p * x;
  const double lo = fma(p, x, -hi) + e * x;
  return hi + lo;
}

__device__ __forceinline__ double div0(double num, double den) { return den != 0.0 ? num / den : 0.0; }

// One photon's clean rows: rows[idx[k] * n_cols + col].
struct Clean {
  const double* rows;
  const int32_t* idx;
  int n_cols;
  double c2;
  __device__ __forceinline__ double eta(int k) const { return rows[(int64_t)idx[k] * n_cols]; }
  __device__ __forceinline__ double dphi(int k) const { return rows[(int64_t)idx[k] * n_cols + 13] * c2; }
  __device__ double term(int j) const;
};

// scipy's _basic_simpson term of the samples (x0, y0), (x1, y1), (x2, y2) (irregular spacing)
__device__ __forceinline__ double simpson_term(double x0, double x1, double x2, double y0, double y1, double y2) {
  const double h0 = x1 - x0, h1 = x2 - x1;
  const double hsum = h0 + h1, hprod = h0 * h1;
  const double h0divh1 = div0(h0, h1);
  const double t0 = y0 * (2.0 - div0(1.0, h0divh1));
  const double t1 = y1 * (hsum * div0(hsum, hprod));
  const double t2 = y2 * (2.0 - h0divh1);
  // hsum / 6 as the correctly rounded quotient from RN(1/6) (div_rn: the IEEE quotient in three
  // FP64 slots instead of about eight); operands below 2^-960, where the remainder could leave
  // the normal range, take the division (the test is on the bits, on the integer pipe)
  const bool big = ((unsigned long long)__double_as_longlong(hsum) & 0x7fffffffffffffffull) >= 0x03f0000000000000ull;
  const double q6 = big ? div_rn(hsum, 6.0, 1.0 / 6.0) : hsum / 6.0;
  return q6 * ((t0 + t1) + t2);
}

// the term of the pair starting at clean sample 2j
__device__ double Clean::term(int j) const {
  const int k = 2 * j;
  return simpson_term(eta(k), eta(k + 1), eta(k + 2), dphi(k), dphi(k + 1), dphi(k + 2));
}

// numpy's pairwise sum of the terms [lo, lo + n) of a block of at most 128: fewer than 8 in
// order, else eight partial sums combined as a balanced tree, then the remainder in order.
__device__ double pairwise_leaf(const Clean& cl, int lo, int n) {
  if (n < 8) {
    double res = -0.0;
    for (int i = 0; i < n; ++i) res += cl.term(lo + i);
    return res;
  }
  double r[8];
  for (int j = 0; j < 8; ++j) r[j] = cl.term(lo + j);
  int i = 8;
  for (; i < n - (n % 8); i += 8)
    for (int j = 0; j < 8; ++j) r[j] += cl.term(lo + i + j);
  double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
  for (; i < n; ++i) res += cl.term(lo + i);
  return res;
}

// numpy's pairwise sum of terms [0, n): a block longer than 128 is split at n/2 rounded down
// to a multiple of 8 and the halves' sums added. Evaluated without recursion (a device stack
// of unknown depth could outgrow the per-thread stack limit): an explicit stack of pending
// splits, at most 26 deep for n < 2^31.
__device__ double pairwise(const Clean& cl, int n) {
  constexpr int kDepth = 32;
  int s_lo[kDepth], s_n[kDepth];
  double s_left[kDepth];
  unsigned char s_phase[kDepth];  // 0: not split yet, 1: left half pending, 2: right half pending
  int sp = 1;
  s_lo[0] = 0;
  s_n[0] = n;
  s_phase[0] = 0;
  while (true) {
    const int t = sp - 1;
    if (s_n[t] > 128 && s_phase[t] == 0 && sp < kDepth) {
      const int n2 = s_n[t] / 2 - (s_n[t] / 2) % 8;
      s_phase[t] = 1;
      s_lo[sp] = s_lo[t];
      s_n[sp] = n2;
      s_phase[sp] = 0;
      ++sp;
      continue;
    }
    double ret = pairwise_leaf(cl, s_lo[t], s_n[t] <= 128 ? s_n[t] : 128);  // (the cap is never hit)
    --sp;
    while (sp > 0) {
      const int p = sp - 1;
      const int n2 = s_n[p] / 2 - (s_n[p] / 2) % 8;
      if (s_phase[p] == 1) {
        s_left[p] = ret;
        s_phase[p] = 2;
        s_lo[sp] = s_lo[p] + n2;
        s_n[sp] = s_n[p] - n2;
        s_phase[sp] = 0;
        ++sp;
        break;
      }
      ret = s_left[p] + ret;
      --sp;
    }
    if (sp == 0) return ret;
  }
}

// scipy.integrate.simpson(dphi, x=eta) over m >= 2 clean samples, given the pairwise sum of the
// pair terms (`pairs`) and the last three samples (x[2] the last; for m == 2, x[1] and x[2]).
__device__ double simpson_finish(int m, double pairs, const double x[3], const double y[3]) {
  if (m % 2 == 1) return 0.0 + pairs;
  if (m == 2) {
    const double last_dx = x[2] - x[1];
    return 0.0 + (0.0 + 0.5 * last_dx * (y[2] + y[1]));
  }
  double result = 0.0 + pairs;
  const double h0 = x[1] - x[0];
  const double h1 = x[2] - x[1];
  // Cartwright's correction of the last interval, with scipy's zero-denominator guards
  const double alpha = div0(2.0 * (h1 * h1) + (3.0 * h0) * h1, 6.0 * (h1 + h0));
  const double beta = div0(h1 * h1 + (3.0 * h0) * h1, 6.0 * h0);
  const double eta = div0(cube_dd(h1), (6.0 * h0) * (h0 + h1));
  result += (alpha * y[2] + beta * y[1]) - eta * y[0];
  return result + 0.0;
}

__device__ double simpson(const Clean& cl, int m) {
  const int n_pairs = (m % 2 == 1) ? (m - 1) / 2 : (m - 2) / 2;
  const double pairs = (m == 2) ? 0.0 : pairwise(cl, n_pairs);
  double x[3], y[3];
  for (int k = 0; k < 3; ++k) {
    const int q = m - 3 + k;
    x[k] = q >= 0 ? cl.eta(q) : 0.0;
    y[k] = q >= 0 ? cl.dphi(q) : 0.0;
  }
  return simpson_finish(m, pairs, x, y);
}

// numpy's pairwise sum of a stream of at most 128 terms, fed in order: the first eight seed the
// eight partial sums, each later complete group of eight adds into them, and the last incomplete
// group is added in order after the partial sums are combined (fewer than eight terms in all:
// added in order to -0.0). The pending group shifts through eight registers, so that every
// index is static (no local-memory array).
struct PairwiseStream {
  double r[8], g[8];
  int ng, groups;
  __device__ __forceinline__ void init() { ng = 0; groups = 0; }
  __device__ __forceinline__ void push(double t) {
#pragma unroll
    for (int j = 0; j < 7; ++j) g[j] = g[j + 1];
    g[7] = t;
    if (++ng == 8) {
#pragma unroll
      for (int j = 0; j < 8; ++j) r[j] = groups ? r[j] + g[j] : g[j];
      ++groups;
      ng = 0;
    }
  }
  __device__ __forceinline__ double sum() const {
    double res = groups ? ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7])) : -0.0;
    // the pending terms are g[8 - ng .. 7], oldest first
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (j >= 8 - ng) res += g[j];
    return res;
  }
};

// np.dot of two 3-vectors, and the square under np.linalg.norm of one: numpy hands both to BLAS
// ddot, whose x86-64 kernel (OpenBLAS, FMA) forms the first product and fuses the other two
// into it in order -- the same bits numpy returns there.
__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return fma(a[2], b[2], fma(a[1], b[1], a[0] * b[0]));
}

// ONE_PASS: n_rows <= 257, so a photon has at most 128 pair terms (one numpy block): the scan
// sums them as it goes and no scratch is used. Otherwise the scan writes the clean rows' indices
// to scratch and the Simpson sum reads them back.
template <bool ONE_PASS>
__global__ void __launch_bounds__(kThreads) record_redshift_kernel(const double* __restrict__ records,
                                                                   int64_t n_photons, int32_t n_rows,
                                                                   int32_t n_cols, double c,
                                                                   const double* __restrict__ v_obs,
                                                                   const double* __restrict__ v_em,
                                                                   int32_t* __restrict__ scratch,
                                                                   double* __restrict__ out) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const double c2 = c * c;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_photons;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double* rows = records + i * (int64_t)n_rows * n_cols;
    int32_t* idx = ONE_PASS ? nullptr : scratch + i * (int64_t)n_rows;
    // the scan: first and last clean rows, the last three samples, the path, the largest |x|
    // and |eta|, and (one pass) the Simpson pair terms
    int m = 0, first = -1, last = -1;
    double x3[3] = {0.0, 0.0, 0.0}, y3[3] = {0.0, 0.0, 0.0}, prev[3] = {0.0, 0.0, 0.0};
    double path = 0.0;
    // compute_time_delay_map's loader keeps a photon whose clean rows stay below 1e26 m and
    // 3e18 s (np.max(np.abs(.)) < limit: every value below it; an infinity is not)
    const unsigned long long pos_lim = (unsigned long long)__double_as_longlong(1e26);
    const unsigned long long eta_lim = (unsigned long long)__double_as_longlong(3e18);
    bool below_lim = true;
    PairwiseStream ps;
    ps.init();
    for (int r = 0; r < n_rows; ++r) {
      const double* row = rows + (int64_t)r * n_cols;
      if (!row_clean(row, n_cols)) continue;
      if (!ONE_PASS) idx[m] = r;
      if (first < 0) first = r;
      last = r;
      x3[0] = x3[1]; x3[1] = x3[2]; x3[2] = row[0];
      y3[0] = y3[1]; y3[1] = y3[2]; y3[2] = row[13] * c2;
      if (ONE_PASS && m >= 2 && (m % 2) == 0) ps.push(simpson_term(x3[0], x3[1], x3[2], y3[0], y3[1], y3[2]));
      if (m >= 1) {
        // compute_travel_time_deflected: path_length += norm(positions[i + 1] - positions[i])
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = row[1 + k] - prev[k];
        path += sqrt(dot3(d, d));
      }
      for (int k = 0; k < 3; ++k) {
        prev[k] = row[1 + k];
        below_lim = below_lim && abs_bits(row[1 + k]) < pos_lim;
      }
      below_lim = below_lim && abs_bits(row[0]) < eta_lim;
      ++m;
    }
    double* o = out + i * EXC_RS_NCOLS;
    for (int k = 0; k < EXC_RS_NCOLS; ++k) o[k] = (k >= EXC_RS_PHI_OBS && k < EXC_RS_N_ROWS) ? nan : 0.0;
    o[EXC_RS_N_ROWS] = (double)m;
    if (m == 0) continue;
    const double* f = rows + (int64_t)first * n_cols;
    const double* l = rows + (int64_t)last * n_cols;
    o[EXC_RS_PHI_OBS] = f[9];
    o[EXC_RS_PHI_EM] = l[9];
    o[EXC_RS_A_OBS] = f[8];
    o[EXC_RS_A_EM] = l[8];
    o[EXC_RS_ETA_OBS] = f[0];
    o[EXC_RS_ETA_EM] = l[0];
    for (int k = 0; k < 3; ++k) {
      o[EXC_RS_X_OBS + k] = f[1 + k];
      o[EXC_RS_X_EM + k] = l[1 + k];
    }
    o[EXC_RS_TD_KEPT] = below_lim ? 1.0 : 0.0;
    if (m < 2) continue;  // compute_redshift_map and compute_time_delays leave such photons at zero
    {
      double X[3];
      for (int k = 0; k < 3; ++k) X[k] = l[1 + k] - f[1 + k];
      const double chord = sqrt(dot3(X, X));
      o[EXC_RS_PATH] = path;
      o[EXC_RS_CHORD] = chord;
      o[EXC_RS_TIME_DELAY] = path / c - chord / c;
    }
    const double z_h = (f[8] / l[8]) - 1.0;
    const double z_sw = (f[9] - l[9]) / c2;
    double z_isw;
    if (ONE_PASS) {
      z_isw = -simpson_finish(m, m == 2 ? 0.0 : ps.sum(), x3, y3) / c2;
    } else {
      const Clean cl{rows, idx, n_cols, c2};
      z_isw = -simpson(cl, m) / c2;
    }
    double z_d = 0.0;
    if (v_obs != nullptr && v_em != nullptr) {
      double d[3], nh[3];
      for (int k = 0; k < 3; ++k) d[k] = l[1 + k] - f[1 + k];
      const double nrm = sqrt(dot3(d, d));
      for (int k = 0; k < 3; ++k) nh[k] = d[k] / nrm;
      z_d = (dot3(v_obs + 3 * i, nh) - dot3(v_em + 3 * i, nh)) / c;
    }
    const double z_v = 0.0;
    o[EXC_RS_Z_H] = z_h;
    o[EXC_RS_Z_SW] = z_sw;
    o[EXC_RS_Z_ISW] = z_isw;
    o[EXC_RS_Z_D] = z_d;
    o[EXC_RS_Z_TOTAL] = (((z_h + z_sw) + z_isw) + z_d) + z_v;
    o[EXC_RS_Z_TOTAL_EXACT] = ((((1.0 + z_h) * (1.0 + z_sw)) * (1.0 + z_isw)) * (1.0 + z_d)) * (1.0 + z_v) - 1.0;
  }
}

// The unit spatial velocity (columns 5..7) of each photon's first clean row; NaN without one.
__global__ void __launch_bounds__(kThreads) sky_directions_kernel(const double* __restrict__ records,
                                                                  int64_t n_photons, int32_t n_rows,
                                                                  int32_t n_cols, double* __restrict__ dirs) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_photons;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double* rows = records + i * (int64_t)n_rows * n_cols;
    double* d = dirs + 3 * i;
    d[0] = d[1] = d[2] = nan;
    for (int r = 0; r < n_rows; ++r) {
      const double* row = rows + (int64_t)r * n_cols;
      if (!row_clean(row, n_cols)) continue;
      const double nrm = sqrt(dot3(row + 5, row + 5));
      for (int k = 0; k < 3; ++k) d[k] = row[5 + k] / nrm;
      break;
    }
  }
}

struct Frame {
  double m[3], bx[3], by[3];
};

// Tangent-plane coordinates of each direction about the mean direction (the angle from it
// along the in-plane unit vector); zero within 1e-10 rad of it, NaN for a NaN direction.
__global__ void __launch_bounds__(kThreads) sky_project_kernel(const double* __restrict__ dirs, int64_t n,
                                                               const Frame fr, double* __restrict__ xp,
                                                               double* __restrict__ yp) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double* d = dirs + 3 * i;
    const double ct = dot3(d, fr.m);
    if (isnan(ct)) {
      xp[i] = yp[i] = ct;
      continue;
    }
    const double th = acos(fmin(fmax(ct, -1.0), 1.0));
    double x = 0.0, y = 0.0;
    if (th > 1e-10) {
      double ip[3];
      for (int k = 0; k < 3; ++k) ip[k] = d[k] - ct * fr.m[k];
      const double ni = sqrt(dot3(ip, ip));
      for (int k = 0; k < 3; ++k) ip[k] = ip[k] / ni;
      x = dot3(ip, fr.bx) * th;
      y = dot3(ip, fr.by) * th;
    }
    xp[i] = x;
    yp[i] = y;
  }
}

struct Extent {
  double x0, x1, y0, y1;
  int nx, ny;
};

__global__ void __launch_bounds__(256) sky_bin_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                                      const double* __restrict__ v, int64_t n, const Extent e,
                                                      double* __restrict__ sum,
                                                      unsigned long long* __restrict__ count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double xi = x[i], yi = y[i], vi = v[i];
    if (!(isfinite(xi) && isfinite(yi) && isfinite(vi))) continue;
    if (xi < e.x0 || xi > e.x1 || yi < e.y0 || yi > e.y1) continue;
    const int ix = min((int)floor((xi - e.x0) / (e.x1 - e.x0) * (double)e.nx), e.nx - 1);
    const int iy = min((int)floor((yi - e.y0) / (e.y1 - e.y0) * (double)e.ny), e.ny - 1);
    const int64_t p = (int64_t)iy * e.nx + ix;
    atomicAdd(sum + p, vi);
    atomicAdd(count + p, 1ull);
  }
}

__global__ void sky_bin_finish_kernel(const double* __restrict__ sum, const unsigned long long* __restrict__ count,
                                      int64_t n_pix, double* __restrict__ mean) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_pix; p += (int64_t)gridDim.x * blockDim.x)
    mean[p] = count[p] ? sum[p] / (double)count[p] : nan;
}

unsigned grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)b;
}

int launch_status() {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    exc::set_last_error(cudaGetErrorString(e));
    return EXC_ERR_CUDA;
  }
  return EXC_SUCCESS;
}

bool rows_ok(const char* who, int64_t n_photons, int32_t n_rows, int32_t n_cols, int32_t min_cols) {
  if (n_photons < 0 || n_rows < 0 || n_cols < min_cols) {
    exc::set_last_error(who);
    return false;
  }
  return true;
}

}  // namespace

extern "C" int exc_record_redshift(const double* records, int64_t n_photons, int32_t n_rows, int32_t n_cols,
                                   double c, const double* v_obs, const double* v_em, int32_t* scratch,
                                   double* out, void* stream) {
  if (!rows_ok("record_redshift: n_photons and n_rows must be >= 0 and n_cols >= 14 (the FLRW record layout)",
               n_photons, n_rows, n_cols, 14))
    return EXC_ERR_INVALID;
  if (n_photons == 0) return EXC_SUCCESS;
  const bool one_pass = n_rows <= kOnePassRows;
  if (!records || !out || (!one_pass && !scratch)) {
    exc::set_last_error("record_redshift: records and out are required, and scratch when n_rows > 257");
    return EXC_ERR_INVALID;
  }
  if ((v_obs == nullptr) != (v_em == nullptr)) {
    exc::set_last_error("record_redshift: give both v_obs and v_em, or neither");
    return EXC_ERR_INVALID;
  }
  if (!(c > 0.0) || !std::isfinite(c)) {
    exc::set_last_error("record_redshift: c must be finite and > 0");
    return EXC_ERR_INVALID;
  }
  if (one_pass)
    record_redshift_kernel<true><<<grid_for(n_photons, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        records, n_photons, n_rows, n_cols, c, v_obs, v_em, nullptr, out);
  else
    record_redshift_kernel<false><<<grid_for(n_photons, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        records, n_photons, n_rows, n_cols, c, v_obs, v_em, scratch, out);
  return launch_status();
}

extern "C" int exc_sky_directions(const double* records, int64_t n_photons, int32_t n_rows, int32_t n_cols,
                                  double* dirs, void* stream) {
  if (!rows_ok("sky_directions: n_photons and n_rows must be >= 0 and n_cols >= 8", n_photons, n_rows, n_cols, 8))
    return EXC_ERR_INVALID;
  if (n_photons == 0) return EXC_SUCCESS;
  if (!records || !dirs) {
    exc::set_last_error("sky_directions: records and dirs are required");
    return EXC_ERR_INVALID;
  }
  sky_directions_kernel<<<grid_for(n_photons, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
      records, n_photons, n_rows, n_cols, dirs);
  return launch_status();
}

extern "C" int exc_sky_project(const double* dirs, int64_t n, const double mean_dir[3], const double basis_x[3],
                               const double basis_y[3], double* x_proj, double* y_proj, void* stream) {
  if (n < 0 || !mean_dir || !basis_x || !basis_y) {
    exc::set_last_error("sky_project: n must be >= 0; mean_dir, basis_x and basis_y are required");
    return EXC_ERR_INVALID;
  }
  if (n == 0) return EXC_SUCCESS;
  if (!dirs || !x_proj || !y_proj) {
    exc::set_last_error("sky_project: dirs, x_proj and y_proj are required");
    return EXC_ERR_INVALID;
  }
  Frame fr;
  for (int k = 0; k < 3; ++k) {
    fr.m[k] = mean_dir[k];
    fr.bx[k] = basis_x[k];
    fr.by[k] = basis_y[k];
  }
  sky_project_kernel<<<grid_for(n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(dirs, n, fr, x_proj, y_proj);
  return launch_status();
}

extern "C" int exc_sky_bin(const double* x, const double* y, const double* values, int64_t n, int32_t nx,
                           int32_t ny, const double extent[4], double* sum, unsigned long long* count, double* mean,
                           void* stream) {
  if (n < 0 || nx < 1 || ny < 1 || (int64_t)nx * ny > ((int64_t)1 << 31) || !extent) {
    exc::set_last_error("sky_bin: n >= 0, nx and ny >= 1 with nx * ny <= 2^31, and extent are required");
    return EXC_ERR_INVALID;
  }
  if (!(extent[1] > extent[0]) || !(extent[3] > extent[2]) || !std::isfinite(extent[1] - extent[0]) ||
      !std::isfinite(extent[3] - extent[2])) {
    exc::set_last_error("sky_bin: extent must be finite with x1 > x0 and y1 > y0");
    return EXC_ERR_INVALID;
  }
  if (!sum || !count || !mean || (n > 0 && (!x || !y || !values))) {
    exc::set_last_error("sky_bin: x, y, values, sum, count and mean are required");
    return EXC_ERR_INVALID;
  }
  const int64_t n_pix = (int64_t)nx * ny;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(sum, 0, n_pix * sizeof(double), s) != cudaSuccess ||
      cudaMemsetAsync(count, 0, n_pix * sizeof(unsigned long long), s) != cudaSuccess)
    return launch_status();
  const Extent e{extent[0], extent[1], extent[2], extent[3], nx, ny};
  if (n > 0) {
    sky_bin_kernel<<<grid_for(n, 256), 256, 0, s>>>(x, y, values, n, e, sum, count);
    const int rc = launch_status();
    if (rc) return rc;
  }
  sky_bin_finish_kernel<<<grid_for(n_pix, 256), 256, 0, s>>>(sum, count, n_pix, mean);
  return launch_status();
}
