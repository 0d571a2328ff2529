// exc_gen.cu -- device-side photon generation (include/excalibur_gb300.h, ExcPhotonGen).
//
// The host generators (photon/photons.py) build millions of initial states in
// numpy and copy them over; here each thread writes one photon's state in
// place and the null condition then sets u^0 (exc_null_init), so a batch of
// any size is produced in two launches with no host work. The arithmetic of
// the patch and cone generators follows the host code operation for
// operation, so the states agree with the host's to the last bit (patch) or
// to the rounding of a 3-term dot product (cone).
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/excalibur_gb300.h"

namespace exc {
void set_last_error(const char* msg);
}

namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// uniform in [0, 1) from the top 53 bits
__device__ __forceinline__ double unit53(uint64_t x) { return (double)(x >> 11) * (1.0 / 9007199254740992.0); }

// CONE_* rotation of the cone-frame direction v onto the cone axis (Rodrigues,
// the host's _rotate_to_direction).
__device__ __forceinline__ void cone_rotate(const ExcPhotonGen& g, const double v[3], double d[3]) {
  const double* k = g.rot_axis;
  const double kv[3] = {k[1] * v[2] - k[2] * v[1], k[2] * v[0] - k[0] * v[2], k[0] * v[1] - k[1] * v[0]};
  const double vk = (v[0] * k[0] + v[1] * k[1]) + v[2] * k[2];
  for (int c = 0; c < 3; ++c) d[c] = (v[c] * g.rot_cos + kv[c] * g.rot_sin) + k[c] * vk * (1.0 - g.rot_cos);
}

// The bin of photon i: the largest ib with bin_offsets[ib] <= i (offsets non-decreasing).
__device__ __forceinline__ int find_bin(const ExcPhotonGen& g, int64_t i) {
  int lo = 0, hi = g.n_bins - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.bin_offsets[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void gen_kernel(const ExcPhotonGen g, int64_t n, double* states) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double d[3];
    double* s = states + i * 8;
    s[0] = g.origin[0];
    s[1] = g.origin[1];
    s[2] = g.origin[2];
    s[3] = g.origin[3];
    s[4] = 0.0;
    if (g.mode == EXC_GEN_IMPACT_BINS) {
      // generate_impact_parameter_bins (photons.py:663-701): screen point, velocity c k
      const int ib = find_bin(g, i);
      const int64_t j = i - g.bin_offsets[ib], nph = g.bin_offsets[ib + 1] - g.bin_offsets[ib];
      const uint64_t h = splitmix64(g.seed ^ splitmix64((uint64_t)i));
      const double p = g.random_phi ? 2.0 * M_PI * unit53(splitmix64(h)) : (double)j * (2.0 * M_PI / (double)nph);
      const double b1 = g.b_edges[ib], b2 = g.b_edges[ib + 1];
      const double b = sqrt(unit53(h) * (b2 * b2 - b1 * b1) + b1 * b1);
      const double cp = cos(p), sp = sin(p);
      double x[3], v[3];
      for (int k = 0; k < 3; ++k) {
        x[k] = g.origin[1 + k] + b * (cp * g.e1[k] + sp * g.e2[k]);
        v[k] = g.axis[k] * g.speed;
      }
      if (!g.spherical) {
        for (int k = 0; k < 3; ++k) { s[1 + k] = x[k]; s[5 + k] = v[k]; }
        continue;
      }
      // cartesian_to_spherical / cartesian_velocity_to_spherical (core/coordinates.py:31-84)
      const double rho2 = x[0] * x[0] + x[1] * x[1];
      const double r2 = rho2 + x[2] * x[2];
      const double r = sqrt(r2);
      s[1] = r;
      s[2] = acos(fmin(1.0, fmax(-1.0, x[2] / r)));
      s[3] = atan2(x[1], x[0]);
      s[5] = (x[0] * v[0] + x[1] * v[1] + x[2] * v[2]) / r;
      s[6] = (x[2] * (x[0] * v[0] + x[1] * v[1]) - rho2 * v[2]) / (r * r * sqrt(rho2));
      s[7] = (x[0] * v[1] - x[1] * v[0]) / rho2;
      continue;
    }
    if (g.mode == EXC_GEN_PATCH_GRID || g.mode == EXC_GEN_PATCH_POINTS) {
      double A, B;
      if (g.mode == EXC_GEN_PATCH_GRID) {
        const int64_t ia = i / g.n_side, ib = i - ia * g.n_side;
        A = ((double)ia + 0.5) / g.n_side * 2.0 - 1.0;
        B = ((double)ib + 0.5) / g.n_side * 2.0 - 1.0;
      } else {
        A = g.uv[2 * i];
        B = g.uv[2 * i + 1];
      }
      const double ah = A * g.half, bh = B * g.half;
      for (int k = 0; k < 3; ++k) d[k] = (g.axis[k] + ah * g.e1[k]) + bh * g.e2[k];
    } else if (g.mode == EXC_GEN_CONE_GRID || g.mode == EXC_GEN_CONE_RANDOM) {
      double th, ph;
      if (g.mode == EXC_GEN_CONE_GRID) {
        const int64_t it = i / g.n_phi, ip = i - it * g.n_phi;
        th = ((double)it + 0.5) * g.half / g.n_theta;
        ph = 2.0 * M_PI * (double)ip / g.n_phi;
      } else {
        // generate_cone_random (photons.py:84-88): theta uniform in [0, cone), azimuth uniform
        const uint64_t h = splitmix64(g.seed ^ splitmix64((uint64_t)i));
        th = g.half * unit53(h);
        ph = 2.0 * M_PI * unit53(splitmix64(h));
      }
      const double v[3] = {sin(th) * cos(ph), sin(th) * sin(ph), cos(th)};
      cone_rotate(g, v, d);
    } else {
      // uniform on the sphere: z uniform in [-1, 1), azimuth uniform in [0, 2 pi)
      const uint64_t h = splitmix64(g.seed ^ splitmix64((uint64_t)i));
      const double z = 1.0 - 2.0 * unit53(h);
      const double p = 2.0 * M_PI * unit53(splitmix64(h));
      const double r = sqrt(fmax(0.0, 1.0 - z * z));
      d[0] = r * cos(p);
      d[1] = r * sin(p);
      d[2] = z;
    }
    const double nrm = sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
    for (int k = 0; k < 3; ++k) s[5 + k] = (d[k] / nrm) * g.speed;
  }
}

}  // namespace

extern "C" int64_t exc_gen_count(const ExcPhotonGen* g) {
  if (!g) return -1;
  switch (g->mode) {
    case EXC_GEN_PATCH_GRID: return (int64_t)g->n_side * g->n_side;
    case EXC_GEN_CONE_GRID: return (int64_t)g->n_theta * g->n_phi;
    case EXC_GEN_PATCH_POINTS:
    case EXC_GEN_FULL_SKY:
    case EXC_GEN_CONE_RANDOM:
    case EXC_GEN_IMPACT_BINS: return g->n;
    default: return -1;
  }
}

extern "C" int exc_generate_photons(const ExcMetric* metric, const ExcPhotonGen* g, double* states, int32_t* status,
                                    void* stream) {
  if (!g || !states) {
    exc::set_last_error("generate: gen and states are required");
    return EXC_ERR_INVALID;
  }
  const int64_t n = exc_gen_count(g);
  if (n < 0) {
    exc::set_last_error("generate: unknown mode");
    return EXC_ERR_INVALID;
  }
  if ((g->mode == EXC_GEN_PATCH_GRID && g->n_side < 1) || (g->mode == EXC_GEN_CONE_GRID && (g->n_theta < 1 || g->n_phi < 1)) ||
      (g->mode == EXC_GEN_PATCH_POINTS && !g->uv)) {
    exc::set_last_error("generate: sizes must be >= 1 (and uv given for PATCH_POINTS)");
    return EXC_ERR_INVALID;
  }
  if (g->mode == EXC_GEN_IMPACT_BINS && (g->n_bins < 1 || !g->b_edges || !g->bin_offsets)) {
    exc::set_last_error("generate: IMPACT_BINS needs n_bins >= 1, b_edges and bin_offsets (device arrays)");
    return EXC_ERR_INVALID;
  }
  if (n == 0) return EXC_SUCCESS;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  gen_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(*g, n, states);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    exc::set_last_error(cudaGetErrorString(e));
    return EXC_ERR_CUDA;
  }
  return exc_null_init(metric, states, g->sign, status, nullptr, n, stream);
}

// ---- lens potential on a grid (objects/spherical_mass.py:29-49) ------------
// One thread per node, grid-stride, coalesced float64 stores: the field the comparison
// runners build with numpy before every run (a 256^3 grid is 134 MB) is written at HBM
// speed instead. Same operations as numpy on the meshgrid of
// linspace(origin, origin + n * spacing, n, endpoint=False): node x_i = i * spacing + origin,
// r = sqrt(((x-x0)^2 + (y-y0)^2) + (z-z0)^2), r = 1e-10 where r == 0, then
// (neg_gm * (three_r2 - r^2)) / two_r3 inside (r < radius) and neg_gm / r outside. The three
// scalar coefficients come from the host, evaluated by Python as the reference writes them
// (-G * M, 3 * R**2, 2 * R**3), so the grid is bit-identical to the reference's. Built with
// --fmad=false: no contraction of the node coordinate or the squares.
namespace {
__global__ void spherical_mass_kernel(int64_t n0, int64_t n1, int64_t n2, double o0, double o1, double o2,
                                      double s0, double s1, double s2, double x0, double y0, double z0,
                                      double radius, double neg_gm, double three_r2, double two_r3,
                                      double* __restrict__ out) {
  const int64_t total = n0 * n1 * n2;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = q % n2, j = (q / n2) % n1, i = q / (n1 * n2);
    const double dx = ((double)i * s0 + o0) - x0;
    const double dy = ((double)j * s1 + o1) - y0;
    const double dz = ((double)k * s2 + o2) - z0;
    double r = sqrt((dx * dx + dy * dy) + dz * dz);
    if (r == 0.0) r = 1e-10;
    out[q] = (r < radius) ? (neg_gm * (three_r2 - r * r)) / two_r3 : neg_gm / r;
  }
}
}  // namespace

extern "C" int exc_spherical_mass_grid(const int64_t n[3], const double origin[3], const double spacing[3],
                                       const double center[3], double radius, double neg_gm, double three_r2,
                                       double two_r3, double* out, void* stream) {
  if (!n || !origin || !spacing || !center || !out) {
    exc::set_last_error("spherical_mass_grid: n, origin, spacing, center and out are required");
    return EXC_ERR_INVALID;
  }
  if (n[0] < 1 || n[1] < 1 || n[2] < 1 || n[0] > (1 << 20) || n[1] > (1 << 20) || n[2] > (1 << 20)) {
    exc::set_last_error("spherical_mass_grid: each n must be in [1, 2^20]");
    return EXC_ERR_INVALID;
  }
  const int64_t total = n[0] * n[1] * n[2];
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  spherical_mass_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      n[0], n[1], n[2], origin[0], origin[1], origin[2], spacing[0], spacing[1], spacing[2], center[0], center[1],
      center[2], radius, neg_gm, three_r2, two_r3, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    exc::set_last_error(cudaGetErrorString(e));
    return EXC_ERR_CUDA;
  }
  return EXC_SUCCESS;
}
