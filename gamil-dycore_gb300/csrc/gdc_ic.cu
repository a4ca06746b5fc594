// gdc_ic.cu -- initial conditions generated in device memory (FP64), the
// device counterparts of the gdc_ic_* host functions in gdc_host.cpp: the
// reference's Rossby-Haurwitz wave, steady geostrophic flow, mountain zonal
// flow and shallow-water wave test cases, and the seeded harmonic state with
// its optional white noise.  The mesh tables and the seeded state's random draws come
// from the host (the same values the host functions use); the per-point
// arithmetic runs here, so a member of any size is admitted without host
// arrays.  Compiled without FMA contraction, like the FP64 kernels.
#include <cuda_runtime.h>

#include "gdc_internal.h"

namespace gdc {
namespace {

constexpr double kG = kGrav;
constexpr int kIcThreads = 256;

struct MeshView {
  const double *full_lat, *half_lat, *full_lon, *half_lon, *full_cos, *half_cos, *full_sin, *half_sin;
  int N, M, Mh;
  double dlon, dlat;
};

__device__ __forceinline__ int grid_stride() { return gridDim.x * blockDim.x; }

// Separable states (Rossby-Haurwitz wave, shallow-water Rossby wave): the
// products of the host's factor tables, with the host's own inline
// evaluators, so the fields equal the gdc_ic_* host arrays bit for bit.
template <int KIND>
__global__ void separable_kernel(MeshView m, const double* t, double* u, double* v, double* gd) {
  const int N = m.N, M = m.M;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < M * N; q += grid_stride()) {
    const int j = q / N, i = q - j * N;
    if (KIND == GDC_IC_ROSSBY_HAURWITZ) {
      u[q] = rh_u(t, N, M, i, j);
      gd[q] = rh_gd(t, N, M, i, j);
      if (j < m.Mh) v[q] = rh_v(t, N, M, i, j);
    } else {
      u[q] = sw_u(t, N, M, i, j);
      gd[q] = sw_gd(t, N, M, i, j);
      if (j < m.Mh) v[q] = sw_v(t, N, M, i, j);
    }
  }
}

// steady_geostrophic_flow (src/test_cases/barotropic/steady_geostrophic_flow_
// test_mod.F90:20-62) and mountain_zonal_flow (mountain_zonal_flow_test_mod.
// F90:28-97): u = u0 cos(lat), v = 0 (alpha = 0), gd = gd0 - (a Omega u0 +
// u0^2/2) sin^2(lat) - ghs, ghs a cone of radius pi/9 around (1.5 pi, pi/6).
__global__ void zonal_kernel(MeshView m, double u0, double gd0, int mountain, double* u, double* v, double* gd,
                             double* ghs) {
  const int N = m.N;
  const double alpha = 0.0, ca = cos(alpha), sa = sin(alpha);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m.M * N; q += grid_stride()) {
    const int j = q / N, i = q - j * N;
    double h = 0.0;
    if (mountain) {
      const double lon0 = kPi * 1.5, lat0 = kPi / 6.0, R = kPi / 9.0, ghs0 = 2000.0 * kG;
      double dl = fabs(m.full_lon[i] - lon0);
      dl = fmin(dl, 2 * kPi - dl);
      const double dp = m.full_lat[j] - lat0;
      const double d = fmin(R, sqrt(dl * dl + dp * dp));
      h = ghs0 * (1.0 - d / R);
    }
    ghs[q] = h;
    u[q] = (j >= 1 && j < m.M - 1) ? u0 * (m.full_cos[j] * ca + cos(m.half_lon[i]) * m.full_sin[j] * sa) : 0.0;
    if (j < m.Mh) v[q] = -u0 * cos(m.full_lon[i]) * sa;
    const double t = m.full_sin[j] * ca - cos(m.full_lon[i]) * m.full_cos[j] * sa;
    gd[q] = gd0 - (kRadius * kOmega * u0 + u0 * u0 * 0.5) * (t * t) - h;
  }
}

// Real spherical-harmonic series sum_{l=1..L} sum_{m=0..l} Pbar_l^m(sin lat)
// (a_lm cos m lon + b_lm sin m lon) with orthonormal associated Legendre
// functions (the standard three-term recurrence, column by column in m).
__device__ double harmonics(const double* a, const double* b, int L, double lat, double lon) {
  const double x = sin(lat), sx = cos(lat);
  double s = 0.0, pmm = sqrt(1.0 / (4 * kPi));
  for (int m = 0; m <= L; ++m) {
    if (m > 0) pmm = sqrt((2.0 * m + 1) / (2.0 * m)) * sx * pmm;
    const double w = m == 0 ? 1.0 : sqrt(2.0);
    const double cm = cos(m * lon), sm = sin(m * lon);
    double p2 = 0.0, p1 = pmm;
    for (int l = m; l <= L; ++l) {
      double p;
      if (l == m) {
        p = pmm;
      } else if (l == m + 1) {
        p = sqrt(2.0 * m + 3) * x * pmm;
      } else {
        const double al = sqrt((4.0 * l * l - 1) / ((double)l * l - (double)m * m));
        const double bl = sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1));
        p = al * (x * p1 - bl * p2);
      }
      if (l > m) {
        p2 = p1;
        p1 = p;
      }
      if (l >= 1) s += w * p * (a[l * (L + 1) + m] * cm + b[l * (L + 1) + m] * sm);
    }
  }
  return s;
}

// gd harmonics at full points, streamfunction harmonics at C-grid corners.
__global__ void seeded_eval_kernel(MeshView m, int L, const double* ag, const double* bg, const double* ap,
                                   const double* bp, double* f, double* psi) {
  const int N = m.N;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m.M * N; q += grid_stride()) {
    const int j = q / N, i = q - j * N;
    f[q] = harmonics(ag, bg, L, m.full_lat[j], m.full_lon[i]);
    if (j < m.Mh) psi[q] = harmonics(ap, bp, L, m.half_lat[j], m.half_lon[i]);
  }
}

// RMS scale factors target / sqrt(mean x^2) of f (n values) and psi: one
// block, FP64 sums.
__global__ void seeded_scale_kernel(const double* f, int nf, const double* psi, int np, double gd_rms,
                                    double psi_rms, double* scale) {
  __shared__ double red[2][kIcThreads];
  double sf = 0.0, sp = 0.0;
  for (int q = threadIdx.x; q < nf; q += blockDim.x) sf += f[q] * f[q];
  for (int q = threadIdx.x; q < np; q += blockDim.x) sp += psi[q] * psi[q];
  red[0][threadIdx.x] = sf;
  red[1][threadIdx.x] = sp;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    scale[0] = red[0][0] > 0 && gd_rms > 0 ? gd_rms / sqrt(red[0][0] / nf) : 0.0;
    scale[1] = red[1][0] > 0 && psi_rms > 0 ? psi_rms / sqrt(red[1][0] / np) : 0.0;
  }
}

// splitmix64 output number k (1-based) of the stream seeded with `seed`:
// the host generator's k-th call, by random access.
__device__ __forceinline__ unsigned long long splitmix(unsigned long long seed, unsigned long long k) {
  unsigned long long z = seed + k * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform_k(unsigned long long seed, unsigned long long k) {
  return ((splitmix(seed, k) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
// Normal number q of the host generator's Box-Muller stream (pairs from
// uniforms 2p+1, 2p+2; the cosine first).
__device__ __forceinline__ double normal_q(unsigned long long seed, unsigned long long q) {
  const unsigned long long p = q >> 1;
  const double u1 = uniform_k(seed, 2 * p + 1), u2 = uniform_k(seed, 2 * p + 2);
  const double r = sqrt(-2.0 * log(u1));
  return (q & 1) ? r * sin(2 * kPi * u2) : r * cos(2 * kPi * u2);
}

// The seeded state from its harmonics: mountains (haversine great-circle
// distance), gd, and u, v differenced from the streamfunction at corners.
__global__ void seeded_assemble_kernel(MeshView m, gdc_ic_spec sp, const double* clat, const double* clon,
                                       const double* f, const double* psi, const double* scale, double* u,
                                       double* v, double* gd, double* ghs) {
  const int N = m.N;
  const double gscale = scale[0], pscale = scale[1];
  const double rr = sp.mountain_radius_deg * kPi / 180.0;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m.M * N; q += grid_stride()) {
    const int j = q / N, i = q - j * N;
    double h = 0.0;
    for (int k = 0; k < sp.n_mountains; ++k) {
      const double dphi = m.full_lat[j] - clat[k], dlam = m.full_lon[i] - clon[k];
      const double s1 = sin(0.5 * dphi), s2 = sin(0.5 * dlam);
      const double hv = s1 * s1 + cos(m.full_lat[j]) * cos(clat[k]) * s2 * s2;
      const double d = 2 * asin(sqrt(fmin(1.0, hv)));
      h += sp.mountain_height * kG * exp(-(d / rr) * (d / rr));
    }
    ghs[q] = h;
    const double t = m.full_sin[j];
    double g = sp.gd0 + gscale * f[q] - (kRadius * kOmega * sp.u0 + sp.u0 * sp.u0 * 0.5) * (t * t) - h;
    if (sp.noise_sigma > 0) g += sp.noise_sigma * normal_q(sp.noise_seed, (unsigned long long)q);
    gd[q] = g;
    u[q] = (j >= 1 && j < m.M - 1)
               ? -(psi[q] * pscale - psi[q - N] * pscale) / (kRadius * m.dlat) + sp.u0 * m.full_cos[j]
               : 0.0;
    if (j < m.Mh) {
      const int im = i > 0 ? i - 1 : N - 1;
      v[q] = (psi[q] * pscale - psi[j * N + im] * pscale) / (kRadius * m.half_cos[j] * m.dlon);
    }
  }
}

// gdc_ic_add_noise for the analytic states.
__global__ void noise_kernel(int n, unsigned long long seed, double sigma, double* gd) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += grid_stride())
    gd[q] += sigma * normal_q(seed, (unsigned long long)q);
}

}  // namespace

int ic_generate(const gdc_ic_spec& spec, int N, int M, const double* tables, double* scratch, double* u,
                double* v, double* gd, double* ghs, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const int Mh = M - 1;
  MeshView m;
  m.full_lat = tables;
  m.half_lat = m.full_lat + M;
  m.full_lon = m.half_lat + Mh;
  m.half_lon = m.full_lon + N;
  m.full_cos = m.half_lon + N;
  m.half_cos = m.full_cos + M;
  m.full_sin = m.half_cos + Mh;
  m.half_sin = m.full_sin + M;
  m.N = N;
  m.M = M;
  m.Mh = Mh;
  m.dlon = 2 * kPi / N;
  m.dlat = kPi / Mh;
  const double* extra = m.half_sin + Mh;
  const int n = M * N;
  const int grid = (n + kIcThreads - 1) / kIcThreads;
  cudaMemsetAsync(v, 0, (size_t)Mh * N * sizeof(double), s);
  cudaMemsetAsync(ghs, 0, (size_t)n * sizeof(double), s);
  switch (spec.kind) {
    case GDC_IC_ROSSBY_HAURWITZ:
      separable_kernel<GDC_IC_ROSSBY_HAURWITZ><<<grid, kIcThreads, 0, s>>>(m, extra, u, v, gd);
      break;
    case GDC_IC_SHALLOW_WATER_WAVES:
      separable_kernel<GDC_IC_SHALLOW_WATER_WAVES><<<grid, kIcThreads, 0, s>>>(m, extra, u, v, gd);
      break;
    case GDC_IC_STEADY_GEOSTROPHIC:
      zonal_kernel<<<grid, kIcThreads, 0, s>>>(m, 2 * kPi * kRadius / (12 * 86400), 2.94e4, 0, u, v, gd, ghs);
      break;
    case GDC_IC_MOUNTAIN_ZONAL_FLOW:
      zonal_kernel<<<grid, kIcThreads, 0, s>>>(m, 20.0, 5960.0 * kG, 1, u, v, gd, ghs);
      break;
    case GDC_IC_SEEDED: {
      const int L = spec.lmax, nc = (L + 1) * (L + 1);
      const double* clat = extra;
      const double* clon = clat + spec.n_mountains;
      const double* ag = clon + spec.n_mountains;
      const double* bg = ag + nc;
      const double* ap = bg + nc;
      const double* bp = ap + nc;
      double* f = scratch;
      double* psi = scratch + n;
      double* scale = scratch + 2 * (size_t)n;
      cudaMemsetAsync(psi, 0, (size_t)n * sizeof(double), s);
      seeded_eval_kernel<<<grid, kIcThreads, 0, s>>>(m, L, ag, bg, ap, bp, f, psi);
      seeded_scale_kernel<<<1, kIcThreads, 0, s>>>(f, n, psi, Mh * N, L > 0 ? spec.gd_rms : 0.0,
                                                  L > 0 ? spec.psi_rms : 0.0, scale);
      seeded_assemble_kernel<<<grid, kIcThreads, 0, s>>>(m, spec, clat, clon, f, psi, scale, u, v, gd, ghs);
      break;
    }
    default:
      return GDC_E_CONFIG;
  }
  if (spec.kind != GDC_IC_SEEDED && spec.noise_sigma > 0)
    noise_kernel<<<grid, kIcThreads, 0, s>>>(n, spec.noise_seed, spec.noise_sigma, gd);
  return cudaGetLastError() == cudaSuccess ? GDC_OK : GDC_E_CUDA;
}

}  // namespace gdc
