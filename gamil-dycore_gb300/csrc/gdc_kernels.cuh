// gdc_kernels.cuh -- sm_103a kernels of the barotropic time step (templates;
// instantiated per arithmetic type by gdc_kernels_f64.cu / gdc_kernels_f32.cu).
//
// One launch of `stage_kernel` evaluates space_operators
// (src/dycore_mod.F90:184-365) for every member of a batch and fuses the
// consumer of the tendency into the same pass (the update_state of a
// predict_correct stage, the tendency store, or the beta inner products).
// Work items are either bulk tiles (R rows x W columns of one member, all
// three staggered fields) or whole-row tasks (pole rows, whose mass-flux
// divergence is a zonal sum, and rows the zonal filter touches, whose
// filter and s1/s2 rescale need the complete latitude circle).
//
// A work item stages gd, ghs, iap u, iap v of its rows +-1 (+2 for gd) and
// columns +-1 (+2) in shared memory, derives iap gd = sqrt(gd),
// u = 2 iap_u / (iap_gd(i) + iap_gd(i+1)) and v = 2 iap_v / (iap_gd(j) +
// iap_gd(j+1)) there (the update_state epilogue of the reference,
// src/dycore_mod.F90:617-645, moved to the consumer so that only
// {gd, iap u, iap v} live in HBM), then evaluates the operators point-wise
// in the reference's order of operations.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "gdc_internal.h"

namespace gdc {

constexpr int kThreads = 256;
constexpr int kRowChunk = 128;  // columns per chunk of a whole-row task
constexpr int kMaxKeep = 128;   // packed FFT coefficients a filter row may keep

// ------------------------------------------------------------ helpers

template <typename A>
__device__ A warp_sum(A v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block-wide sum (fixed shuffle tree + fixed warp order).
template <typename A>
__device__ A block_sum(A v, A* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    A s = (l < nw) ? red[l] : A(0);
    s = warp_sum(s);
    if (l == 0) red[0] = s;
  }
  __syncthreads();
  A r = red[0];
  __syncthreads();
  return r;
}

template <typename T>
struct TileSmem {
  T *gd, *ghs, *iu, *iv, *ig, *u, *v;
  int R, W, SW, rows;  // SW = W + 3 columns, rows = R + 3
  int j0, i0;
};

template <typename T>
__device__ inline T cf(const MemberDev<T>& md, int k, int j) {
  return md.coef[cf_off(k, md.M) + j];
}
template <typename T>
__device__ inline T ch(const MemberDev<T>& md, int k, int jh) {  // jh in -1..Mh
  return md.coef[ch_off(k, md.M) + jh + 1];
}

// Partition of a staging buffer of `words` T values into the seven arrays.
template <typename T>
__device__ TileSmem<T> carve_tile(T* base, int R, int W, int j0, int i0) {
  TileSmem<T> t;
  t.R = R;
  t.W = W;
  t.SW = W + 3;
  t.rows = R + 3;
  t.j0 = j0;
  t.i0 = i0;
  const int n = t.rows * t.SW;
  t.gd = base;
  t.ghs = base + n;
  t.iu = base + 2 * n;
  t.iv = base + 3 * n;
  t.ig = base + 4 * n;
  t.u = base + 5 * n;
  t.v = base + 6 * n;
  return t;
}

// Load rows j0-1 .. j0+R+1 (full) and half rows j0-1 .. j0+R+1, columns
// i0-1 .. i0+W+1 (periodic), then derive iap gd, u and v.  Rows outside
// the sphere are the reference's never-filled latitude halo: 0.
template <typename T>
__device__ void stage_tile(const MemberDev<T>& md, const T* __restrict__ gd,
                           const T* __restrict__ iu, const T* __restrict__ iv, TileSmem<T>& t,
                           bool u_halo_row = false) {
  const int N = md.N, M = md.M, Mh = md.Mh;
  const int SW = t.SW, n = t.rows * SW;
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    const int rr = p / SW, cc = p - rr * SW;
    const int j = t.j0 - 1 + rr;
    int i = t.i0 - 1 + cc;
    i = i < 0 ? i + N : (i >= N ? i - N : i);
    T g = 0, gh = 0, a = 0, b = 0;
    if (j >= 0 && j < M) {
      const size_t o = (size_t)j * N + i;
      g = gd[o];
      gh = md.ghs[o];
      a = iu[o];
      if (j < Mh) b = iv[o];
    }
    t.gd[p] = g;
    t.ghs[p] = gh;
    t.iu[p] = a;
    t.iv[p] = b;
    t.ig[p] = sqrt(g);
  }
  __syncthreads();
  // u on full rows j0..j0+R (local 1..R+1; from local 0 when the stencil
  // also needs row j0-1), v on half rows j0-1..j0+R (local 0..R+1),
  // columns i0-1..i0+W (local 0..W+1).
  const int urow0 = u_halo_row ? 0 : 1;
  const int nd = (t.R + 2) * (t.W + 2);
  for (int q = threadIdx.x; q < nd; q += blockDim.x) {
    const int rr = q / (t.W + 2), cc = q - rr * (t.W + 2);
    const int p = rr * SW + cc;
    const int j = t.j0 - 1 + rr;
    T uu = 0, vv = 0;
    if (rr >= urow0 && j >= 1 && j <= M - 2) uu = t.iu[p] * T(2) / (t.ig[p] + t.ig[p + 1]);
    if (j >= 0 && j < Mh) vv = t.iv[p] * T(2) / (t.ig[p] + t.ig[p + SW]);
    t.u[p] = uu;
    t.v[p] = vv;
  }
  __syncthreads();
}

// ----------------------------------------------------- point operators
// (rr, cc) is the local position of full row j / half row j, column i.

template <typename T, int PASS, int ADV>
__device__ inline T point_du(const MemberDev<T>& md, const TileSmem<T>& t, int j, int p,
                             T beta_lon, T beta_lat) {
  const int SW = t.SW;
  T r = 0;
  if (PASS != kFastPass) {
    // src/dycore_mod.F90:376-392 / :393-415
    const T uc = t.u[p], um = t.u[p - 1], up = t.u[p + 1];
    const T u1 = uc + um, u2 = uc + up;
    T adv_lon;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lon = cf(md, CF_RADVLON, j) * (u2 * t.iu[p + 1] - u1 * t.iu[p - 1]);
    } else {
      const T ic = t.iu[p], ip = t.iu[p + 1], im = t.iu[p - 1];
      adv_lon = cf(md, CF_RADVLON, j) * (u2 * (ic + ip) - beta_lon * fabs(u2) * (ip - ic) -
                                         u1 * (ic + im) + beta_lon * fabs(u1) * (ic - im) -
                                         (u2 - u1) * ic);
    }
    // src/dycore_mod.F90:433-439 / :450-459
    const T v1 = (t.v[p - SW] + t.v[p - SW + 1]) * ch(md, CH_COS, j - 1);
    const T v2 = (t.v[p] + t.v[p + 1]) * ch(md, CH_COS, j);
    T adv_lat;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lat = cf(md, CF_RADVLAT, j) * (v2 * t.iu[p + SW] - v1 * t.iu[p - SW]);
    } else {
      const T ic = t.iu[p], ip = t.iu[p + SW], im = t.iu[p - SW];
      adv_lat = cf(md, CF_RADVLAT, j) * (v2 * (ic + ip) - beta_lat * fabs(v2) * (ip - ic) -
                                         v1 * (ic + im) + beta_lat * fabs(v1) * (ic - im) -
                                         (v2 - v1) * ic);
    }
    r = -adv_lon - adv_lat;
  }
  if (PASS != kSlowPass) {
    // src/dycore_mod.F90:485-493
    const T fv = T(0.25) * (cf(md, CF_F, j) + cf(md, CF_C, j) * t.u[p]) *
                 (cf(md, CF_C1, j) * (t.iv[p - SW] + t.iv[p - SW + 1]) +
                  cf(md, CF_C2, j) * (t.iv[p] + t.iv[p + 1]));
    // src/dycore_mod.F90:514-519
    const T pgf = T(0.5) * (t.ig[p] + t.ig[p + 1]) / cf(md, CF_DLON, j) *
                  (t.gd[p + 1] + t.ghs[p + 1] - t.gd[p] - t.ghs[p]);
    if (PASS == kAllPass)
      r = r + fv - pgf;
    else
      r = fv - pgf;
  }
  return r;
}

template <typename T, int PASS, int ADV>
__device__ inline T point_dv(const MemberDev<T>& md, const TileSmem<T>& t, int jh, int p,
                             T beta_lon, T beta_lat) {
  const int SW = t.SW;
  T r = 0;
  if (PASS != kFastPass) {
    // src/dycore_mod.F90:386-391 / :406-414
    const T u1 = t.u[p - 1] + t.u[p + SW - 1];
    const T u2 = t.u[p] + t.u[p + SW];
    T adv_lon;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lon = ch(md, CH_RADVLON, jh) * (u2 * t.iv[p + 1] - u1 * t.iv[p - 1]);
    } else {
      const T ic = t.iv[p], ip = t.iv[p + 1], im = t.iv[p - 1];
      adv_lon = ch(md, CH_RADVLON, jh) * (u2 * (ic + ip) - beta_lon * fabs(u2) * (ip - ic) -
                                          u1 * (ic + im) + beta_lon * fabs(u1) * (ic - im) -
                                          (u2 - u1) * ic);
    }
    // src/dycore_mod.F90:441-446 / :461-469
    const T vc = t.v[p] * ch(md, CH_COS, jh);
    const T v1 = vc + t.v[p - SW] * ch(md, CH_COS, jh - 1);
    const T v2 = vc + t.v[p + SW] * ch(md, CH_COS, jh + 1);
    T adv_lat;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lat = ch(md, CH_RADVLAT, jh) * (v2 * t.iv[p + SW] - v1 * t.iv[p - SW]);
    } else {
      const T ic = t.iv[p], ip = t.iv[p + SW], im = t.iv[p - SW];
      adv_lat = ch(md, CH_RADVLAT, jh) * (v2 * (ic + ip) - beta_lat * fabs(v2) * (ip - ic) -
                                          v1 * (ic + im) + beta_lat * fabs(v1) * (ic - im) -
                                          (v2 - v1) * ic);
    }
    r = -adv_lon - adv_lat;
  }
  if (PASS != kSlowPass) {
    // src/dycore_mod.F90:495-503
    const T f0 = cf(md, CF_F, jh), c0 = cf(md, CF_C, jh);
    const T f1 = cf(md, CF_F, jh + 1), c1 = cf(md, CF_C, jh + 1);
    const T fu = T(0.25) * ((f0 + c0 * t.u[p]) * t.iu[p] + (f0 + c0 * t.u[p - 1]) * t.iu[p - 1] +
                            (f1 + c1 * t.u[p + SW]) * t.iu[p + SW] +
                            (f1 + c1 * t.u[p + SW - 1]) * t.iu[p + SW - 1]);
    // src/dycore_mod.F90:530-535
    const T pgf = T(0.5) * (t.ig[p] + t.ig[p + SW]) / ch(md, CH_DLAT, jh) * ch(md, CH_COS, jh) *
                  (t.gd[p + SW] + t.ghs[p + SW] - t.gd[p] - t.ghs[p]);
    if (PASS == kAllPass)
      r = r - fu - pgf;
    else
      r = -fu - pgf;
  }
  return r;
}

// Interior rows only (1..M-2); pole rows come from the zonal-sum cap.
template <typename T, int PASS>
__device__ inline T point_dgd(const MemberDev<T>& md, const TileSmem<T>& t, int j, int p) {
  if (PASS == kSlowPass) return T(0);  // src/dycore_mod.F90:297
  const int SW = t.SW;
  // src/dycore_mod.F90:546-552
  const T mdlon = ((t.ig[p] + t.ig[p + 1]) * t.iu[p] - (t.ig[p] + t.ig[p - 1]) * t.iu[p - 1]) *
                  T(0.5) / cf(md, CF_DLON, j);
  // src/dycore_mod.F90:564-570
  const T mdlat = ((t.ig[p] + t.ig[p + SW]) * t.iv[p] * ch(md, CH_COS, j) -
                   (t.ig[p] + t.ig[p - SW]) * t.iv[p - SW] * ch(md, CH_COS, j - 1)) *
                  T(0.5) / cf(md, CF_DLAT, j);
  return -mdlon - mdlat;
}

// ------------------------------------------------------- consumers

// Per-point consumer of one tendency value of field f at (row j, column i).
template <typename T>
struct Emit {
  const MemberDev<T>& md;
  const StageArgs& a;
  T h, s2;
  T ip1 = 0, ip2 = 0;
  __device__ Emit(const MemberDev<T>& m, const StageArgs& s, T h_) : md(m), a(s), h(h_), s2(T(s.scale2)) {}

  __device__ void put(int f, int j, int i, T val, T wcos) {
    const size_t o = (size_t)j * md.N + i;
    if (a.taccum >= 0) {
      // add_data(tend, accum_fast_tend), src/dycore_mod.F90:721
      T* acc = md.td[a.taccum][f];
      acc[o] = (a.accum_init ? T(0) : acc[o]) + val;
    }
    if (a.tadd >= 0) {
      // add_data / sub_data(slow_tend, tend), src/types_mod.F90:284-324
      const T sv = md.td[a.tadd][f][o];
      val = a.tadd_sign > 0 ? val + sv : val - sv;
    }
    if (a.tadd2 >= 0) val = val + md.td[a.tadd2][f][o] * s2;  // scale_data then add_data
    if (a.tout >= 0) md.td[a.tout][f][o] = val;
    if (a.out_slot >= 0) {
      // update_state, src/dycore_mod.F90:609-633 (new = old + dt * tend)
      md.st[a.out_slot][f][o] = md.st[a.base_slot][f][o] + h * val;
    }
    if (a.do_ip) {
      // inner_product_tend_tend / _tend_state, src/types_mod.F90:347-397
      const T pv = a.beta_mode == 0 ? md.td[a.tprev][f][o] : md.st[a.ip_slot][f][o];
      ip1 += pv * val * wcos;
      ip2 += val * val * wcos;
    }
  }
};

// Zonal filter of one row held in shared memory (src/filter_mod.F90:
// 105-167 with FFTPACK 5.1's packing, lib/fft/rfftf1.f:87-109 and
// lib/fft/rfftb1.f:43-59).  The kept coefficients (packed indices
// 0..keep-1: a0, (a_k, b_k) for k <= cutoff, and a_(cutoff+1)) are
// projected directly: forward sums by warps, reconstruction per point in
// packed-index order.
template <typename T>
__device__ void filter_project(const MemberDev<T>& md, T* x, int keep, T* coefs) {
  const int N = md.N;
  const T* ctab = md.twid;
  const T* stab = md.twid + N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  for (int p = warp; p < keep; p += nw) {
    T acc = 0;
    if (p == 0) {
      for (int n = lane; n < N; n += 32) acc += x[n];
    } else {
      const int k = (p + 1) >> 1;
      const T* tab = (p & 1) ? ctab : stab;
      for (int n = lane; n < N; n += 32) acc += x[n] * tab[(k * n) % N];
    }
    acc = warp_sum(acc);
    if (lane == 0) coefs[p] = acc * (p == 0 ? T(1.0) / T(N) : T(2.0) / T(N));
  }
  __syncthreads();
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    T y = 0;
    for (int p = 0; p < keep; ++p) {
      if (p == 0) {
        y = y + coefs[0];
      } else {
        const int k = (p + 1) >> 1;
        y = y + coefs[p] * ((p & 1) ? ctab : stab)[(k * n) % N];
      }
    }
    x[n] = y;
  }
  __syncthreads();
}

// The s1/s2-rescaled tendency filter of src/dycore_mod.F90:212-219.  With
// rtol > 0 (an extension; 0 is the reference) the rescale is skipped when
// s1 or s2 is zero to within rtol of the sum of the magnitudes of its terms.
template <typename T>
__device__ void filter_rescale(const MemberDev<T>& md, T* x, const T* __restrict__ w1,
                               const T* __restrict__ w2, int keep, T* coefs, T* red, double rtol) {
  const int N = md.N;
  T s = 0, sa = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const T t = x[i] * (w2 ? (w1[i] + w2[i]) : w1[i]);
    s += t;
    sa += fabs(t);
  }
  const T s1 = block_sum(s, red);
  const T a1 = rtol > 0 ? block_sum(sa, red) : T(0);
  if (!(fabs(s1) > T(1.0e-16))) return;  // src/filter_mod.F90:31
  filter_project(md, x, keep, coefs);
  s = 0;
  sa = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const T t = x[i] * (w2 ? (w1[i] + w2[i]) : w1[i]);
    s += t;
    sa += fabs(t);
  }
  const T s2 = block_sum(s, red);
  const T a2 = rtol > 0 ? block_sum(sa, red) : T(0);
  if (rtol > 0 && (fabs(s1) <= T(rtol) * a1 || fabs(s2) <= T(rtol) * a2)) return;
  for (int i = threadIdx.x; i < N; i += blockDim.x) x[i] = x[i] * s1 / s2;
  __syncthreads();
}

// Last block of a member to finish reduces that member's partials in a
// fixed order (deterministic), then re-arms the counter.
static __device__ bool last_block_of_member(unsigned* counters, int member, int nitems, unsigned* flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(&counters[member], 1u);
    *flag = (prev == (unsigned)(nitems - 1)) ? 1u : 0u;
  }
  __syncthreads();
  const bool last = *flag != 0;
  if (last) __threadfence();
  return last;
}

static __device__ void reduce_member_partials2(const double* partials, int b, int n, double* out,
                                        double* red) {
  for (int k = 0; k < 2; ++k) {
    double s = 0;
    for (int q = (int)threadIdx.x; q < n; q += blockDim.x) s += __ldcg(&partials[2 * (size_t)(b + q) + k]);
    out[k] = block_sum(s, red);
  }
}

// --------------------------------------------------------- stage kernel

template <typename T, int PASS, int ADV>
__global__ void __launch_bounds__(kThreads)
    stage_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl,
                 StageArgs a, int staging_words, int max_n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* staging = reinterpret_cast<T*>(smem_raw);
  T* rows = staging + staging_words;  // 3 * max_n (row tasks)
  T* coefs = rows + 3 * max_n;        // kMaxKeep
  T* redT = coefs + kMaxKeep;         // 32
  double* redD = reinterpret_cast<double*>(redT + 32);  // 32
  __shared__ unsigned last_flag;

  const WorkItem w = wl[blockIdx.x];
  const MemberDev<T>& md = mems[w.member];
  const int N = md.N, M = md.M, Mh = md.Mh;
  const T* gd_in = md.st[a.in_slot][F_GD];
  const T* iu_in = md.st[a.in_slot][F_IU];
  const T* iv_in = md.st[a.in_slot][F_IV];
  const double hstep = md.pcdt[PASS] * a.h_scale;
  Emit<T> em(md, a, T(hstep));
  const T ub_lon = T(a.ub_lon), ub_lat = T(a.ub_lat);

  if (w.kind == 0) {
    // ---------------- bulk tile: rows j0..j0+R-1 are ordinary rows
    TileSmem<T> t = carve_tile(staging, w.rows, w.cols, w.j0, w.i0);
    stage_tile(md, gd_in, iu_in, iv_in, t);
    const int npts = w.rows * w.cols;
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
      const int r = q / w.cols, c = q - r * w.cols;
      const int j = w.j0 + r, i = w.i0 + c;
      const int p = (r + 1) * t.SW + (c + 1);
      const T du = point_du<T, PASS, ADV>(md, t, j, p, ub_lon, ub_lat);
      const T dv = point_dv<T, PASS, ADV>(md, t, j, p, ub_lon, ub_lat);
      const T dg = point_dgd<T, PASS>(md, t, j, p);
      em.put(F_IU, j, i, du, cf(md, CF_COS, j));
      em.put(F_IV, j, i, dv, ch(md, CH_COS, j));
      em.put(F_GD, j, i, dg, cf(md, CF_COS, j));
    }
  } else {
    // ---------------- whole-row task: row index j (full row j, half row j)
    const int j = w.j0;
    const int info = md.rowinfo[j];
    const bool has_du = (j >= 1 && j <= M - 2);
    const bool has_dv = (j <= Mh - 1);
    const bool south = (j == 0), north = (j == M - 1);
    T* rdu = rows;
    T* rdv = rows + max_n;
    T* rdg = rows + 2 * max_n;
    double cap = 0;
    for (int c0 = 0; c0 < N; c0 += kRowChunk) {
      const int W = min(kRowChunk, N - c0);
      TileSmem<T> t = carve_tile(staging, 1, W, j, c0);
      __syncthreads();
      stage_tile(md, gd_in, iu_in, iv_in, t);
      for (int c = threadIdx.x; c < W; c += blockDim.x) {
        const int p = t.SW + (c + 1);
        const int i = c0 + c;
        rdu[i] = has_du ? point_du<T, PASS, ADV>(md, t, j, p, ub_lon, ub_lat) : T(0);
        rdv[i] = has_dv ? point_dv<T, PASS, ADV>(md, t, j, p, ub_lon, ub_lat) : T(0);
        if (south || north) {
          // src/dycore_mod.F90:572-596: sp += (ig(j)+ig(j+1)) iv(j);
          // np -= (ig(j)+ig(j-1)) iv(j-1).  Accumulated in FP64.
          if (PASS != kSlowPass) {
            if (south)
              cap += ((double)t.ig[p] + (double)t.ig[p + t.SW]) * (double)t.iv[p];
            else
              cap += ((double)t.ig[p] + (double)t.ig[p - t.SW]) * (double)t.iv[p - t.SW];
          }
          rdg[i] = T(0);
        } else {
          rdg[i] = point_dgd<T, PASS>(md, t, j, p);
        }
      }
    }
    __syncthreads();
    if ((south || north) && PASS != kSlowPass) {
      double s = block_sum(cap, redD);
      if (north) s = -s;
      s = s * 2.0 / N / kRadius / (kPi / Mh);
      // dgd = - mass_div_lon - mass_div_lat with mass_div_lon = 0 at poles
      const T val = T(-0.0) - T(s);
      for (int i = threadIdx.x; i < N; i += blockDim.x) rdg[i] = val;
      __syncthreads();
    }
    const size_t ro = (size_t)j * N;
    if (has_du && (info & RI_FLAG_FULL))
      filter_rescale(md, rdu, iu_in + ro, (const T*)nullptr, ri_keep_full(info), coefs, redT, a.rescale_rtol);
    if (has_dv && (info & RI_FLAG_HALF))
      filter_rescale(md, rdv, iv_in + ro, (const T*)nullptr, ri_keep_half(info), coefs, redT, a.rescale_rtol);
    if (PASS != kSlowPass && (info & RI_FLAG_FULL))
      filter_rescale(md, rdg, gd_in + ro, md.ghs + ro, ri_keep_full(info), coefs, redT, a.rescale_rtol);
    const T cj = cf(md, CF_COS, j);
    const T chj = has_dv ? ch(md, CH_COS, j) : T(0);
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      // du is 0 on pole rows (never assigned by the reference); inner
      // products skip pole-row du (src/types_mod.F90:355).
      if (has_du)
        em.put(F_IU, j, i, rdu[i], cj);
      else
        em.put(F_IU, j, i, T(0), T(0));
      if (has_dv) em.put(F_IV, j, i, rdv[i], chj);
      em.put(F_GD, j, i, rdg[i], cj);
    }
  }

  if (a.do_ip) {
    // Per-item partials, then the member's last block forms beta
    // (src/dycore_mod.F90:784-786; isp: :743-746).
    const double s1 = block_sum((double)em.ip1, redD);
    const double s2 = block_sum((double)em.ip2, redD);
    if (threadIdx.x == 0) {
      a.partials[2 * (size_t)w.pidx] = s1;
      a.partials[2 * (size_t)w.pidx + 1] = s2;
    }
    if (last_block_of_member(a.counters, w.member, md.pcount, &last_flag)) {
      double tot[2];
      reduce_member_partials2(a.partials, md.pbase, md.pcount, tot, redD);
      if (threadIdx.x == 0) {
        const double ip1 = tot[0], ip2 = tot[1];
        double beta = (a.qcon && ip1 != 0.0 && ip2 != 0.0) ? ip1 / ip2 : 1.0;
        if (a.beta_mode == 1) beta = beta * 4.0 / md.dt;
        a.beta[w.member] = beta;
        a.counters[w.member] = 0;
      }
    }
  }
}

// ------------------------------------------------------ final update
// update_state(time_step_size * beta, tend(new), state(old), state(new))
// (src/dycore_mod.F90:789-790) over every point of the member.  FP32 time
// levels carry a compensation word: new = (hi + lo) + dt*T via TwoSum.

template <typename T>
__device__ inline void final_point(const MemberDev<T>& md, const FinalArgs& a, int f, size_t o,
                                   double hstep) {
  const T tv = md.td[a.tslot][f][o];
  const T hi = md.st[a.base_slot][f][o];
  if (a.use_lo) {
    const T lo = md.lo[a.base_slot][f][o];
    const T y = lo + T(hstep) * tv;
    const T s = hi + y;
    const T bp = s - hi;
    const T err = (hi - (s - bp)) + (y - bp);
    md.st[a.out_slot][f][o] = s;
    md.lo[a.out_slot][f][o] = err;
  } else {
    md.st[a.out_slot][f][o] = hi + T(hstep) * tv;
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    final_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl,
                 FinalArgs a) {
  const WorkItem w = wl[blockIdx.x];
  const MemberDev<T>& md = mems[w.member];
  const int N = md.N, Mh = md.Mh;
  double hstep = md.pcdt[a.pass] * a.h_scale;
  if (a.beta) hstep = md.pcdt[a.pass] * a.h_scale * a.beta[w.member];
  if (w.kind == 0) {
    const int npts = w.rows * w.cols;
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
      const int r = q / w.cols, c = q - r * w.cols;
      const size_t o = (size_t)(w.j0 + r) * N + (w.i0 + c);
      final_point(md, a, F_GD, o, hstep);
      final_point(md, a, F_IU, o, hstep);
      final_point(md, a, F_IV, o, hstep);
    }
  } else {
    const int j = w.j0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      const size_t o = (size_t)j * N + i;
      final_point(md, a, F_GD, o, hstep);
      final_point(md, a, F_IU, o, hstep);
      if (j <= Mh - 1) final_point(md, a, F_IV, o, hstep);
    }
  }
}

// ------------------------------------------------------------- diag
// diag_run totals (src/diag_mod.F90:301-317, 98-121) in FP64.

template <typename T>
__device__ inline double val64(const MemberDev<T>& md, int slot, int f, size_t o) {
  double v = (double)md.st[slot][f][o];
  if (md.lo[slot][f]) v += (double)md.lo[slot][f][o];
  return v;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    diag_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl,
                DiagArgs a) {
  __shared__ double red[32];
  __shared__ unsigned last_flag;
  const WorkItem w = wl[blockIdx.x];
  const MemberDev<T>& md = mems[w.member];
  const int N = md.N, M = md.M, Mh = md.Mh;
  const double* dc = md.dcoef;
  double mass = 0, en = 0;
  auto point = [&](int j, int i, bool hv) {
    const size_t o = (size_t)j * N + i;
    const double g = val64(md, a.slot, F_GD, o);
    const double gh = (double)md.ghs[o];
    mass = mass + dc[j] * g;
    if (j >= 1 && j <= M - 2) {
      const double uu = val64(md, a.slot, F_IU, o);
      en = en + uu * uu * dc[M + j];
    }
    if (hv) {
      const double vv = val64(md, a.slot, F_IV, o);
      en = en + vv * vv * dc[2 * M + j];
    }
    const double hh = g + gh;
    en = en + hh * hh * dc[M + j];
  };
  if (w.kind == 0) {
    const int npts = w.rows * w.cols;
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
      const int r = q / w.cols, c = q - r * w.cols;
      point(w.j0 + r, w.i0 + c, true);
    }
  } else {
    for (int i = threadIdx.x; i < N; i += blockDim.x) point(w.j0, i, w.j0 <= Mh - 1);
  }
  const double sm = block_sum(mass, red);
  const double se = block_sum(en, red);
  if (threadIdx.x == 0) {
    a.partials[2 * (size_t)w.pidx] = sm;
    a.partials[2 * (size_t)w.pidx + 1] = se;
  }
  if (last_block_of_member(a.counters, w.member, md.pcount, &last_flag)) {
    double tot[2];
    reduce_member_partials2(a.partials, md.pbase, md.pcount, tot, red);
    if (threadIdx.x == 0) {
      const double total_mass = tot[0] * (kRadius * kRadius);
      const double total_energy = tot[1];
      a.diag[3 * w.member] = total_mass;
      a.diag[3 * w.member + 1] = total_energy;
      a.diag[3 * w.member + 2] = a.beta ? a.beta[w.member] : 1.0;
      const long long step = a.steps[w.member] + 1;
      a.steps[w.member] = step;
      if ((isnan(total_mass) || isnan(total_energy)) && a.nan_step[w.member] < 0)
        a.nan_step[w.member] = step;
      a.counters[w.member] = 0;
    }
  }
}

// -------------------------------------------------------- diffusion
// ordinary_diffusion with diffusion_order = 2 (src/diffusion_mod.F90:
// 74-217).  Pass 1 forms the Laplacians of gd, u, v (pole caps from zonal
// sums, the zonal filter without rescale on flagged rows) and writes
// gd' = gd + c gdd, u' = u + c ud, v' = v + c vd into slot SA; pass 2 is
// the iap_transform of (gd', u', v') back into the state slot.

template <typename T>
__device__ inline T lap_lon(const T* f, int p, T d) {
  return (f[p + 1] - T(2) * f[p] + f[p - 1]) / (d * d);
}

template <typename T>
__device__ inline T point_gdd_like(const MemberDev<T>& md, const TileSmem<T>& t, const T* f, int j,
                                   int p) {
  // src/diffusion_mod.F90:109-115 (and :135-143 for u)
  const int SW = t.SW;
  const T dl = cf(md, CF_DLAT, j);
  return lap_lon(f, p, cf(md, CF_DLON, j)) +
         ((f[p + SW] - f[p]) * ch(md, CH_COS, j) - (f[p] - f[p - SW]) * ch(md, CH_COS, j - 1)) /
             (dl * dl) * cf(md, CF_COS, j);
}

template <typename T>
__device__ inline T point_vd(const MemberDev<T>& md, const TileSmem<T>& t, int jh, int p) {
  // src/diffusion_mod.F90:145-171
  const int SW = t.SW, Mh = md.Mh;
  const T* v = t.v;
  T vd = lap_lon(v, p, ch(md, CH_DLON, jh));
  const T dl = ch(md, CH_DLAT, jh);
  if (jh >= 1 && jh <= Mh - 2) {
    vd = vd + ((v[p + SW] - v[p]) * cf(md, CF_COS, jh + 1) - (v[p] - v[p - SW]) * cf(md, CF_COS, jh)) /
                  (dl * dl) * ch(md, CH_COS, jh);
  } else if (jh == 0) {
    vd = vd + (v[p + SW] - v[p]) * cf(md, CF_COS, jh + 1) / (dl * dl) * ch(md, CH_COS, jh);
  } else {
    vd = vd - (v[p] - v[p - SW]) * cf(md, CF_COS, jh) / (dl * dl) * ch(md, CH_COS, jh);
  }
  return vd;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    diffusion_lap_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl,
                         int slot, double c, int staging_words, int max_n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* staging = reinterpret_cast<T*>(smem_raw);
  T* rows = staging + staging_words;
  T* coefs = rows + 3 * max_n;
  double* redD = reinterpret_cast<double*>(coefs + kMaxKeep + 32);
  const WorkItem w = wl[blockIdx.x];
  const MemberDev<T>& md = mems[w.member];
  const int N = md.N, M = md.M, Mh = md.Mh;
  const T* gd_in = md.st[slot][F_GD];
  T* go = md.st[SL_SA][F_GD];
  T* uo = md.st[SL_SA][F_IU];
  T* vo = md.st[SL_SA][F_IV];
  const T cc_ = T(c);
  if (w.kind == 0) {
    TileSmem<T> t = carve_tile(staging, w.rows, w.cols, w.j0, w.i0);
    stage_tile(md, gd_in, md.st[slot][F_IU], md.st[slot][F_IV], t, true);
    const int npts = w.rows * w.cols;
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
      const int r = q / w.cols, cl = q - r * w.cols;
      const int j = w.j0 + r, i = w.i0 + cl;
      const int p = (r + 1) * t.SW + (cl + 1);
      const size_t o = (size_t)j * N + i;
      go[o] = t.gd[p] + cc_ * point_gdd_like(md, t, t.gd, j, p);
      uo[o] = t.u[p] + cc_ * point_gdd_like(md, t, t.u, j, p);
      vo[o] = t.v[p] + cc_ * point_vd(md, t, j, p);
    }
  } else {
    const int j = w.j0;
    const int info = md.rowinfo[j];
    const bool has_u = (j >= 1 && j <= M - 2);
    const bool has_v = (j <= Mh - 1);
    const bool pole = (j == 0 || j == M - 1);
    T* rg = rows;
    T* ru = rows + max_n;
    T* rv = rows + 2 * max_n;
    T* rg0 = nullptr;
    double cap = 0;
    for (int c0 = 0; c0 < N; c0 += kRowChunk) {
      const int W = min(kRowChunk, N - c0);
      TileSmem<T> t = carve_tile(staging, 1, W, j, c0);
      __syncthreads();
      stage_tile(md, gd_in, md.st[slot][F_IU], md.st[slot][F_IV], t, true);
      for (int cl = threadIdx.x; cl < W; cl += blockDim.x) {
        const int p = t.SW + (cl + 1);
        const int i = c0 + cl;
        if (pole) {
          // sp = sp + gd(i,j+1) - gd(i,j); np = np - (gd(i,j) - gd(i,j-1))
          if (j == 0)
            cap += (double)t.gd[p + t.SW] - (double)t.gd[p];
          else
            cap -= (double)t.gd[p] - (double)t.gd[p - t.SW];
          rg[i] = T(0);
        } else {
          rg[i] = point_gdd_like(md, t, t.gd, j, p);
        }
        ru[i] = has_u ? point_gdd_like(md, t, t.u, j, p) : T(0);
        rv[i] = has_v ? point_vd(md, t, j, p) : T(0);
        // keep the state values of this row for the update below
        go[(size_t)j * N + i] = t.gd[p];
        uo[(size_t)j * N + i] = t.u[p];
        if (has_v) vo[(size_t)j * N + i] = t.v[p];
      }
    }
    __syncthreads();
    if (pole) {
      const double s = block_sum(cap, redD);
      const int jh = (j == 0) ? 0 : Mh - 1;
      const double dl = (double)cf(md, CF_DLAT, j);
      const double val = s * (double)ch(md, CH_COS, jh) / (dl * dl) * (double)cf(md, CF_COS, j) / N;
      for (int i = threadIdx.x; i < N; i += blockDim.x) rg[i] = T(val);
      __syncthreads();
    }
    (void)rg0;
    if (has_u && (info & RI_FLAG_FULL)) {
      filter_project(md, rg, ri_keep_full(info), coefs);
      filter_project(md, ru, ri_keep_full(info), coefs);
    }
    if (has_v && (info & RI_FLAG_HALF)) filter_project(md, rv, ri_keep_half(info), coefs);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      const size_t o = (size_t)j * N + i;
      go[o] = go[o] + cc_ * rg[i];
      uo[o] = uo[o] + cc_ * ru[i];
      if (has_v) vo[o] = vo[o] + cc_ * rv[i];
    }
  }
}

// iap_transform (src/types_mod.F90:399-426) of SA = (gd', u', v') into slot.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    diffusion_iap_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl,
                         int slot) {
  const WorkItem w = wl[blockIdx.x];
  const MemberDev<T>& md = mems[w.member];
  const int N = md.N, Mh = md.Mh;
  const T* g = md.st[SL_SA][F_GD];
  const T* u = md.st[SL_SA][F_IU];
  const T* v = md.st[SL_SA][F_IV];
  auto point = [&](int j, int i, bool hv) {
    const size_t o = (size_t)j * N + i;
    const int ip = (i + 1 == N) ? 0 : i + 1;
    const T ig = sqrt(g[o]);
    md.st[slot][F_GD][o] = g[o];
    md.st[slot][F_IU][o] = T(0.5) * (ig + sqrt(g[(size_t)j * N + ip])) * u[o];
    if (hv) md.st[slot][F_IV][o] = T(0.5) * (ig + sqrt(g[o + N])) * v[o];
    if (md.lo[slot][F_GD]) {
      md.lo[slot][F_GD][o] = T(0);
      md.lo[slot][F_IU][o] = T(0);
      if (hv) md.lo[slot][F_IV][o] = T(0);
    }
  };
  if (w.kind == 0) {
    const int npts = w.rows * w.cols;
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
      const int r = q / w.cols, c = q - r * w.cols;
      point(w.j0 + r, w.i0 + c, true);
    }
  } else {
    for (int i = threadIdx.x; i < N; i += blockDim.x) point(w.j0, i, w.j0 <= Mh - 1);
  }
}

// copy_data(state1, state2) (src/types_mod.F90:229-241) of the prognostic
// words, compensation included.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    copy_state_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl,
                      int from, int to) {
  const WorkItem w = wl[blockIdx.x];
  const MemberDev<T>& md = mems[w.member];
  const int N = md.N, Mh = md.Mh;
  auto point = [&](int j, int i, bool hv) {
    const size_t o = (size_t)j * N + i;
    for (int f = 0; f < 3; ++f) {
      if (f == F_IV && !hv) continue;
      md.st[to][f][o] = md.st[from][f][o];
      if (md.lo[to][f]) md.lo[to][f][o] = md.lo[from][f] ? md.lo[from][f][o] : T(0);
    }
  };
  if (w.kind == 0) {
    const int npts = w.rows * w.cols;
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
      const int r = q / w.cols, c = q - r * w.cols;
      point(w.j0 + r, w.i0 + c, true);
    }
  } else {
    for (int i = threadIdx.x; i < N; i += blockDim.x) point(w.j0, i, w.j0 <= Mh - 1);
  }
}

// --------------------------------------------------------- launchers

static inline int check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "gdc: kernel launch failed: %s\n", cudaGetErrorString(e));
    return GDC_E_CUDA;
  }
  return GDC_OK;
}

template <typename T>
size_t stage_smem_bytes(int tile_rows, int tile_cols, int max_n, int* staging_words) {
  const int bulk = 7 * (tile_rows + 3) * (tile_cols + 3);
  const int row = 7 * 4 * (kRowChunk + 3);
  // Rounded to 4 words and max_n to an even count so that the FP64
  // reduction buffer after the T arrays stays 8-byte aligned.
  const int sw = ((bulk > row ? bulk : row) + 3) & ~3;
  max_n = (max_n + 1) & ~1;
  if (staging_words) *staging_words = sw;
  return (size_t)(sw + 3 * max_n + kMaxKeep + 32) * sizeof(T) + 32 * sizeof(double) + 16;
}

template <typename T, int PASS, int ADV>
static int launch_stage_t(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int tile_rows,
                          int tile_cols, int max_n, const StageArgs& a, cudaStream_t s) {
  int sw = 0;
  max_n = (max_n + 1) & ~1;
  const size_t smem = stage_smem_bytes<T>(tile_rows, tile_cols, max_n, &sw);
  static size_t configured = 0;
  if (smem > configured) {
    if (cudaFuncSetAttribute(stage_kernel<T, PASS, ADV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return check_launch();
    configured = smem;
  }
  stage_kernel<T, PASS, ADV><<<nwork, kThreads, smem, s>>>(mem, wl, a, sw, max_n);
  return check_launch();
}

template <typename T>
int launch_stage(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int adv, int tile_rows,
                 int tile_cols, int max_n, const StageArgs& a, void* stream) {
  if (nwork <= 0) return GDC_OK;
  cudaStream_t s = (cudaStream_t)stream;
#define GDC_DISPATCH(P, A) \
  if (a.pass == P && adv == A) return launch_stage_t<T, P, A>(mem, wl, nwork, tile_rows, tile_cols, max_n, a, s);
  GDC_DISPATCH(kAllPass, GDC_ADV_CENTER_DIFF)
  GDC_DISPATCH(kFastPass, GDC_ADV_CENTER_DIFF)
  GDC_DISPATCH(kSlowPass, GDC_ADV_CENTER_DIFF)
  GDC_DISPATCH(kAllPass, GDC_ADV_UPWIND)
  GDC_DISPATCH(kFastPass, GDC_ADV_UPWIND)
  GDC_DISPATCH(kSlowPass, GDC_ADV_UPWIND)
#undef GDC_DISPATCH
  return GDC_E_CONFIG;
}

template <typename T>
int launch_final(const MemberDev<T>* mem, const WorkItem* wl, int nwork, const FinalArgs& a,
                 void* stream) {
  if (nwork <= 0) return GDC_OK;
  final_kernel<T><<<nwork, kThreads, 0, (cudaStream_t)stream>>>(mem, wl, a);
  return check_launch();
}

template <typename T>
int launch_diag(const MemberDev<T>* mem, const WorkItem* wl, int nwork, const DiagArgs& a,
                void* stream) {
  if (nwork <= 0) return GDC_OK;
  diag_kernel<T><<<nwork, kThreads, 0, (cudaStream_t)stream>>>(mem, wl, a);
  return check_launch();
}

template <typename T>
int launch_diffusion(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int tile_rows,
                     int tile_cols, int max_n, int slot, double sign_dt_coef, void* stream) {
  if (nwork <= 0) return GDC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int sw = 0;
  max_n = (max_n + 1) & ~1;
  const size_t smem = stage_smem_bytes<T>(tile_rows, tile_cols, max_n, &sw);
  static size_t configured = 0;
  if (smem > configured) {
    if (cudaFuncSetAttribute(diffusion_lap_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return check_launch();
    configured = smem;
  }
  diffusion_lap_kernel<T><<<nwork, kThreads, smem, s>>>(mem, wl, slot, sign_dt_coef, sw, max_n);
  int rc = check_launch();
  if (rc != GDC_OK) return rc;
  diffusion_iap_kernel<T><<<nwork, kThreads, 0, s>>>(mem, wl, slot);
  return check_launch();
}

template <typename T>
int launch_copy_state(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int from_slot,
                      int to_slot, void* stream) {
  if (nwork <= 0) return GDC_OK;
  copy_state_kernel<T><<<nwork, kThreads, 0, (cudaStream_t)stream>>>(mem, wl, from_slot, to_slot);
  return check_launch();
}

}  // namespace gdc
