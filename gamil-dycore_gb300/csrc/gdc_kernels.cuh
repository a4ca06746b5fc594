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
// A work item copies gd, ghs, iap u, iap v of its rows +-1 (+2 for gd) and
// columns +-1 (+2) into shared memory with cp.async (every load of the
// tile in flight at once; rows off the sphere are zero-filled, as the
// reference's never-filled latitude halo), derives iap gd = sqrt(gd),
// u = 2 iap_u / (iap_gd(i) + iap_gd(i+1)) and v = 2 iap_v / (iap_gd(j) +
// iap_gd(j+1)) there (the update_state epilogue of the reference,
// src/dycore_mod.F90:617-645, moved to the consumer so that only
// {gd, iap u, iap v} live in HBM), then evaluates the operators point-wise
// in the reference's order of operations.
//
// Sums: in FP64 every reduction the reference performs (filter s1/s2 and
// projections, pole caps, beta's inner products, the diagnostics) is
// accumulated in double-double and rounded once, i.e. it is the correctly
// rounded sum of the reference's (rounded) terms, independent of the order
// the GPU adds them in.
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

// Sum accumulator: double-double (Knuth TwoSum, exact without FMA) for
// FP64, plain float for FP32.
template <typename T>
struct Acc;
template <>
struct Acc<double> {
  double s = 0, c = 0;
  __device__ void add(double x) {
    const double t = s + x;
    const double bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
  }
  __device__ void merge(double os, double oc) {
    add(os);
    c += oc;
  }
  __device__ double value() const { return s + c; }
};
template <>
struct Acc<float> {
  float s = 0, c = 0;
  __device__ void add(float x) { s += x; }
  __device__ void merge(float os, float oc) { s += os + oc; }
  __device__ float value() const { return s + c; }
};

template <typename A>
__device__ inline A warp_sum(A v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Plain FP64 running sum (the FP32 path's diagnostics: FP64, but without
// the double-double cost -- FP64 arithmetic is the scarce unit).
struct PlainD {
  double s = 0, c = 0;
  __device__ void add(double x) { s += x; }
  __device__ void merge(double os, double oc) { s += os + oc; }
  __device__ double value() const { return s + c; }
};
template <typename T>
struct DiagAcc {
  using type = Acc<double>;
};
template <>
struct DiagAcc<float> {
  using type = PlainD;
};

template <typename A>
__device__ inline void warp_acc(A& a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const auto os = __shfl_xor_sync(0xffffffffu, a.s, o);
    const auto oc = __shfl_xor_sync(0xffffffffu, a.c, o);
    a.merge(os, oc);
  }
}

// Block-wide accumulation; `red` holds 64 values.  Every thread gets the
// result.
template <typename A, typename V>
__device__ A block_acc(A a, V* red) {
  warp_acc(a);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) {
    red[2 * w] = a.s;
    red[2 * w + 1] = a.c;
  }
  __syncthreads();
  if (w == 0) {
    A b;
    if (l < nw) {
      b.s = red[2 * l];
      b.c = red[2 * l + 1];
    }
    warp_acc(b);
    if (l == 0) {
      red[0] = b.s;
      red[1] = b.c;
    }
  }
  __syncthreads();
  A r;
  r.s = red[0];
  r.c = red[1];
  __syncthreads();
  return r;
}

template <typename A, typename V>
__device__ inline V block_value(A a, V* red) {
  return block_acc(a, red).value();
}

// 4- or 8-byte asynchronous global->shared copy; src-size 0 zero-fills.
template <typename T>
__device__ __forceinline__ void cp_async(T* smem, const T* gmem, bool valid) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  const int n = valid ? (int)sizeof(T) : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gmem), "n"(sizeof(T)),
               "r"(n)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename T>
__device__ inline T cf(const MemberDev<T>& md, int k, int j) {
  return md.coef[cf_off(k, md.M) + j];
}
template <typename T>
__device__ inline T ch(const MemberDev<T>& md, int k, int jh) {  // jh in -1..Mh
  return md.coef[ch_off(k, md.M) + jh + 1];
}

// Shared-memory tile of R x W output points with compile-time shape: rows
// j0-1 .. j0+R+1 and columns i0-1 .. i0+W+1 of gd, ghs, iap u, iap v, plus
// the derived iap gd, u and v.  Rows are padded so that column i0 starts on
// a 16-byte boundary (the row interiors are copied 16 bytes at a time).
// Partial tiles (the last row band of a run, the last column block of a
// row) stage only what their valid points use.  `cfull` / `chalf` hold the
// row coefficients of full rows j0-1..j0+R and half rows j0-1..j0+R.
template <typename T, int R_, int W_>
struct Tile {
  static constexpr int R = R_, W = W_;
  static constexpr int VEC = 16 / (int)sizeof(T);  // elements per 16-byte copy
  static constexpr int OFF = VEC - 1;              // so that column i0 is aligned
  static constexpr int SW = ((W_ + 3 + OFF + VEC - 1) / VEC) * VEC;
  static constexpr int ROWS = R_ + 3, NS = ROWS * SW;
  static constexpr int CR = R_ + 2;                // coefficient rows
  T *gd, *ghs, *iu, *iv, *ig, *u, *v;
  T *cfull, *chalf;
  int j0, i0, vrows, vcols;
  __device__ static int pos(int rr, int cc) { return rr * SW + cc + OFF; }
  __device__ T cf(int k, int j) const { return cfull[k * CR + (j - j0 + 1)]; }
  __device__ T ch(int k, int jh) const { return chalf[k * CR + (jh - j0 + 1)]; }
};

// Full-row coefficients a tile reads, and the half-row ones.
enum TileFull { TF_RADVLON, TF_RADVLAT, TF_F, TF_C, TF_C1, TF_C2, TF_DLON, TF_DLAT, TF_COS, TF_N };
enum TileHalf { TH_COS, TH_RADVLON, TH_RADVLAT, TH_DLAT, TH_DLON, TH_N };
__device__ __constant__ const int kTileFullSrc[TF_N] = {CF_RADVLON, CF_RADVLAT, CF_F, CF_C, CF_C1,
                                                        CF_C2, CF_DLON, CF_DLAT, CF_COS};
__device__ __constant__ const int kTileHalfSrc[TH_N] = {CH_COS, CH_RADVLON, CH_RADVLAT, CH_DLAT, CH_DLON};

template <typename T, int R, int W>
constexpr int tile_words() {
  return 7 * Tile<T, R, W>::NS + (TF_N + TH_N) * Tile<T, R, W>::CR;
}

template <typename T, int R, int W>
__device__ inline Tile<T, R, W> carve(T* base, int j0, int i0, int vrows, int vcols) {
  Tile<T, R, W> t;
  constexpr int n = Tile<T, R, W>::NS;
  t.gd = base;
  t.ghs = base + n;
  t.iu = base + 2 * n;
  t.iv = base + 3 * n;
  t.ig = base + 4 * n;
  t.u = base + 5 * n;
  t.v = base + 6 * n;
  t.cfull = base + 7 * n;
  t.chalf = t.cfull + TF_N * Tile<T, R, W>::CR;
  t.j0 = j0;
  t.i0 = i0;
  t.vrows = vrows;
  t.vcols = vcols;
  return t;
}

template <typename T>
__device__ __forceinline__ void cp_async16(T* smem, const T* gmem, bool valid) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}

// Issue the tile's copies (completed by cp_async_wait_all).  Positions off
// the sphere are zero-filled (the reference's never-filled latitude halo);
// positions beyond a partial tile's halo are not staged and never read
// (tile_derive masks them, the stencils stop at the halo).  With `given`, u and v
// are copied too (the level's u, v were supplied with its state).  The
// row interiors (columns i0 .. i0+vcols-1, never wrapping) go 16 bytes at a
// time; the halo columns i0-1, i0+vcols, i0+vcols+1 element by element.
// Requires num_lon and i0 to be multiples of VEC (checked at admission).
template <typename T, int R, int W>
__device__ void tile_issue(const MemberDev<T>& md, const T* __restrict__ gd, const T* __restrict__ iu,
                           const T* __restrict__ iv, Tile<T, R, W>& t, bool given = false) {
  using TL = Tile<T, R, W>;
  constexpr int VEC = TL::VEC, NCH = W / VEC;
  const int N = md.N, M = md.M, Mh = md.Mh;
  const int nfield = given ? 6 : 4;
  // interiors
  for (int q = threadIdx.x; q < TL::ROWS * NCH; q += kThreads) {
    const int rr = q / NCH, k = q - rr * NCH;
    const int j = t.j0 - 1 + rr;
    // Chunks past a partial tile are not issued at all: a zero-filling
    // copy there would overlap the halo columns written by other threads.
    if (rr > t.vrows + 2 || k * VEC >= t.vcols) continue;
    const bool vf = j >= 0 && j < M, vh = j >= 0 && j < Mh;
    const size_t o = vf ? (size_t)j * N + t.i0 + k * VEC : 0;
    const int dp = TL::pos(rr, 1 + k * VEC);
    cp_async16(&t.gd[dp], gd + o, vf);
    cp_async16(&t.ghs[dp], md.ghs + o, vf);
    cp_async16(&t.iu[dp], iu + o, vf);
    cp_async16(&t.iv[dp], iv + (vh ? o : 0), vh);
    if (given) {
      cp_async16(&t.u[dp], md.given_u + o, vf);
      cp_async16(&t.v[dp], md.given_v + (vh ? o : 0), vh);
    }
  }
  // halo columns
  for (int q = threadIdx.x; q < TL::ROWS * 3; q += kThreads) {
    const int rr = q / 3, h = q - rr * 3;
    const int cc = h == 0 ? 0 : t.vcols + h;
    const int j = t.j0 - 1 + rr;
    int i = t.i0 - 1 + cc;
    i = i < 0 ? i + N : (i >= N ? i - N : i);
    if (rr > t.vrows + 2) continue;
    const bool vf = j >= 0 && j < M, vh = j >= 0 && j < Mh;
    const size_t o = vf ? (size_t)j * N + i : 0;
    const int dp = TL::pos(rr, cc);
    cp_async(&t.gd[dp], gd + o, vf);
    cp_async(&t.ghs[dp], md.ghs + o, vf);
    cp_async(&t.iu[dp], iu + o, vf);
    cp_async(&t.iv[dp], iv + (vh ? o : 0), vh);
    if (given) {
      cp_async(&t.u[dp], md.given_u + o, vf);
      cp_async(&t.v[dp], md.given_v + (vh ? o : 0), vh);
    }
  }
  (void)nfield;
  // row coefficients of full rows j0-1..j0+R and half rows j0-1..j0+R
  for (int q = threadIdx.x; q < (TF_N + TH_N) * TL::CR; q += kThreads) {
    const int k = q / TL::CR, lr = q - k * TL::CR;
    const int j = t.j0 - 1 + lr;
    T val = T(0);
    if (k < TF_N) {
      if (j >= 0 && j < M) val = md.coef[cf_off(kTileFullSrc[k], M) + j];
    } else if (j >= -1 && j <= Mh) {
      val = md.coef[ch_off(kTileHalfSrc[k - TF_N], M) + j + 1];
    }
    t.cfull[q] = val;  // cfull and chalf are contiguous
  }
}

// After the copies: iap gd, then u on full rows j0..j0+R (local 1..R+1;
// from local 0 when the stencil also needs row j0-1), v on half rows
// j0-1..j0+R (local 0..R+1), columns i0-1..i0+W (local 0..W+1).
template <typename T, int R, int W>
__device__ void tile_derive(const MemberDev<T>& md, Tile<T, R, W>& t, bool u_halo_row = false,
                            bool given = false) {
  using TL = Tile<T, R, W>;
  const int M = md.M, Mh = md.Mh;
  cp_async_wait_all();
  __syncthreads();
  for (int p = threadIdx.x; p < TL::NS; p += kThreads) t.ig[p] = sqrt(t.gd[p]);
  __syncthreads();
  if (given) return;
  const int urow0 = u_halo_row ? 0 : 1;
  constexpr int DW = W + 2, ND = (R + 2) * (W + 2);
  for (int q = threadIdx.x; q < ND; q += kThreads) {
    const int rr = q / DW, cc = q - rr * DW;
    const int p = TL::pos(rr, cc);
    const int j = t.j0 - 1 + rr;
    const bool need = rr <= t.vrows + 1 && cc <= t.vcols + 1;
    T uu = 0, vv = 0;
    if (need && rr >= urow0 && j >= 1 && j <= M - 2) uu = t.iu[p] * T(2) / (t.ig[p] + t.ig[p + 1]);
    if (need && j >= 0 && j < Mh) vv = t.iv[p] * T(2) / (t.ig[p] + t.ig[p + TL::SW]);
    t.u[p] = uu;
    t.v[p] = vv;
  }
  __syncthreads();
}

// Member descriptor copied to shared memory once per block.
template <typename T>
__device__ inline void load_member(const MemberDev<T>* __restrict__ mems, int member, MemberDev<T>* smd) {
  const unsigned* src = reinterpret_cast<const unsigned*>(mems + member);
  unsigned* dst = reinterpret_cast<unsigned*>(smd);
  constexpr int nw = sizeof(MemberDev<T>) / 4;
  for (int k = threadIdx.x; k < nw; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
}

// ----------------------------------------------------- point operators
// p is the local position of full row j / half row j, column i.

template <typename T, int PASS, int ADV, class TL>
__device__ inline T point_du(const MemberDev<T>& md, const TL& t, int j, int p, T beta_lon,
                             T beta_lat) {
  constexpr int SW = TL::SW;
  T r = 0;
  if (PASS != kFastPass) {
    // src/dycore_mod.F90:376-392 / :393-415
    const T uc = t.u[p], um = t.u[p - 1], up = t.u[p + 1];
    const T u1 = uc + um, u2 = uc + up;
    T adv_lon;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lon = t.cf(TF_RADVLON, j) * (u2 * t.iu[p + 1] - u1 * t.iu[p - 1]);
    } else {
      const T ic = t.iu[p], ip = t.iu[p + 1], im = t.iu[p - 1];
      adv_lon = t.cf(TF_RADVLON, j) * (u2 * (ic + ip) - beta_lon * fabs(u2) * (ip - ic) - u1 * (ic + im) +
                                         beta_lon * fabs(u1) * (ic - im) - (u2 - u1) * ic);
    }
    // src/dycore_mod.F90:433-439 / :450-459
    const T v1 = (t.v[p - SW] + t.v[p - SW + 1]) * t.ch(TH_COS, j - 1);
    const T v2 = (t.v[p] + t.v[p + 1]) * t.ch(TH_COS, j);
    T adv_lat;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lat = t.cf(TF_RADVLAT, j) * (v2 * t.iu[p + SW] - v1 * t.iu[p - SW]);
    } else {
      const T ic = t.iu[p], ip = t.iu[p + SW], im = t.iu[p - SW];
      adv_lat = t.cf(TF_RADVLAT, j) * (v2 * (ic + ip) - beta_lat * fabs(v2) * (ip - ic) - v1 * (ic + im) +
                                         beta_lat * fabs(v1) * (ic - im) - (v2 - v1) * ic);
    }
    r = -adv_lon - adv_lat;
  }
  if (PASS != kSlowPass) {
    // src/dycore_mod.F90:485-493
    const T fv = T(0.25) * (t.cf(TF_F, j) + t.cf(TF_C, j) * t.u[p]) *
                 (t.cf(TF_C1, j) * (t.iv[p - SW] + t.iv[p - SW + 1]) + t.cf(TF_C2, j) * (t.iv[p] + t.iv[p + 1]));
    // src/dycore_mod.F90:514-519
    const T pgf = T(0.5) * (t.ig[p] + t.ig[p + 1]) / t.cf(TF_DLON, j) *
                  (t.gd[p + 1] + t.ghs[p + 1] - t.gd[p] - t.ghs[p]);
    if (PASS == kAllPass)
      r = r + fv - pgf;
    else
      r = fv - pgf;
  }
  return r;
}

template <typename T, int PASS, int ADV, class TL>
__device__ inline T point_dv(const MemberDev<T>& md, const TL& t, int jh, int p, T beta_lon,
                             T beta_lat) {
  constexpr int SW = TL::SW;
  T r = 0;
  if (PASS != kFastPass) {
    // src/dycore_mod.F90:386-391 / :406-414
    const T u1 = t.u[p - 1] + t.u[p + SW - 1];
    const T u2 = t.u[p] + t.u[p + SW];
    T adv_lon;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lon = t.ch(TH_RADVLON, jh) * (u2 * t.iv[p + 1] - u1 * t.iv[p - 1]);
    } else {
      const T ic = t.iv[p], ip = t.iv[p + 1], im = t.iv[p - 1];
      adv_lon = t.ch(TH_RADVLON, jh) * (u2 * (ic + ip) - beta_lon * fabs(u2) * (ip - ic) - u1 * (ic + im) +
                                          beta_lon * fabs(u1) * (ic - im) - (u2 - u1) * ic);
    }
    // src/dycore_mod.F90:441-446 / :461-469
    const T vc = t.v[p] * t.ch(TH_COS, jh);
    const T v1 = vc + t.v[p - SW] * t.ch(TH_COS, jh - 1);
    const T v2 = vc + t.v[p + SW] * t.ch(TH_COS, jh + 1);
    T adv_lat;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lat = t.ch(TH_RADVLAT, jh) * (v2 * t.iv[p + SW] - v1 * t.iv[p - SW]);
    } else {
      const T ic = t.iv[p], ip = t.iv[p + SW], im = t.iv[p - SW];
      adv_lat = t.ch(TH_RADVLAT, jh) * (v2 * (ic + ip) - beta_lat * fabs(v2) * (ip - ic) - v1 * (ic + im) +
                                          beta_lat * fabs(v1) * (ic - im) - (v2 - v1) * ic);
    }
    r = -adv_lon - adv_lat;
  }
  if (PASS != kSlowPass) {
    // src/dycore_mod.F90:495-503
    const T f0 = t.cf(TF_F, jh), c0 = t.cf(TF_C, jh);
    const T f1 = t.cf(TF_F, jh + 1), c1 = t.cf(TF_C, jh + 1);
    const T fu = T(0.25) * ((f0 + c0 * t.u[p]) * t.iu[p] + (f0 + c0 * t.u[p - 1]) * t.iu[p - 1] +
                            (f1 + c1 * t.u[p + SW]) * t.iu[p + SW] + (f1 + c1 * t.u[p + SW - 1]) * t.iu[p + SW - 1]);
    // src/dycore_mod.F90:530-535
    const T pgf = T(0.5) * (t.ig[p] + t.ig[p + SW]) / t.ch(TH_DLAT, jh) * t.ch(TH_COS, jh) *
                  (t.gd[p + SW] + t.ghs[p + SW] - t.gd[p] - t.ghs[p]);
    if (PASS == kAllPass)
      r = r - fu - pgf;
    else
      r = -fu - pgf;
  }
  return r;
}

// Interior rows only (1..M-2); pole rows come from the zonal-sum cap.
template <typename T, int PASS, class TL>
__device__ inline T point_dgd(const MemberDev<T>& md, const TL& t, int j, int p) {
  if (PASS == kSlowPass) return T(0);  // src/dycore_mod.F90:297
  constexpr int SW = TL::SW;
  // src/dycore_mod.F90:546-552
  const T mdlon = ((t.ig[p] + t.ig[p + 1]) * t.iu[p] - (t.ig[p] + t.ig[p - 1]) * t.iu[p - 1]) * T(0.5) /
                  t.cf(TF_DLON, j);
  // src/dycore_mod.F90:564-570
  const T mdlat = ((t.ig[p] + t.ig[p + SW]) * t.iv[p] * t.ch(TH_COS, j) -
                   (t.ig[p] + t.ig[p - SW]) * t.iv[p - SW] * t.ch(TH_COS, j - 1)) *
                  T(0.5) / t.cf(TF_DLAT, j);
  return -mdlon - mdlat;
}

// ------------------------------------------------------- consumers

// Consumer of one tendency value of field f at offset o.  `base` and
// `prev` are the update operand and the previous tendency, supplied by the
// caller (prefetched for bulk tiles).
template <typename T>
struct Emit {
  const MemberDev<T>& md;
  const StageArgs& a;
  T h, s2;
  Acc<T> ip1, ip2;
  __device__ Emit(const MemberDev<T>& m, const StageArgs& s, T h_) : md(m), a(s), h(h_), s2(T(s.scale2)) {}

  __device__ void put(int f, size_t o, T val, T wcos, T base, T prev) {
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
    // update_state, src/dycore_mod.F90:609-633 (new = old + dt * tend)
    if (a.out_slot >= 0) md.st[a.out_slot][f][o] = base + h * val;
    if (a.do_ip) {
      // inner_product_tend_tend / _tend_state, src/types_mod.F90:347-397
      ip1.add(prev * val * wcos);
      ip2.add(val * val * wcos);
    }
  }
  // Operands read straight from global memory (row tasks, isp modes).
  __device__ T base_of(int f, size_t o) const { return a.out_slot >= 0 ? md.st[a.base_slot][f][o] : T(0); }
  __device__ T prev_of(int f, size_t o) const {
    if (!a.do_ip) return T(0);
    return a.beta_mode == 0 ? md.td[a.tprev][f][o] : md.st[a.ip_slot][f][o];
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
    Acc<T> acc;
    if (p == 0) {
      for (int n = lane; n < N; n += 32) acc.add(x[n]);
    } else {
      const int k = (p + 1) >> 1;
      const T* tab = (p & 1) ? ctab : stab;
      for (int n = lane; n < N; n += 32) acc.add(x[n] * tab[(k * n) % N]);
    }
    warp_acc(acc);
    if (lane == 0) coefs[p] = acc.value() * (p == 0 ? T(1.0) / T(N) : T(2.0) / T(N));
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
__device__ void filter_rescale(const MemberDev<T>& md, T* x, const T* __restrict__ w1, const T* __restrict__ w2,
                               int keep, T* coefs, T* red, double rtol) {
  const int N = md.N;
  Acc<T> s, sa;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const T t = x[i] * (w2 ? (w1[i] + w2[i]) : w1[i]);
    s.add(t);
    sa.add(fabs(t));
  }
  const T s1 = block_value(s, red);
  const T a1 = rtol > 0 ? block_value(sa, red) : T(0);
  if (!(fabs(s1) > T(1.0e-16))) return;  // src/filter_mod.F90:31
  filter_project(md, x, keep, coefs);
  Acc<T> q, qa;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const T t = x[i] * (w2 ? (w1[i] + w2[i]) : w1[i]);
    q.add(t);
    qa.add(fabs(t));
  }
  const T s2 = block_value(q, red);
  const T a2 = rtol > 0 ? block_value(qa, red) : T(0);
  if (rtol > 0 && (fabs(s1) <= T(rtol) * a1 || fabs(s2) <= T(rtol) * a2)) return;
  for (int i = threadIdx.x; i < N; i += blockDim.x) x[i] = x[i] * s1 / s2;
  __syncthreads();
}

// --------------------------------------------------------- stage kernel

template <typename T>
struct StageOcc {
  static constexpr int kMinBlocks = sizeof(T) == 4 ? 4 : 2;
};

template <typename T, int PASS, int ADV, int R, int W>
__global__ void __launch_bounds__(kThreads, StageOcc<T>::kMinBlocks)
    stage_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl, StageArgs a,
                 int staging_words, int max_n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* staging = reinterpret_cast<T*>(smem_raw);
  T* rows = staging + staging_words;  // 3 * max_n (row tasks)
  T* coefs = rows + 3 * max_n;        // kMaxKeep
  T* redT = coefs + kMaxKeep;         // 64
  __shared__ MemberDev<T> smd;

  const WorkItem w = wl[blockIdx.x];
  load_member(mems, w.member, &smd);
  const MemberDev<T>& md = smd;
  const int N = md.N, M = md.M, Mh = md.Mh;
  const T* gd_in = md.st[a.in_slot][F_GD];
  const T* iu_in = md.st[a.in_slot][F_IU];
  const T* iv_in = md.st[a.in_slot][F_IV];
  const double hstep = md.pcdt[PASS] * a.h_scale;
  Emit<T> em(md, a, T(hstep));
  const T ub_lon = T(a.ub_lon), ub_lat = T(a.ub_lat);
  const bool plain_ops = a.taccum < 0 && a.tadd < 0 && a.tadd2 < 0;
  // u, v supplied with this level (initial condition, diffusion): used as
  // given, as the reference's space_operators reads state%u / state%v.
  const bool given = a.uvslot && a.uvslot[w.member] == a.in_slot;
  if (a.uvslot && a.out_slot >= 0 && threadIdx.x == 0 && a.uvslot[w.member] == a.out_slot)
    a.uvslot[w.member] = -1;  // level overwritten: u, v derived from now on

  if (w.kind == 0) {
    // ---------------- bulk tile: rows j0..j0+R-1 are ordinary rows
    using TL = Tile<T, R, W>;
    constexpr int PPT = (R * W + kThreads - 1) / kThreads;
    TL t = carve<T, R, W>(staging, w.j0, w.i0, w.rows, w.cols);
    tile_issue(md, gd_in, iu_in, iv_in, t, given);
    // While the tile is in flight, fetch the per-point update operands.
    const bool base_in_tile = a.out_slot >= 0 && a.base_slot == a.in_slot;
    T pre_b[PPT][3], pre_p[PPT][3];
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      const int q = threadIdx.x + k * kThreads;
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        pre_b[k][f] = T(0);
        pre_p[k][f] = T(0);
      }
      const int r = q / W, c = q - r * W;
      if (q < R * W && r < w.rows && c < w.cols) {
        const size_t o = (size_t)(w.j0 + r) * N + (w.i0 + c);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
          if (a.out_slot >= 0 && !base_in_tile) pre_b[k][f] = md.st[a.base_slot][f][o];
          if (a.do_ip) pre_p[k][f] = a.beta_mode == 0 ? md.td[a.tprev][f][o] : md.st[a.ip_slot][f][o];
        }
      }
    }
    tile_derive(md, t, false, given);
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      const int q = threadIdx.x + k * kThreads;
      const int r = q / W, c = q - r * W;
      if (q >= R * W || r >= w.rows || c >= w.cols) continue;
      const int j = w.j0 + r, i = w.i0 + c;
      const int p = TL::pos(r + 1, c + 1);
      const size_t o = (size_t)j * N + i;
      if (base_in_tile) {
        pre_b[k][F_GD] = t.gd[p];
        pre_b[k][F_IU] = t.iu[p];
        pre_b[k][F_IV] = t.iv[p];
      }
      const T du = point_du<T, PASS, ADV>(md, t, j, p, ub_lon, ub_lat);
      const T dv = point_dv<T, PASS, ADV>(md, t, j, p, ub_lon, ub_lat);
      const T dg = point_dgd<T, PASS>(md, t, j, p);
      if (plain_ops) {
        em.put(F_IU, o, du, t.cf(TF_COS, j), pre_b[k][F_IU], pre_p[k][F_IU]);
        em.put(F_IV, o, dv, t.ch(TH_COS, j), pre_b[k][F_IV], pre_p[k][F_IV]);
        em.put(F_GD, o, dg, t.cf(TF_COS, j), pre_b[k][F_GD], pre_p[k][F_GD]);
      } else {
        em.put(F_IU, o, du, t.cf(TF_COS, j), em.base_of(F_IU, o), em.prev_of(F_IU, o));
        em.put(F_IV, o, dv, t.ch(TH_COS, j), em.base_of(F_IV, o), em.prev_of(F_IV, o));
        em.put(F_GD, o, dg, t.cf(TF_COS, j), em.base_of(F_GD, o), em.prev_of(F_GD, o));
      }
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
    Acc<double> cap;
    using TR = Tile<T, 1, kRowChunk>;
    for (int c0 = 0; c0 < N; c0 += kRowChunk) {
      const int vw = min(kRowChunk, N - c0);
      TR t = carve<T, 1, kRowChunk>(staging, j, c0, 1, vw);
      __syncthreads();
      tile_issue(md, gd_in, iu_in, iv_in, t, given);
      tile_derive(md, t, false, given);
      for (int c = threadIdx.x; c < vw; c += blockDim.x) {
        const int p = TR::pos(1, c + 1);
        const int i = c0 + c;
        rdu[i] = has_du ? point_du<T, PASS, ADV>(md, t, j, p, ub_lon, ub_lat) : T(0);
        rdv[i] = has_dv ? point_dv<T, PASS, ADV>(md, t, j, p, ub_lon, ub_lat) : T(0);
        if (south || north) {
          // src/dycore_mod.F90:572-596: sp += (ig(j)+ig(j+1)) iv(j);
          // np -= (ig(j)+ig(j-1)) iv(j-1).  Terms and sum in FP64.
          if (PASS != kSlowPass) {
            if (south)
              cap.add(((double)t.ig[p] + (double)t.ig[p + TR::SW]) * (double)t.iv[p]);
            else
              cap.add(((double)t.ig[p] + (double)t.ig[p - TR::SW]) * (double)t.iv[p - TR::SW]);
          }
          rdg[i] = T(0);
        } else {
          rdg[i] = point_dgd<T, PASS>(md, t, j, p);
        }
      }
    }
    __syncthreads();
    if ((south || north) && PASS != kSlowPass) {
      double* redD = reinterpret_cast<double*>(redT + 64);
      double s = block_value(cap, redD);
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
      const size_t o = ro + i;
      // du is 0 on pole rows (never assigned by the reference); inner
      // products skip pole-row du (src/types_mod.F90:355).
      if (has_du)
        em.put(F_IU, o, rdu[i], cj, em.base_of(F_IU, o), em.prev_of(F_IU, o));
      else
        em.put(F_IU, o, T(0), T(0), em.base_of(F_IU, o), T(0));
      if (has_dv) em.put(F_IV, o, rdv[i], chj, em.base_of(F_IV, o), em.prev_of(F_IV, o));
      em.put(F_GD, o, rdg[i], cj, em.base_of(F_GD, o), em.prev_of(F_GD, o));
    }
  }

  if (a.do_ip) {
    // Per-item partials of the inner products (src/dycore_mod.F90:784-785;
    // isp :743-744); beta_kernel reduces them per member.  FP64 reduces in
    // double-double, FP32 in FP32 (FP64 arithmetic is the scarce unit).
    const Acc<T> s1 = block_acc(em.ip1, redT);
    const Acc<T> s2 = block_acc(em.ip2, redT);
    if (threadIdx.x == 0) {
      double* pp = a.partials + 4 * (size_t)w.pidx;
      pp[0] = (double)s1.s;
      pp[1] = (double)s1.c;
      pp[2] = (double)s2.s;
      pp[3] = (double)s2.c;
    }
  }
}

// beta of predict_correct (src/dycore_mod.F90:784-786) or isp (:743-746),
// one block per member over that member's partials.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    beta_kernel(const MemberDev<T>* __restrict__ mems, const int* __restrict__ slots, const double* partials,
                double* beta, int qcon, int beta_mode) {
  __shared__ double red[64];
  const int s = slots[blockIdx.x];
  const MemberDev<T>& md = mems[s];
  Acc<double> a1, a2;
  for (int q = threadIdx.x; q < md.pcount; q += blockDim.x) {
    const double* pp = partials + 4 * (size_t)(md.pbase + q);
    a1.merge(pp[0], pp[1]);
    a2.merge(pp[2], pp[3]);
  }
  const double ip1 = block_value(a1, red);
  const double ip2 = block_value(a2, red);
  if (threadIdx.x == 0) {
    double b = (qcon && ip1 != 0.0 && ip2 != 0.0) ? ip1 / ip2 : 1.0;
    if (beta_mode == 1) b = b * 4.0 / md.dt;
    beta[s] = b;
  }
}

// ------------------------------------------------------ final update
// update_state(time_step_size * beta, tend(new), state(old), state(new))
// (src/dycore_mod.F90:789-790) over every point of the member.  FP32 time
// levels carry a compensation word: new = (hi + lo) + dt*T via TwoSum.

template <typename T>
__device__ inline void final_point(const MemberDev<T>& md, const FinalArgs& a, int f, size_t o, double hstep) {
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
    final_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl, FinalArgs a) {
  __shared__ MemberDev<T> smd;
  const WorkItem w = wl[blockIdx.x];
  load_member(mems, w.member, &smd);
  const MemberDev<T>& md = smd;
  const int N = md.N, Mh = md.Mh;
  double hstep = md.pcdt[a.pass] * a.h_scale;
  if (a.beta) hstep = md.pcdt[a.pass] * a.h_scale * a.beta[w.member];
  // This level's u, v are derived from its new state from now on.
  if (a.uvslot && threadIdx.x == 0 && a.uvslot[w.member] == a.out_slot) a.uvslot[w.member] = -1;
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
    diag_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl, DiagArgs a) {
  __shared__ double red[64];
  __shared__ MemberDev<T> smd;
  const WorkItem w = wl[blockIdx.x];
  load_member(mems, w.member, &smd);
  const MemberDev<T>& md = smd;
  const int N = md.N, M = md.M, Mh = md.Mh;
  const double* dc = md.dcoef;
  typename DiagAcc<T>::type mass, en;
  auto point = [&](int j, int i, bool hv) {
    const size_t o = (size_t)j * N + i;
    const double g = val64(md, a.slot, F_GD, o);
    const double gh = (double)md.ghs[o];
    mass.add(dc[j] * g);
    if (j >= 1 && j <= M - 2) {
      const double uu = val64(md, a.slot, F_IU, o);
      en.add(uu * uu * dc[M + j]);
    }
    if (hv) {
      const double vv = val64(md, a.slot, F_IV, o);
      en.add(vv * vv * dc[2 * M + j]);
    }
    const double hh = g + gh;
    en.add(hh * hh * dc[M + j]);
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
  const auto sm = block_acc(mass, red);
  const auto se = block_acc(en, red);
  if (threadIdx.x == 0) {
    double* pp = a.partials + 4 * (size_t)w.pidx;
    pp[0] = sm.s;
    pp[1] = sm.c;
    pp[2] = se.s;
    pp[3] = se.c;
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    diag_finalize_kernel(const MemberDev<T>* __restrict__ mems, const int* __restrict__ slots, DiagArgs a) {
  __shared__ double red[64];
  const int s = slots[blockIdx.x];
  const MemberDev<T>& md = mems[s];
  Acc<double> m, e;
  for (int q = threadIdx.x; q < md.pcount; q += blockDim.x) {
    const double* pp = a.partials + 4 * (size_t)(md.pbase + q);
    m.merge(pp[0], pp[1]);
    e.merge(pp[2], pp[3]);
  }
  const double tm = block_value(m, red);
  const double te = block_value(e, red);
  if (threadIdx.x == 0) {
    const double total_mass = tm * (kRadius * kRadius);
    a.diag[3 * s] = total_mass;
    a.diag[3 * s + 1] = te;
    a.diag[3 * s + 2] = a.beta ? a.beta[s] : 1.0;
    const long long step = a.steps[s] + (a.count_step ? 1 : 0);
    a.steps[s] = step;
    if ((isnan(total_mass) || isnan(te)) && a.nan_step[s] < 0) a.nan_step[s] = step;
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

template <typename T, class TL>
__device__ inline T point_gdd_like(const MemberDev<T>& md, const TL& t, const T* f, int j, int p) {
  // src/diffusion_mod.F90:109-115 (and :135-143 for u)
  constexpr int SW = TL::SW;
  const T dl = t.cf(TF_DLAT, j);
  return lap_lon(f, p, t.cf(TF_DLON, j)) +
         ((f[p + SW] - f[p]) * t.ch(TH_COS, j) - (f[p] - f[p - SW]) * t.ch(TH_COS, j - 1)) / (dl * dl) *
             t.cf(TF_COS, j);
}

template <typename T, class TL>
__device__ inline T point_vd(const MemberDev<T>& md, const TL& t, int jh, int p) {
  // src/diffusion_mod.F90:145-171
  constexpr int SW = TL::SW;
  const int Mh = md.Mh;
  const T* v = t.v;
  T vd = lap_lon(v, p, t.ch(TH_DLON, jh));
  const T dl = t.ch(TH_DLAT, jh);
  if (jh >= 1 && jh <= Mh - 2) {
    vd = vd + ((v[p + SW] - v[p]) * t.cf(TF_COS, jh + 1) - (v[p] - v[p - SW]) * t.cf(TF_COS, jh)) / (dl * dl) *
                  t.ch(TH_COS, jh);
  } else if (jh == 0) {
    vd = vd + (v[p + SW] - v[p]) * t.cf(TF_COS, jh + 1) / (dl * dl) * t.ch(TH_COS, jh);
  } else {
    vd = vd - (v[p] - v[p - SW]) * t.cf(TF_COS, jh) / (dl * dl) * t.ch(TH_COS, jh);
  }
  return vd;
}

template <typename T, int R, int W>
__global__ void __launch_bounds__(kThreads)
    diffusion_lap_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl, int slot, double c,
                         int staging_words, int max_n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* staging = reinterpret_cast<T*>(smem_raw);
  T* rows = staging + staging_words;
  T* coefs = rows + 3 * max_n;
  T* redT = coefs + kMaxKeep;
  double* redD = reinterpret_cast<double*>(redT + 64);
  __shared__ MemberDev<T> smd;
  const WorkItem w = wl[blockIdx.x];
  load_member(mems, w.member, &smd);
  const MemberDev<T>& md = smd;
  const int N = md.N, M = md.M, Mh = md.Mh;
  const T* gd_in = md.st[slot][F_GD];
  T* go = md.st[SL_SA][F_GD];
  T* uo = md.st[SL_SA][F_IU];
  T* vo = md.st[SL_SA][F_IV];
  const T cc_ = T(c);
  if (w.kind == 0) {
    using TL = Tile<T, R, W>;
    TL t = carve<T, R, W>(staging, w.j0, w.i0, w.rows, w.cols);
    tile_issue(md, gd_in, md.st[slot][F_IU], md.st[slot][F_IV], t);
    tile_derive(md, t, true);
    const int npts = w.rows * w.cols;
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
      const int r = q / w.cols, cl = q - r * w.cols;
      const int j = w.j0 + r, i = w.i0 + cl;
      const int p = TL::pos(r + 1, cl + 1);
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
    Acc<double> cap;
    using TR = Tile<T, 1, kRowChunk>;
    for (int c0 = 0; c0 < N; c0 += kRowChunk) {
      const int vw = min(kRowChunk, N - c0);
      TR t = carve<T, 1, kRowChunk>(staging, j, c0, 1, vw);
      __syncthreads();
      tile_issue(md, gd_in, md.st[slot][F_IU], md.st[slot][F_IV], t);
      tile_derive(md, t, true);
      for (int cl = threadIdx.x; cl < vw; cl += blockDim.x) {
        const int p = TR::pos(1, cl + 1);
        const int i = c0 + cl;
        if (pole) {
          // sp = sp + gd(i,j+1) - gd(i,j); np = np - (gd(i,j) - gd(i,j-1)):
          // the terms +gd(j+1), -gd(j) (south) and -gd(j), +gd(j-1) (north).
          if (j == 0) {
            cap.add((double)t.gd[p + TR::SW]);
            cap.add(-(double)t.gd[p]);
          } else {
            cap.add(-(double)t.gd[p]);
            cap.add((double)t.gd[p - TR::SW]);
          }
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
      const double s = block_value(cap, redD);
      const int jh = (j == 0) ? 0 : Mh - 1;
      const double dl = (double)cf(md, CF_DLAT, j);
      const double val = s * (double)ch(md, CH_COS, jh) / (dl * dl) * (double)cf(md, CF_COS, j) / N;
      for (int i = threadIdx.x; i < N; i += blockDim.x) rg[i] = T(val);
      __syncthreads();
    }
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
    diffusion_iap_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl, int slot,
                         int* uvslot) {
  __shared__ MemberDev<T> smd;
  const WorkItem w = wl[blockIdx.x];
  load_member(mems, w.member, &smd);
  const MemberDev<T>& md = smd;
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
    // The next step's first stage reads the diffused u, v themselves.
    md.given_u[o] = u[o];
    if (hv) md.given_v[o] = v[o];
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
  if (uvslot && threadIdx.x == 0) uvslot[w.member] = slot;
}

// copy_data(state1, state2) (src/types_mod.F90:229-241) of the prognostic
// words, compensation included.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    copy_state_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl, int from, int to) {
  __shared__ MemberDev<T> smd;
  const WorkItem w = wl[blockIdx.x];
  load_member(mems, w.member, &smd);
  const MemberDev<T>& md = smd;
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
  int bulk = 0;
  if (tile_rows == 8 && tile_cols == 32) bulk = tile_words<T, 8, 32>();
  if (tile_rows == 8 && tile_cols == 64) bulk = tile_words<T, 8, 64>();
  if (tile_rows == 4 && tile_cols == 128) bulk = tile_words<T, 4, 128>();
  const int row = tile_words<T, 1, kRowChunk>();
  // Rounded to 4 words and max_n to an even count so that the FP64
  // reduction buffer after the T arrays stays 8-byte aligned.
  const int sw = ((bulk > row ? bulk : row) + 3) & ~3;
  max_n = (max_n + 1) & ~1;
  if (staging_words) *staging_words = sw;
  return (size_t)(sw + 3 * max_n + kMaxKeep + 64) * sizeof(T) + 64 * sizeof(double) + 16;
}

template <typename T, int PASS, int ADV, int R, int W>
static int launch_stage_t(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int max_n, const StageArgs& a,
                          cudaStream_t s) {
  int sw = 0;
  max_n = (max_n + 1) & ~1;
  const size_t smem = stage_smem_bytes<T>(R, W, max_n, &sw);
  static size_t configured = 0;
  if (smem > configured) {
    if (cudaFuncSetAttribute(stage_kernel<T, PASS, ADV, R, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return check_launch();
    configured = smem;
  }
  stage_kernel<T, PASS, ADV, R, W><<<nwork, kThreads, smem, s>>>(mem, wl, a, sw, max_n);
  return check_launch();
}

template <typename T, int R, int W>
static int launch_stage_shape(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int adv, int max_n,
                              const StageArgs& a, cudaStream_t s) {
#define GDC_DISPATCH(P, A) \
  if (a.pass == P && adv == A) return launch_stage_t<T, P, A, R, W>(mem, wl, nwork, max_n, a, s);
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
int launch_stage(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int adv, int tile_rows, int tile_cols,
                 int max_n, const StageArgs& a, void* stream) {
  if (nwork <= 0) return GDC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (tile_rows == 8 && tile_cols == 32) return launch_stage_shape<T, 8, 32>(mem, wl, nwork, adv, max_n, a, s);
  if (tile_rows == 8 && tile_cols == 64) return launch_stage_shape<T, 8, 64>(mem, wl, nwork, adv, max_n, a, s);
  if (tile_rows == 4 && tile_cols == 128) return launch_stage_shape<T, 4, 128>(mem, wl, nwork, adv, max_n, a, s);
  return GDC_E_CONFIG;
}

template <typename T>
int launch_beta(const MemberDev<T>* mem, const int* slots, int nmembers, const double* partials, double* beta,
                int qcon, int beta_mode, void* stream) {
  if (nmembers <= 0) return GDC_OK;
  beta_kernel<T><<<nmembers, kThreads, 0, (cudaStream_t)stream>>>(mem, slots, partials, beta, qcon, beta_mode);
  return check_launch();
}

template <typename T>
int launch_final(const MemberDev<T>* mem, const WorkItem* wl, int nwork, const FinalArgs& a, void* stream) {
  if (nwork <= 0) return GDC_OK;
  final_kernel<T><<<nwork, kThreads, 0, (cudaStream_t)stream>>>(mem, wl, a);
  return check_launch();
}

template <typename T>
int launch_diag(const MemberDev<T>* mem, const WorkItem* wl, int nwork, const int* slots, int nmembers,
                const DiagArgs& a, void* stream) {
  if (nwork <= 0) return GDC_OK;
  diag_kernel<T><<<nwork, kThreads, 0, (cudaStream_t)stream>>>(mem, wl, a);
  int rc = check_launch();
  if (rc) return rc;
  diag_finalize_kernel<T><<<nmembers, kThreads, 0, (cudaStream_t)stream>>>(mem, slots, a);
  return check_launch();
}

template <typename T>
int launch_diffusion(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int tile_rows, int tile_cols,
                     int max_n, int slot, double sign_dt_coef, int* uvslot, void* stream) {
  if (nwork <= 0) return GDC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int sw = 0;
  max_n = (max_n + 1) & ~1;
  const size_t smem = stage_smem_bytes<T>(tile_rows, tile_cols, max_n, &sw);
  static size_t configured = 0;
  auto lap = diffusion_lap_kernel<T, 8, 32>;
  if (tile_rows == 8 && tile_cols == 64)
    lap = diffusion_lap_kernel<T, 8, 64>;
  else if (tile_rows == 4 && tile_cols == 128)
    lap = diffusion_lap_kernel<T, 4, 128>;
  else if (!(tile_rows == 8 && tile_cols == 32))
    return GDC_E_CONFIG;
  if (smem > configured) {
    for (auto k : {diffusion_lap_kernel<T, 8, 32>, diffusion_lap_kernel<T, 8, 64>, diffusion_lap_kernel<T, 4, 128>})
      if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch();
    configured = smem;
  }
  lap<<<nwork, kThreads, smem, s>>>(mem, wl, slot, sign_dt_coef, sw, max_n);
  int rc = check_launch();
  if (rc != GDC_OK) return rc;
  diffusion_iap_kernel<T><<<nwork, kThreads, 0, s>>>(mem, wl, slot, uvslot);
  return check_launch();
}

template <typename T>
int launch_copy_state(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int from_slot, int to_slot,
                      void* stream) {
  if (nwork <= 0) return GDC_OK;
  copy_state_kernel<T><<<nwork, kThreads, 0, (cudaStream_t)stream>>>(mem, wl, from_slot, to_slot);
  return check_launch();
}

}  // namespace gdc
