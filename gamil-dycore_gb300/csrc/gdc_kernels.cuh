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

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>

#include <cooperative_groups.h>

#include "gdc_internal.h"

namespace gdc {

constexpr int kThreads = 256;
constexpr int kRowChunk = 128;  // columns per chunk of a whole-row task
#ifndef GDC_STRIP_BLOCKS
#define GDC_STRIP_BLOCKS 2  // resident strip blocks per SM (FP32)
#endif
#ifndef GDC_STAGE_BLOCKS
#define GDC_STAGE_BLOCKS 4  // resident stage blocks per SM the FP32 register budget targets
#endif

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
// FP32 sums are compensated too: beta = ip1 / ip2 differs from 1 by about
// the step's relative change (1e-6), so a plain FP32 sum (relative error
// ~1e-7 per block) would put percent-level errors on beta - 1.
template <>
struct Acc<float> {
  float s = 0, c = 0;
  __device__ void add(float x) {
    const float t = s + x;
    const float bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
  }
  __device__ void merge(float os, float oc) {
    add(os);
    c += oc;
  }
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

// The 16-byte vector of a compute type.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
};
template <>
struct Vec16<double> {
  using type = double2;
};

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
// row) stage only what their valid points use.  `rc` holds the coefficient
// records of rows j0-1..j0+R (full row j and half row j in each).
template <typename T, int R_, int W_>
struct Tile {
  static constexpr int R = R_, W = W_;
  static constexpr int VEC = 16 / (int)sizeof(T);  // elements per 16-byte copy
  static constexpr int OFF = VEC - 1;              // so that column i0 is aligned
  static constexpr int SW = ((W_ + 3 + OFF + VEC - 1) / VEC) * VEC;
  static constexpr int ROWS = R_ + 3, NS = ROWS * SW;
  static constexpr int CR = R_ + 2;                // coefficient rows
  T *gd, *ghs, *iu, *iv, *ig, *u, *v;
  T* rc;
  int j0, i0, vrows, vcols;
  __device__ static int pos(int rr, int cc) { return rr * SW + cc + OFF; }
  __device__ T cf(int k, int j) const { return rc[(j - j0 + 1) * kRecWords + k]; }
  __device__ T ch(int k, int jh) const { return rc[(jh - j0 + 1) * kRecWords + k]; }
};

template <typename T, int R, int W>
GDC_HD constexpr int tile_words() {
  return 7 * Tile<T, R, W>::NS + kRecWords * Tile<T, R, W>::CR;
}

// Words of a whole-row task's staging tile, rounded to 16 bytes.
template <typename T>
GDC_HD constexpr int row_task_words() {
  return (tile_words<T, 1, kRowChunk>() + 3) & ~3;
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
  t.rc = base + 7 * n;
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
// With `tend` (a fused final update), the tendencies of the level's update
// are staged into the ig, u and v areas (free until tile_derive).
template <typename T, int R, int W>
__device__ void tile_issue(const MemberDev<T>& md, const T* __restrict__ gd, const T* __restrict__ iu,
                           const T* __restrict__ iv, Tile<T, R, W>& t, bool given = false, bool want_ghs = true,
                           T* const* tend = nullptr) {
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
    if (want_ghs) cp_async16(&t.ghs[dp], md.ghs + o, vf);
    cp_async16(&t.iu[dp], iu + o, vf);
    cp_async16(&t.iv[dp], iv + (vh ? o : 0), vh);
    if (given) {
      cp_async16(&t.u[dp], md.given_u + o, vf);
      cp_async16(&t.v[dp], md.given_v + (vh ? o : 0), vh);
    }
    if (tend) {
      cp_async16(&t.ig[dp], tend[F_GD] + o, vf);
      cp_async16(&t.u[dp], tend[F_IU] + o, vf);
      cp_async16(&t.v[dp], tend[F_IV] + (vh ? o : 0), vh);
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
    if (want_ghs) cp_async(&t.ghs[dp], md.ghs + o, vf);
    cp_async(&t.iu[dp], iu + o, vf);
    cp_async(&t.iv[dp], iv + (vh ? o : 0), vh);
    if (given) {
      cp_async(&t.u[dp], md.given_u + o, vf);
      cp_async(&t.v[dp], md.given_v + (vh ? o : 0), vh);
    }
    if (tend) {
      cp_async(&t.ig[dp], tend[F_GD] + o, vf);
      cp_async(&t.u[dp], tend[F_IU] + o, vf);
      cp_async(&t.v[dp], tend[F_IV] + (vh ? o : 0), vh);
    }
  }
  (void)nfield;
  // coefficient records of rows j0-1..j0+R (records exist for rows -1..M)
  constexpr int RCH = kRecWords / VEC;  // 16-byte copies per record
  for (int q = threadIdx.x; q < TL::CR * RCH; q += kThreads) {
    const int lr = q / RCH, k = q - lr * RCH;
    const int j = t.j0 - 1 + lr;
    if (j > M) continue;  // beyond a partial tile: never read
    cp_async16(&t.rc[lr * kRecWords + k * VEC], md.rowc + (size_t)(j + 1) * kRecWords + k * VEC, true);
  }
}

// The fused final update (StageArgs::fuse): after the copies, every staged
// position of gd, iap u, iap v becomes the previous predict_correct's new
// level, fin_base + h T_new with h = pcdt[fin_pass] * fin_h_scale * beta --
// in FP32 with its compensation word, TwoSum of lo + h T onto hi, exactly
// as final_kernel forms it -- and the block writes the level (and its
// compensation words) for the points it owns: rows 1..vrows, columns
// 1..vcols of the tile, of the fields in `own_fields` (bit f for field f).
// Row interiors go 16 bytes at a time (shared, compensation words and the
// level's stores), the three halo columns element by element.
template <typename T>
__device__ __forceinline__ T combine_level(T x, const T* lo, T tv, T h, T* e) {
  if (lo) {
    const T y = *lo + h * tv;
    const T sum = x + y;
    const T bp = sum - x;
    *e = (x - (sum - bp)) + (y - bp);
    return sum;
  }
  return x + h * tv;
}

template <typename T, int R, int W>
__device__ void tile_combine(const MemberDev<T>& md, const StageArgs& a, int member, Tile<T, R, W>& t,
                             int own_fields) {
  using TL = Tile<T, R, W>;
  using V = typename Vec16<T>::type;
  constexpr int VEC = TL::VEC, NCH = W / VEC;
  const int N = md.N, M = md.M, Mh = md.Mh;
  const T h = T(md.pcdt[a.fin_pass] * a.fin_h_scale * a.beta[member]);
  T* const* lo = md.lo[a.fin_base];
  T* const* out = md.st[a.in_slot];
  T* const* olo = md.lo[a.in_slot];
  T* hi[3] = {t.gd, t.iu, t.iv};
  const T* tt[3] = {t.ig, t.u, t.v};
  cp_async_wait_all();
  __syncthreads();
  // row interiors (columns i0 .. i0+vcols-1, never wrapping, 16-byte aligned)
  for (int q = threadIdx.x; q < TL::ROWS * NCH; q += kThreads) {
    const int rr = q / NCH, k = q - rr * NCH;
    if (rr > t.vrows + 2 || k * VEC >= t.vcols) continue;  // not staged
    const int j = t.j0 - 1 + rr;
    if (j < 0 || j >= M) continue;  // off the sphere: zero, as staged
    const int p = TL::pos(rr, 1 + k * VEC);
    const size_t o = (size_t)j * N + t.i0 + k * VEC;
    const bool own = rr >= 1 && rr <= t.vrows;
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      if (f == F_IV && j >= Mh) continue;
      V x = *reinterpret_cast<const V*>(hi[f] + p);
      const V tv = *reinterpret_cast<const V*>(tt[f] + p);
      V l, e;
      if (lo[f]) l = *reinterpret_cast<const V*>(lo[f] + o);
      T* xs = reinterpret_cast<T*>(&x);
      const T* ts = reinterpret_cast<const T*>(&tv);
      const T* ls = reinterpret_cast<const T*>(&l);
      T* es = reinterpret_cast<T*>(&e);
#pragma unroll
      for (int m = 0; m < VEC; ++m) xs[m] = combine_level(xs[m], lo[f] ? ls + m : nullptr, ts[m], h, es + m);
      *reinterpret_cast<V*>(hi[f] + p) = x;
      if (own && (own_fields >> f & 1)) {
        *reinterpret_cast<V*>(out[f] + o) = x;
        if (lo[f]) *reinterpret_cast<V*>(olo[f] + o) = e;
      }
    }
  }
  // halo columns i0-1, i0+vcols, i0+vcols+1 (periodic): never owned
  for (int q = threadIdx.x; q < TL::ROWS * 3; q += kThreads) {
    const int rr = q / 3, hh = q - rr * 3;
    if (rr > t.vrows + 2) continue;
    const int j = t.j0 - 1 + rr;
    if (j < 0 || j >= M) continue;
    const int cc = hh == 0 ? 0 : t.vcols + hh;
    int i = t.i0 - 1 + cc;
    i = i < 0 ? i + N : (i >= N ? i - N : i);
    const int p = TL::pos(rr, cc);
    const size_t o = (size_t)j * N + i;
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      if (f == F_IV && j >= Mh) continue;
      T e;
      hi[f][p] = combine_level(hi[f][p], lo[f] ? lo[f] + o : nullptr, tt[f][p], h, &e);
    }
  }
  __syncthreads();
}

// After the copies: iap gd, then u on full rows j0..j0+R (local 1..R+1;
// from local 0 when the stencil also needs row j0-1), v on half rows
// j0-1..j0+R (local 0..R+1), columns i0-1..i0+W (local 0..W+1).
// Local tile rows (inclusive) on which iap gd, u and v are derived; an
// empty range (lo > hi) derives none.  Whole tiles derive every row their
// stencils may read; a whole-row task for one field derives only the rows
// that field's stencil reads (row_task_rows).
struct DeriveRows {
  int ig0 = 0, ig1 = 1 << 20, u0 = 0, u1 = 1 << 20, v0 = 0, v1 = 1 << 20;
};

// A one-row tile (the task's row at local row 1) computing the tendency of
// field f alone (f < 0: all three), pass `pass` (src/dycore_mod.F90:
// 367-598): du reads u on its row (and v on the half rows around it in the
// advection), dv reads u on its row and the next and v on three half rows,
// dgd only iap gd.
__device__ inline DeriveRows row_task_rows(int pass, int f) {
  DeriveRows d;
  if (f < 0) return d;
  if (f == F_GD) {
    d.ig0 = 0, d.ig1 = 2, d.u0 = 1, d.u1 = 0, d.v0 = 1, d.v1 = 0;
  } else if (f == F_IU) {
    if (pass == kFastPass)
      d.ig0 = 1, d.ig1 = 1, d.u0 = 1, d.u1 = 1, d.v0 = 1, d.v1 = 0;
    else
      d.ig0 = 0, d.ig1 = 2, d.u0 = 1, d.u1 = 1, d.v0 = 0, d.v1 = 1;
  } else {
    if (pass == kFastPass)
      d.ig0 = 1, d.ig1 = 2, d.u0 = 1, d.u1 = 2, d.v0 = 1, d.v1 = 0;
    else
      d.ig0 = 0, d.ig1 = 3, d.u0 = 1, d.u1 = 2, d.v0 = 0, d.v1 = 2;
  }
  return d;
}

template <typename T, int R, int W>
__device__ void tile_derive(const MemberDev<T>& md, Tile<T, R, W>& t, bool u_halo_row = false,
                            bool given = false, bool want_v = true, DeriveRows rows = DeriveRows()) {
  using TL = Tile<T, R, W>;
  const int M = md.M, Mh = md.Mh;
  const int urow0 = max(u_halo_row ? 0 : 1, rows.u0);
  constexpr int DW = W + 2, ND = (R + 2) * (W + 2);
  cp_async_wait_all();
  __syncthreads();
  if constexpr (sizeof(T) == 4) {
    // FP32: one pass and one barrier fewer -- each position takes the
    // square roots it divides by itself (the same values as ig).
    for (int q = threadIdx.x; q < ND; q += kThreads) {
      const int rr = q / DW, cc = q - rr * DW;
      const int p = TL::pos(rr, cc);
      if (rr > t.vrows + 1 || cc > t.vcols + 1) continue;
      const int j = t.j0 - 1 + rr;
      const T g0 = sqrt(t.gd[p]);
      if (rr >= rows.ig0 && rr <= rows.ig1) t.ig[p] = g0;
      if (given) continue;
      T uu = 0, vv = 0;
      if (rr >= urow0 && rr <= rows.u1 && j >= 1 && j <= M - 2) uu = t.iu[p] * T(2) / (g0 + sqrt(t.gd[p + 1]));
      if (want_v && rr >= rows.v0 && rr <= rows.v1 && j >= 0 && j < Mh)
        vv = t.iv[p] * T(2) / (g0 + sqrt(t.gd[p + TL::SW]));
      t.u[p] = uu;
      t.v[p] = vv;
    }
    __syncthreads();
    return;
  }
  for (int p = threadIdx.x; p < TL::NS; p += kThreads) {
    const int rr = p / TL::SW;
    if (rr >= rows.ig0 && rr <= rows.ig1) t.ig[p] = sqrt(t.gd[p]);
  }
  __syncthreads();
  if (given) return;
  for (int q = threadIdx.x; q < ND; q += kThreads) {
    const int rr = q / DW, cc = q - rr * DW;
    const int p = TL::pos(rr, cc);
    const int j = t.j0 - 1 + rr;
    const bool need = rr <= t.vrows + 1 && cc <= t.vcols + 1;
    T uu = 0, vv = 0;
    if (need && rr >= urow0 && rr <= rows.u1 && j >= 1 && j <= M - 2) uu = t.iu[p] * T(2) / (t.ig[p] + t.ig[p + 1]);
    if (want_v && need && rr >= rows.v0 && rr <= rows.v1 && j >= 0 && j < Mh)
      vv = t.iv[p] * T(2) / (t.ig[p] + t.ig[p + TL::SW]);
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

// Stencil views: s.f(dr, dc) is field f at row offset dr and column offset
// dc (-1..1) from the point, s.cf / s.ch the row coefficients, s.j the row.
// TileView reads a shared-memory tile; the strip kernel has its own view
// over registers.  The point operators below are written once for both.
template <typename T, class TL>
struct TileView {
  const TL& t;
  int p, j;
  __device__ __forceinline__ T u(int dr, int dc) const { return t.u[p + dr * TL::SW + dc]; }
  __device__ __forceinline__ T v(int dr, int dc) const { return t.v[p + dr * TL::SW + dc]; }
  __device__ __forceinline__ T iu(int dr, int dc) const { return t.iu[p + dr * TL::SW + dc]; }
  __device__ __forceinline__ T iv(int dr, int dc) const { return t.iv[p + dr * TL::SW + dc]; }
  __device__ __forceinline__ T ig(int dr, int dc) const { return t.ig[p + dr * TL::SW + dc]; }
  __device__ __forceinline__ T gd(int dr, int dc) const { return t.gd[p + dr * TL::SW + dc]; }
  __device__ __forceinline__ T ghs(int dr, int dc) const { return t.ghs[p + dr * TL::SW + dc]; }
  __device__ __forceinline__ T cf(int k, int jj) const { return t.cf(k, jj); }
  __device__ __forceinline__ T ch(int k, int jj) const { return t.ch(k, jj); }
};

// `wadv`: the WENO advection term -(u_adv_lon + u_adv_lat) of this point,
// computed beforehand by weno_kernel (uv_adv_scheme weno only).
template <typename T, int PASS, int ADV, class S>
__device__ __forceinline__ T point_du(const S& s, T beta_lon, T beta_lat, T wadv = T(0)) {
  const int j = s.j;
  T r = 0;
  if (PASS != kFastPass && ADV == GDC_ADV_WENO) r = wadv;
  if (PASS != kFastPass && ADV != GDC_ADV_WENO) {
    // src/dycore_mod.F90:376-392 / :393-415
    const T uc = s.u(0, 0), um = s.u(0, -1), up = s.u(0, 1);
    const T u1 = uc + um, u2 = uc + up;
    T adv_lon;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lon = s.cf(TF_RADVLON, j) * (u2 * s.iu(0, 1) - u1 * s.iu(0, -1));
    } else {
      const T ic = s.iu(0, 0), ip = s.iu(0, 1), im = s.iu(0, -1);
      adv_lon = s.cf(TF_RADVLON, j) * (u2 * (ic + ip) - beta_lon * fabs(u2) * (ip - ic) - u1 * (ic + im) +
                                         beta_lon * fabs(u1) * (ic - im) - (u2 - u1) * ic);
    }
    // src/dycore_mod.F90:433-439 / :450-459
    const T v1 = (s.v(-1, 0) + s.v(-1, 1)) * s.ch(TH_COS, j - 1);
    const T v2 = (s.v(0, 0) + s.v(0, 1)) * s.ch(TH_COS, j);
    T adv_lat;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lat = s.cf(TF_RADVLAT, j) * (v2 * s.iu(1, 0) - v1 * s.iu(-1, 0));
    } else {
      const T ic = s.iu(0, 0), ip = s.iu(1, 0), im = s.iu(-1, 0);
      adv_lat = s.cf(TF_RADVLAT, j) * (v2 * (ic + ip) - beta_lat * fabs(v2) * (ip - ic) - v1 * (ic + im) +
                                         beta_lat * fabs(v1) * (ic - im) - (v2 - v1) * ic);
    }
    r = -adv_lon - adv_lat;
  }
  if (PASS != kSlowPass) {
    // src/dycore_mod.F90:485-493
    const T fv = T(0.25) * (s.cf(TF_F, j) + s.cf(TF_C, j) * s.u(0, 0)) *
                 (s.cf(TF_C1, j) * (s.iv(-1, 0) + s.iv(-1, 1)) + s.cf(TF_C2, j) * (s.iv(0, 0) + s.iv(0, 1)));
    // src/dycore_mod.F90:514-519
    const T pgf = T(0.5) * (s.ig(0, 0) + s.ig(0, 1)) / s.cf(TF_DLON, j) *
                  (s.gd(0, 1) + s.ghs(0, 1) - s.gd(0, 0) - s.ghs(0, 0));
    if (PASS == kAllPass)
      r = r + fv - pgf;
    else
      r = fv - pgf;
  }
  return r;
}

template <typename T, int PASS, int ADV, class S>
__device__ __forceinline__ T point_dv(const S& s, T beta_lon, T beta_lat, T wadv = T(0)) {
  const int jh = s.j;
  T r = 0;
  if (PASS != kFastPass && ADV == GDC_ADV_WENO) r = wadv;
  if (PASS != kFastPass && ADV != GDC_ADV_WENO) {
    // src/dycore_mod.F90:386-391 / :406-414
    const T u1 = s.u(0, -1) + s.u(1, -1);
    const T u2 = s.u(0, 0) + s.u(1, 0);
    T adv_lon;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lon = s.ch(TH_RADVLON, jh) * (u2 * s.iv(0, 1) - u1 * s.iv(0, -1));
    } else {
      const T ic = s.iv(0, 0), ip = s.iv(0, 1), im = s.iv(0, -1);
      adv_lon = s.ch(TH_RADVLON, jh) * (u2 * (ic + ip) - beta_lon * fabs(u2) * (ip - ic) - u1 * (ic + im) +
                                          beta_lon * fabs(u1) * (ic - im) - (u2 - u1) * ic);
    }
    // src/dycore_mod.F90:441-446 / :461-469
    const T vc = s.v(0, 0) * s.ch(TH_COS, jh);
    const T v1 = vc + s.v(-1, 0) * s.ch(TH_COS, jh - 1);
    const T v2 = vc + s.v(1, 0) * s.ch(TH_COS, jh + 1);
    T adv_lat;
    if (ADV == GDC_ADV_CENTER_DIFF) {
      adv_lat = s.ch(TH_RADVLAT, jh) * (v2 * s.iv(1, 0) - v1 * s.iv(-1, 0));
    } else {
      const T ic = s.iv(0, 0), ip = s.iv(1, 0), im = s.iv(-1, 0);
      adv_lat = s.ch(TH_RADVLAT, jh) * (v2 * (ic + ip) - beta_lat * fabs(v2) * (ip - ic) - v1 * (ic + im) +
                                          beta_lat * fabs(v1) * (ic - im) - (v2 - v1) * ic);
    }
    r = -adv_lon - adv_lat;
  }
  if (PASS != kSlowPass) {
    // src/dycore_mod.F90:495-503
    const T f0 = s.cf(TF_F, jh), c0 = s.cf(TF_C, jh);
    const T f1 = s.cf(TF_F, jh + 1), c1 = s.cf(TF_C, jh + 1);
    const T fu = T(0.25) * ((f0 + c0 * s.u(0, 0)) * s.iu(0, 0) + (f0 + c0 * s.u(0, -1)) * s.iu(0, -1) +
                            (f1 + c1 * s.u(1, 0)) * s.iu(1, 0) + (f1 + c1 * s.u(1, -1)) * s.iu(1, -1));
    // src/dycore_mod.F90:530-535
    const T pgf = T(0.5) * (s.ig(0, 0) + s.ig(1, 0)) / s.ch(TH_DLAT, jh) * s.ch(TH_COS, jh) *
                  (s.gd(1, 0) + s.ghs(1, 0) - s.gd(0, 0) - s.ghs(0, 0));
    if (PASS == kAllPass)
      r = r - fu - pgf;
    else
      r = -fu - pgf;
  }
  return r;
}

// Interior rows only (1..M-2); pole rows come from the zonal-sum cap.
template <typename T, int PASS, class S>
__device__ __forceinline__ T point_dgd(const S& s) {
  if (PASS == kSlowPass) return T(0);  // src/dycore_mod.F90:297
  const int j = s.j;
  // src/dycore_mod.F90:546-552
  const T mdlon = ((s.ig(0, 0) + s.ig(0, 1)) * s.iu(0, 0) - (s.ig(0, 0) + s.ig(0, -1)) * s.iu(0, -1)) * T(0.5) /
                  s.cf(TF_DLON, j);
  // src/dycore_mod.F90:564-570
  const T mdlat = ((s.ig(0, 0) + s.ig(1, 0)) * s.iv(0, 0) * s.ch(TH_COS, j) -
                   (s.ig(0, 0) + s.ig(-1, 0)) * s.iv(-1, 0) * s.ch(TH_COS, j - 1)) *
                  T(0.5) / s.cf(TF_DLAT, j);
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

  // One point's terms of predict_correct's inner products (beta_mode 0).
  // FP64 adds prev*val*w and val*val*w to <T_old, T_new> and <T_new, T_new>
  // as the reference does (double-double: the oracle's exact sums).  FP32
  // forms d = <T_old - T_new, T_new> in place of <T_old, T_new>, so that
  // beta = 1 + d / <T_new, T_new> (the same ratio): beta - 1 is carried by
  // d itself instead of by the difference of two nearly equal sums, and
  // plain float sums local to the thread suffice; ip_flush folds them into
  // the compensated block sums.
  T l1 = T(0), l2 = T(0);
  __device__ __forceinline__ void ip_point(T prev, T val, T w) {
    if constexpr (sizeof(T) == 4) {
      l1 += (prev - val) * val * w;
      l2 += val * val * w;
    } else {
      ip1.add(prev * val * w);
      ip2.add(val * val * w);
    }
  }
  __device__ __forceinline__ void ip_flush() {
    if constexpr (sizeof(T) == 4) {
      ip1.add(l1);
      ip2.add(l2);
      l1 = l2 = T(0);
    }
  }

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
      if (a.beta_mode == 0) {
        ip_point(prev, val, wcos);
      } else {
        ip1.add(prev * val * wcos);
        ip2.add(val * val * wcos);
      }
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
// `tw` holds the member's twiddles in shared memory: cos(2 pi m/N) at
// tw[m], sin at tw[N + m] (copied by twiddles_to_shared).  Indices k n mod
// N advance by additions.
//
// A whole-row task split over the two blocks of a cluster (RowPair::on):
// both blocks hold the whole row, each forms the coefficients of its parity
// (p % 2 == part) and writes them to its own and its partner's shared
// memory, and a cluster barrier before the writes (the partner has started
// and is done with the previous filter's coefficients) and one after them
// make all of them visible to both; each block then reconstructs the whole
// row.  Every coefficient is the same sum as in one block.
struct RowPair {
  bool on = false;
  int part = 0;
};

template <typename T>
__device__ void filter_project(const MemberDev<T>& md, T* x, int keep, T* coefs, const T* tw,
                               RowPair pr = RowPair()) {
  const int N = md.N;
  const T* ctab = tw;
  const T* stab = tw + N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T* remote = nullptr;
  if (pr.on) {
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    cl.sync();
    remote = cl.map_shared_rank(coefs, (int)cl.block_rank() ^ 1);
  } else {
    __syncthreads();
  }
  const int p0 = pr.on ? 2 * warp + pr.part : warp, dp = pr.on ? 2 * nw : nw;
  for (int p = p0; p < keep; p += dp) {
    Acc<T> acc;
    if (p == 0) {
      for (int n = lane; n < N; n += 32) acc.add(x[n]);
    } else {
      const int k = (p + 1) >> 1;
      const T* tab = (p & 1) ? ctab : stab;
      const int step = (32 * k) % N;
      int idx = (k * lane) % N;
      for (int n = lane; n < N; n += 32) {
        acc.add(x[n] * tab[idx]);
        idx += step;
        if (idx >= N) idx -= N;
      }
    }
    warp_acc(acc);
    if (lane == 0) {
      // a0 and, when every mode is kept, the Nyquist term r(N) = (1/N)
      // sum x (-1)^n (the cosine table is exactly +-1 there) take 1/N
      const bool single = p == 0 || (p == N - 1 && N % 2 == 0);
      const T c = acc.value() * (single ? T(1.0) / T(N) : T(2.0) / T(N));
      coefs[p] = c;
      if (remote) remote[p] = c;
    }
  }
  if (pr.on)
    cooperative_groups::this_cluster().sync();
  else
    __syncthreads();
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    T y = 0;
    y = y + coefs[0];
    int idx = 0;  // k n mod N for the current k
    for (int p = 1; p < keep; ++p) {
      if (p & 1) {
        idx += n;
        if (idx >= N) idx -= N;
        y = y + coefs[p] * ctab[idx];
      } else {
        y = y + coefs[p] * stab[idx];
      }
    }
    x[n] = y;
  }
  __syncthreads();
}

// Copy the member's twiddle tables (2N values) to shared memory.
template <typename T>
__device__ inline void twiddles_to_shared(const MemberDev<T>& md, T* tw) {
  for (int i = threadIdx.x; i < 2 * md.N; i += blockDim.x) tw[i] = md.twid[i];
}

// The s1/s2-rescaled tendency filter of src/dycore_mod.F90:212-219.  With
// rtol > 0 (an extension; 0 is the reference) the rescale is skipped when
// s1 or s2 is zero to within rtol of the sum of the magnitudes of its terms.
template <typename T>
__device__ void filter_rescale(const MemberDev<T>& md, T* x, const T* __restrict__ w1, const T* __restrict__ w2,
                               int keep, T* coefs, T* red, double rtol, const T* tw, RowPair pr = RowPair()) {
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
  filter_project(md, x, keep, coefs, tw, pr);
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

// ------------------------------------------------------------- WENO
// uv_adv_scheme weno (src/weno_mod.F90, weno_order 2): the momentum
// advection terms of every point, written to md.wadv for the stage kernel.
// One point per thread, straight from global memory: the reference's
// Lax-Friedrichs split fluxes and interface fluxes are recomputed at each
// point that reads them (the 5-point stencil and its u/v derivation are
// cached in L1), in the reference's order of operations.  Kept as the
// reference has them: u_adv_lon divides by half_dlon of the row's half row
// (:153-154), u_adv_lat's correction takes v at lon i-1, i (:281-282), and
// the split fluxes are zero on the pole and lat-halo rows (those halos are
// never filled).
template <typename T>
struct WenoIn {
  const T *gd, *iu, *iv, *gu, *gv;
  int N, M, Mh;
  bool given;
  __device__ __forceinline__ int wrap(int i) const { return i < 0 ? i + N : (i >= N ? i - N : i); }
  // u at column i (periodic), full row j; zero on the pole rows
  __device__ __forceinline__ T u(int i, int j) const {
    if (j < 1 || j > M - 2) return T(0);
    i = wrap(i);
    if (given) return gu[j * N + i];
    const int ip = i + 1 == N ? 0 : i + 1;
    return iu[j * N + i] * T(2) / (sqrt(gd[j * N + i]) + sqrt(gd[j * N + ip]));
  }
  // v at column i (periodic), half row j; zero off the half rows
  __device__ __forceinline__ T v(int i, int j) const {
    if (j < 0 || j > Mh - 1) return T(0);
    i = wrap(i);
    if (given) return gv[j * N + i];
    return iv[j * N + i] * T(2) / (sqrt(gd[j * N + i]) + sqrt(gd[(j + 1) * N + i]));
  }
  __device__ __forceinline__ T iu_(int i, int j) const { return iu[j * N + wrap(i)]; }
  __device__ __forceinline__ T iv_(int i, int j) const { return iv[j * N + wrap(i)]; }
};

// weno_2nd_order_pass (src/weno_mod.F90:249-298, coefficients :41-46)
template <typename T>
__device__ __forceinline__ T weno2(T fp1, T fp2, T fp3, T fn2, T fn3, T fn4) {
  const T c11 = T(-0.5), c21 = T(1.5), c12 = T(0.5), c22 = T(0.5);
  const T wo1 = T(1.0 / 3.0), wo2 = T(2.0 / 3.0), eps = T(1.0e-6);
  T fs1 = c11 * fp1 + c21 * fp2, fs2 = c12 * fp2 + c22 * fp3;
  T b1 = (fp2 - fp1) * (fp2 - fp1), b2 = (fp3 - fp2) * (fp3 - fp2);
  T w1 = wo1 / ((eps + b1) * (eps + b1)), w2 = wo2 / ((eps + b2) * (eps + b2));
  T sw = w1 + w2;
  w1 = w1 / sw;
  w2 = w2 / sw;
  const T f = w1 * fs1 + w2 * fs2;
  fs1 = c11 * fn4 + c21 * fn3;
  fs2 = c12 * fn3 + c22 * fn2;
  b1 = (fn3 - fn4) * (fn3 - fn4);
  b2 = (fn2 - fn3) * (fn2 - fn3);
  w1 = wo1 / ((eps + b1) * (eps + b1));
  w2 = wo2 / ((eps + b2) * (eps + b2));
  sw = w1 + w2;
  w1 = w1 / sw;
  w2 = w2 / sw;
  return f + (w1 * fs1 + w2 * fs2);
}

// -(u_adv_lon + u_adv_lat) at u point (i, full row j), 1 <= j <= M-2
// (src/weno_mod.F90:66-73, 102-110, 151-155; :169-177, 199-206, 225-229).
template <typename T>
__device__ T weno_point_u(const WenoIn<T>& s, const T* coef, int i, int j) {
  const int M = s.M;
  const T umax = T(20), vmax = T(20), h = T(0.5), q = T(0.25);
  // zonal: split fluxes of row j at columns i-2..i+2
  T fp[5], fn[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const T uk = s.u(i - 2 + k, j), ik = s.iu_(i - 2 + k, j);
    fp[k] = h * (uk + umax) * ik;
    fn[k] = h * (uk - umax) * ik;
  }
  const T fi = weno2(fp[1], fp[2], fp[3], fn[2], fn[3], fn[4]);
  const T fim = weno2(fp[0], fp[1], fp[2], fn[1], fn[2], fn[3]);
  const T ual = (fi - fim - (s.u(i + 1, j) - s.u(i - 1, j)) * s.iu_(i, j) * q) / coef[ch_off(CH_DLON, M) + j + 1];
  // meridional: split fluxes of column i at rows j-2..j+2 (zero off 1..M-2)
  T mp[5], mn[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int r = j - 2 + k;
    if (r >= 1 && r <= M - 2) {
      const T vb = q * (s.v(i, r - 1) + s.v(i, r) + s.v(i + 1, r - 1) + s.v(i + 1, r));
      const T ik = s.iu_(i, r);
      mp[k] = h * (vb + vmax) * ik;
      mn[k] = h * (vb - vmax) * ik;
    } else {
      mp[k] = T(0);
      mn[k] = T(0);
    }
  }
  const T gj = weno2(mp[1], mp[2], mp[3], mn[2], mn[3], mn[4]);
  const T gjm = j - 1 >= 1 ? weno2(mp[0], mp[1], mp[2], mn[1], mn[2], mn[3]) : T(0);
  const T uat = (gj - gjm - (s.v(i - 1, j) + s.v(i, j) - s.v(i - 1, j - 1) - s.v(i, j - 1)) * s.iu_(i, j) * q) /
                coef[cf_off(CF_DLAT, M) + j];
  return -ual - uat;
}

// -(v_adv_lon + v_adv_lat) at v point (i, half row j), 0 <= j <= Mh-1
// (src/weno_mod.F90:75-85, 111-118, 156-158; :179-186, 208-215, 230-234).
template <typename T>
__device__ T weno_point_v(const WenoIn<T>& s, const T* coef, int i, int j) {
  const int M = s.M, Mh = s.Mh;
  const T umax = T(20), vmax = T(20), h = T(0.5), q = T(0.25);
  T fp[5], fn[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int c = i - 2 + k;
    const T ub = q * (s.u(c - 1, j) + s.u(c - 1, j + 1) + s.u(c, j) + s.u(c, j + 1));
    const T ik = s.iv_(c, j);
    fp[k] = h * (ub + umax) * ik;
    fn[k] = h * (ub - umax) * ik;
  }
  const T fi = weno2(fp[1], fp[2], fp[3], fn[2], fn[3], fn[4]);
  const T fim = weno2(fp[0], fp[1], fp[2], fn[1], fn[2], fn[3]);
  const T val = (fi - fim - (s.u(i, j) + s.u(i, j + 1) - s.u(i - 1, j) - s.u(i - 1, j + 1)) * s.iv_(i, j) * q) /
                coef[ch_off(CH_DLON, M) + j + 1];
  T mp[5], mn[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int r = j - 2 + k;
    if (r >= 0 && r <= Mh - 1) {
      const T vk = s.v(i, r), ik = s.iv_(i, r);
      mp[k] = h * (vk + vmax) * ik;
      mn[k] = h * (vk - vmax) * ik;
    } else {
      mp[k] = T(0);
      mn[k] = T(0);
    }
  }
  const T gj = weno2(mp[1], mp[2], mp[3], mn[2], mn[3], mn[4]);
  const T gjm = j - 1 >= 0 ? weno2(mp[0], mp[1], mp[2], mn[1], mn[2], mn[3]) : T(0);
  const T vat = (gj - gjm - (s.v(i, j + 1) - s.v(i, j - 1)) * s.iv_(i, j) * q) / coef[ch_off(CH_DLAT, M) + j + 1];
  return -val - vat;
}

// One flat item of a member's iap u or iap v field per block (gd items
// return at once): the WENO terms of the stage's input level.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    weno_kernel(const MemberDev<T>* __restrict__ mems, const FlatItem* __restrict__ fl, int in_slot,
                const int* __restrict__ uvslot) {
  const FlatItem w = fl[blockIdx.x];
  if (w.field == F_GD) return;
  const MemberDev<T>& md = mems[w.member];
  WenoIn<T> s;
  s.gd = md.st[in_slot][F_GD];
  s.iu = md.st[in_slot][F_IU];
  s.iv = md.st[in_slot][F_IV];
  s.gu = md.given_u;
  s.gv = md.given_v;
  s.N = md.N;
  s.M = md.M;
  s.Mh = md.Mh;
  s.given = uvslot && uvslot[w.member] == in_slot;
  const int N = md.N;
  T* out = md.wadv[w.field == F_IU ? 0 : 1];
  for (int k = threadIdx.x; k < w.count; k += kThreads) {
    const int q = w.begin + k, j = q / N, i = q - j * N;
    T r = T(0);
    if (w.field == F_IU) {
      if (j >= 1 && j <= md.M - 2) r = weno_point_u(s, md.coef, i, j);
    } else {
      r = weno_point_v(s, md.coef, i, j);
    }
    out[q] = r;
  }
}

// --------------------------------------------------------- stage kernel

// One bulk tile (rows j0..j0+rows-1, all ordinary; columns i0..i0+cols-1).
// Thread t owns column t % W and RPT consecutive rows from (t / W) * RPT;
// UF fixes the update form at compile time (UF_GENERAL: any StageArgs).
template <typename T, int PASS, int ADV, int R, int W, int UF>
__device__ __forceinline__ void bulk_tile(const MemberDev<T>& md, const StageArgs& a, const WorkItem& w,
                                          T* staging, bool given, const T* gd_in, const T* iu_in,
                                          const T* iv_in, T ub_lon, T ub_lat, Emit<T>& em) {
  using TL = Tile<T, R, W>;
  // Rows per thread; a tile with fewer points than threads leaves the
  // threads past R*W without points (they stage and derive only).
  constexpr int RPT = R * W >= kThreads ? R * W / kThreads : 1;
  static_assert(R * W < kThreads ? kThreads % W == 0 : RPT * kThreads == R * W,
                "a tile is a whole number of rows per thread");
  const int N = md.N;
  TL t = carve<T, R, W>(staging, w.j0, w.i0, w.rows, w.cols);
  const bool fuse = UF == UF_PREDICT_IN && a.fuse;
  // The slow pass (advection) reads no ghs, the fast pass no v.
  tile_issue(md, gd_in, iu_in, iv_in, t, given, PASS != kSlowPass, fuse ? md.td[TS_NEW] : nullptr);
  const int c = threadIdx.x % W, r0 = (threadIdx.x / W) * RPT;
  const bool cval = c < w.cols;
  const int ob = (w.j0 + r0) * N + w.i0 + c;  // the thread's first point
  // Operands fetched while the tile is in flight: the base level
  // (predict 2) or the previous tendency (correct).
  T pre[RPT][3];
  if (UF == UF_PREDICT_OUT || UF == UF_CORRECT) {
    T* const* src = UF == UF_PREDICT_OUT ? md.st[a.base_slot] : md.td[a.tprev];
#pragma unroll
    for (int k = 0; k < RPT; ++k)
#pragma unroll
      for (int f = 0; f < 3; ++f) pre[k][f] = (cval && r0 + k < w.rows) ? src[f][ob + k * N] : T(0);
  }
  if (fuse) tile_combine(md, a, w.member, t, 7);
  tile_derive(md, t, false, given, PASS != kFastPass);
  T* dst[3] = {nullptr, nullptr, nullptr};
  T* tdst[3] = {nullptr, nullptr, nullptr};
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    if (UF == UF_PREDICT_IN || UF == UF_PREDICT_OUT) dst[f] = md.st[a.out_slot][f];
    if (UF == UF_PREDICT_OUT || UF == UF_CORRECT) tdst[f] = md.td[a.tout][f];
  }
  const T h = em.h;
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int r = r0 + k;
    if (!cval || r >= w.rows) continue;
    const int j = w.j0 + r, o = ob + k * N;
    const int p = TL::pos(r + 1, c + 1);
    const TileView<T, TL> sv{t, p, j};
    T wu = T(0), wv = T(0);
    if (ADV == GDC_ADV_WENO && PASS != kFastPass) {
      wu = md.wadv[0][o];
      wv = md.wadv[1][o];
    }
    const T du = point_du<T, PASS, ADV>(sv, ub_lon, ub_lat, wu);
    const T dv = point_dv<T, PASS, ADV>(sv, ub_lon, ub_lat, wv);
    const T dg = point_dgd<T, PASS>(sv);
    if (UF == UF_PREDICT_IN) {
      // update_state from the input level (src/dycore_mod.F90:609-633)
      dst[F_IU][o] = t.iu[p] + h * du;
      dst[F_IV][o] = t.iv[p] + h * dv;
      dst[F_GD][o] = t.gd[p] + h * dg;
    } else if (UF == UF_PREDICT_OUT) {
      tdst[F_IU][o] = du;
      dst[F_IU][o] = pre[k][F_IU] + h * du;
      tdst[F_IV][o] = dv;
      dst[F_IV][o] = pre[k][F_IV] + h * dv;
      tdst[F_GD][o] = dg;
      dst[F_GD][o] = pre[k][F_GD] + h * dg;
    } else if (UF == UF_CORRECT) {
      // inner_product_tend_tend (src/types_mod.F90:347-372), same order
      // of terms as Emit::put
      const T wf = t.cf(TF_COS, j), wh = t.ch(TH_COS, j);
      tdst[F_IU][o] = du;
      em.ip_point(pre[k][F_IU], du, wf);
      tdst[F_IV][o] = dv;
      em.ip_point(pre[k][F_IV], dv, wh);
      tdst[F_GD][o] = dg;
      em.ip_point(pre[k][F_GD], dg, wf);
    } else {
      em.put(F_IU, o, du, t.cf(TF_COS, j), em.base_of(F_IU, o), em.prev_of(F_IU, o));
      em.put(F_IV, o, dv, t.ch(TH_COS, j), em.base_of(F_IV, o), em.prev_of(F_IV, o));
      em.put(F_GD, o, dg, t.cf(TF_COS, j), em.base_of(F_GD, o), em.prev_of(F_GD, o));
    }
  }
  em.ip_flush();
}

// ------------------------------------------------- column pairs (FP32)
// FP32 bulk tiles may advance two adjacent columns per thread: each stencil
// operand of the pair is one or two 8-byte shared loads instead of two
// 4-byte ones, the results go out as 8-byte stores, and the point
// operators run on F2 (component-wise float arithmetic, contracted to FMA
// as the scalar path is).  The values are the scalar path's.
#ifndef GDC_PAIR
#define GDC_PAIR 1
#endif

struct F2 {
  float x, y;
  F2() = default;
  __device__ __forceinline__ F2(float a) : x(a), y(a) {}
  __device__ __forceinline__ F2(float a, float b) : x(a), y(b) {}
  __device__ __forceinline__ explicit F2(double a) : x((float)a), y((float)a) {}
  __device__ __forceinline__ F2(int a) : x((float)a), y((float)a) {}
};
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return F2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return F2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return F2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ F2 operator/(F2 a, F2 b) { return F2(a.x / b.x, a.y / b.y); }
__device__ __forceinline__ F2 operator-(F2 a) { return F2(-a.x, -a.y); }
__device__ __forceinline__ F2 fabs(F2 a) { return F2(fabsf(a.x), fabsf(a.y)); }
__device__ __forceinline__ F2 ld2(const float* p) {
  const float2 v = *reinterpret_cast<const float2*>(p);
  return F2(v.x, v.y);
}
__device__ __forceinline__ void st2(float* p, F2 v) { *reinterpret_cast<float2*>(p) = make_float2(v.x, v.y); }

// Stencil view of a column pair: p is the (even) tile position of its
// first column; offsets dc = -1, 0, 1 come from the aligned pairs at
// p - 2, p, p + 2.
template <class TL>
struct TileView2 {
  const TL& t;
  int p, j;
  __device__ __forceinline__ F2 at(const float* a, int dr, int dc) const {
    const float* b = a + p + dr * TL::SW;
    const F2 c = ld2(b);
    if (dc == 0) return c;
    if (dc < 0) return F2(ld2(b - 2).y, c.x);
    return F2(c.y, ld2(b + 2).x);
  }
  __device__ __forceinline__ F2 u(int dr, int dc) const { return at(t.u, dr, dc); }
  __device__ __forceinline__ F2 v(int dr, int dc) const { return at(t.v, dr, dc); }
  __device__ __forceinline__ F2 iu(int dr, int dc) const { return at(t.iu, dr, dc); }
  __device__ __forceinline__ F2 iv(int dr, int dc) const { return at(t.iv, dr, dc); }
  __device__ __forceinline__ F2 ig(int dr, int dc) const { return at(t.ig, dr, dc); }
  __device__ __forceinline__ F2 gd(int dr, int dc) const { return at(t.gd, dr, dc); }
  __device__ __forceinline__ F2 ghs(int dr, int dc) const { return at(t.ghs, dr, dc); }
  __device__ __forceinline__ float cf(int k, int jj) const { return t.cf(k, jj); }
  __device__ __forceinline__ float ch(int k, int jj) const { return t.ch(k, jj); }
};

// bulk_tile for FP32 with column pairs: thread t owns columns c, c+1
// (c = 2 (t % (W/2))) of RPT consecutive rows.  Tile columns are even in
// number (num_lon and i0 are multiples of 4), so a pair never straddles a
// partial tile's edge.
template <int PASS, int ADV, int R, int W, int UF>
__device__ __forceinline__ void bulk_tile_pair(const MemberDev<float>& md, const StageArgs& a, const WorkItem& w,
                                               float* staging, bool given, const float* gd_in, const float* iu_in,
                                               const float* iv_in, float ub_lon, float ub_lat, Emit<float>& em) {
  using T = float;
  using TL = Tile<T, R, W>;
  constexpr int PW = W / 2, RPT = R * PW / kThreads;
  static_assert(RPT * kThreads == R * PW, "a tile is a whole number of pair rows per thread");
  const int N = md.N;
  TL t = carve<T, R, W>(staging, w.j0, w.i0, w.rows, w.cols);
  const bool fuse = UF == UF_PREDICT_IN && a.fuse;
  tile_issue(md, gd_in, iu_in, iv_in, t, given, PASS != kSlowPass, fuse ? md.td[TS_NEW] : nullptr);
  const int c = 2 * (threadIdx.x % PW), r0 = (threadIdx.x / PW) * RPT;
  const bool cval = c < w.cols;
  const int ob = (w.j0 + r0) * N + w.i0 + c;
  F2 pre[RPT][3];
  if (UF == UF_PREDICT_OUT || UF == UF_CORRECT) {
    T* const* src = UF == UF_PREDICT_OUT ? md.st[a.base_slot] : md.td[a.tprev];
#pragma unroll
    for (int k = 0; k < RPT; ++k)
#pragma unroll
      for (int f = 0; f < 3; ++f) pre[k][f] = (cval && r0 + k < w.rows) ? ld2(src[f] + ob + k * N) : F2(0.0f);
  }
  if (fuse) tile_combine(md, a, w.member, t, 7);
  tile_derive(md, t, false, given, PASS != kFastPass);
  T* dst[3] = {nullptr, nullptr, nullptr};
  T* tdst[3] = {nullptr, nullptr, nullptr};
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    if (UF == UF_PREDICT_IN || UF == UF_PREDICT_OUT) dst[f] = md.st[a.out_slot][f];
    if (UF == UF_PREDICT_OUT || UF == UF_CORRECT) tdst[f] = md.td[a.tout][f];
  }
  const F2 h(em.h);
  // All of the thread's tendencies first, then its stores: the stencil
  // values its rows share are loaded from shared memory once (a global
  // store between them would make the compiler load them again).
  F2 tdu[RPT], tdv[RPT], tdg[RPT];
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int r = r0 + k;
    const int j = w.j0 + r, o = ob + k * N;
    const int p = TL::pos(r + 1, c + 1);
    const TileView2<TL> sv{t, p, j};
    F2 wu(0.0f), wv(0.0f);
    if (ADV == GDC_ADV_WENO && PASS != kFastPass && cval && r < w.rows) {
      wu = ld2(md.wadv[0] + o);
      wv = ld2(md.wadv[1] + o);
    }
    tdu[k] = point_du<F2, PASS, ADV>(sv, F2(ub_lon), F2(ub_lat), wu);
    tdv[k] = point_dv<F2, PASS, ADV>(sv, F2(ub_lon), F2(ub_lat), wv);
    tdg[k] = point_dgd<F2, PASS>(sv);
  }
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int r = r0 + k;
    if (!cval || r >= w.rows) continue;
    const int j = w.j0 + r, o = ob + k * N;
    const int p = TL::pos(r + 1, c + 1);
    const F2 du = tdu[k], dv = tdv[k], dg = tdg[k];
    if (UF == UF_PREDICT_IN) {
      st2(dst[F_IU] + o, ld2(t.iu + p) + h * du);
      st2(dst[F_IV] + o, ld2(t.iv + p) + h * dv);
      st2(dst[F_GD] + o, ld2(t.gd + p) + h * dg);
    } else if (UF == UF_PREDICT_OUT) {
      st2(tdst[F_IU] + o, du);
      st2(dst[F_IU] + o, pre[k][F_IU] + h * du);
      st2(tdst[F_IV] + o, dv);
      st2(dst[F_IV] + o, pre[k][F_IV] + h * dv);
      st2(tdst[F_GD] + o, dg);
      st2(dst[F_GD] + o, pre[k][F_GD] + h * dg);
    } else if (UF == UF_CORRECT) {
      const T wf = t.cf(TF_COS, j), wh = t.ch(TH_COS, j);
      st2(tdst[F_IU] + o, du);
      st2(tdst[F_IV] + o, dv);
      st2(tdst[F_GD] + o, dg);
      // the scalar path's order of terms, point by point
      em.ip_point(pre[k][F_IU].x, du.x, wf);
      em.ip_point(pre[k][F_IV].x, dv.x, wh);
      em.ip_point(pre[k][F_GD].x, dg.x, wf);
      em.ip_point(pre[k][F_IU].y, du.y, wf);
      em.ip_point(pre[k][F_IV].y, dv.y, wh);
      em.ip_point(pre[k][F_GD].y, dg.y, wf);
    } else {
      const T wf = t.cf(TF_COS, j), wh = t.ch(TH_COS, j);
      em.put(F_IU, o, du.x, wf, em.base_of(F_IU, o), em.prev_of(F_IU, o));
      em.put(F_IV, o, dv.x, wh, em.base_of(F_IV, o), em.prev_of(F_IV, o));
      em.put(F_GD, o, dg.x, wf, em.base_of(F_GD, o), em.prev_of(F_GD, o));
      em.put(F_IU, o + 1, du.y, wf, em.base_of(F_IU, o + 1), em.prev_of(F_IU, o + 1));
      em.put(F_IV, o + 1, dv.y, wh, em.base_of(F_IV, o + 1), em.prev_of(F_IV, o + 1));
      em.put(F_GD, o + 1, dg.y, wf, em.base_of(F_GD, o + 1), em.prev_of(F_GD, o + 1));
    }
  }
  em.ip_flush();
}

// The bulk tile of a stage: column pairs for FP32 tiles whose pair count
// divides evenly among the threads, else one column per thread.
template <typename T, int PASS, int ADV, int R, int W, int UF>
__device__ __forceinline__ void bulk_tile_any(const MemberDev<T>& md, const StageArgs& a, const WorkItem& w,
                                              T* staging, bool given, const T* gd_in, const T* iu_in,
                                              const T* iv_in, T ub_lon, T ub_lat, Emit<T>& em) {
  if constexpr (GDC_PAIR && sizeof(T) == 4 && (R * W / 2) % kThreads == 0)
    bulk_tile_pair<PASS, ADV, R, W, UF>(md, a, w, staging, given, gd_in, iu_in, iv_in, ub_lon, ub_lat, em);
  else
    bulk_tile<T, PASS, ADV, R, W, UF>(md, a, w, staging, given, gd_in, iu_in, iv_in, ub_lon, ub_lat, em);
}

// ------------------------------------------------------------ warp strips
// One warp advances one strip: output columns i0..i0+cols-1 (cols <= 30) of
// rows j0..j0+rows-1, all ordinary.  Lane L holds column i0-1+L (mod N) of
// every field for the rows j-1, j, j+1 around the output row j in
// registers; east and west neighbours come by shuffles, so the strip needs
// no shared memory and no block barrier.  Lanes 1..cols emit.

template <typename T, bool GIVEN>
struct StripRaw;  // one row of one column as loaded (off the sphere: 0)
template <typename T>
struct StripRaw<T, false> {
  T gd, ghs, iu, iv, gdx, ig;  // gdx: gd one column east (lane 31 only)
};
template <typename T>
struct StripRaw<T, true> {
  T gd, ghs, iu, iv, gdx, ig, gu, gv;  // gu, gv: the level's given u, v
};
template <typename T>
struct StripRow {  // a row with its derived iap gd, u and v
  T gd, ghs, iu, iv, ig, u, v;
};

// Coefficients come by shuffles: lanes 0..15 hold the record of row j,
// lanes 16..31 that of row j+1; the one row j-1 coefficient the operators
// read (half-row cos) is carried from the previous row.  Every lane must
// evaluate the operators (shuffles need the whole warp).
template <typename T>
struct StripView {
  int j;
  T rec;       // this lane's coefficient record word
  T cos_prev;  // ch(TH_COS, j - 1)
  T u_[3][3], v_[3][3], iu_[3][3], iv_[3][3], ig_[3][3], gd_[3][3], ghs_[3][3];
  __device__ __forceinline__ T u(int dr, int dc) const { return u_[dr + 1][dc + 1]; }
  __device__ __forceinline__ T v(int dr, int dc) const { return v_[dr + 1][dc + 1]; }
  __device__ __forceinline__ T iu(int dr, int dc) const { return iu_[dr + 1][dc + 1]; }
  __device__ __forceinline__ T iv(int dr, int dc) const { return iv_[dr + 1][dc + 1]; }
  __device__ __forceinline__ T ig(int dr, int dc) const { return ig_[dr + 1][dc + 1]; }
  __device__ __forceinline__ T gd(int dr, int dc) const { return gd_[dr + 1][dc + 1]; }
  __device__ __forceinline__ T ghs(int dr, int dc) const { return ghs_[dr + 1][dc + 1]; }
  __device__ __forceinline__ T cf(int k, int jj) const { return coef(k, jj); }
  __device__ __forceinline__ T ch(int k, int jj) const { return coef(k, jj); }
  __device__ __forceinline__ T coef(int k, int jj) const {
    if (jj == j - 1) return cos_prev;  // k == TH_COS
    return __shfl_sync(0xffffffffu, rec, (jj == j ? 0 : kRecWords) + k);
  }
};

template <typename T>
__device__ __forceinline__ T shfl_dn(T x) {
  return __shfl_down_sync(0xffffffffu, x, 1);
}
template <typename T>
__device__ __forceinline__ T shfl_up(T x) {
  return __shfl_up_sync(0xffffffffu, x, 1);
}

// Per-warp constants of a strip.
template <typename T>
struct StripCtx {
  int c, cx, N, M, Mh;
  bool east;
  const T* __restrict__ gd;
  const T* __restrict__ ghs;
  const T* __restrict__ iu;
  const T* __restrict__ iv;
  const T* __restrict__ gu;
  const T* __restrict__ gv;
};

template <typename T, bool GIVEN>
__device__ __forceinline__ StripRaw<T, GIVEN> strip_load(const StripCtx<T>& x, int r) {
  StripRaw<T, GIVEN> q;
  const bool vf = r >= 0 && r < x.M, vh = r >= 0 && r < x.Mh;
  const int o = r * x.N + x.c;
  q.gd = vf ? x.gd[o] : T(0);
  q.ghs = vf ? x.ghs[o] : T(0);
  q.iu = vf ? x.iu[o] : T(0);
  q.iv = vh ? x.iv[o] : T(0);
  q.gdx = (vf && x.east) ? x.gd[r * x.N + x.cx] : T(0);
  q.ig = T(0);
  if constexpr (GIVEN) {
    q.gu = vf ? x.gu[o] : T(0);
    q.gv = vh ? x.gv[o] : T(0);
  }
  return q;
}

// Derive row r (raw a, iap gd already set) given the iap gd of row r+1.
template <typename T, bool GIVEN>
__device__ __forceinline__ StripRow<T> strip_derive(const StripCtx<T>& x, const StripRaw<T, GIVEN>& a, T ig_next,
                                                    int r) {
  StripRow<T> d;
  d.gd = a.gd;
  d.ghs = a.ghs;
  d.iu = a.iu;
  d.iv = a.iv;
  d.ig = a.ig;
  if constexpr (GIVEN) {
    d.u = a.gu;
    d.v = a.gv;
  } else {
    const T ige = shfl_dn(a.ig);  // iap gd one column east
    const T ig_e = x.east ? sqrt(a.gdx) : ige;
    d.u = (r >= 1 && r <= x.M - 2) ? a.iu * T(2) / (a.ig + ig_e) : T(0);
    d.v = (r >= 0 && r < x.Mh) ? a.iv * T(2) / (a.ig + ig_next) : T(0);
  }
  return d;
}

template <typename T, int PASS, int ADV, int UF, bool GIVEN>
__device__ void strip_warp(const MemberDev<T>& md, const WorkItem& w, const StageArgs& a) {
  using Raw = StripRaw<T, GIVEN>;
  const int lane = threadIdx.x & 31;
  StripCtx<T> x;
  x.N = md.N;
  x.M = md.M;
  x.Mh = md.Mh;
  const int N = x.N;
  x.c = ((w.i0 - 1 + lane) % N + N) % N;
  x.cx = x.c + 1 < N ? x.c + 1 : 0;
  x.east = lane == 31;
  x.gd = md.st[a.in_slot][F_GD];
  x.iu = md.st[a.in_slot][F_IU];
  x.iv = md.st[a.in_slot][F_IV];
  x.ghs = md.ghs;
  x.gu = md.given_u;
  x.gv = md.given_v;
  const int c = x.c;
  const bool emit = lane >= 1 && lane <= w.cols;
  Emit<T> em(md, a, T(md.pcdt[PASS] * a.h_scale));
  const T ub_lon = T(a.ub_lon), ub_lat = T(a.ub_lat);
  const T h = em.h;
  T* dst[3] = {nullptr, nullptr, nullptr};
  T* tdst[3] = {nullptr, nullptr, nullptr};
  const T* src[3] = {nullptr, nullptr, nullptr};
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    if (UF == UF_PREDICT_IN || UF == UF_PREDICT_OUT) dst[f] = md.st[a.out_slot][f];
    if (UF == UF_PREDICT_OUT || UF == UF_CORRECT) tdst[f] = md.td[a.tout][f];
    if (UF == UF_PREDICT_OUT) src[f] = md.st[a.base_slot][f];
    if (UF == UF_CORRECT) src[f] = md.td[a.tprev][f];
  }
  // Member fields the loop reads, in registers: the stores below could
  // otherwise alias the descriptor and force reloads.
  const T* __restrict__ rc = md.rowc;
  const int j0 = w.j0, jend = w.j0 + w.rows;  // output rows j0..jend-1
  // Window: rows j0-1, j0, j0+1 derived; raw rows j0+2, j0+3 in hand (the
  // loads of a row are issued two iterations before its derivation).
  Raw r0 = strip_load<T, GIVEN>(x, j0 - 1);
  Raw r1 = strip_load<T, GIVEN>(x, j0);
  Raw r2 = strip_load<T, GIVEN>(x, j0 + 1);
  Raw p1 = strip_load<T, GIVEN>(x, j0 + 2);
  Raw p2 = strip_load<T, GIVEN>(x, j0 + 3);
  T pre[3] = {T(0), T(0), T(0)};
  if (UF == UF_PREDICT_OUT || UF == UF_CORRECT) {
#pragma unroll
    for (int f = 0; f < 3; ++f) pre[f] = emit ? src[f][j0 * N + c] : T(0);
  }
  r0.ig = sqrt(r0.gd);
  r1.ig = sqrt(r1.gd);
  r2.ig = sqrt(r2.gd);
  p1.ig = sqrt(p1.gd);
  StripRow<T> d0 = strip_derive<T, GIVEN>(x, r0, r1.ig, j0 - 1);
  StripRow<T> d1 = strip_derive<T, GIVEN>(x, r1, r2.ig, j0);
  StripRow<T> d2 = strip_derive<T, GIVEN>(x, r2, p1.ig, j0 + 1);
  T d0_v_e = shfl_dn(d0.v), d0_iv_e = shfl_dn(d0.iv);  // row j-1, one column east
  T d1_u_w = shfl_up(d1.u), d1_iu_w = shfl_up(d1.iu);  // row j, one column west
  // Coefficient records of rows j, j+1 (one word per lane), of j+1, j+2
  // for the next row, and the half-row cos of row j-1.
  static_assert(2 * kRecWords == 32, "two records per warp");
  T rec = __ldg(rc + (j0 + 1) * kRecWords + lane);
  T cos_prev = __ldg(rc + j0 * kRecWords + TH_COS);
  for (int j = j0; j < jend; ++j) {
    // Loads for later rows: raw row j+4, update operands of row j+1.
    Raw q;
    if (j + 4 <= jend + 1)
      q = strip_load<T, GIVEN>(x, j + 4);
    else
      q = Raw{};
    const T rec_next = j + 1 < jend ? __ldg(rc + (j + 2) * kRecWords + lane) : T(0);
    T pre_next[3] = {T(0), T(0), T(0)};
    if (UF == UF_PREDICT_OUT || UF == UF_CORRECT) {
      if (j + 1 < jend && emit) {
#pragma unroll
        for (int f = 0; f < 3; ++f) pre_next[f] = src[f][(j + 1) * N + c];
      }
    }
    StripView<T> s;
    s.j = j;
    s.rec = rec;
    s.cos_prev = cos_prev;
    // row j-1
    s.v_[0][1] = d0.v;
    s.v_[0][2] = d0_v_e;
    s.iu_[0][1] = d0.iu;
    s.iv_[0][1] = d0.iv;
    s.iv_[0][2] = d0_iv_e;
    s.ig_[0][1] = d0.ig;
    // row j
    s.u_[1][0] = d1_u_w;
    s.u_[1][1] = d1.u;
    s.u_[1][2] = shfl_dn(d1.u);
    s.v_[1][1] = d1.v;
    s.v_[1][2] = shfl_dn(d1.v);
    s.iu_[1][0] = d1_iu_w;
    s.iu_[1][1] = d1.iu;
    s.iu_[1][2] = shfl_dn(d1.iu);
    s.iv_[1][0] = shfl_up(d1.iv);
    s.iv_[1][1] = d1.iv;
    s.iv_[1][2] = shfl_dn(d1.iv);
    s.ig_[1][0] = shfl_up(d1.ig);
    s.ig_[1][1] = d1.ig;
    s.ig_[1][2] = shfl_dn(d1.ig);
    s.gd_[1][1] = d1.gd;
    s.gd_[1][2] = shfl_dn(d1.gd);
    s.ghs_[1][1] = d1.ghs;
    s.ghs_[1][2] = shfl_dn(d1.ghs);
    // row j+1
    const T d2_u_w = shfl_up(d2.u), d2_iu_w = shfl_up(d2.iu);
    s.u_[2][0] = d2_u_w;
    s.u_[2][1] = d2.u;
    s.v_[2][1] = d2.v;
    s.iu_[2][0] = d2_iu_w;
    s.iu_[2][1] = d2.iu;
    s.iv_[2][1] = d2.iv;
    s.ig_[2][1] = d2.ig;
    s.gd_[2][1] = d2.gd;
    s.ghs_[2][1] = d2.ghs;
    const T du = point_du<T, PASS, ADV>(s, ub_lon, ub_lat);
    const T dv = point_dv<T, PASS, ADV>(s, ub_lon, ub_lat);
    const T dg = point_dgd<T, PASS>(s);
    const T wf = s.cf(TF_COS, j), wh = s.ch(TH_COS, j);
    if (emit) {
      const int o = j * N + c;
      if (UF == UF_PREDICT_IN) {
        dst[F_IU][o] = d1.iu + h * du;
        dst[F_IV][o] = d1.iv + h * dv;
        dst[F_GD][o] = d1.gd + h * dg;
      } else if (UF == UF_PREDICT_OUT) {
        tdst[F_IU][o] = du;
        dst[F_IU][o] = pre[F_IU] + h * du;
        tdst[F_IV][o] = dv;
        dst[F_IV][o] = pre[F_IV] + h * dv;
        tdst[F_GD][o] = dg;
        dst[F_GD][o] = pre[F_GD] + h * dg;
      } else if (UF == UF_CORRECT) {
        tdst[F_IU][o] = du;
        em.ip_point(pre[F_IU], du, wf);
        tdst[F_IV][o] = dv;
        em.ip_point(pre[F_IV], dv, wh);
        tdst[F_GD][o] = dg;
        em.ip_point(pre[F_GD], dg, wf);
      } else {
        em.put(F_IU, o, du, wf, em.base_of(F_IU, o), em.prev_of(F_IU, o));
        em.put(F_IV, o, dv, wh, em.base_of(F_IV, o), em.prev_of(F_IV, o));
        em.put(F_GD, o, dg, wf, em.base_of(F_GD, o), em.prev_of(F_GD, o));
      }
    }
    em.ip_flush();  // one row of the strip
    cos_prev = wh;
    rec = rec_next;
    // Advance the window by one row: derive row j+2 (raw p1, with the iap
    // gd of row j+3 from p2).
    p2.ig = sqrt(p2.gd);
    const StripRow<T> d3 = strip_derive<T, GIVEN>(x, p1, p2.ig, j + 2);
    d0_v_e = s.v_[1][2];
    d0_iv_e = s.iv_[1][2];
    d1_u_w = d2_u_w;
    d1_iu_w = d2_iu_w;
    d0 = d1;
    d1 = d2;
    d2 = d3;
    p1 = p2;
    p2 = q;
#pragma unroll
    for (int f = 0; f < 3; ++f) pre[f] = pre_next[f];
  }
  if (a.do_ip) {
    warp_acc(em.ip1);
    warp_acc(em.ip2);
    if (lane == 0) {
      double* pp = a.partials + 4 * (size_t)w.pidx;
      pp[0] = (double)em.ip1.s;
      pp[1] = (double)em.ip1.c;
      pp[2] = (double)em.ip2.s;
      pp[3] = (double)em.ip2.c;
    }
  }
}

template <typename T, int PASS, int ADV, int UF>
__device__ __forceinline__ void strip_item(const MemberDev<T>& md, const WorkItem& w, const StageArgs& a) {
  // u, v supplied with this level (initial condition, diffusion): used as
  // given, as the reference's space_operators reads state%u / state%v.
  const bool given = a.uvslot && a.uvslot[w.member] == a.in_slot;
  if (a.uvslot && a.out_slot >= 0 && (threadIdx.x & 31) == 0 && a.uvslot[w.member] == a.out_slot)
    a.uvslot[w.member] = -1;  // level overwritten: u, v derived from now on
  if (given)
    strip_warp<T, PASS, ADV, UF, true>(md, w, a);
  else
    strip_warp<T, PASS, ADV, UF, false>(md, w, a);
}

// The end of a whole-row task for field f once the row's raw tendency is in
// shared memory (x, N values): the pole cap of dgd (from the FP64 sum `cap`
// of this block), the zonal filter of that field, and its update.
template <typename T, int PASS>
__device__ void row_tail(const MemberDev<T>& md, const StageArgs& a, Emit<T>& em, int j, int f, T* x,
                         const Acc<double>& cap, T* coefs, T* redT, const T* gd_in, const T* iu_in,
                         const T* iv_in, const T* tw, RowPair pr) {
  const int N = md.N, M = md.M, Mh = md.Mh;
  const int info = md.rowinfo[j];
  const bool has_du = (j >= 1 && j <= M - 2);
  const bool south = (j == 0), north = (j == M - 1);
  if (f == F_GD && (south || north) && PASS != kSlowPass) {
    double* redD = reinterpret_cast<double*>(redT + 64);
    double s = block_value(cap, redD);
    if (north) s = -s;
    s = s * 2.0 / N / kRadius / (kPi / Mh);
    // dgd = - mass_div_lon - mass_div_lat with mass_div_lon = 0 at poles
    const T val = T(-0.0) - T(s);
    for (int i = threadIdx.x; i < N; i += blockDim.x) x[i] = val;
    __syncthreads();
  }
  const size_t ro = (size_t)j * N;
  if (f == F_IU && has_du && (info & RI_FLAG_FULL))
    filter_rescale(md, x, iu_in + ro, (const T*)nullptr, ri_keep_full(info), coefs, redT, a.rescale_rtol, tw, pr);
  if (f == F_IV && (info & RI_FLAG_HALF))
    filter_rescale(md, x, iv_in + ro, (const T*)nullptr, ri_keep_half(info), coefs, redT, a.rescale_rtol, tw, pr);
  if (f == F_GD && PASS != kSlowPass && (info & RI_FLAG_FULL))
    filter_rescale(md, x, gd_in + ro, md.ghs + ro, ri_keep_full(info), coefs, redT, a.rescale_rtol, tw, pr);
  const T w = f == F_IV ? ch(md, CH_COS, j) : cf(md, CF_COS, j);
  // a block of a pair updates its half of the row (num_lon is a multiple of 4)
  const int i_end = pr.on ? (pr.part + 1) * (N / 2) : N;
  for (int i = (pr.on ? pr.part * (N / 2) : 0) + threadIdx.x; i < i_end; i += blockDim.x) {
    const size_t o = ro + i;
    // du is 0 on pole rows (never assigned by the reference); inner
    // products skip pole-row du (src/types_mod.F90:355).
    if (f == F_IU && !has_du)
      em.put(F_IU, o, T(0), T(0), em.base_of(F_IU, o), T(0));
    else
      em.put(f, o, x[i], w, em.base_of(f, o), em.prev_of(f, o));
  }
  em.ip_flush();
}

template <typename T>
struct StageOcc {
  static constexpr int kMinBlocks = sizeof(T) == 4 ? GDC_STAGE_BLOCKS : 2;
};

// One work item of a stage (a bulk tile or a whole-row task), by the block.
template <typename T, int PASS, int ADV, int R, int W>
__device__ __forceinline__ void stage_item(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl,
                                           const StageArgs& a, unsigned char* smem_raw, int staging_words,
                                           int max_n) {
  const WorkItem w = wl[blockIdx.x];
  if (w.kind > 1) return;  // padding of a paired launch to an even count
  // A whole-row task split over a block pair (two consecutive items, parts
  // 0 and 1, the pair's blocks of one cluster).  Both blocks decide alike
  // (from the two items and the launch), so both or neither take the
  // cluster barriers; an item whose partner is not there (a launch without
  // clusters) is done whole by part 0, and part 1 contributes nothing.
  RowPair pr;
  if constexpr (sizeof(T) == 8) {  // FP64 only: FP32 launches have many items per SM
  if (w.kind == 1 && w.rows == 2) {
    bool paired = false;
    if (a.pair && (int)cooperative_groups::this_cluster().num_blocks() == 2) {
      const WorkItem q = wl[blockIdx.x ^ 1];
      paired = q.kind == 1 && q.rows == 2 && q.member == w.member && q.j0 == w.j0 && q.field == w.field &&
               q.i0 == (w.i0 ^ 1) && (int)(blockIdx.x & 1) == w.i0;
    }
    if (paired) {
      pr.on = true;
      pr.part = w.i0;
    } else if (w.i0 == 1) {
      if (a.do_ip && threadIdx.x == 0) {
        double* pp = a.partials + 4 * (size_t)w.pidx;
        pp[0] = pp[1] = pp[2] = pp[3] = 0.0;
      }
      return;
    }
  }
  }
  T* staging = reinterpret_cast<T*>(smem_raw);  // bulk tile, or the row task's tile, then:
  T* rows = staging + row_task_words<T>();      // 3 * max_n (row tasks)
  T* coefs = rows + 3 * max_n;                  // max_n (a row keeps at most num_lon)
  T* tw = coefs + max_n;                        // 2 * max_n twiddles
  T* redT = staging + staging_words;            // 64, then 64 doubles
  // The member descriptor is read in place (read-only, L1-cached): copying
  // it to shared memory cost a barrier per block.
  const MemberDev<T>& md = mems[w.member];
  const int N = md.N, M = md.M, Mh = md.Mh;
  // A fused final update stages its base level (and forms in_slot from it).
  const bool fuse = a.fuse && a.form == UF_PREDICT_IN;
  const int src_slot = fuse ? a.fin_base : a.in_slot;
  const T* gd_in = md.st[src_slot][F_GD];
  const T* iu_in = md.st[src_slot][F_IU];
  const T* iv_in = md.st[src_slot][F_IV];
  const double hstep = md.pcdt[PASS] * a.h_scale;
  Emit<T> em(md, a, T(hstep));
  const T ub_lon = T(a.ub_lon), ub_lat = T(a.ub_lat);
  // u, v supplied with this level (initial condition, diffusion): used as
  // given, as the reference's space_operators reads state%u / state%v.  A
  // level formed by a fused update is never given: u, v derived from now on.
  const bool given = !fuse && a.uvslot && a.uvslot[w.member] == a.in_slot;
  if (a.uvslot && threadIdx.x == 0) {
    const int g = a.uvslot[w.member];
    if ((a.out_slot >= 0 && g == a.out_slot) || (fuse && g == a.in_slot))
      a.uvslot[w.member] = -1;  // level overwritten: u, v derived from now on
  }

  if (w.kind == 0) {
    // ---------------- bulk tile: rows j0..j0+R-1 are ordinary rows
#define GDC_BULK(F)                                                                                   \
  bulk_tile_any<T, PASS, ADV, R, W, F>(md, a, w, staging, given, gd_in, iu_in, iv_in, ub_lon, ub_lat, em); \
  break;
    switch (a.form) {
      case UF_PREDICT_IN:
        GDC_BULK(UF_PREDICT_IN)
      case UF_PREDICT_OUT:
        GDC_BULK(UF_PREDICT_OUT)
      case UF_CORRECT:
        GDC_BULK(UF_CORRECT)
      default:
        GDC_BULK(UF_GENERAL)
    }
#undef GDC_BULK
  } else {
    // ---------------- whole-row task: row j (full row j for gd and iap u,
    // half row j for iap v), field w.field or all three (w.field < 0)
    const int j = w.j0, f = w.field;
    twiddles_to_shared(md, tw);
    const bool has_du = (j >= 1 && j <= M - 2);
    const bool has_dv = (j <= Mh - 1);
    const bool south = (j == 0), north = (j == M - 1);
    const bool want_u = f < 0 || f == F_IU, want_v = has_dv && (f < 0 || f == F_IV), want_g = f < 0 || f == F_GD;
    T* xr[3] = {rows + 2 * max_n, rows, rows + max_n};  // by field: gd, iap u, iap v
    if (f >= 0) xr[f] = rows;
    // A pair splits the columns of a row without a pole cap: each block
    // computes the raw tendencies of its columns (split at a multiple of 4,
    // the staging copies' alignment) into its own and its partner's rows.
    const bool split_cols = pr.on && !south && !north;
    T* rx[3] = {nullptr, nullptr, nullptr};
    int cb = 0, ce = N;
    if (split_cols) {
      cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
      cl.sync();  // the partner has started
      const int other = (int)cl.block_rank() ^ 1;
      for (int q = 0; q < 3; ++q) rx[q] = cl.map_shared_rank(xr[q], other);
      const int sp = (N / 2) & ~3;
      cb = pr.part ? sp : 0;
      ce = pr.part ? N : sp;
    }
    Acc<double> cap;
    using TR = Tile<T, 1, kRowChunk>;
    for (int c0 = cb; c0 < ce; c0 += kRowChunk) {
      const int vw = min(kRowChunk, ce - c0);
      TR t = carve<T, 1, kRowChunk>(staging, j, c0, 1, vw);
      __syncthreads();
      tile_issue(md, gd_in, iu_in, iv_in, t, given, PASS != kSlowPass, fuse ? md.td[TS_NEW] : nullptr);
      if (fuse) tile_combine(md, a, w.member, t, f < 0 ? 7 : (1 << f));
      // only the rows this task's field reads
      tile_derive(md, t, false, given, PASS != kFastPass, row_task_rows(PASS, f));
      for (int c = threadIdx.x; c < vw; c += blockDim.x) {
        const int p = TR::pos(1, c + 1);
        const int i = c0 + c;
        const TileView<T, TR> sv{t, p, j};
        const bool wl = ADV == GDC_ADV_WENO && PASS != kFastPass;
        if (want_u) {
          const T x = has_du ? point_du<T, PASS, ADV>(sv, ub_lon, ub_lat, wl ? md.wadv[0][j * N + i] : T(0)) : T(0);
          xr[F_IU][i] = x;
          if (split_cols) rx[F_IU][i] = x;
        }
        if (want_v) {
          const T x = point_dv<T, PASS, ADV>(sv, ub_lon, ub_lat, wl ? md.wadv[1][j * N + i] : T(0));
          xr[F_IV][i] = x;
          if (split_cols) rx[F_IV][i] = x;
        }
        if (!want_g) continue;
        if (south || north) {
          // src/dycore_mod.F90:572-596: sp += (ig(j)+ig(j+1)) iv(j);
          // np -= (ig(j)+ig(j-1)) iv(j-1).  Terms and sum in FP64.
          if (PASS != kSlowPass) {
            if (south)
              cap.add(((double)t.ig[p] + (double)t.ig[p + TR::SW]) * (double)t.iv[p]);
            else
              cap.add(((double)t.ig[p] + (double)t.ig[p - TR::SW]) * (double)t.iv[p - TR::SW]);
          }
          xr[F_GD][i] = T(0);
        } else {
          const T x = point_dgd<T, PASS>(sv);
          xr[F_GD][i] = x;
          if (split_cols) rx[F_GD][i] = x;
        }
      }
    }
    if (split_cols)
      cooperative_groups::this_cluster().sync();  // both halves in both blocks' rows
    else
      __syncthreads();
    // The filter's weights are the input level: with a fused update, the
    // level this block has just formed and written for its own field(s) of
    // row j (visible to the block after the barrier above).
    const T* wg = fuse ? md.st[a.in_slot][F_GD] : gd_in;
    const T* wu = fuse ? md.st[a.in_slot][F_IU] : iu_in;
    const T* wv = fuse ? md.st[a.in_slot][F_IV] : iv_in;
    if (want_u) row_tail<T, PASS>(md, a, em, j, F_IU, xr[F_IU], cap, coefs, redT, wg, wu, wv, tw, pr);
    if (want_v) row_tail<T, PASS>(md, a, em, j, F_IV, xr[F_IV], cap, coefs, redT, wg, wu, wv, tw, pr);
    if (want_g) row_tail<T, PASS>(md, a, em, j, F_GD, xr[F_GD], cap, coefs, redT, wg, wu, wv, tw, pr);
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

// A stage launch: one block per work item (clusters of two blocks when
// StageArgs::pair: then whole-row tasks may be split over a pair).
template <typename T, int PASS, int ADV, int R, int W>
__global__ void __launch_bounds__(kThreads, StageOcc<T>::kMinBlocks)
    stage_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl, StageArgs a,
                 int staging_words, int max_n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_item<T, PASS, ADV, R, W>(mems, wl, a, smem_raw, staging_words, max_n);
}

// Warp strips, one per warp (items cover every row of their members).
template <typename T>
struct StripOcc {
  static constexpr int kMinBlocks = sizeof(T) == 4 ? GDC_STRIP_BLOCKS : 2;
};

template <typename T, int PASS, int ADV>
__global__ void __launch_bounds__(kThreads, StripOcc<T>::kMinBlocks)
    strip_kernel(const MemberDev<T>* __restrict__ mems, const WorkItem* __restrict__ wl, int nitems, StageArgs a) {
  const int item = (int)blockIdx.x * (kThreads / 32) + (int)(threadIdx.x >> 5);
  if (item >= nitems) return;
  const WorkItem w = wl[item];
  const MemberDev<T>& md = mems[w.member];
  switch (a.form) {
    case UF_PREDICT_IN:
      strip_item<T, PASS, ADV, UF_PREDICT_IN>(md, w, a);
      break;
    case UF_PREDICT_OUT:
      strip_item<T, PASS, ADV, UF_PREDICT_OUT>(md, w, a);
      break;
    case UF_CORRECT:
      strip_item<T, PASS, ADV, UF_CORRECT>(md, w, a);
      break;
    default:
      strip_item<T, PASS, ADV, UF_GENERAL>(md, w, a);
  }
}

// beta of predict_correct (src/dycore_mod.F90:784-786) or isp (:743-746),
// one block per member over that member's partials.
// beta of member slot s from its md.pcount partials (src/dycore_mod.F90:
// 784-787; isp :743-747), reduced by the whole block in a fixed order.
// FP64: double-double (the oracle's correctly rounded sums); FP32: the
// partials carry FP32 rounding, a plain FP64 sum loses nothing.
// The two sums over a member's partial slots (4 doubles each: two
// accumulators as value and compensation) by one warp.  A member has one
// slot per work item -- tens to a few hundred -- and in FP64 every further
// warp's share of the merge tree is FP64 work on the SM's narrow FP64 pipe.
template <typename A>
__device__ void warp_partials(const double* partials, int base, int count, A& a1, A& a2) {
  for (int q = threadIdx.x & 31; q < count; q += 32) {
    const double* pp = partials + 4 * (size_t)(base + q);
    a1.merge(pp[0], pp[1]);
    a2.merge(pp[2], pp[3]);
  }
  warp_acc(a1);
  warp_acc(a2);
}

// The partial sums of a member: one warp in FP64 (double-double merges on
// the narrow FP64 pipe), the whole block in FP32 (plain FP64 merges: the
// latency of a longer serial merge per lane is what counts there).
template <typename T, typename A>
__device__ void member_partials(const double* partials, int base, int count, A& a1, A& a2) {
  if constexpr (sizeof(T) == 8) {
    warp_partials(partials, base, count, a1, a2);
  } else {
    __shared__ double red[64];
    for (int q = threadIdx.x; q < count; q += blockDim.x) {
      const double* pp = partials + 4 * (size_t)(base + q);
      a1.merge(pp[0], pp[1]);
      a2.merge(pp[2], pp[3]);
    }
    a1 = block_acc(a1, red);
    a2 = block_acc(a2, red);
  }
}
// Threads of a beta or diag_finalize block.
template <typename T>
constexpr int partial_threads() { return sizeof(T) == 8 ? 32 : kThreads; }

template <typename T>
__device__ void member_beta(const MemberDev<T>& md, int s, const double* partials, double* beta, int qcon,
                            int beta_mode) {
  typename DiagAcc<T>::type a1, a2;
  member_partials<T>(partials, md.pbase, md.pcount, a1, a2);
  const double ip1 = a1.value(), ip2 = a2.value();
  if (threadIdx.x == 0) {
    double b;
    if (sizeof(T) == 4 && beta_mode == 0) {
      // FP32 partials carry d = <T_old - T_new, T_new> (Emit::ip_point):
      // <T_old, T_new> = ip2 + d and beta = 1 + d / ip2.
      b = (qcon && ip2 + ip1 != 0.0 && ip2 != 0.0) ? 1.0 + ip1 / ip2 : 1.0;
    } else {
      b = (qcon && ip1 != 0.0 && ip2 != 0.0) ? ip1 / ip2 : 1.0;
    }
    if (beta_mode == 1) b = b * 4.0 / md.dt;
    beta[s] = b;
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    beta_kernel(const MemberDev<T>* __restrict__ mems, const int* __restrict__ slots, const double* partials,
                double* beta, int qcon, int beta_mode) {
  const int s = slots[blockIdx.x];
  member_beta<T>(mems[s], s, partials, beta, qcon, beta_mode);
}

// ------------------------------------------------------ final update
// update_state(time_step_size * beta, tend(new), state(old), state(new))
// (src/dycore_mod.F90:789-790) over every point of the member.  FP32 time
// levels carry a compensation word: new = (hi + lo) + dt*T via TwoSum.


// One flat item: a contiguous run of one field, 16 bytes per access.  All
// of a thread's loads are issued before its first store.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    final_kernel(const MemberDev<T>* __restrict__ mems, const FlatItem* __restrict__ fl, FinalArgs a) {
  using V = typename Vec16<T>::type;
  constexpr int VEC = 16 / (int)sizeof(T), U = flat_chunk<T>() / (VEC * kThreads);
  const FlatItem w = fl[blockIdx.x];
  const MemberDev<T>& md = mems[w.member];
  double hstep = md.pcdt[a.pass] * a.h_scale;
  if (a.beta) hstep = md.pcdt[a.pass] * a.h_scale * a.beta[w.member];
  // This level's u, v are derived from its new state from now on.
  if (a.uvslot && threadIdx.x == 0 && w.field == 0 && w.begin == 0 && a.uvslot[w.member] == a.out_slot)
    a.uvslot[w.member] = -1;
  const int f = w.field, nv = w.count / VEC;
  const T h = T(hstep);
  const V* __restrict__ tv = reinterpret_cast<const V*>(md.td[a.tslot][f] + w.begin);
  const V* __restrict__ hi = reinterpret_cast<const V*>(md.st[a.base_slot][f] + w.begin);
  V* __restrict__ out = reinterpret_cast<V*>(md.st[a.out_slot][f] + w.begin);
  V x[U], t[U], l[U];
#pragma unroll
  for (int k = 0; k < U; ++k) {
    const int q = threadIdx.x + k * kThreads;
    if (q < nv) {
      x[k] = hi[q];
      t[k] = tv[q];
    }
  }
  if (a.use_lo) {
    const V* __restrict__ lo = reinterpret_cast<const V*>(md.lo[a.base_slot][f] + w.begin);
    V* __restrict__ olo = reinterpret_cast<V*>(md.lo[a.out_slot][f] + w.begin);
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int q = threadIdx.x + k * kThreads;
      if (q < nv) l[k] = lo[q];
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int q = threadIdx.x + k * kThreads;
      if (q >= nv) continue;
      V sv, ev;
      const T* xs = reinterpret_cast<const T*>(&x[k]);
      const T* ls = reinterpret_cast<const T*>(&l[k]);
      const T* ts = reinterpret_cast<const T*>(&t[k]);
      T* ss = reinterpret_cast<T*>(&sv);
      T* es = reinterpret_cast<T*>(&ev);
#pragma unroll
      for (int m = 0; m < VEC; ++m) {
        const T y = ls[m] + h * ts[m];
        const T sum = xs[m] + y;
        const T bp = sum - xs[m];
        ss[m] = sum;
        es[m] = (xs[m] - (sum - bp)) + (y - bp);
      }
      out[q] = sv;
      olo[q] = ev;
    }
  } else {
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int q = threadIdx.x + k * kThreads;
      if (q >= nv) continue;
      V sv;
      const T* xs = reinterpret_cast<const T*>(&x[k]);
      const T* ts = reinterpret_cast<const T*>(&t[k]);
      T* ss = reinterpret_cast<T*>(&sv);
#pragma unroll
      for (int m = 0; m < VEC; ++m) ss[m] = xs[m] + h * ts[m];
      out[q] = sv;
    }
  }
}

// ------------------------------------------------------------- diag
// diag_run totals (src/diag_mod.F90:301-317, 98-121) in FP64.

// One row j of the diag sums, by one warp.  FP64 members add the weighted
// point terms in double-double (as the oracle's exact sums); FP32 members
// sum each row's unweighted terms in float-float (the state is hi + lo) and
// apply the row's FP64 weights once per row.
struct FF {
  float hi = 0.f, lo = 0.f;
  __device__ void add(float x) {
    const float t = hi + x;
    const float bp = t - hi;
    lo += (hi - (t - bp)) + (x - bp);
    hi = t;
  }
  __device__ void add_sq(float xh, float xl) {  // (xh + xl)^2, dropping xl^2
    const float p = xh * xh;
    float e = fmaf(xh, xh, -p);
    e = fmaf(2.0f * xh, xl, e);
    add(p);
    lo += e;
  }
  __device__ double value() const { return (double)hi + (double)lo; }
};

__device__ inline void diag_row(const MemberDev<double>& md, int slot, int j, int lane, Acc<double>& mass,
                                Acc<double>& en) {
  const int N = md.N, M = md.M, Mh = md.Mh;
  const double* dc = md.dcoef;
  const bool hu = j >= 1 && j <= M - 2, hv = j < Mh;
  const size_t ro = (size_t)j * N;
  const double2* g2 = reinterpret_cast<const double2*>(md.st[slot][F_GD] + ro);
  const double2* h2 = reinterpret_cast<const double2*>(md.ghs + ro);
  const double2* u2 = reinterpret_cast<const double2*>(md.st[slot][F_IU] + ro);
  const double2* v2 = reinterpret_cast<const double2*>(md.st[slot][F_IV] + (hv ? ro : 0));
  const double wm = dc[j], wf = dc[M + j], wh = hv ? dc[2 * M + j] : 0.0;
  for (int q = lane; q < N / 2; q += 32) {
    const double2 g = g2[q], gh = h2[q];
    const double2 uu = hu ? u2[q] : make_double2(0, 0);
    const double2 vv = hv ? v2[q] : make_double2(0, 0);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const double gk = k ? g.y : g.x, hk = k ? gh.y : gh.x;
      const double uk = k ? uu.y : uu.x, vk = k ? vv.y : vv.x;
      mass.add(wm * gk);
      if (hu) en.add(uk * uk * wf);
      if (hv) en.add(vk * vk * wh);
      const double hh = gk + hk;
      en.add(hh * hh * wf);
    }
  }
}

__device__ inline void diag_row(const MemberDev<float>& md, int slot, int j, int lane, PlainD& mass, PlainD& en) {
  const int N = md.N, M = md.M, Mh = md.Mh;
  const double* dc = md.dcoef;
  const bool hu = j >= 1 && j <= M - 2, hv = j < Mh;
  const size_t ro = (size_t)j * N;
  const float4* gH = reinterpret_cast<const float4*>(md.st[slot][F_GD] + ro);
  const float4* gL = reinterpret_cast<const float4*>(md.lo[slot][F_GD] + ro);
  const float4* hS = reinterpret_cast<const float4*>(md.ghs + ro);
  const float4* uH = reinterpret_cast<const float4*>(md.st[slot][F_IU] + ro);
  const float4* uL = reinterpret_cast<const float4*>(md.lo[slot][F_IU] + ro);
  const float4* vH = reinterpret_cast<const float4*>(md.st[slot][F_IV] + (hv ? ro : 0));
  const float4* vL = reinterpret_cast<const float4*>(md.lo[slot][F_IV] + (hv ? ro : 0));
  FF sg, su, sv, sh;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int q = lane; q < N / 4; q += 32) {
    const float4 gh = gH[q], gl = gL[q], hs = hS[q];
    const float4 uh = hu ? uH[q] : z, ul = hu ? uL[q] : z;
    const float4 vh = hv ? vH[q] : z, vl = hv ? vL[q] : z;
    const float* a0 = &gh.x;
    const float* a1 = &gl.x;
    const float* a2 = &hs.x;
    const float* a3 = &uh.x;
    const float* a4 = &ul.x;
    const float* a5 = &vh.x;
    const float* a6 = &vl.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      sg.add(a0[k]);
      sg.lo += a1[k];
      su.add_sq(a3[k], a4[k]);
      sv.add_sq(a5[k], a6[k]);
      // hh = g + ghs as a float pair
      const float t = a0[k] + a2[k];
      const float bp = t - a0[k];
      const float e = (a0[k] - (t - bp)) + (a2[k] - bp) + a1[k];
      sh.add_sq(t, e);
    }
  }
  mass.add(dc[j] * sg.value());
  if (hu) en.add(dc[M + j] * su.value());
  if (hv) en.add(dc[2 * M + j] * sv.value());
  en.add(dc[M + j] * sh.value());
}

// Warp w of item (member, rows begin..begin+count-1) sums row begin + w.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    diag_kernel(const MemberDev<T>* __restrict__ mems, const FlatItem* __restrict__ dl, DiagArgs a) {
  __shared__ double red[64];
  const FlatItem w = dl[blockIdx.x];
  const MemberDev<T>& md = mems[w.member];
  typename DiagAcc<T>::type mass, en;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp < w.count) diag_row(md, a.slot, w.begin + warp, lane, mass, en);
  const auto sm = block_acc(mass, red);
  const auto se = block_acc(en, red);
  if (threadIdx.x == 0) {
    double* pp = a.partials + 4 * (size_t)blockIdx.x;
    pp[0] = sm.s;
    pp[1] = sm.c;
    pp[2] = se.s;
    pp[3] = se.c;
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    diag_finalize_kernel(const MemberDev<T>* __restrict__ mems, const int* __restrict__ slots, DiagArgs a) {
  const int s = slots[blockIdx.x];
  const MemberDev<T>& md = mems[s];
  Acc<double> m, e;
  member_partials<T>(a.partials, md.dbase, md.dcount, m, e);
  const double tm = m.value(), te = e.value();
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
  // The stage kernel's layout (stage_smem_bytes): a bulk tile, or the row
  // task's tile, rows, kept coefficients and twiddles, in one area.
  T* staging = reinterpret_cast<T*>(smem_raw);
  T* rows = staging + row_task_words<T>();
  T* coefs = rows + 3 * max_n;
  T* tw = coefs + max_n;  // 2 * max_n twiddles
  T* redT = staging + staging_words;
  double* redD = reinterpret_cast<double*>(redT + 64);
  __shared__ MemberDev<T> smd;
  const WorkItem w = wl[blockIdx.x];
  if (w.kind == 1 && w.field > 0) return;  // one block per whole row here (field -1 or F_GD)
  load_member(mems, w.member, &smd);
  const MemberDev<T>& md = smd;
  const int N = md.N, M = md.M, Mh = md.Mh;
  const T* gd_in = md.st[slot][F_GD];
  if (w.kind != 0) twiddles_to_shared(md, tw);
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
      filter_project(md, rg, ri_keep_full(info), coefs, tw);
      filter_project(md, ru, ri_keep_full(info), coefs, tw);
    }
    if (has_v && (info & RI_FLAG_HALF)) filter_project(md, rv, ri_keep_half(info), coefs, tw);
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
  if (w.kind == 1 && w.field > 0) return;  // one block per whole row here (field -1 or F_GD)
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
  if (w.kind == 1 && w.field > 0) return;  // one block per whole row here (field -1 or F_GD)
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

// ------------------------------------------------------------ history
// History output of one member's state(old) in FP64 (src/history_mod.F90:
// 101-108 and diag_run's div, vor, src/diag_mod.F90:49-68): u, v on the A
// grid, gh = gd + ghs, divergence on full rows 1..M-2 (0 on the pole rows),
// vorticity on half rows.  u, v are the level's given ones or recovered as
// update_state does (src/dycore_mod.F90:636-645); FP32 levels are read as
// hi + lo.  One block per full row.

template <typename T>
__device__ inline double hist_val(const T* hi, const T* lo, size_t o) {
  double v = (double)hi[o];
  if (lo) v += (double)lo[o];
  return v;
}

template <typename T>
__device__ inline double hist_u(const MemberDev<T>& md, int lvl, bool given, int i, int j) {
  const int N = md.N, M = md.M;
  if (j < 0 || j >= M) return 0.0;  // zero latitude halo
  i = i < 0 ? i + N : (i >= N ? i - N : i);
  const size_t o = (size_t)j * N + i;
  if (given) return (double)md.given_u[o];
  if (j == 0 || j == M - 1) return 0.0;
  const size_t oe = (size_t)j * N + (i + 1 < N ? i + 1 : 0);
  const double g0 = sqrt(hist_val(md.st[lvl][F_GD], md.lo[lvl][F_GD], o));
  const double g1 = sqrt(hist_val(md.st[lvl][F_GD], md.lo[lvl][F_GD], oe));
  return hist_val(md.st[lvl][F_IU], md.lo[lvl][F_IU], o) * 2.0 / (g0 + g1);
}

template <typename T>
__device__ inline double hist_v(const MemberDev<T>& md, int lvl, bool given, int i, int jh) {
  const int N = md.N, Mh = md.Mh;
  if (jh < 0 || jh >= Mh) return 0.0;
  i = i < 0 ? i + N : (i >= N ? i - N : i);
  const size_t o = (size_t)jh * N + i;
  if (given) return (double)md.given_v[o];
  const double g0 = sqrt(hist_val(md.st[lvl][F_GD], md.lo[lvl][F_GD], o));
  const double g1 = sqrt(hist_val(md.st[lvl][F_GD], md.lo[lvl][F_GD], o + N));
  return hist_val(md.st[lvl][F_IV], md.lo[lvl][F_IV], o) * 2.0 / (g0 + g1);
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    history_kernel(const MemberDev<T>* __restrict__ mems, int slot, int lvl, int given, double* ua, double* va,
                   double* gh, double* div, double* vor) {
  const MemberDev<T>& md = mems[slot];
  const int N = md.N, M = md.M, Mh = md.Mh;
  const int j = blockIdx.x;
  const bool gv = given != 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const size_t o = (size_t)j * N + i;
    const double uc = hist_u(md, lvl, gv, i, j), uw = hist_u(md, lvl, gv, i - 1, j);
    const double vc = hist_v(md, lvl, gv, i, j), vs = hist_v(md, lvl, gv, i, j - 1);
    ua[o] = 0.5 * (uc + uw);
    va[o] = 0.5 * (vc + vs);
    gh[o] = hist_val(md.st[lvl][F_GD], md.lo[lvl][F_GD], o) + (double)md.ghs[o];
    double d = 0.0;
    if (j >= 1 && j <= M - 2) {
      const double vm1 = vs * (double)ch(md, CH_COS, j - 1);
      const double vp1 = vc * (double)ch(md, CH_COS, j);
      d = (uc - uw) / (double)cf(md, CF_DLON, j) + (vp1 - vm1) / (double)cf(md, CF_DLAT, j);
    }
    div[o] = d;
    if (j < Mh) {
      const double vm1 = vc, vp1 = hist_v(md, lvl, gv, i + 1, j);
      const double um1 = uc, up1 = hist_u(md, lvl, gv, i, j + 1);
      vor[o] = (vp1 - vm1) / (double)ch(md, CH_DLON, j) - (up1 - um1) / (double)ch(md, CH_DLAT, j);
    }
  }
}

// --------------------------------------------------------- launchers

// Dynamic shared memory already allowed for one kernel, per device: the
// attribute is a per-device setting, and launches may come from several
// host threads (one batch engine each).
struct SmemConfigured {
  static constexpr int kDevices = 64;
  std::atomic<size_t> bytes[kDevices];
  SmemConfigured() {
    for (auto& b : bytes) b.store(0);
  }
  // True when `smem` bytes are already allowed on the current device.
  bool covers(size_t smem, int* dev) {
    if (cudaGetDevice(dev) != cudaSuccess || *dev < 0 || *dev >= kDevices) {
      *dev = -1;
      return false;
    }
    return smem <= bytes[*dev].load();
  }
  void record(int dev, size_t smem) {
    if (dev < 0) return;
    size_t cur = bytes[dev].load();
    while (smem > cur && !bytes[dev].compare_exchange_weak(cur, smem)) {
    }
  }
};

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
  if (tile_rows == 16 && tile_cols == 64) bulk = tile_words<T, 16, 64>();
  if (tile_rows == 4 && tile_cols == 128) bulk = tile_words<T, 4, 128>();
  if (tile_rows == 4 && tile_cols == 32) bulk = tile_words<T, 4, 32>();
  // A block is a bulk tile or a whole-row task: the row task's tile, rows,
  // kept coefficients and twiddles share the bulk tile's staging area.
  // Rounded to 4 words and max_n to an even count so that the FP64
  // reduction buffer after the area stays 8-byte aligned.
  max_n = (max_n + 1) & ~1;
  const int row = row_task_words<T>() + 3 * max_n + max_n + 2 * max_n;
  const int sw = ((bulk > row ? bulk : row) + 3) & ~3;
  if (staging_words) *staging_words = sw;
  return (size_t)(sw + 64) * sizeof(T) + 64 * sizeof(double) + 16;
}

template <typename T, int PASS, int ADV, int R, int W>
static int launch_stage_t(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int max_n, const StageArgs& a,
                          cudaStream_t s) {
  int sw = 0;
  max_n = (max_n + 1) & ~1;
  const size_t smem = stage_smem_bytes<T>(R, W, max_n, &sw);
  static SmemConfigured configured;
  int dev = -1;
  if (!configured.covers(smem, &dev)) {
    if (cudaFuncSetAttribute(stage_kernel<T, PASS, ADV, R, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return check_launch();
    configured.record(dev, smem);
  }
  if (!a.pair) {
    stage_kernel<T, PASS, ADV, R, W><<<nwork, kThreads, smem, s>>>(mem, wl, a, sw, max_n);
    return check_launch();
  }
  if (nwork % 2) return GDC_E_CONFIG;  // clusters of two need an even count
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nwork);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, stage_kernel<T, PASS, ADV, R, W>, mem, wl, a, sw, max_n);
  return check_launch();
}

// One tile shape's stage kernels (three passes x two advection schemes).
// Each (real type, shape) pair is instantiated in a translation unit of its
// own (gdc_stage_shape.cu built once per pair) so that the library's
// kernels compile in parallel.
template <typename T, int R, int W>
int launch_stage_shape(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int adv, int max_n,
                       const StageArgs& a, cudaStream_t s);
#ifdef GDC_STAGE_SHAPE_UNIT
template <typename T, int R, int W>
int launch_stage_shape(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int adv, int max_n,
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
#endif

// WENO members use 8x32 tiles only (one instantiation per pass; the fast
// pass has no advection and runs the centred kernel).
template <typename T>
static int launch_stage_weno(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int max_n, const StageArgs& a,
                             cudaStream_t s) {
  if (a.pass == kAllPass) return launch_stage_t<T, kAllPass, GDC_ADV_WENO, 8, 32>(mem, wl, nwork, max_n, a, s);
  if (a.pass == kSlowPass) return launch_stage_t<T, kSlowPass, GDC_ADV_WENO, 8, 32>(mem, wl, nwork, max_n, a, s);
  return launch_stage_t<T, kFastPass, GDC_ADV_CENTER_DIFF, 8, 32>(mem, wl, nwork, max_n, a, s);
}

template <typename T>
int launch_stage(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int adv, int tile_rows, int tile_cols,
                 int max_n, const StageArgs& args, void* stream) {
  if (nwork <= 0) return GDC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  StageArgs a = args;
  a.form = update_form(args);
  if (adv == GDC_ADV_WENO)
    return tile_rows == 8 && tile_cols == 32 ? launch_stage_weno<T>(mem, wl, nwork, max_n, a, s) : GDC_E_CONFIG;
  if (tile_rows == 8 && tile_cols == 32) return launch_stage_shape<T, 8, 32>(mem, wl, nwork, adv, max_n, a, s);
  if (tile_rows == 8 && tile_cols == 64) return launch_stage_shape<T, 8, 64>(mem, wl, nwork, adv, max_n, a, s);
  if (tile_rows == 16 && tile_cols == 64) return launch_stage_shape<T, 16, 64>(mem, wl, nwork, adv, max_n, a, s);
  if (tile_rows == 4 && tile_cols == 128) return launch_stage_shape<T, 4, 128>(mem, wl, nwork, adv, max_n, a, s);
  if constexpr (sizeof(T) == 8)
    if (tile_rows == 4 && tile_cols == 32) return launch_stage_shape<T, 4, 32>(mem, wl, nwork, adv, max_n, a, s);
  return GDC_E_CONFIG;
}

template <typename T, int PASS, int ADV>
static int launch_strips_t(const WorkItem* strips, int nstrip, const MemberDev<T>* mem, const StageArgs& a,
                           cudaStream_t s) {
  if (nstrip <= 0) return GDC_OK;
  const int per = kThreads / 32;
  strip_kernel<T, PASS, ADV><<<(nstrip + per - 1) / per, kThreads, 0, s>>>(mem, strips, nstrip, a);
  return check_launch();
}

template <typename T>
int launch_stage_strips(const MemberDev<T>* mem, const WorkItem* strips, int nstrip, int adv, const StageArgs& args,
                        void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  StageArgs a = args;
  a.form = update_form(args);
#define GDC_DISPATCH(P, A) \
  if (a.pass == P && adv == A) return launch_strips_t<T, P, A>(strips, nstrip, mem, a, s);
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
int launch_history(const MemberDev<T>* mem, int slot, int lvl, int given, int num_lat, double* ua, double* va,
                   double* gh, double* div, double* vor, void* stream) {
  history_kernel<T><<<num_lat, kThreads, 0, (cudaStream_t)stream>>>(mem, slot, lvl, given, ua, va, gh, div, vor);
  return check_launch();
}

// iap_transform (src/types_mod.F90:399-426) of an FP64 initial condition
// into member `slot`'s time level `lvl`, with the FP32 compensation words
// where the level has them; the condition's own u, v become the level's
// given u, v.  The inputs point at element (0, 0) of rows `ld` apart
// (compact device arrays: ld = N; the caller's padded host arrays, read in
// place where the device reads pageable host memory: their interior).  FP64
// arithmetic with explicit roundings, as on the host.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    ic_iap_kernel(const MemberDev<T>* __restrict__ mems, int slot, int lvl, const double* __restrict__ u,
                  const double* __restrict__ v, const double* __restrict__ gd, const double* __restrict__ ghs,
                  int ld) {
  const MemberDev<T>& d = mems[slot];
  const int N = d.N, Mh = d.Mh, n = d.M * N;
  auto put = [](T* hi, T* lo, int q, double x) {
    const T h = T(x);
    hi[q] = h;
    if (lo) lo[q] = T(__dsub_rn(x, (double)h));
  };
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int j = q / N, i = q - j * N;
    const size_t r = (size_t)j * ld + i;
    const double g = gd[r], sg = __dsqrt_rn(g);
    put(d.st[lvl][F_GD], d.lo[lvl][F_GD], q, g);
    d.ghs[q] = T(ghs[r]);
    const size_t rp = i + 1 == N ? r + 1 - N : r + 1;
    put(d.st[lvl][F_IU], d.lo[lvl][F_IU], q, __dmul_rn(__dmul_rn(0.5, __dadd_rn(sg, __dsqrt_rn(gd[rp]))), u[r]));
    d.given_u[q] = T(u[r]);
    if (j < Mh) {
      put(d.st[lvl][F_IV], d.lo[lvl][F_IV], q,
          __dmul_rn(__dmul_rn(0.5, __dadd_rn(sg, __dsqrt_rn(gd[r + ld]))), v[r]));
      d.given_v[q] = T(v[r]);
    }
  }
}

template <typename T>
int launch_ic_iap(const MemberDev<T>* mem, int slot, int lvl, int N, int M, const double* u, const double* v,
                  const double* gd, const double* ghs, int ld, void* stream) {
  const int n = N * M, grid = (n + kThreads - 1) / kThreads;
  ic_iap_kernel<T><<<grid, kThreads, 0, (cudaStream_t)stream>>>(mem, slot, lvl, u, v, gd, ghs, ld);
  return check_launch();
}

// A member's level `lvl` read back in FP64 (hi + lo), compact: gd, u, v,
// iap u, iap v, iap gd (sqrt gd) -- u, v derived as update_state recovers them
// (src/dycore_mod.F90:636-645; zero on the pole rows) with uv_mode 0, the
// level's given u, v with 1, not written with 2.  Explicitly rounded FP64
// operations: the same values as the same arithmetic on the host.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    state_out_kernel(const MemberDev<T>* __restrict__ mems, int slot, int lvl, int uv_mode, double* __restrict__ out) {
  const MemberDev<T>& d = mems[slot];
  const int N = d.N, M = d.M, Mh = d.Mh;
  const size_t n = (size_t)M * N, nh = (size_t)Mh * N;
  double* og = out;
  double* ouu = og + n;
  double* ovv = ouu + n;
  double* ou = ovv + nh;
  double* ov = ou + n;
  double* oi = ov + nh;
  const T *gh = d.st[lvl][F_GD], *gl = d.lo[lvl][F_GD];
  auto level = [](const T* hi, const T* lo, size_t q) {
    return __dadd_rn((double)hi[q], lo ? (double)lo[q] : 0.0);
  };
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(q / N), i = (int)(q - (size_t)j * N);
    const double g = level(gh, gl, q), sg = __dsqrt_rn(g);
    const double iu = level(d.st[lvl][F_IU], d.lo[lvl][F_IU], q);
    og[q] = g;
    ou[q] = iu;
    oi[q] = sg;
    if (j < Mh) ov[q] = level(d.st[lvl][F_IV], d.lo[lvl][F_IV], q);
    if (uv_mode == 1) {
      ouu[q] = __dadd_rn((double)d.given_u[q], 0.0);
      if (j < Mh) ovv[q] = __dadd_rn((double)d.given_v[q], 0.0);
    } else if (uv_mode == 0) {
      const size_t qp = i + 1 == N ? q + 1 - N : q + 1;
      ouu[q] = (j == 0 || j == M - 1) ? 0.0
                                      : __ddiv_rn(__dmul_rn(iu, 2.0), __dadd_rn(sg, __dsqrt_rn(level(gh, gl, qp))));
      if (j < Mh)
        ovv[q] = __ddiv_rn(__dmul_rn(ov[q], 2.0), __dadd_rn(sg, __dsqrt_rn(level(gh, gl, q + N))));
    }
  }
}

template <typename T>
int launch_state_out(const MemberDev<T>* mem, int slot, int lvl, int uv_mode, int N, int M, double* out,
                     void* stream) {
  const int grid = (int)std::min<size_t>(((size_t)N * M + kThreads - 1) / kThreads, 4096);
  state_out_kernel<T><<<grid, kThreads, 0, (cudaStream_t)stream>>>(mem, slot, lvl, uv_mode, out);
  return check_launch();
}

template <typename T>
int launch_weno(const MemberDev<T>* mem, const FlatItem* fl, int nflat, int in_slot, const int* uvslot,
                void* stream) {
  if (nflat <= 0) return GDC_OK;
  weno_kernel<T><<<nflat, kThreads, 0, (cudaStream_t)stream>>>(mem, fl, in_slot, uvslot);
  return check_launch();
}

template <typename T>
int launch_beta(const MemberDev<T>* mem, const int* slots, int nmembers, const double* partials, double* beta,
                int qcon, int beta_mode, void* stream) {
  if (nmembers <= 0) return GDC_OK;
  beta_kernel<T><<<nmembers, partial_threads<T>(), 0, (cudaStream_t)stream>>>(mem, slots, partials, beta, qcon,
                                                                             beta_mode);
  return check_launch();
}

template <typename T>
int launch_final(const MemberDev<T>* mem, const FlatItem* fl, int nflat, const FinalArgs& a, void* stream) {
  if (nflat <= 0) return GDC_OK;
  final_kernel<T><<<nflat, kThreads, 0, (cudaStream_t)stream>>>(mem, fl, a);
  return check_launch();
}

template <typename T>
int launch_diag(const MemberDev<T>* mem, const FlatItem* dl, int ndl, const int* slots, int nmembers,
                const DiagArgs& a, void* stream) {
  if (ndl <= 0) return GDC_OK;
  diag_kernel<T><<<ndl, 32 * diag_rows<T>(), 0, (cudaStream_t)stream>>>(mem, dl, a);
  int rc = check_launch();
  if (rc) return rc;
  diag_finalize_kernel<T><<<nmembers, partial_threads<T>(), 0, (cudaStream_t)stream>>>(mem, slots, a);
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
  static SmemConfigured configured;
  int dev = -1;
  auto lap = diffusion_lap_kernel<T, 8, 32>;
  if (tile_rows == 8 && tile_cols == 64)
    lap = diffusion_lap_kernel<T, 8, 64>;
  else if (tile_rows == 4 && tile_cols == 128)
    lap = diffusion_lap_kernel<T, 4, 128>;
  else if (!(tile_rows == 8 && tile_cols == 32))
    return GDC_E_CONFIG;
  if (!configured.covers(smem, &dev)) {
    for (auto k : {diffusion_lap_kernel<T, 8, 32>, diffusion_lap_kernel<T, 8, 64>, diffusion_lap_kernel<T, 4, 128>})
      if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch();
    configured.record(dev, smem);
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
