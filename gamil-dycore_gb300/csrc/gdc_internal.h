// gdc_internal.h -- types shared by the host engine (gdc_engine.cpp,
// gdc_host.cpp) and the CUDA kernels (gdc_kernels.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/gdc.h"

#ifdef __CUDACC__
#define GDC_HD __host__ __device__
#else
#define GDC_HD
#endif

namespace gdc {

// src/params_mod.F90:6-11 (FP64).
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kOmega = 2.0 * kPi / 86400.0;
constexpr double kRadius = 6.37122e6;
constexpr double kGrav = 9.80616;  // src/params_mod.F90:11

// ---------------------------------------------------------------- host mesh
struct Mesh {
  int N = 0, M = 0, Mh = 0;
  double dlon = 0, dlat = 0;
  std::vector<double> full_lat, half_lat, full_lon, half_lon;
  std::vector<double> full_cos, half_cos, full_sin, half_sin;
};
struct Coef {
  std::vector<double> full_cos, full_f, full_c, full_dlon, full_dlat;  // M
  std::vector<double> half_cos, half_dlon, half_dlat;                  // Mh
};
Mesh make_mesh(int N, int M);
Coef make_coef(const Mesh& m);
void make_filter_rows(const Mesh& m, const gdc_params& p, std::vector<int>& flag_full,
                      std::vector<int>& keep_full, std::vector<int>& flag_half,
                      std::vector<int>& keep_half);
void seeded_draws(unsigned long long seed, int lmax, int n_mountains, std::vector<double>& clat,
                  std::vector<double>& clon, std::vector<double>& ag, std::vector<double>& bg,
                  std::vector<double>& ap, std::vector<double>& bp);

// Separable initial conditions: per-row and per-column factor tables built
// on the host (the transcendental functions, O(M + N) values) and the
// per-point products, evaluated by the same inline functions on the host
// and on the device (no FMA contraction on either), so both give the same
// bits.  Rossby-Haurwitz wave (src/test_cases/barotropic/rossby_haurwitz_
// wave_test_mod.F90:33-85): rows ua, ub, uc, vb, ga, gb, gc (M each; vb
// Mh used), columns cu, sv, cg1, cg2 (N each).
void rh_tables(const Mesh& m, std::vector<double>& t);
GDC_HD inline size_t rh_table_words(int N, int M) { return 7 * (size_t)M + 4 * (size_t)N; }
GDC_HD inline double rh_u(const double* t, int N, int M, int i, int j) {
  const double omg = 7.848e-6;
  const double* col = t + 7 * (size_t)M;
  const double b = t[M + j] * col[i], c = t[2 * M + j] * col[i];
  return kRadius * omg * (t[j] + b - c);
}
GDC_HD inline double rh_v(const double* t, int N, int M, int i, int j) {
  const double omg = 7.848e-6;
  const double a = t[3 * (size_t)M + j] * t[7 * (size_t)M + N + i];
  return -kRadius * omg * a;
}
GDC_HD inline double rh_gd(const double* t, int N, int M, int i, int j) {
  const double gd0 = 8.0e3 * kGrav;
  const double* col = t + 7 * (size_t)M;
  return gd0 + kRadius * kRadius *
                   (t[4 * (size_t)M + j] + t[5 * (size_t)M + j] * col[2 * N + i] + t[6 * (size_t)M + j] * col[3 * N + i]);
}
// Shallow-water Rossby wave of Shamir and Paldor (src/test_cases/barotropic/
// shallow_water_waves_test_mod.F90:97-135, 232-298): rows uTilde, vTilde,
// hTilde at the full latitudes (v's half row j takes vTilde of full row j,
// as the reference's getFields does), columns cos(k lon) at half and full
// longitudes and cos(k lon - pi/2); gd = g h + 5e4.  Pole-row u (below
// 1e-100 in the reference) is set to zero.
void sw_waves_tables(const Mesh& m, std::vector<double>& t);
double sw_waves_phase_speed(int wave_flag);
GDC_HD inline size_t sw_table_words(int N, int M) { return 3 * (size_t)M + 3 * (size_t)N; }
GDC_HD inline double sw_u(const double* t, int N, int M, int i, int j) {
  return (j == 0 || j == M - 1) ? 0.0 : t[j] * t[3 * (size_t)M + i];
}
GDC_HD inline double sw_v(const double* t, int N, int M, int i, int j) {
  return t[(size_t)M + j] * t[3 * (size_t)M + N + i];
}
GDC_HD inline double sw_gd(const double* t, int N, int M, int i, int j) {
  return kGrav * (t[2 * (size_t)M + j] * t[3 * (size_t)M + 2 * N + i]) + 5.0e4;
}

// Device initial conditions (gdc_ic.cu): FP64 fields, interior only, lon
// fastest: u, gd, ghs num_lat rows, v num_lat - 1.  `tables` holds the mesh
// (full_lat, half_lat, full_lon, half_lon, full_cos, half_cos, full_sin,
// half_sin: M, Mh, N, N, M, Mh, M, Mh values) followed, for the separable
// states, by their factor tables (rh_tables, sw_waves_tables) and, for the
// seeded state, by the mountain centres (lat, lon) and the harmonic
// coefficients (gd a, b, streamfunction a, b; (lmax+1)^2 each); `scratch`
// 2 M N + 2 doubles.
int ic_generate(const gdc_ic_spec& spec, int N, int M, const double* tables, double* scratch, double* u,
                double* v, double* gd, double* ghs, void* stream);

// ------------------------------------------------------------ device layout
// Passes of space_operators (src/dycore_mod.F90:34-36).
enum Pass { kAllPass = 0, kFastPass = 1, kSlowPass = 2 };

// Row coefficient table, per member, in the compute type.  Full-row tables
// have M entries; half-row tables have Mh+2 entries with index 0 standing
// for half row -1 and index Mh+1 for half row Mh (both 0.0: the reference
// reads those out of bounds only to multiply a zero latitude halo).
enum FullCoef {
  CF_COS = 0,   // full_cos_lat after reset_cos_lat_at_poles
  CF_F,         // 2 Omega sin
  CF_C,         // sin / cos / a (0 at poles)
  CF_RADVLON,   // 0.25 / full_dlon
  CF_RADVLAT,   // 0.25 / full_dlat
  CF_DLON,      // full_dlon
  CF_DLAT,      // full_dlat
  CF_C1,        // half_cos(j-1) / full_cos(j)
  CF_C2,        // half_cos(j) / full_cos(j)
  CF_MASSW,     // full_cos * dlon * dlat (diag total_mass weight)
  CF_NFULL
};
enum HalfCoef {
  CH_COS = 0,   // half_cos_lat
  CH_RADVLON,   // 0.25 / half_dlon
  CH_RADVLAT,   // 0.25 / half_dlat
  CH_DLON,      // half_dlon
  CH_DLAT,      // half_dlat
  CH_NHALF
};
inline size_t coef_words(int M) { return (size_t)CF_NFULL * M + (size_t)CH_NHALF * (M + 1); }
// Offset of table k: full tables first, then half tables (Mh+2 = M+1 each).
GDC_HD inline size_t cf_off(int k, int M) { return (size_t)k * M; }
GDC_HD inline size_t ch_off(int k, int M) { return (size_t)CF_NFULL * M + (size_t)k * (M + 1); }

// Per-row coefficient records for the stencil tiles: record j+1 holds, for
// row j = -1..M, the full-row coefficients of row j in TileFull order and
// the half-row coefficients of half row j in TileHalf order, 16 words per
// record so that a tile copies its rows 16 bytes at a time.  Entries of rows
// outside the tables are 0.0, as in the table above.
enum TileFull { TF_RADVLON, TF_RADVLAT, TF_F, TF_C, TF_C1, TF_C2, TF_DLON, TF_DLAT, TF_COS, TF_N };
enum TileHalf { TH_COS = TF_N, TH_RADVLON, TH_RADVLAT, TH_DLAT, TH_DLON, TH_END };
constexpr int kRecWords = 16;
static_assert(TH_END <= kRecWords, "coefficient record overflow");
inline size_t rec_words(int M) { return (size_t)(M + 2) * kRecWords; }
template <typename T>
std::vector<T> row_records(const std::vector<T>& coef, int M) {
  static const int fsrc[TF_N] = {CF_RADVLON, CF_RADVLAT, CF_F, CF_C, CF_C1, CF_C2, CF_DLON, CF_DLAT, CF_COS};
  static const int hsrc[TH_END - TH_COS] = {CH_COS, CH_RADVLON, CH_RADVLAT, CH_DLAT, CH_DLON};
  std::vector<T> rec(rec_words(M), T(0));
  for (int j = -1; j <= M; ++j) {
    T* r = rec.data() + (size_t)(j + 1) * kRecWords;
    if (j >= 0 && j < M)
      for (int k = 0; k < TF_N; ++k) r[k] = coef[cf_off(fsrc[k], M) + j];
    if (j >= -1 && j <= M - 1)
      for (int k = 0; k < TH_END - TH_COS; ++k) r[TH_COS + k] = coef[ch_off(hsrc[k], M) + j + 1];
  }
  return rec;
}

// Row information bits (per row index j = 0..M-1).
enum RowBits {
  RI_SPECIAL = 1,    // handled by a whole-row task (pole or filtered row)
  RI_FLAG_FULL = 2,  // full row j is filtered
  RI_FLAG_HALF = 4,  // half row j is filtered
};
// rowinfo[j] = bits | keep_full << 8 | keep_half << 20 (packed-coefficient
// counts kept by the factor rows, 0..2046).
GDC_HD inline int ri_keep_full(int r) { return (r >> 8) & 0xfff; }
GDC_HD inline int ri_keep_half(int r) { return (r >> 20) & 0x7ff; }

// Buffer slots of a member: time levels 0,1,2 of the reference
// (state(0..2)), the isp saved state (state(-1)), and two stage states.
enum Slot { SL_L0 = 0, SL_L1, SL_L2, SL_SAVED, SL_SA, SL_SB, SL_N };
// Tendency slots (du, dv, dgd each).
enum TSlot { TS_OLD = 0, TS_NEW, TS_SLOW, TS_ACCUM, TS_N };

template <typename T>
struct MemberDev {
  int N, M, Mh;
  int pbase, pcount;      // partial-sum slots of this member's work items
  int dbase, dcount;      // partial-sum slots of this member's diag items
  int pad0, pad1;
  double pcdt[3];         // predict_correct time_step_size per Pass
  double dt;              // time_step_size
  T* st[SL_N][3];         // state slots: gd, iap u, iap v
  T* lo[SL_N][3];         // compensation words (FP32 time levels), else null
  T* td[TS_N][3];         // tendency slots: dgd, du, dv
  T* ghs;
  const T* coef;
  const T* rowc;          // coefficient records of rows -1..M (kRecWords each)
  const T* twid;          // cos(2 pi m/N), m<N, then sin(2 pi m/N)
  const int* rowinfo;
  const double* dcoef;    // FP64 diag weights: mass weight [M], full cos [M], half cos [Mh]
  T* given_u;             // u and v supplied with the state of level uvslot[member]
  T* given_v;             // (initial condition, diffusion) rather than derived
  T* wadv[2];             // uv_adv_scheme weno: -(u_adv_lon + u_adv_lat) [M N] and
                          // -(v_adv_lon + v_adv_lat) [Mh N] of the stage's input, else null
};

enum Field { F_GD = 0, F_IU = 1, F_IV = 2 };

struct WorkItem {
  int member;  // member slot
  int kind;    // 0 bulk tile, 1 whole-row task, 3 nothing (padding)
  int j0;      // first row index (row task: the row)
  int i0;      // first column (tile); row task: its part (0, 1) of a pair
  int rows;    // tile rows; row task: 1, or 2 when split over a block pair
  int cols;    // tile columns
  int pidx;    // partial-sum slot
  int field;   // whole-row task: the one field it computes (F_GD, F_IU, F_IV), or -1 for all three
};

// What a stage launch does with the tendency T = space_operators(in):
//   T' = T (+/- T_add) (+ scale2 * T_add2)           combine
//   accum = (init ? 0 : accum) + T                    (isp fast sum)
//   T_out = T'; S_out = base + h T'                   store / update
//   partials of <P, T'> and <T', T'> with P = T_prev (beta_mode 0) or the
//   state slot `ip_slot` (beta_mode 1), and the member's beta.
struct StageArgs {
  int pass;
  int in_slot, base_slot, out_slot;  // Slot values (-1 unused)
  int tout, tprev;                   // TSlot values (-1 unused)
  int tadd, tadd_sign;               // TSlot added (+1) or subtracted (-1)
  int tadd2;                         // TSlot added after scaling by scale2
  double scale2;
  int taccum, accum_init;            // TSlot accumulating T (pre-combine)
  double h_scale;                    // update step = pcdt[pass] * h_scale
  int do_ip;                         // form partials and beta
  int beta_mode;                     // 0 predict_correct, 1 isp
  int ip_slot;                       // state slot for beta_mode 1
  double* partials;                  // 4 doubles per partial slot
  double* beta;                      // per member
  int qcon;
  double ub_lon, ub_lat;             // uv_adv_upwind_{lon,lat}_beta
  double rescale_rtol;               // gdc_params::filter_rescale_rtol
  int* uvslot;                       // per member: slot whose u, v are given (-1 none)
  int form;                          // UpdateForm, set by the launchers
  // Fused final update (predict form only): the input level in_slot is
  // first formed, for every point the block stages, as the previous
  // predict_correct's update in_slot = fin_base + pcdt[fin_pass] *
  // fin_h_scale * beta * T_new (compensated in FP32, as final_kernel), and
  // the block writes it for its own points.
  int fuse;
  int fin_base, fin_pass;
  double fin_h_scale;
  // Launched as clusters of two blocks: a whole-row task listed as two
  // items (WorkItem rows == 2, parts i0 = 0, 1 at an even and the next odd
  // index) runs on the pair.
  int pair;
};

// Warp strips: output columns per warp (lanes 1..30 of the 32), and the
// band heights (rows marched by one warp) the engine offers.
constexpr int kStripCols = 30;

// Update forms the bulk tiles specialise (the three stages of
// predict_correct); anything else takes the general path.
enum UpdateForm {
  UF_PREDICT_IN = 0,   // out = in + h T                    (base is the input level)
  UF_PREDICT_OUT = 1,  // out = base + h T, tout = T
  UF_CORRECT = 2,      // tout = T, inner products with tprev
  UF_GENERAL = 3,
};
inline int update_form(const StageArgs& a) {
  const bool plain = a.taccum < 0 && a.tadd < 0 && a.tadd2 < 0;
  if (!plain) return UF_GENERAL;
  if (a.out_slot >= 0 && a.base_slot == a.in_slot && a.tout < 0 && !a.do_ip) return UF_PREDICT_IN;
  if (a.out_slot >= 0 && a.base_slot != a.in_slot && a.tout >= 0 && !a.do_ip) return UF_PREDICT_OUT;
  if (a.out_slot < 0 && a.tout >= 0 && a.do_ip && a.beta_mode == 0 && a.tprev >= 0) return UF_CORRECT;
  return UF_GENERAL;
}

// A contiguous run of one field of one member: elements [begin, begin+count)
// of the field's array (gd, iap u: M rows; iap v: M-1 rows; N per row).
struct FlatItem {
  int member;
  int field;
  int begin;
  int count;
};
// Elements per flat item: 4 16-byte vectors per thread of a 256-thread block.
template <typename T>
GDC_HD constexpr int flat_chunk() {
  return 256 * 4 * (16 / (int)sizeof(T));
}

struct FinalArgs {
  int base_slot, out_slot, tslot;
  int pass;
  int use_lo;          // write compensated result (time level)
  double h_scale;      // step = pcdt[pass] * h_scale * beta (or * 1)
  const double* beta;  // per member or null
  int* uvslot;         // per member; cleared when out_slot overwrites that level
};

struct DiagArgs {
  int slot;
  int count_step;        // 1: this diag closes a model step
  double* partials;      // 4 doubles per partial slot
  double* diag;          // per member: mass, energy, beta
  const double* beta;
  long long* steps;      // per member: steps completed (incremented here)
  long long* nan_step;   // per member: first step with NaN mass/energy
};

// Tile shapes compiled for the stage and diffusion kernels (rows x columns),
// and the warp-strip layouts of the stage kernel (band rows x kStripCols).
// 4x32 (fewer points than threads: finer load balance where FP64 work per
// point is large) is compiled for FP64 only.
inline bool tile_shape_supported(int r, int c, bool fp64) {
  return (r == 8 && c == 32) || (r == 8 && c == 64) || (r == 4 && c == 128) || (r == 16 && c == 64) ||
         (fp64 && r == 4 && c == 32);
}
inline bool strip_shape_supported(int r, int c) { return c == kStripCols && (r == 8 || r == 16 || r == 32 || r == 64); }

// Kernel launchers (gdc_kernels_f64.cu / gdc_kernels_f32.cu).
template <typename T>
int launch_stage(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int adv, int tile_rows,
                 int tile_cols, int max_n, const StageArgs& a, void* stream);
template <typename T>
int launch_final(const MemberDev<T>* mem, const FlatItem* fl, int nflat, const FinalArgs& a,
                 void* stream);
// Per-item partial sums, then one block per member (`slots`) forms the totals.
template <typename T>
int launch_diag(const MemberDev<T>* mem, const FlatItem* dl, int ndl, const int* slots,
                int nmembers, const DiagArgs& a, void* stream);
// Rows per diag item (one warp per row): 8 in FP32; 2 in FP64, whose row
// sums are double-double FP64 work -- few rows per block spread it over
// more SMs' FP64 pipes.
template <typename T>
constexpr int diag_rows() { return sizeof(T) == 8 ? 2 : 8; }
// beta of each member in `slots` from the stage kernel's partials.
template <typename T>
int launch_beta(const MemberDev<T>* mem, const int* slots, int nmembers, const double* partials,
                double* beta, int qcon, int beta_mode, void* stream);
// ordinary_diffusion (order 2): Laplacians of state `slot` into SA as
// (gd', u', v'), then iap_transform of SA back into `slot`.
template <typename T>
int launch_diffusion(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int tile_rows,
                     int tile_cols, int max_n, int slot, double sign_dt_coef, int* uvslot,
                     void* stream);
template <typename T>
int launch_copy_state(const MemberDev<T>* mem, const WorkItem* wl, int nwork, int from_slot,
                      int to_slot, void* stream);
// Warp strips of one stage (one warp per item; ordinary rows only: the
// whole-row tasks go to launch_stage).
template <typename T>
int launch_stage_strips(const MemberDev<T>* mem, const WorkItem* strips, int nstrip, int adv, const StageArgs& a,
                        void* stream);
// History output of member `slot` at level `lvl` into device FP64 buffers
// (num_lat x num_lon each; vor num_lat - 1 rows).
// iap_transform of an FP64 initial condition into member `slot`'s level
// `lvl`, its given u, v and ghs (src/types_mod.F90:399-426); inputs point at
// element (0, 0), rows `ld` apart.
template <typename T>
int launch_ic_iap(const MemberDev<T>* mem, int slot, int lvl, int N, int M, const double* u, const double* v,
                  const double* gd, const double* ghs, int ld, void* stream);
// Member `slot`'s level `lvl` in FP64, compact: gd [M N], u [M N],
// v [Mh N], iap u [M N], iap v [Mh N], iap gd [M N]; u, v derived
// (uv_mode 0), the given ones (1) or not written (2).
template <typename T>
int launch_state_out(const MemberDev<T>* mem, int slot, int lvl, int uv_mode, int N, int M, double* out,
                     void* stream);
// The WENO advection terms of every member's level `in_slot` (flat items
// of the iap u and v fields; gd items are skipped).
template <typename T>
int launch_weno(const MemberDev<T>* mem, const FlatItem* fl, int nflat, int in_slot, const int* uvslot,
                void* stream);
template <typename T>
int launch_history(const MemberDev<T>* mem, int slot, int lvl, int given, int num_lat, double* ua, double* va,
                   double* gh, double* div, double* vor, void* stream);
// Shared-memory bytes of one stage launch.
template <typename T>
size_t stage_smem_bytes(int tile_rows, int tile_cols, int max_n, int* staging_words);

}  // namespace gdc
