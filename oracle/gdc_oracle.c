/*
 * gdc_oracle.c -- CPU restatement (FP64, single thread) of the gamil-dycore
 * barotropic time step.  TEST INFRASTRUCTURE ONLY: the parity reference for
 * the CUDA path and the timed CPU baseline.  Nothing in the product links it.
 *
 * Parity status: unpinned by reference outputs (the Fortran reference cannot
 * be built here and ships no golden vectors); pinned by the known-answer
 * checks in tests/.
 *
 * Every routine keeps the reference's Fortran indices (1-based interior,
 * halo width 2) and its evaluation order, and cites the file:line it follows
 * (paths relative to the gamil-dycore project root).  Build with
 * -O2 -ffp-contract=off so that no FMA contraction or reassociation changes
 * the order of operations.
 *
 * Sums: the reference's reductions (filter s1/s2 and FFT coefficients, the
 * pole caps, beta's inner products, the diagnostics) are evaluated as the
 * correctly rounded sum of the same rounded terms (exact expansion
 * arithmetic, Shewchuk 1997).  The reference's own summation order is not
 * fixed -- it is built with -Ofast, which lets the compiler reassociate --
 * and the correctly rounded sum is the order-independent value every
 * order approximates; the CUDA path computes the same value.
 *
 * Reference-order build (-DGDO_PLAIN_SUMS, compiled -O2 without
 * contraction): every reduction is instead the reference's own running sum
 * in its loop order (s = s + term, j outer, i inner), and with
 * gdo_set_fft(m, 1) the filter runs FFTPACK's transforms (gdc_fftpack.c)
 * instead of the projection -- the reference's arithmetic as written,
 * evaluated in source order.
 */
#include "gdc_oracle.h"

#include <math.h>

#include "gdc_fftpack.h"
#include <stdlib.h>
#include <string.h>

/* src/params_mod.F90:6-11 (compiled with -fdefault-real-8: all FP64). */
#define PI (atan(1.0) * 4.0)
#define OMEGA (2.0 * PI / 86400.0)
#define RADIUS 6.37122e6

enum { NO_SPLIT = 0, CSP2 = 2, ISP = 3 };
enum { ALL_PASS = 0, FAST_PASS = 1, SLOW_PASS = 2 };
enum { CENTER_DIFF = 0, UPWIND = 1, WENO = 2 };

/* src/types_mod.F90:58-72 */
enum {
  T_U_ADV_LON, T_U_ADV_LAT, T_V_ADV_LON, T_V_ADV_LAT, T_FU, T_FV, T_U_PGF,
  T_V_PGF, T_MDLON, T_MDLAT, T_DU, T_DV, T_DGD, T_NFIELD
};
/* Which tendency arrays are v-shaped (half lat rows). */
static const int tend_is_half[T_NFIELD] = {0, 0, 1, 1, 1, 0, 0, 1, 0, 0, 0, 1, 0};

typedef struct {
  double *u, *v, *gd, *iu, *iv, *ig; /* src/types_mod.F90:41-52 */
} state_t;

typedef struct {
  double* a[T_NFIELD];
} tend_t;

struct gdo_model {
  /* params */
  int N, M, Mh, NP;
  double dt;
  int subcycles, split, qcon, adv;
  double beta_lon, beta_lat;
  int use_filter, cutoff[20];
  int use_diff, diff_order;
  double diff_coef;
  double rescale_rtol; /* extension guard, 0 = reference behaviour */
  /* Conditioning record of the s1/s2 rescale (diagnostic): the largest
   * sum|t w| / |s| seen for s1 and s2 since the last gdo_rescale_record
   * call, and where (field: 0 du, 1 dv, 2 dgd; Fortran row index). */
  double rc_cond[2];
  int rc_field[2], rc_row[2];
  int cur_field, cur_row;
  /* mesh (1-based; index 0 and R+1 are zero pads standing for the
   * out-of-bounds reads described at v_adv_lat) */
  double dlon, dlat;
  double *full_lat, *half_lat, *full_cos, *half_cos, *full_sin, *half_sin;
  /* coef, src/types_mod.F90:25-38 */
  double *full_f, *half_f, *full_c, *half_c, *full_dlon, *half_dlon,
      *full_dlat, *half_dlat;
  /* data, src/data_mod.F90:19-22: state(-1:2), tend(-2:2) */
  state_t state_mem[4];
  tend_t tend_mem[5];
  double* ghs;
  /* filter, src/filter_mod.F90:22-31 */
  int *flag_full, *flag_half;    /* 1-based */
  double *ffac_full, *ffac_half; /* [lat][N], 1-based lat, 0-based lon */
  double *ctab, *stab;           /* cos/sin(2 pi m / N), m = 0..N-1 */
  /* Filter arithmetic: 0 = projection onto the kept modes (the CUDA
   * path's), 1 = FFTPACK's forward and backward transforms (the
   * reference's, gdc_fftpack.c). */
  int fft;
  gdo_rfft plan;
  double *fft_r, *fft_w;
  /* WENO scratch, src/weno_mod.F90:26-31: split and interface fluxes
   * (u-shaped fp_u, fn_u, f_u; v-shaped fp_v, fn_v, f_v).  Zeroed once
   * (parallel_allocate, src/parallel_mod.F90:312-313); the pole and
   * lat-halo rows are never written afterwards. */
  double *w_fpu, *w_fnu, *w_fu, *w_fpv, *w_fnv, *w_fv;
  /* diffusion scratch, src/diffusion_mod.F90:20-26 */
  double *d_ud, *d_vd, *d_gdd, *d_u, *d_v, *d_gd;
  /* time_mod indices and diag */
  int old, new_;
  double total_mass, total_energy, last_beta;
};

#define STATE(m, k) (&(m)->state_mem[(k) + 1])
#define TEND(m, k) (&(m)->tend_mem[(k) + 2])
/* Fortran element (i,j) of a padded field: lon -1..N+2, lat -1..R+2. */
#define AT(m, f, i, j) ((f)[((j) + 1) * (m)->NP + ((i) + 1)])

static double* zalloc(size_t n) { return (double*)calloc(n, sizeof(double)); }

/* ---- correctly rounded summation ------------------------------------
 * A nonoverlapping expansion of increasing magnitude grown term by term
 * with Knuth's TwoSum (zero components dropped), then rounded once to
 * nearest-even (Shewchuk, "Adaptive Precision Floating-Point Arithmetic
 * and Fast Robust Geometric Predicates", 1997). */
typedef struct {
  double p[80];
  int n;
  double special; /* running sum of infinities / NaNs */
  int has_special;
} xsum;

static void xs_init(xsum* x) { x->n = 0; x->special = 0.0; x->has_special = 0; }

#ifdef GDO_PLAIN_SUMS
/* Timing build (the CPU baseline): the reference's plain running sums,
 * compiled like the reference (-Ofast). */
static void xs_add(xsum* x, double v) {
  if (x->n == 0) {
    x->p[0] = 0.0;
    x->n = 1;
  }
  x->p[0] += v;
}
static double xs_value(const xsum* x) { return x->n ? x->p[0] : 0.0; }
#else
static void xs_add(xsum* x, double v) {
  if (!isfinite(v)) {
    x->special += v;
    x->has_special = 1;
    return;
  }
  int k = 0;
  for (int q = 0; q < x->n; ++q) {
    double y = x->p[q];
    double hi = v + y;
    double bp = hi - v;
    double lo = (v - (hi - bp)) + (y - bp);
    if (lo != 0.0) x->p[k++] = lo;
    v = hi;
  }
  x->p[k++] = v;
  x->n = k;
}

static double xs_value(const xsum* x) {
  if (x->has_special) return x->special;
  int n = x->n;
  if (n == 0) return 0.0;
  double hi = x->p[--n];
  double lo = 0.0;
  while (n > 0) {
    double a = hi, b = x->p[--n];
    hi = a + b;
    double bv = hi - a;
    lo = b - bv;
    if (lo != 0.0) break;
  }
  /* Round-half-even correction: when the remainder is exactly half an ulp
   * and the next component has the same sign, the true sum lies beyond
   * the halfway point. */
  if (n > 0 && ((lo < 0.0 && x->p[n - 1] < 0.0) || (lo > 0.0 && x->p[n - 1] > 0.0))) {
    double b = lo * 2.0;
    double a = hi + b;
    double bv = a - hi;
    if (b == bv) hi = a;
  }
  return hi;
}
#endif
static size_t full_sz(const gdo_model* m) { return (size_t)(m->M + 4) * m->NP; }
static size_t half_sz(const gdo_model* m) { return (size_t)(m->Mh + 4) * m->NP; }

/* src/parallel_mod.F90:466-524 -- periodic lon halo, every padded row.
 * Lat halo rows are never filled (they stay 0.0, src/parallel_mod.F90:313). */
static void fill_halo(const gdo_model* m, double* f, int half) {
  int rows = (half ? m->Mh : m->M) + 4, N = m->N;
  for (int r = 0; r < rows; ++r) {
    double* row = f + (size_t)r * m->NP;
    row[0] = row[N];         /* (-1) <- (N-1) */
    row[1] = row[N + 1];     /* (0)  <- (N)   */
    row[N + 2] = row[2];     /* (N+1) <- (1)  */
    row[N + 3] = row[3];     /* (N+2) <- (2)  */
  }
}

/* ---------------------------------------------------------------- init */

/* src/mesh_mod.F90:44-114 */
static void mesh_init(gdo_model* m) {
  int N = m->N, M = m->M, Mh = m->Mh;
  m->full_lat = zalloc(M + 2); m->half_lat = zalloc(Mh + 2);
  m->full_cos = zalloc(M + 2); m->half_cos = zalloc(Mh + 2);
  m->full_sin = zalloc(M + 2); m->half_sin = zalloc(Mh + 2);
  m->dlon = 2 * PI / N;
  m->dlat = PI / Mh;
  for (int j = 1; j <= Mh; ++j) {
    m->full_lat[j] = -0.5 * PI + (j - 1) * m->dlat;
    m->half_lat[j] = m->full_lat[j] + 0.5 * m->dlat;
  }
  m->full_lat[M] = 0.5 * PI;
  for (int j = 1; j <= Mh; ++j) {
    m->half_cos[j] = cos(m->half_lat[j]);
    m->half_sin[j] = sin(m->half_lat[j]);
  }
  for (int j = 1; j <= M; ++j) {
    m->full_cos[j] = cos(m->full_lat[j]);
    m->full_sin[j] = sin(m->full_lat[j]);
  }
  m->full_cos[1] = 0.0;
  m->full_cos[M] = 0.0;
  m->full_sin[1] = -1.0;
  m->full_sin[M] = 1.0;
}

/* src/data_mod.F90:26-59 */
static void data_init(gdo_model* m) {
  int M = m->M, Mh = m->Mh;
  m->full_f = zalloc(M + 2); m->full_c = zalloc(M + 2);
  m->full_dlon = zalloc(M + 2); m->full_dlat = zalloc(M + 2);
  m->half_f = zalloc(Mh + 2); m->half_c = zalloc(Mh + 2);
  m->half_dlon = zalloc(Mh + 2); m->half_dlat = zalloc(Mh + 2);
  for (int j = 1; j <= M; ++j) {
    m->full_f[j] = 2.0 * OMEGA * m->full_sin[j];
    if (j == 1 || j == M)
      m->full_c[j] = 0.0;
    else
      m->full_c[j] = m->full_sin[j] / m->full_cos[j] / RADIUS;
    m->full_dlon[j] = RADIUS * m->dlon * m->full_cos[j];
    m->full_dlat[j] = RADIUS * m->dlat * m->full_cos[j];
  }
  for (int j = 1; j <= Mh; ++j) {
    m->half_f[j] = 2.0 * OMEGA * m->half_sin[j];
    m->half_c[j] = m->half_sin[j] / m->half_cos[j] / RADIUS;
    m->half_dlon[j] = RADIUS * m->dlon * m->half_cos[j];
    m->half_dlat[j] = RADIUS * m->dlat * m->half_cos[j];
  }
  for (int k = 0; k < 4; ++k) {
    state_t* s = &m->state_mem[k];
    s->u = zalloc(full_sz(m)); s->gd = zalloc(full_sz(m));
    s->iu = zalloc(full_sz(m)); s->ig = zalloc(full_sz(m));
    s->v = zalloc(half_sz(m)); s->iv = zalloc(half_sz(m));
  }
  for (int k = 0; k < 5; ++k)
    for (int f = 0; f < T_NFIELD; ++f)
      m->tend_mem[k].a[f] = zalloc(tend_is_half[f] ? half_sz(m) : full_sz(m));
  m->ghs = zalloc(full_sz(m));
}

/* src/filter_mod.F90:35-103.  The north half-row flag is set at
 * full_lat_end_idx-j+1 (:56) while its factors go to half_lat_end_idx-j+1
 * (:94-95); the flag for j=1 lands one past the last half row (an
 * out-of-bounds write in the reference, dropped here). */
static void filter_init(gdo_model* m) {
  int N = m->N, M = m->M, Mh = m->Mh;
  m->flag_full = (int*)calloc(M + 2, sizeof(int));
  m->flag_half = (int*)calloc(Mh + 3, sizeof(int));
  m->ffac_full = zalloc((size_t)(M + 2) * N);
  m->ffac_half = zalloc((size_t)(Mh + 2) * N);
  if (m->use_filter) {
    for (int j = 1; j <= 20; ++j) {
      if (m->cutoff[j - 1] != 0) {
        m->flag_full[1 + j] = 1;
        m->flag_half[1 + j - 1] = 1;
      }
    }
    for (int j = 1; j <= 20; ++j) {
      if (m->cutoff[j - 1] != 0) {
        m->flag_full[M - j] = 1;
        if (M - j + 1 <= Mh) m->flag_half[M - j + 1] = 1;
      }
    }
  }
  for (int j = 1; j <= 20; ++j) {
    int c = m->cutoff[j - 1];
    if (c == 0) continue;
    for (int i = 1; i <= c + 1; ++i) {
      /* factor index 2i-1 and 2i (1-based) -> 0-based 2i-2 and 2i-1 */
      m->ffac_full[(size_t)(1 + j) * N + 2 * i - 2] = 1.0;
      m->ffac_full[(size_t)(1 + j) * N + 2 * i - 1] = 1.0;
      m->ffac_half[(size_t)(1 + j - 1) * N + 2 * i - 2] = 1.0;
      m->ffac_half[(size_t)(1 + j - 1) * N + 2 * i - 1] = 1.0;
      m->ffac_full[(size_t)(M - j) * N + 2 * i - 2] = 1.0;
      m->ffac_full[(size_t)(M - j) * N + 2 * i - 1] = 1.0;
      m->ffac_half[(size_t)(Mh - j + 1) * N + 2 * i - 2] = 1.0;
      m->ffac_half[(size_t)(Mh - j + 1) * N + 2 * i - 1] = 1.0;
    }
  }
  m->ctab = zalloc(N);
  m->stab = zalloc(N);
  for (int k = 0; k < N; ++k) {
    m->ctab[k] = cos(2.0 * PI * k / N);
    m->stab[k] = sin(2.0 * PI * k / N);
  }
}

gdo_model* gdo_create(int num_lon, int num_lat, double time_step_size,
                      int subcycles, int split_scheme, int qcon_modified,
                      int uv_adv_scheme, double upwind_lon_beta,
                      double upwind_lat_beta, int use_zonal_tend_filter,
                      const int* cutoff, int use_diffusion,
                      double diffusion_coef, int diffusion_order) {
  gdo_model* m = (gdo_model*)calloc(1, sizeof(gdo_model));
  m->N = num_lon; m->M = num_lat; m->Mh = num_lat - 1; m->NP = num_lon + 4;
  m->dt = time_step_size;
  m->subcycles = subcycles;
  m->split = (split_scheme == CSP2 || split_scheme == ISP) ? split_scheme : NO_SPLIT;
  m->qcon = qcon_modified;
  m->adv = uv_adv_scheme;
  m->beta_lon = upwind_lon_beta;
  m->beta_lat = upwind_lat_beta;
  m->use_filter = use_zonal_tend_filter;
  for (int k = 0; k < 20; ++k) m->cutoff[k] = cutoff ? cutoff[k] : 0;
  m->use_diff = use_diffusion;
  m->diff_coef = diffusion_coef;
  m->diff_order = diffusion_order;
  mesh_init(m);
  data_init(m);
  filter_init(m);
  m->d_ud = zalloc(full_sz(m)); m->d_gdd = zalloc(full_sz(m));
  m->d_u = zalloc(full_sz(m)); m->d_gd = zalloc(full_sz(m));
  m->d_vd = zalloc(half_sz(m)); m->d_v = zalloc(half_sz(m));
  if (m->adv == WENO) {
    m->w_fpu = zalloc(full_sz(m)); m->w_fnu = zalloc(full_sz(m)); m->w_fu = zalloc(full_sz(m));
    m->w_fpv = zalloc(half_sz(m)); m->w_fnv = zalloc(half_sz(m)); m->w_fv = zalloc(half_sz(m));
  }
  m->old = 1; m->new_ = 2; /* src/time_mod.F90:68-69 */
  m->last_beta = 1.0;
  return m;
}

void gdo_set_rescale_rtol(gdo_model* m, double rtol) { m->rescale_rtol = rtol; }

void gdo_rescale_record(gdo_model* m, double* cond, int* field, int* row) {
  for (int k = 0; k < 2; ++k) {
    cond[k] = m->rc_cond[k];
    field[k] = m->rc_field[k];
    row[k] = m->rc_row[k];
    m->rc_cond[k] = 0.0;
  }
}

int gdo_set_fft(gdo_model* m, int on) {
  if (!on) {
    m->fft = 0;
    return 0;
  }
  if (!m->plan.ok) {
    if (gdo_rfft_init(&m->plan, m->N) != 0) return -1;
    m->fft_r = zalloc(m->N);
    m->fft_w = zalloc(m->N);
  }
  m->fft = 1;
  return 0;
}

int gdo_rfft_row(int n, int backward, double* x) {
  gdo_rfft p;
  if (gdo_rfft_init(&p, n) != 0) {
    gdo_rfft_free(&p);
    return -1;
  }
  double* w = zalloc(n);
  if (backward)
    gdo_rfft_backward(&p, x, w);
  else
    gdo_rfft_forward(&p, x, w);
  free(w);
  gdo_rfft_free(&p);
  return 0;
}

double gdo_fsum(const double* x, int n) {
  xsum acc;
  xs_init(&acc);
  for (int k = 0; k < n; ++k) xs_add(&acc, x[k]);
  return xs_value(&acc);
}

void gdo_destroy(gdo_model* m) {
  if (!m) return;
  double* bufs[] = {m->full_lat, m->half_lat, m->full_cos, m->half_cos,
                    m->full_sin, m->half_sin, m->full_f, m->half_f, m->full_c,
                    m->half_c, m->full_dlon, m->half_dlon, m->full_dlat,
                    m->half_dlat, m->ghs, m->ffac_full, m->ffac_half, m->ctab,
                    m->stab, m->d_ud, m->d_vd, m->d_gdd, m->d_u, m->d_v, m->d_gd,
                    m->w_fpu, m->w_fnu, m->w_fu, m->w_fpv, m->w_fnv, m->w_fv};
  for (size_t k = 0; k < sizeof(bufs) / sizeof(bufs[0]); ++k) free(bufs[k]);
  for (int k = 0; k < 4; ++k) {
    state_t* s = &m->state_mem[k];
    free(s->u); free(s->v); free(s->gd); free(s->iu); free(s->iv); free(s->ig);
  }
  for (int k = 0; k < 5; ++k)
    for (int f = 0; f < T_NFIELD; ++f) free(m->tend_mem[k].a[f]);
  free(m->flag_full); free(m->flag_half);
  gdo_rfft_free(&m->plan);
  free(m->fft_r); free(m->fft_w);
  free(m);
}

/* ------------------------------------------------------------- filter */

/* src/filter_mod.F90:105-167 with FFTPACK 5.1 rfft1f/rfft1b
 * (lib/fft/rfftf1.f:87-109 packing, lib/fft/rfftb1.f:43-59 unpacking).
 * The packed forward transform is r(1) = a0 = (1/N) sum x, r(2k) = a_k =
 * (2/N) sum x cos(2 pi k n/N), r(2k+1) = b_k = (2/N) sum x sin(...), and
 * r(N) = (1/N) sum x (-1)^n for even N; backward rebuilds x_n = a0 +
 * sum_k (a_k cos + b_k sin) + r(N)(-1)^n.  Coefficients whose factor is 0
 * drop out, so only the kept ones are evaluated. */
/* src/filter_mod.F90:105-135 as the reference computes it: the row through
 * rfft1f, times the factor row, back through rfft1b. */
static void filter_row_fftpack(const gdo_model* m, const double* fac, double* x) {
  int N = m->N;
  double *r = m->fft_r, *w = m->fft_w;
  for (int i = 1; i <= N; ++i) r[i - 1] = x[i + 1];
  gdo_rfft_forward(&m->plan, r, w);
  for (int p = 0; p < N; ++p) r[p] = r[p] * fac[p];
  gdo_rfft_backward(&m->plan, r, w);
  for (int i = 1; i <= N; ++i) x[i + 1] = r[i - 1];
}

static void filter_row(const gdo_model* m, const double* fac, double* x) {
  int N = m->N;
  if (m->fft) {
    filter_row_fftpack(m, fac, x);
    return;
  }
  double* local = zalloc(N);
  double* coefs = zalloc(N);
  for (int i = 1; i <= N; ++i) local[i - 1] = x[i + 1];
  for (int p = 0; p < N; ++p) { /* p = packed index - 1 */
    if (fac[p] == 0.0) continue;
    xsum acc;
    xs_init(&acc);
    double s;
    if (p == 0) {
      for (int n = 0; n < N; ++n) xs_add(&acc, local[n]);
      s = xs_value(&acc) * (1.0 / N);
    } else if (N % 2 == 0 && p == N - 1) {
      for (int n = 0; n < N; ++n) xs_add(&acc, (n & 1) ? -local[n] : local[n]);
      s = xs_value(&acc) * (1.0 / N);
    } else {
      int k = (p + 1) / 2;
      const double* tab = (p % 2 == 1) ? m->ctab : m->stab;
      for (int n = 0; n < N; ++n) xs_add(&acc, local[n] * tab[(int)(((long)k * n) % N)]);
      s = xs_value(&acc) * (2.0 / N);
    }
    coefs[p] = s * fac[p];
  }
  for (int n = 0; n < N; ++n) {
    double y = 0.0;
    for (int p = 0; p < N; ++p) {
      if (fac[p] == 0.0) continue;
      if (p == 0) {
        y = y + coefs[p];
      } else if (N % 2 == 0 && p == N - 1) {
        y = y + ((n & 1) ? -coefs[p] : coefs[p]);
      } else {
        int k = (p + 1) / 2;
        const double* tab = (p % 2 == 1) ? m->ctab : m->stab;
        y = y + coefs[p] * tab[(int)(((long)k * n) % N)];
      }
    }
    local[n] = y;
  }
  for (int i = 1; i <= N; ++i) x[i + 1] = local[i - 1];
  free(local);
  free(coefs);
}

void gdo_filter_row(const gdo_model* m, int half, int lat_idx, double* x) {
  const double* fac = (half ? m->ffac_half : m->ffac_full) + (size_t)lat_idx * m->N;
  filter_row(m, fac, x);
}

void gdo_filter_flags(const gdo_model* m, int* out_full, int* out_half,
                      int* cut_full, int* cut_half) {
  for (int j = 1; j <= m->M; ++j) {
    if (out_full) out_full[j - 1] = m->flag_full[j];
    if (cut_full) {
      const double* f = m->ffac_full + (size_t)j * m->N;
      int c = -1;
      for (int p = 0; p < m->N; ++p)
        if (f[p] != 0.0) c = p;
      cut_full[j - 1] = c < 0 ? -1 : (c + 1) / 2 - 1;
    }
  }
  for (int j = 1; j <= m->Mh; ++j) {
    if (out_half) out_half[j - 1] = m->flag_half[j];
    if (cut_half) {
      const double* f = m->ffac_half + (size_t)j * m->N;
      int c = -1;
      for (int p = 0; p < m->N; ++p)
        if (f[p] != 0.0) c = p;
      cut_half[j - 1] = c < 0 ? -1 : (c + 1) / 2 - 1;
    }
  }
}

/* ---------------------------------------------------------- operators */

/* ------------------------------------------------------------ WENO
 * src/weno_mod.F90 with weno_order = 2, restated as the reference runs it:
 * Lax-Friedrichs split fluxes with u_max = v_max = 20, the two-stencil
 * weno_2nd_order_pass, and the reference's index choices kept as they are:
 * u_adv_lon divides by coef%half_dlon(j) (:153-154), u_adv_lat's correction
 * term takes v at lon i-1, i (:281-282), and the lat halos of the split
 * fluxes are never filled (parallel_fill_halo fills lon halos only,
 * src/parallel_mod.F90:466-524), so the pole and lat-halo rows of every
 * split and interface flux are zero. */
#define WENO_EPS 1.0e-6
#define WENO_UMAX 20.0
#define WENO_VMAX 20.0

/* src/weno_mod.F90:249-298 (coefficients :41-46) */
static double weno_2nd_order_pass(double fp1, double fp2, double fp3, double fn2, double fn3, double fn4) {
  const double c11 = -(1.0 / 2.0), c21 = 3.0 / 2.0, c12 = 1.0 / 2.0, c22 = 1.0 / 2.0;
  const double wo1 = 1.0 / 3.0, wo2 = 2.0 / 3.0;
  double fs1 = c11 * fp1 + c21 * fp2, fs2 = c12 * fp2 + c22 * fp3;
  double b1 = (fp2 - fp1) * (fp2 - fp1), b2 = (fp3 - fp2) * (fp3 - fp2);
  double w1 = wo1 / ((WENO_EPS + b1) * (WENO_EPS + b1)), w2 = wo2 / ((WENO_EPS + b2) * (WENO_EPS + b2));
  double sw = w1 + w2;
  w1 = w1 / sw;
  w2 = w2 / sw;
  double f = w1 * fs1 + w2 * fs2;
  fs1 = c11 * fn4 + c21 * fn3;
  fs2 = c12 * fn3 + c22 * fn2;
  b1 = (fn3 - fn4) * (fn3 - fn4);
  b2 = (fn2 - fn3) * (fn2 - fn3);
  w1 = wo1 / ((WENO_EPS + b1) * (WENO_EPS + b1));
  w2 = wo2 / ((WENO_EPS + b2) * (WENO_EPS + b2));
  sw = w1 + w2;
  w1 = w1 / sw;
  w2 = w2 / sw;
  return f + (w1 * fs1 + w2 * fs2);
}

/* src/weno_mod.F90:58-159 */
static void weno_zonal(gdo_model* m, const state_t* s, tend_t* t) {
  int N = m->N, M = m->M, Mh = m->Mh;
  double *fpu = m->w_fpu, *fnu = m->w_fnu, *fu = m->w_fu, *fpv = m->w_fpv, *fnv = m->w_fnv, *fv = m->w_fv;
  double *ual = t->a[T_U_ADV_LON], *val = t->a[T_V_ADV_LON];
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i) {
      AT(m, fpu, i, j) = 0.5 * (AT(m, s->u, i, j) + WENO_UMAX) * AT(m, s->iu, i, j);
      AT(m, fnu, i, j) = 0.5 * (AT(m, s->u, i, j) - WENO_UMAX) * AT(m, s->iu, i, j);
    }
  fill_halo(m, fpu, 0);
  fill_halo(m, fnu, 0);
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i) {
      double u = 0.25 * (AT(m, s->u, i - 1, j) + AT(m, s->u, i - 1, j + 1) + AT(m, s->u, i, j) + AT(m, s->u, i, j + 1));
      AT(m, fpv, i, j) = 0.5 * (u + WENO_UMAX) * AT(m, s->iv, i, j);
      AT(m, fnv, i, j) = 0.5 * (u - WENO_UMAX) * AT(m, s->iv, i, j);
    }
  fill_halo(m, fpv, 1);
  fill_halo(m, fnv, 1);
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, fu, i, j) = weno_2nd_order_pass(AT(m, fpu, i - 1, j), AT(m, fpu, i, j), AT(m, fpu, i + 1, j),
                                            AT(m, fnu, i, j), AT(m, fnu, i + 1, j), AT(m, fnu, i + 2, j));
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, fv, i, j) = weno_2nd_order_pass(AT(m, fpv, i - 1, j), AT(m, fpv, i, j), AT(m, fpv, i + 1, j),
                                            AT(m, fnv, i, j), AT(m, fnv, i + 1, j), AT(m, fnv, i + 2, j));
  fill_halo(m, fu, 0);
  fill_halo(m, fv, 1);
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, ual, i, j) = (AT(m, fu, i, j) - AT(m, fu, i - 1, j) -
                          (AT(m, s->u, i + 1, j) - AT(m, s->u, i - 1, j)) * AT(m, s->iu, i, j) * 0.25) /
                         m->half_dlon[j];
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, val, i, j) = (AT(m, fv, i, j) - AT(m, fv, i - 1, j) -
                          (AT(m, s->u, i, j) + AT(m, s->u, i, j + 1) - AT(m, s->u, i - 1, j) -
                           AT(m, s->u, i - 1, j + 1)) * AT(m, s->iv, i, j) * 0.25) /
                         m->half_dlon[j];
}

/* src/weno_mod.F90:161-247 */
static void weno_meridional(gdo_model* m, const state_t* s, tend_t* t) {
  int N = m->N, M = m->M, Mh = m->Mh;
  double *fpu = m->w_fpu, *fnu = m->w_fnu, *fu = m->w_fu, *fpv = m->w_fpv, *fnv = m->w_fnv, *fv = m->w_fv;
  double *ual = t->a[T_U_ADV_LAT], *val = t->a[T_V_ADV_LAT];
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i) {
      double v = 0.25 * (AT(m, s->v, i, j - 1) + AT(m, s->v, i, j) + AT(m, s->v, i + 1, j - 1) + AT(m, s->v, i + 1, j));
      AT(m, fpu, i, j) = 0.5 * (v + WENO_VMAX) * AT(m, s->iu, i, j);
      AT(m, fnu, i, j) = 0.5 * (v - WENO_VMAX) * AT(m, s->iu, i, j);
    }
  fill_halo(m, fpu, 0);
  fill_halo(m, fnu, 0);
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i) {
      AT(m, fpv, i, j) = 0.5 * (AT(m, s->v, i, j) + WENO_VMAX) * AT(m, s->iv, i, j);
      AT(m, fnv, i, j) = 0.5 * (AT(m, s->v, i, j) - WENO_VMAX) * AT(m, s->iv, i, j);
    }
  fill_halo(m, fpv, 1);
  fill_halo(m, fnv, 1);
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, fu, i, j) = weno_2nd_order_pass(AT(m, fpu, i, j - 1), AT(m, fpu, i, j), AT(m, fpu, i, j + 1),
                                            AT(m, fnu, i, j), AT(m, fnu, i, j + 1), AT(m, fnu, i, j + 2));
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, fv, i, j) = weno_2nd_order_pass(AT(m, fpv, i, j - 1), AT(m, fpv, i, j), AT(m, fpv, i, j + 1),
                                            AT(m, fnv, i, j), AT(m, fnv, i, j + 1), AT(m, fnv, i, j + 2));
  fill_halo(m, fu, 0);
  fill_halo(m, fv, 1);
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, ual, i, j) = (AT(m, fu, i, j) - AT(m, fu, i, j - 1) -
                          (AT(m, s->v, i - 1, j) + AT(m, s->v, i, j) - AT(m, s->v, i - 1, j - 1) -
                           AT(m, s->v, i, j - 1)) * AT(m, s->iu, i, j) * 0.25) /
                         m->full_dlat[j];
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, val, i, j) = (AT(m, fv, i, j) - AT(m, fv, i, j - 1) -
                          (AT(m, s->v, i, j + 1) - AT(m, s->v, i, j - 1)) * AT(m, s->iv, i, j) * 0.25) /
                         m->half_dlat[j];
}

/* src/dycore_mod.F90:367-420 */
static void zonal_momentum_advection(gdo_model* m, const state_t* s, tend_t* t) {
  int N = m->N, M = m->M, Mh = m->Mh;
  if (m->adv == WENO) {
    weno_zonal(m, s, t);
    return;
  }
  double *ual = t->a[T_U_ADV_LON], *val = t->a[T_V_ADV_LON];
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i) {
      double u1 = AT(m, s->u, i, j) + AT(m, s->u, i - 1, j);
      double u2 = AT(m, s->u, i, j) + AT(m, s->u, i + 1, j);
      if (m->adv == CENTER_DIFF) {
        AT(m, ual, i, j) = 0.25 / m->full_dlon[j] *
                           (u2 * AT(m, s->iu, i + 1, j) - u1 * AT(m, s->iu, i - 1, j));
      } else {
        AT(m, ual, i, j) = 0.25 / m->full_dlon[j] *
            (u2 * (AT(m, s->iu, i, j) + AT(m, s->iu, i + 1, j)) -
             m->beta_lon * fabs(u2) * (AT(m, s->iu, i + 1, j) - AT(m, s->iu, i, j)) -
             u1 * (AT(m, s->iu, i, j) + AT(m, s->iu, i - 1, j)) +
             m->beta_lon * fabs(u1) * (AT(m, s->iu, i, j) - AT(m, s->iu, i - 1, j)) -
             (u2 - u1) * AT(m, s->iu, i, j));
      }
    }
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i) {
      double u1 = AT(m, s->u, i - 1, j) + AT(m, s->u, i - 1, j + 1);
      double u2 = AT(m, s->u, i, j) + AT(m, s->u, i, j + 1);
      if (m->adv == CENTER_DIFF) {
        AT(m, val, i, j) = 0.25 / m->half_dlon[j] *
                           (u2 * AT(m, s->iv, i + 1, j) - u1 * AT(m, s->iv, i - 1, j));
      } else {
        AT(m, val, i, j) = 0.25 / m->half_dlon[j] *
            (u2 * (AT(m, s->iv, i, j) + AT(m, s->iv, i + 1, j)) -
             m->beta_lon * fabs(u2) * (AT(m, s->iv, i + 1, j) - AT(m, s->iv, i, j)) -
             u1 * (AT(m, s->iv, i, j) + AT(m, s->iv, i - 1, j)) +
             m->beta_lon * fabs(u1) * (AT(m, s->iv, i, j) - AT(m, s->iv, i - 1, j)) -
             (u2 - u1) * AT(m, s->iv, i, j));
      }
    }
}

/* src/dycore_mod.F90:422-475.  half_cos(0) and half_cos(Mh+1) are read out
 * of bounds by the reference at :443-444 and :463-464; they always multiply
 * a zero lat-halo v, so the pads hold 0.0 and the product is 0. */
static void meridional_momentum_advection(gdo_model* m, const state_t* s, tend_t* t) {
  int N = m->N, M = m->M, Mh = m->Mh;
  if (m->adv == WENO) {
    weno_meridional(m, s, t);
    return;
  }
  double *ual = t->a[T_U_ADV_LAT], *val = t->a[T_V_ADV_LAT];
  const double* hc = m->half_cos;
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i) {
      double v1 = (AT(m, s->v, i, j - 1) + AT(m, s->v, i + 1, j - 1)) * hc[j - 1];
      double v2 = (AT(m, s->v, i, j) + AT(m, s->v, i + 1, j)) * hc[j];
      if (m->adv == CENTER_DIFF) {
        AT(m, ual, i, j) = 0.25 / m->full_dlat[j] *
                           (v2 * AT(m, s->iu, i, j + 1) - v1 * AT(m, s->iu, i, j - 1));
      } else {
        AT(m, ual, i, j) = 0.25 / m->full_dlat[j] *
            (v2 * (AT(m, s->iu, i, j) + AT(m, s->iu, i, j + 1)) -
             m->beta_lat * fabs(v2) * (AT(m, s->iu, i, j + 1) - AT(m, s->iu, i, j)) -
             v1 * (AT(m, s->iu, i, j) + AT(m, s->iu, i, j - 1)) +
             m->beta_lat * fabs(v1) * (AT(m, s->iu, i, j) - AT(m, s->iu, i, j - 1)) -
             (v2 - v1) * AT(m, s->iu, i, j));
      }
    }
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i) {
      double v1 = AT(m, s->v, i, j) * hc[j] + AT(m, s->v, i, j - 1) * hc[j - 1];
      double v2 = AT(m, s->v, i, j) * hc[j] + AT(m, s->v, i, j + 1) * hc[j + 1];
      if (m->adv == CENTER_DIFF) {
        AT(m, val, i, j) = 0.25 / m->half_dlat[j] *
                           (v2 * AT(m, s->iv, i, j + 1) - v1 * AT(m, s->iv, i, j - 1));
      } else {
        AT(m, val, i, j) = 0.25 / m->half_dlat[j] *
            (v2 * (AT(m, s->iv, i, j) + AT(m, s->iv, i, j + 1)) -
             m->beta_lat * fabs(v2) * (AT(m, s->iv, i, j + 1) - AT(m, s->iv, i, j)) -
             v1 * (AT(m, s->iv, i, j) + AT(m, s->iv, i, j - 1)) +
             m->beta_lat * fabs(v1) * (AT(m, s->iv, i, j) - AT(m, s->iv, i, j - 1)) -
             (v2 - v1) * AT(m, s->iv, i, j));
      }
    }
}

/* src/dycore_mod.F90:477-505 */
static void coriolis(gdo_model* m, const state_t* s, tend_t* t) {
  int N = m->N, M = m->M, Mh = m->Mh;
  double *fv = t->a[T_FV], *fu = t->a[T_FU];
  for (int j = 2; j <= M - 1; ++j) {
    double c1 = m->half_cos[j - 1] / m->full_cos[j];
    double c2 = m->half_cos[j] / m->full_cos[j];
    for (int i = 1; i <= N; ++i)
      AT(m, fv, i, j) = 0.25 * (m->full_f[j] + m->full_c[j] * AT(m, s->u, i, j)) *
                        (c1 * (AT(m, s->iv, i, j - 1) + AT(m, s->iv, i + 1, j - 1)) +
                         c2 * (AT(m, s->iv, i, j) + AT(m, s->iv, i + 1, j)));
  }
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, fu, i, j) = 0.25 *
          ((m->full_f[j] + m->full_c[j] * AT(m, s->u, i, j)) * AT(m, s->iu, i, j) +
           (m->full_f[j] + m->full_c[j] * AT(m, s->u, i - 1, j)) * AT(m, s->iu, i - 1, j) +
           (m->full_f[j + 1] + m->full_c[j + 1] * AT(m, s->u, i, j + 1)) * AT(m, s->iu, i, j + 1) +
           (m->full_f[j + 1] + m->full_c[j + 1] * AT(m, s->u, i - 1, j + 1)) * AT(m, s->iu, i - 1, j + 1));
}

/* src/dycore_mod.F90:507-537 */
static void pressure_gradient(gdo_model* m, const state_t* s, tend_t* t) {
  int N = m->N, M = m->M, Mh = m->Mh;
  double *up = t->a[T_U_PGF], *vp = t->a[T_V_PGF];
  const double* ghs = m->ghs;
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, up, i, j) = 0.5 * (AT(m, s->ig, i, j) + AT(m, s->ig, i + 1, j)) / m->full_dlon[j] *
                        (AT(m, s->gd, i + 1, j) + AT(m, ghs, i + 1, j) - AT(m, s->gd, i, j) - AT(m, ghs, i, j));
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, vp, i, j) = 0.5 * (AT(m, s->ig, i, j) + AT(m, s->ig, i, j + 1)) / m->half_dlat[j] * m->half_cos[j] *
                        (AT(m, s->gd, i, j + 1) + AT(m, ghs, i, j + 1) - AT(m, s->gd, i, j) - AT(m, ghs, i, j));
}

/* src/dycore_mod.F90:539-598 (pole caps :572-596; parallel_zonal_sum is an
 * empty stub, src/parallel_mod.F90:604-610, so the local sum is final). */
static void mass_divergence(gdo_model* m, const state_t* s, tend_t* t) {
  int N = m->N, M = m->M;
  double *ml = t->a[T_MDLON], *mt = t->a[T_MDLAT];
  const double* hc = m->half_cos;
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, ml, i, j) = ((AT(m, s->ig, i, j) + AT(m, s->ig, i + 1, j)) * AT(m, s->iu, i, j) -
                         (AT(m, s->ig, i, j) + AT(m, s->ig, i - 1, j)) * AT(m, s->iu, i - 1, j)) *
                        0.5 / m->full_dlon[j];
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, mt, i, j) = ((AT(m, s->ig, i, j) + AT(m, s->ig, i, j + 1)) * AT(m, s->iv, i, j) * hc[j] -
                         (AT(m, s->ig, i, j) + AT(m, s->ig, i, j - 1)) * AT(m, s->iv, i, j - 1) * hc[j - 1]) *
                        0.5 / m->full_dlat[j];
  {
    int j = 1;
    xsum acc;
    xs_init(&acc);
    for (int i = 1; i <= N; ++i)
      xs_add(&acc, (AT(m, s->ig, i, j) + AT(m, s->ig, i, j + 1)) * AT(m, s->iv, i, j));
    double sp = xs_value(&acc);
    sp = sp * 2.0 / N / RADIUS / m->dlat;
    for (int i = 1; i <= N; ++i) AT(m, mt, i, j) = sp;
  }
  {
    int j = M;
    xsum acc;
    xs_init(&acc);
    for (int i = 1; i <= N; ++i)
      xs_add(&acc, (AT(m, s->ig, i, j) + AT(m, s->ig, i, j - 1)) * AT(m, s->iv, i, j - 1));
    double np = -xs_value(&acc);
    np = np * 2.0 / N / RADIUS / m->dlat;
    for (int i = 1; i <= N; ++i) AT(m, mt, i, j) = np;
  }
}

/* s1/s2 rescaled row filter, src/dycore_mod.F90:212-219 and repeats.  With
 * rescale_rtol > 0 (an extension shared with the CUDA path; 0 is the
 * reference) the rescale is skipped when s1 or s2 is zero to within rtol of
 * the sum of its terms' magnitudes. */
static void filter_tend_row(gdo_model* m, const double* fac, double* trow,
                            const double* w1, const double* w2) {
  int N = m->N;
  double s1, s2, a1 = 0.0, a2 = 0.0;
  xsum acc;
  xs_init(&acc);
  for (int i = 1; i <= N; ++i) {
    double t = trow[i + 1] * (w2 ? (w1[i + 1] + w2[i + 1]) : w1[i + 1]);
    xs_add(&acc, t);
    a1 = a1 + fabs(t);
  }
  s1 = xs_value(&acc);
  if (fabs(s1) > 1.0e-16 && a1 / fabs(s1) > m->rc_cond[0]) {
    m->rc_cond[0] = a1 / fabs(s1);
    m->rc_field[0] = m->cur_field;
    m->rc_row[0] = m->cur_row;
  }
  if (fabs(s1) > 1.0e-16) { /* src/filter_mod.F90:31 */
    filter_row(m, fac, trow);
    xs_init(&acc);
    for (int i = 1; i <= N; ++i) {
      double t = trow[i + 1] * (w2 ? (w1[i + 1] + w2[i + 1]) : w1[i + 1]);
      xs_add(&acc, t);
      a2 = a2 + fabs(t);
    }
    s2 = xs_value(&acc);
    if (a2 / fabs(s2) > m->rc_cond[1]) {
      m->rc_cond[1] = a2 / fabs(s2);
      m->rc_field[1] = m->cur_field;
      m->rc_row[1] = m->cur_row;
    }
    if (m->rescale_rtol > 0 && (fabs(s1) <= m->rescale_rtol * a1 || fabs(s2) <= m->rescale_rtol * a2)) return;
    for (int i = 1; i <= N; ++i) trow[i + 1] = trow[i + 1] * s1 / s2;
  }
}

#define ROW(m, f, j) ((f) + (size_t)((j) + 1) * (m)->NP)

/* src/dycore_mod.F90:184-365 */
static void space_operators(gdo_model* m, const state_t* s, tend_t* t, int pass) {
  int N = m->N, M = m->M, Mh = m->Mh;
  double *du = t->a[T_DU], *dv = t->a[T_DV], *dgd = t->a[T_DGD];
  if (pass == ALL_PASS || pass == SLOW_PASS) {
    zonal_momentum_advection(m, s, t);
    meridional_momentum_advection(m, s, t);
  }
  if (pass == ALL_PASS || pass == FAST_PASS) {
    coriolis(m, s, t);
    pressure_gradient(m, s, t);
    mass_divergence(m, s, t);
  }
  const double *ual = t->a[T_U_ADV_LON], *uat = t->a[T_U_ADV_LAT], *fv = t->a[T_FV],
               *up = t->a[T_U_PGF], *val = t->a[T_V_ADV_LON], *vat = t->a[T_V_ADV_LAT],
               *fu = t->a[T_FU], *vp = t->a[T_V_PGF], *ml = t->a[T_MDLON], *mt = t->a[T_MDLAT];
  /* dgd first in the fast pass (:311-325), last in the all pass (:239-253);
   * the order does not matter for the values. */
  if (pass == ALL_PASS || pass == FAST_PASS) {
    for (int j = 1; j <= M; ++j) {
      for (int i = 1; i <= N; ++i) AT(m, dgd, i, j) = -AT(m, ml, i, j) - AT(m, mt, i, j);
      if (m->flag_full[j]) {
        m->cur_field = 2;
        m->cur_row = j;
        filter_tend_row(m, m->ffac_full + (size_t)j * N, ROW(m, dgd, j), ROW(m, s->gd, j), ROW(m, m->ghs, j));
      }
    }
  } else {
    memset(dgd, 0, full_sz(m) * sizeof(double)); /* :297 */
  }
  for (int j = 2; j <= M - 1; ++j) {
    for (int i = 1; i <= N; ++i) {
      if (pass == ALL_PASS)
        AT(m, du, i, j) = -AT(m, ual, i, j) - AT(m, uat, i, j) + AT(m, fv, i, j) - AT(m, up, i, j);
      else if (pass == SLOW_PASS)
        AT(m, du, i, j) = -AT(m, ual, i, j) - AT(m, uat, i, j);
      else
        AT(m, du, i, j) = AT(m, fv, i, j) - AT(m, up, i, j);
    }
    if (m->flag_full[j]) {
      m->cur_field = 0;
      m->cur_row = j;
      filter_tend_row(m, m->ffac_full + (size_t)j * N, ROW(m, du, j), ROW(m, s->iu, j), NULL);
    }
  }
  for (int j = 1; j <= Mh; ++j) {
    for (int i = 1; i <= N; ++i) {
      if (pass == ALL_PASS)
        AT(m, dv, i, j) = -AT(m, val, i, j) - AT(m, vat, i, j) - AT(m, fu, i, j) - AT(m, vp, i, j);
      else if (pass == SLOW_PASS)
        AT(m, dv, i, j) = -AT(m, val, i, j) - AT(m, vat, i, j);
      else
        AT(m, dv, i, j) = -AT(m, fu, i, j) - AT(m, vp, i, j);
    }
    if (m->flag_half[j]) {
      m->cur_field = 1;
      m->cur_row = j;
      filter_tend_row(m, m->ffac_half + (size_t)j * N, ROW(m, dv, j), ROW(m, s->iv, j), NULL);
    }
  }
}

/* src/dycore_mod.F90:600-652 */
static void update_state(gdo_model* m, double dt, const tend_t* t, const state_t* o, state_t* n) {
  int N = m->N, M = m->M, Mh = m->Mh;
  const double *du = t->a[T_DU], *dv = t->a[T_DV], *dgd = t->a[T_DGD];
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i) AT(m, n->gd, i, j) = AT(m, o->gd, i, j) + dt * AT(m, dgd, i, j);
  fill_halo(m, n->gd, 0);
  for (size_t k = 0; k < full_sz(m); ++k) n->ig[k] = sqrt(n->gd[k]);
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i) AT(m, n->iu, i, j) = AT(m, o->iu, i, j) + dt * AT(m, du, i, j);
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i) AT(m, n->iv, i, j) = AT(m, o->iv, i, j) + dt * AT(m, dv, i, j);
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, n->u, i, j) = AT(m, n->iu, i, j) * 2.0 / (AT(m, n->ig, i, j) + AT(m, n->ig, i + 1, j));
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, n->v, i, j) = AT(m, n->iv, i, j) * 2.0 / (AT(m, n->ig, i, j) + AT(m, n->ig, i, j + 1));
  fill_halo(m, n->iu, 0);
  fill_halo(m, n->iv, 1);
  fill_halo(m, n->u, 0);
  fill_halo(m, n->v, 1);
}

/* src/types_mod.F90:347-371 */
static double ip_tend_tend(const gdo_model* m, const tend_t* a, const tend_t* b) {
  int N = m->N, M = m->M, Mh = m->Mh;
  xsum res;
  xs_init(&res);
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      xs_add(&res, AT(m, a->a[T_DU], i, j) * AT(m, b->a[T_DU], i, j) * m->full_cos[j]);
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      xs_add(&res, AT(m, a->a[T_DV], i, j) * AT(m, b->a[T_DV], i, j) * m->half_cos[j]);
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i)
      xs_add(&res, AT(m, a->a[T_DGD], i, j) * AT(m, b->a[T_DGD], i, j) * m->full_cos[j]);
  return xs_value(&res);
}

/* src/types_mod.F90:373-397 */
static double ip_tend_state(const gdo_model* m, const tend_t* a, const state_t* s) {
  int N = m->N, M = m->M, Mh = m->Mh;
  xsum res;
  xs_init(&res);
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      xs_add(&res, AT(m, a->a[T_DU], i, j) * AT(m, s->iu, i, j) * m->full_cos[j]);
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      xs_add(&res, AT(m, a->a[T_DV], i, j) * AT(m, s->iv, i, j) * m->half_cos[j]);
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i)
      xs_add(&res, AT(m, a->a[T_DGD], i, j) * AT(m, s->gd, i, j) * m->full_cos[j]);
  return xs_value(&res);
}

/* src/dycore_mod.F90:754-792 */
static void predict_correct(gdo_model* m, double time_step_size, int old, int new_, int pass) {
  state_t *so = STATE(m, old), *sn = STATE(m, new_);
  tend_t *to = TEND(m, old), *tn = TEND(m, new_);
  double dt = time_step_size * 0.5;
  space_operators(m, so, to, pass);
  update_state(m, dt, to, so, sn);
  space_operators(m, sn, to, pass);
  update_state(m, dt, to, so, sn);
  space_operators(m, sn, tn, pass);
  double ip1 = ip_tend_tend(m, to, tn);
  double ip2 = ip_tend_tend(m, tn, tn);
  double beta = (m->qcon && ip1 != 0.0 && ip2 != 0.0) ? ip1 / ip2 : 1.0;
  m->last_beta = beta;
  dt = time_step_size * beta;
  update_state(m, dt, tn, so, sn);
}

/* src/dycore_mod.F90:671-687 */
static void csp2_splitting(gdo_model* m) {
  double fast_dt = m->dt / m->subcycles;
  int t1 = 0, t2 = m->old;
  predict_correct(m, 0.5 * m->dt, m->old, t1, SLOW_PASS);
  for (int k = 1; k <= m->subcycles; ++k) {
    predict_correct(m, fast_dt, t1, t2, FAST_PASS);
    int tmp = t1; t1 = t2; t2 = tmp;
  }
  predict_correct(m, 0.5 * m->dt, t1, m->new_, SLOW_PASS);
}

/* src/types_mod.F90:229-345, only du/dv/dgd reach update_state and the
 * inner products, so only they are carried. */
static void tend_axpy(const gdo_model* m, double a, const tend_t* x, tend_t* y) {
  const int f3[3] = {T_DU, T_DV, T_DGD};
  for (int k = 0; k < 3; ++k) {
    size_t n = tend_is_half[f3[k]] ? half_sz(m) : full_sz(m);
    for (size_t q = 0; q < n; ++q) y->a[f3[k]][q] = y->a[f3[k]][q] + a * x->a[f3[k]][q];
  }
}
static void tend_add(const gdo_model* m, const tend_t* x, tend_t* y) {
  const int f3[3] = {T_DU, T_DV, T_DGD};
  for (int k = 0; k < 3; ++k) {
    size_t n = tend_is_half[f3[k]] ? half_sz(m) : full_sz(m);
    for (size_t q = 0; q < n; ++q) y->a[f3[k]][q] = y->a[f3[k]][q] + x->a[f3[k]][q];
  }
}
static void tend_sub(const gdo_model* m, const tend_t* x, tend_t* y) {
  const int f3[3] = {T_DU, T_DV, T_DGD};
  for (int k = 0; k < 3; ++k) {
    size_t n = tend_is_half[f3[k]] ? half_sz(m) : full_sz(m);
    for (size_t q = 0; q < n; ++q) y->a[f3[k]][q] = y->a[f3[k]][q] - x->a[f3[k]][q];
  }
}
static void tend_scale(const gdo_model* m, double a, tend_t* y) {
  const int f3[3] = {T_DU, T_DV, T_DGD};
  for (int k = 0; k < 3; ++k) {
    size_t n = tend_is_half[f3[k]] ? half_sz(m) : full_sz(m);
    for (size_t q = 0; q < n; ++q) y->a[f3[k]][q] = y->a[f3[k]][q] * a;
  }
}
static void state_copy(const gdo_model* m, const state_t* a, state_t* b) {
  memcpy(b->u, a->u, full_sz(m) * sizeof(double));
  memcpy(b->gd, a->gd, full_sz(m) * sizeof(double));
  memcpy(b->iu, a->iu, full_sz(m) * sizeof(double));
  memcpy(b->ig, a->ig, full_sz(m) * sizeof(double));
  memcpy(b->v, a->v, half_sz(m) * sizeof(double));
  memcpy(b->iv, a->iv, half_sz(m) * sizeof(double));
}

/* src/dycore_mod.F90:689-752 */
static void isp_splitting(gdo_model* m) {
  double fast_dt = m->dt / m->subcycles;
  double half_dt = m->dt * 0.5;
  int t1 = m->old, t2 = 0;
  state_t* saved = STATE(m, -1);
  tend_t* slow = TEND(m, -2);
  tend_t* accum = TEND(m, -1);
  state_copy(m, STATE(m, m->old), saved);
  tend_scale(m, 0.0, accum);
  space_operators(m, STATE(m, m->old), slow, SLOW_PASS);
  for (int k = 1; k <= m->subcycles; ++k) {
    space_operators(m, STATE(m, t1), TEND(m, t1), FAST_PASS);
    tend_add(m, slow, TEND(m, t1));
    update_state(m, fast_dt * 0.5, TEND(m, t1), STATE(m, t1), STATE(m, t2));
    space_operators(m, STATE(m, t2), TEND(m, t1), FAST_PASS);
    tend_add(m, slow, TEND(m, t1));
    update_state(m, fast_dt * 0.5, TEND(m, t1), STATE(m, t1), STATE(m, t2));
    space_operators(m, STATE(m, t2), TEND(m, t2), FAST_PASS);
    tend_add(m, TEND(m, t2), accum);
    tend_add(m, slow, TEND(m, t2));
    update_state(m, fast_dt, TEND(m, t2), STATE(m, t1), STATE(m, t2));
    int tmp = t1; t1 = t2; t2 = tmp;
  }
  tend_scale(m, 2.0 / m->subcycles, accum);
  space_operators(m, STATE(m, t1), TEND(m, t1), SLOW_PASS);
  tend_sub(m, slow, TEND(m, t1));
  update_state(m, half_dt, TEND(m, t1), STATE(m, t1), STATE(m, m->new_));
  space_operators(m, STATE(m, m->new_), TEND(m, t1), SLOW_PASS);
  tend_sub(m, slow, TEND(m, t1));
  update_state(m, half_dt, TEND(m, t1), STATE(m, t1), STATE(m, m->new_));
  space_operators(m, STATE(m, m->new_), TEND(m, m->new_), SLOW_PASS);
  tend_add(m, slow, TEND(m, m->new_));
  tend_add(m, accum, TEND(m, m->new_));
  double ip1 = ip_tend_state(m, TEND(m, m->new_), saved);
  double ip2 = ip_tend_tend(m, TEND(m, m->new_), TEND(m, m->new_));
  double beta = (m->qcon && ip1 != 0.0 && ip2 != 0.0) ? ip1 / ip2 : 1.0;
  beta = beta * 4.0 / m->dt;
  m->last_beta = beta;
  half_dt = half_dt * beta;
  update_state(m, half_dt, TEND(m, m->new_), saved, STATE(m, m->new_));
  (void)tend_axpy;
}

/* src/types_mod.F90:399-426 */
static void iap_transform(gdo_model* m, state_t* s) {
  int N = m->N, M = m->M, Mh = m->Mh;
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i) AT(m, s->ig, i, j) = sqrt(AT(m, s->gd, i, j));
  fill_halo(m, s->ig, 0);
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, s->iu, i, j) = 0.5 * (AT(m, s->ig, i, j) + AT(m, s->ig, i + 1, j)) * AT(m, s->u, i, j);
  fill_halo(m, s->iu, 0);
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, s->iv, i, j) = 0.5 * (AT(m, s->ig, i, j) + AT(m, s->ig, i, j + 1)) * AT(m, s->v, i, j);
  fill_halo(m, s->iv, 1);
}

/* src/diffusion_mod.F90:74-217 */
static void ordinary_diffusion(gdo_model* m, double dt, state_t* s) {
  int N = m->N, M = m->M, Mh = m->Mh;
  double *u = m->d_u, *v = m->d_v, *gd = m->d_gd, *ud = m->d_ud, *vd = m->d_vd, *gdd = m->d_gdd;
  const double *fc = m->full_cos, *hc = m->half_cos;
  memcpy(u, s->u, full_sz(m) * sizeof(double));
  memcpy(v, s->v, half_sz(m) * sizeof(double));
  memcpy(gd, s->gd, full_sz(m) * sizeof(double));
  for (int order = 1; order <= m->diff_order / 2; ++order) {
    for (int j = 2; j <= M - 1; ++j)
      for (int i = 1; i <= N; ++i)
        AT(m, gdd, i, j) = (AT(m, gd, i + 1, j) - 2 * AT(m, gd, i, j) + AT(m, gd, i - 1, j)) /
                               (m->full_dlon[j] * m->full_dlon[j]) +
                           ((AT(m, gd, i, j + 1) - AT(m, gd, i, j)) * hc[j] -
                            (AT(m, gd, i, j) - AT(m, gd, i, j - 1)) * hc[j - 1]) /
                               (m->full_dlat[j] * m->full_dlat[j]) * fc[j];
    {
      int j = 1;
      xsum acc;
      xs_init(&acc);
      for (int i = 1; i <= N; ++i) {
        xs_add(&acc, AT(m, gd, i, j + 1));
        xs_add(&acc, -AT(m, gd, i, j));
      }
      double sp = xs_value(&acc);
      double val = sp * hc[j] / (m->full_dlat[j] * m->full_dlat[j]) * fc[j] / N;
      for (int i = -1; i <= N + 2; ++i) AT(m, gdd, i, j) = val;
    }
    {
      int j = M;
      xsum acc;
      xs_init(&acc);
      for (int i = 1; i <= N; ++i) {
#ifdef GDO_PLAIN_SUMS
        /* np = np - (gd(i,j) - gd(i,j-1)), src/diffusion_mod.F90:126-128 */
        xs_add(&acc, -(AT(m, gd, i, j) - AT(m, gd, i, j - 1)));
#else
        xs_add(&acc, -AT(m, gd, i, j));
        xs_add(&acc, AT(m, gd, i, j - 1));
#endif
      }
      double np = xs_value(&acc);
      double val = np * hc[j - 1] / (m->full_dlat[j] * m->full_dlat[j]) * fc[j] / N;
      for (int i = -1; i <= N + 2; ++i) AT(m, gdd, i, j) = val;
    }
    for (int j = 2; j <= M - 1; ++j)
      for (int i = 1; i <= N; ++i)
        AT(m, ud, i, j) = (AT(m, u, i + 1, j) - 2 * AT(m, u, i, j) + AT(m, u, i - 1, j)) /
                              (m->full_dlon[j] * m->full_dlon[j]) +
                          ((AT(m, u, i, j + 1) - AT(m, u, i, j)) * hc[j] -
                           (AT(m, u, i, j) - AT(m, u, i, j - 1)) * hc[j - 1]) /
                              (m->full_dlat[j] * m->full_dlat[j]) * fc[j];
    for (int j = 1; j <= Mh; ++j)
      for (int i = 1; i <= N; ++i)
        AT(m, vd, i, j) = (AT(m, v, i + 1, j) - 2 * AT(m, v, i, j) + AT(m, v, i - 1, j)) /
                          (m->half_dlon[j] * m->half_dlon[j]);
    for (int j = 2; j <= Mh - 1; ++j)
      for (int i = 1; i <= N; ++i)
        AT(m, vd, i, j) = AT(m, vd, i, j) +
                          ((AT(m, v, i, j + 1) - AT(m, v, i, j)) * fc[j + 1] -
                           (AT(m, v, i, j) - AT(m, v, i, j - 1)) * fc[j]) /
                              (m->half_dlat[j] * m->half_dlat[j]) * hc[j];
    {
      int j = 1;
      for (int i = 1; i <= N; ++i)
        AT(m, vd, i, j) = AT(m, vd, i, j) + (AT(m, v, i, j + 1) - AT(m, v, i, j)) * fc[j + 1] /
                                                (m->half_dlat[j] * m->half_dlat[j]) * hc[j];
    }
    {
      int j = Mh;
      for (int i = 1; i <= N; ++i)
        AT(m, vd, i, j) = AT(m, vd, i, j) - (AT(m, v, i, j) - AT(m, v, i, j - 1)) * fc[j] /
                                                (m->half_dlat[j] * m->half_dlat[j]) * hc[j];
    }
    if (order != m->diff_order / 2) {
      fill_halo(m, gdd, 0);
      fill_halo(m, ud, 0);
      fill_halo(m, vd, 1);
      memcpy(gd, gdd, full_sz(m) * sizeof(double));
      memcpy(u, ud, full_sz(m) * sizeof(double));
      memcpy(v, vd, half_sz(m) * sizeof(double));
    }
  }
  for (int j = 2; j <= M - 1; ++j)
    if (m->flag_full[j]) {
      filter_row(m, m->ffac_full + (size_t)j * N, ROW(m, gdd, j));
      filter_row(m, m->ffac_full + (size_t)j * N, ROW(m, ud, j));
    }
  for (int j = 1; j <= Mh; ++j)
    if (m->flag_half[j]) filter_row(m, m->ffac_half + (size_t)j * N, ROW(m, vd, j));
  int half_order = m->diff_order / 2 + 1;
  int sign = (half_order % 2 == 0) ? 1 : -1; /* (-1)**(diffusion_order/2+1) */
  for (int j = 1; j <= M; ++j) {
    for (int i = 1; i <= N; ++i)
      AT(m, s->gd, i, j) = AT(m, s->gd, i, j) + sign * dt * m->diff_coef * AT(m, gdd, i, j);
    for (int i = 1; i <= N; ++i)
      AT(m, s->u, i, j) = AT(m, s->u, i, j) + sign * dt * m->diff_coef * AT(m, ud, i, j);
  }
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      AT(m, s->v, i, j) = AT(m, s->v, i, j) + sign * dt * m->diff_coef * AT(m, vd, i, j);
  fill_halo(m, s->gd, 0);
  fill_halo(m, s->u, 0);
  fill_halo(m, s->v, 1);
  iap_transform(m, s);
}

/* src/diag_mod.F90:71-87, 98-121 */
static int diag_run(gdo_model* m, const state_t* s) {
  int N = m->N, M = m->M, Mh = m->Mh;
  xsum am, ae;
  xs_init(&am);
  xs_init(&ae);
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i)
      xs_add(&am, m->full_cos[j] * m->dlon * m->dlat * AT(m, s->gd, i, j));
  double mass = xs_value(&am) * (RADIUS * RADIUS);
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i)
      xs_add(&ae, AT(m, s->iu, i, j) * AT(m, s->iu, i, j) * m->full_cos[j]);
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i)
      xs_add(&ae, AT(m, s->iv, i, j) * AT(m, s->iv, i, j) * m->half_cos[j]);
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i) {
      double h = AT(m, s->gd, i, j) + AT(m, m->ghs, i, j);
      xs_add(&ae, h * h * m->full_cos[j]);
    }
  double e = xs_value(&ae);
  m->total_mass = mass;
  m->total_energy = e;
  return (isnan(mass) || isnan(e)) ? 1 : 0;
}

/* ------------------------------------------------------------ driver */

void gdo_set_state(gdo_model* m, const double* u, const double* v,
                   const double* gd, const double* ghs) {
  state_t* s = STATE(m, 1);
  memcpy(s->u, u, full_sz(m) * sizeof(double));
  memcpy(s->v, v, half_sz(m) * sizeof(double));
  memcpy(s->gd, gd, full_sz(m) * sizeof(double));
  memcpy(m->ghs, ghs, full_sz(m) * sizeof(double));
}

/* src/dycore_mod.F90:121-129 and :159-173 */
void gdo_run_init(gdo_model* m) {
  int j = 1;
  m->full_cos[j] = m->half_cos[1] * 0.25;
  m->full_dlon[j] = RADIUS * m->dlon * m->full_cos[j];
  m->full_dlat[j] = RADIUS * m->dlat * m->full_cos[j];
  j = m->M;
  m->full_cos[j] = m->half_cos[m->Mh] * 0.25;
  m->full_dlon[j] = RADIUS * m->dlon * m->full_cos[j];
  m->full_dlat[j] = RADIUS * m->dlat * m->full_cos[j];
  iap_transform(m, STATE(m, m->old));
  diag_run(m, STATE(m, m->old));
}

/* src/dycore_mod.F90:131-140, :654-669; src/time_mod.F90:106-130 */
int gdo_step(gdo_model* m, int nsteps) {
  for (int k = 0; k < nsteps; ++k) {
    if (m->split == CSP2)
      csp2_splitting(m);
    else if (m->split == ISP)
      isp_splitting(m);
    else
      predict_correct(m, m->dt, m->old, m->new_, ALL_PASS);
    if (m->use_diff) ordinary_diffusion(m, m->dt, STATE(m, m->new_));
    int tmp = m->old; m->old = m->new_; m->new_ = tmp;
    if (diag_run(m, STATE(m, m->old))) return 1;
  }
  return 0;
}

void gdo_get_state(const gdo_model* m, double* u, double* v, double* gd,
                   double* iap_u, double* iap_v, double* iap_gd) {
  const state_t* s = &m->state_mem[m->old + 1];
  if (u) memcpy(u, s->u, full_sz(m) * sizeof(double));
  if (v) memcpy(v, s->v, half_sz(m) * sizeof(double));
  if (gd) memcpy(gd, s->gd, full_sz(m) * sizeof(double));
  if (iap_u) memcpy(iap_u, s->iu, full_sz(m) * sizeof(double));
  if (iap_v) memcpy(iap_v, s->iv, half_sz(m) * sizeof(double));
  if (iap_gd) memcpy(iap_gd, s->ig, full_sz(m) * sizeof(double));
}

void gdo_diag(const gdo_model* m, double* total_mass, double* total_energy, double* last_beta) {
  if (total_mass) *total_mass = m->total_mass;
  if (total_energy) *total_energy = m->total_energy;
  if (last_beta) *last_beta = m->last_beta;
}

void gdo_tendency(gdo_model* m, int pass, double* du, double* dv, double* dgd) {
  tend_t* t = TEND(m, 0);
  space_operators(m, STATE(m, m->old), t, pass);
  if (du) memcpy(du, t->a[T_DU], full_sz(m) * sizeof(double));
  if (dv) memcpy(dv, t->a[T_DV], half_sz(m) * sizeof(double));
  if (dgd) memcpy(dgd, t->a[T_DGD], full_sz(m) * sizeof(double));
}

/* history_write_state's A-grid wind and gh (src/history_mod.F90:101-108) and
 * diag_run's div and vor (src/diag_mod.F90:49-68) of state(old), in the
 * padded layout (halos 0).  div is left 0 on the pole rows, as the reference
 * never assigns them. */
void gdo_history(const gdo_model* m, double* ua, double* va, double* gh, double* div, double* vor) {
  const int N = m->N, M = m->M, Mh = m->Mh;
  const state_t* s = &m->state_mem[m->old + 1];
  memset(ua, 0, full_sz(m) * sizeof(double));
  memset(va, 0, full_sz(m) * sizeof(double));
  memset(gh, 0, full_sz(m) * sizeof(double));
  memset(div, 0, full_sz(m) * sizeof(double));
  memset(vor, 0, half_sz(m) * sizeof(double));
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i) {
      AT(m, ua, i, j) = 0.5 * (AT(m, s->u, i, j) + AT(m, s->u, i - 1, j));
      AT(m, va, i, j) = 0.5 * (AT(m, s->v, i, j) + AT(m, s->v, i, j - 1));
      AT(m, gh, i, j) = AT(m, s->gd, i, j) + AT(m, m->ghs, i, j);
    }
  for (int j = 2; j <= M - 1; ++j)
    for (int i = 1; i <= N; ++i) {
      const double um1 = AT(m, s->u, i - 1, j), up1 = AT(m, s->u, i, j);
      const double vm1 = AT(m, s->v, i, j - 1) * m->half_cos[j - 1];
      const double vp1 = AT(m, s->v, i, j) * m->half_cos[j];
      AT(m, div, i, j) = (up1 - um1) / m->full_dlon[j] + (vp1 - vm1) / m->full_dlat[j];
    }
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i) {
      const double um1 = AT(m, s->u, i, j), up1 = AT(m, s->u, i, j + 1);
      const double vm1 = AT(m, s->v, i, j), vp1 = AT(m, s->v, i + 1, j);
      AT(m, vor, i, j) = (vp1 - vm1) / m->half_dlon[j] - (up1 - um1) / m->half_dlat[j];
    }
}

/* src/dycore_mod.F90:794-851 (disabled in the reference, :363). */
void gdo_antisymmetry(const gdo_model* m, double* out4) {
  int N = m->N, M = m->M, Mh = m->Mh;
  const tend_t* t = &m->tend_mem[2];
  const state_t* s = &m->state_mem[m->old + 1];
  double ual = 0, uat = 0, fv = 0, up = 0, val = 0, vat = 0, fu = 0, vp = 0, ml = 0, mt = 0;
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i) {
      double w = AT(m, s->iu, i, j) * m->full_cos[j];
      ual = ual + AT(m, t->a[T_U_ADV_LON], i, j) * w;
      uat = uat + AT(m, t->a[T_U_ADV_LAT], i, j) * w;
      fv = fv + AT(m, t->a[T_FV], i, j) * w;
      up = up + AT(m, t->a[T_U_PGF], i, j) * w;
    }
  for (int j = 1; j <= Mh; ++j)
    for (int i = 1; i <= N; ++i) {
      double w = AT(m, s->iv, i, j) * m->half_cos[j];
      val = val + AT(m, t->a[T_V_ADV_LON], i, j) * w;
      vat = vat + AT(m, t->a[T_V_ADV_LAT], i, j) * w;
      fu = fu + AT(m, t->a[T_FU], i, j) * w;
      vp = vp + AT(m, t->a[T_V_PGF], i, j) * w;
    }
  for (int j = 1; j <= M; ++j)
    for (int i = 1; i <= N; ++i) {
      double w = (AT(m, s->gd, i, j) + AT(m, m->ghs, i, j)) * m->full_cos[j];
      ml = ml + AT(m, t->a[T_MDLON], i, j) * w;
      mt = mt + AT(m, t->a[T_MDLAT], i, j) * w;
    }
  out4[0] = ual + val + uat + vat;
  out4[1] = up + ml;
  out4[2] = fv - fu;
  out4[3] = vp + mt;
}
