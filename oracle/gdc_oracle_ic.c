/*
 * gdc_oracle_ic.c -- the seeded initial state of the benchmark
 * configurations, restated for the oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * The benchmark's states (a gd0 + spherical-harmonic gd rescaled to an RMS,
 * a nondivergent wind from a streamfunction of the same family differenced
 * at C-grid corners, optional seeded Gaussian mountains and a balanced
 * zonal flow, and per-member N(0, sigma) noise on gd) are defined by the
 * library's gdc_ic_seeded / gdc_ic_add_noise; they have no counterpart in
 * the reference's test cases.  This file evaluates the same definition with
 * the same operations in the same order, so that the reference arm of the
 * benchmark and the tests can build those states without loading the
 * product library (a test checks the two agree bit for bit).
 *
 * Arrays use the reference's padded layout (halo 2, lon fastest, ld N+4).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gdc_oracle.h"

#define PI_ (atan(1.0) * 4.0)
#define GRAV 9.80616
#define RAD 6.37122e6

typedef struct {
  uint64_t s;
  int have;
  double spare;
} rng_t;

/* splitmix64 */
static uint64_t rng_next(rng_t* r) {
  uint64_t z = (r->s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double rng_uniform(rng_t* r) { return ((double)(rng_next(r) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
/* Box-Muller, the cosine normal first and the sine one kept for the next call. */
static double rng_normal(rng_t* r) {
  if (r->have) {
    r->have = 0;
    return r->spare;
  }
  const double u1 = rng_uniform(r), u2 = rng_uniform(r);
  const double rad = sqrt(-2.0 * log(u1));
  r->spare = rad * sin(2 * PI_ * u2);
  r->have = 1;
  return rad * cos(2 * PI_ * u2);
}

/* Coefficients a_lm, b_lm (index l (L+1) + m) drawn for l = 1..L, m = 0..l. */
static void draw_harmonics(rng_t* r, int L, double* a, double* b) {
  for (int l = 1; l <= L; ++l)
    for (int m = 0; m <= l; ++m) {
      a[l * (L + 1) + m] = rng_normal(r);
      if (m > 0) b[l * (L + 1) + m] = rng_normal(r);
    }
}

/* sum_{l=1..L} sum_{m=0..l} w_m Pbar_l^m(sin lat) (a cos m lon + b sin m lon),
 * orthonormal associated Legendre functions by the three-term recurrence. */
static double eval_harmonics(int L, const double* a, const double* b, double* P, double lat, double lon) {
  const double x = sin(lat), sx = cos(lat);
  memset(P, 0, sizeof(double) * (size_t)(L + 1) * (L + 1));
  P[0] = sqrt(1.0 / (4 * PI_));
  for (int m = 1; m <= L; ++m) P[m * (L + 1) + m] = sqrt((2.0 * m + 1) / (2.0 * m)) * sx * P[(m - 1) * (L + 1) + m - 1];
  for (int m = 0; m < L; ++m) P[(m + 1) * (L + 1) + m] = sqrt(2.0 * m + 3) * x * P[m * (L + 1) + m];
  for (int m = 0; m <= L; ++m)
    for (int l = m + 2; l <= L; ++l) {
      const double al = sqrt((4.0 * l * l - 1) / ((double)l * l - (double)m * m));
      const double bl = sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1));
      P[l * (L + 1) + m] = al * (x * P[(l - 1) * (L + 1) + m] - bl * P[(l - 2) * (L + 1) + m]);
    }
  double s = 0;
  for (int l = 1; l <= L; ++l)
    for (int m = 0; m <= l; ++m) {
      const double w = (m == 0 ? 1.0 : sqrt(2.0)) * P[l * (L + 1) + m];
      s += w * (a[l * (L + 1) + m] * cos(m * lon) + b[l * (L + 1) + m] * sin(m * lon));
    }
  return s;
}

#define AT0(f, ld, i0, j0) (f)[(size_t)((j0) + 2) * (ld) + ((i0) + 2)]

static void lon_halo(double* f, int ld, int N, int rows) {
  for (int j = 0; j < rows + 4; ++j) {
    double* row = f + (size_t)j * ld;
    row[0] = row[N];
    row[1] = row[N + 1];
    row[N + 2] = row[2];
    row[N + 3] = row[3];
  }
}

int gdo_ic_seeded(int N, int M, unsigned long long seed, int lmax, double gd0, double gd_rms, double psi_rms,
                  double u0, int n_mountains, double mountain_height, double mountain_radius_deg, double* u,
                  double* v, double* gd, double* ghs) {
  if (N < 4 || M < 5 || lmax < 0 || lmax > 64 || n_mountains < 0) return -1;
  const int Mh = M - 1, ld = N + 4;
  const double dlon = 2 * PI_ / N, dlat = PI_ / Mh;
  double* full_lat = calloc(M, sizeof(double));
  double* half_lat = calloc(Mh, sizeof(double));
  double* full_lon = calloc(N, sizeof(double));
  double* half_lon = calloc(N, sizeof(double));
  double* full_cos = calloc(M, sizeof(double));
  double* full_sin = calloc(M, sizeof(double));
  double* half_cos = calloc(Mh, sizeof(double));
  for (int j = 0; j < Mh; ++j) {
    full_lat[j] = -0.5 * PI_ + j * dlat;
    half_lat[j] = full_lat[j] + 0.5 * dlat;
  }
  full_lat[M - 1] = 0.5 * PI_;
  for (int i = 0; i < N; ++i) {
    full_lon[i] = i * dlon;
    half_lon[i] = full_lon[i] + 0.5 * dlon;
  }
  for (int j = 0; j < Mh; ++j) half_cos[j] = cos(half_lat[j]);
  for (int j = 0; j < M; ++j) {
    full_cos[j] = cos(full_lat[j]);
    full_sin[j] = sin(full_lat[j]);
  }
  full_cos[0] = full_cos[M - 1] = 0.0;
  full_sin[0] = -1.0;
  full_sin[M - 1] = 1.0;
  memset(u, 0, sizeof(double) * (size_t)ld * (M + 4));
  memset(v, 0, sizeof(double) * (size_t)ld * (Mh + 4));
  memset(gd, 0, sizeof(double) * (size_t)ld * (M + 4));
  memset(ghs, 0, sizeof(double) * (size_t)ld * (M + 4));

  rng_t r = {seed, 0, 0.0};
  /* draw order: mountain centres, then the gd and streamfunction sets */
  double* clat = calloc(n_mountains + 1, sizeof(double));
  double* clon = calloc(n_mountains + 1, sizeof(double));
  for (int k = 0; k < n_mountains; ++k) {
    clon[k] = 2 * PI_ * rng_uniform(&r);
    clat[k] = asin(2 * rng_uniform(&r) - 1);
  }
  const size_t nc = (size_t)(lmax + 1) * (lmax + 1);
  double* ag = calloc(nc, sizeof(double));
  double* bg = calloc(nc, sizeof(double));
  double* ap = calloc(nc, sizeof(double));
  double* bp = calloc(nc, sizeof(double));
  double* P = calloc(nc, sizeof(double));
  draw_harmonics(&r, lmax, ag, bg);
  draw_harmonics(&r, lmax, ap, bp);

  double* f = calloc((size_t)M * N, sizeof(double));
  double ss = 0;
  if (lmax > 0 && gd_rms > 0)
    for (int j = 0; j < M; ++j)
      for (int i = 0; i < N; ++i) {
        f[(size_t)j * N + i] = eval_harmonics(lmax, ag, bg, P, full_lat[j], full_lon[i]);
        ss += f[(size_t)j * N + i] * f[(size_t)j * N + i];
      }
  const double gscale = ss > 0 ? gd_rms / sqrt(ss / ((double)M * N)) : 0.0;
  const double rr = mountain_radius_deg * PI_ / 180.0;
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < N; ++i) {
      double h = 0;
      for (int k = 0; k < n_mountains; ++k) {
        const double dphi = full_lat[j] - clat[k], dlam = full_lon[i] - clon[k];
        const double s1 = sin(0.5 * dphi), s2 = sin(0.5 * dlam);
        const double hv = s1 * s1 + cos(full_lat[j]) * cos(clat[k]) * s2 * s2;
        const double d = 2 * asin(sqrt(fmin(1.0, hv)));
        h += mountain_height * GRAV * exp(-(d / rr) * (d / rr));
      }
      AT0(ghs, ld, i, j) = h;
      const double t = full_sin[j];
      const double omega = 2.0 * PI_ / 86400.0;
      AT0(gd, ld, i, j) = gd0 + gscale * f[(size_t)j * N + i] - (RAD * omega * u0 + u0 * u0 * 0.5) * (t * t) - h;
    }
  double* psi = calloc((size_t)Mh * N, sizeof(double));
  ss = 0;
  if (lmax > 0 && psi_rms > 0)
    for (int j = 0; j < Mh; ++j)
      for (int i = 0; i < N; ++i) {
        psi[(size_t)j * N + i] = eval_harmonics(lmax, ap, bp, P, half_lat[j], half_lon[i]);
        ss += psi[(size_t)j * N + i] * psi[(size_t)j * N + i];
      }
  const double pscale = ss > 0 ? psi_rms / sqrt(ss / ((double)Mh * N)) : 0.0;
  for (size_t q = 0; q < (size_t)Mh * N; ++q) psi[q] *= pscale;
  for (int j = 1; j < M - 1; ++j)
    for (int i = 0; i < N; ++i)
      AT0(u, ld, i, j) = -(psi[(size_t)j * N + i] - psi[(size_t)(j - 1) * N + i]) / (RAD * dlat) + u0 * full_cos[j];
  for (int j = 0; j < Mh; ++j)
    for (int i = 0; i < N; ++i) {
      const int im = (i + N - 1) % N;
      AT0(v, ld, i, j) = (psi[(size_t)j * N + i] - psi[(size_t)j * N + im]) / (RAD * half_cos[j] * dlon);
    }
  lon_halo(u, ld, N, M);
  lon_halo(v, ld, N, Mh);
  lon_halo(gd, ld, N, M);
  lon_halo(ghs, ld, N, M);
  free(full_lat); free(half_lat); free(full_lon); free(half_lon);
  free(full_cos); free(full_sin); free(half_cos);
  free(clat); free(clon); free(ag); free(bg); free(ap); free(bp); free(P); free(f); free(psi);
  return 0;
}

int gdo_ic_add_noise(int N, int M, unsigned long long seed, double sigma, double* gd) {
  if (N < 4 || M < 5) return -1;
  const int ld = N + 4;
  rng_t r = {seed, 0, 0.0};
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < N; ++i) AT0(gd, ld, i, j) += sigma * rng_normal(&r);
  lon_halo(gd, ld, N, M);
  return 0;
}
