/*
 * gdc_fftpack.c -- the real single-sequence transform of FFTPACK 5.1 as the
 * reference's zonal filter calls it (rfft1i / rfft1f / rfft1b, vendored in
 * the reference as lib/fft/*.f).  TEST INFRASTRUCTURE ONLY: the oracle's
 * transform-order filter, used by tests/ and the CPU baseline; the product
 * library never links it.
 *
 * Restated from the published mixed-radix algorithm (Swarztrauber's
 * FFTPACK) with the same factorisation, twiddle table, pass order and
 * butterfly arithmetic as the reference's copy, so that each output is
 * rounded the way the reference's FP64 build (-fdefault-real-8) rounds it
 * when it evaluates the F77 expressions in source order: every butterfly
 * below names its intermediate sums and forms them in the order the
 * reference's expressions group them (where the reference's radix-5
 * forward pass adds four products left to right instead of pairing them,
 * so does this).  Radices 2, 3, 4 and 5 are covered -- every grid of the
 * reference's test cases and of the benchmark configurations (N = 144,
 * 180, 200, 360, 720, 1440, ...) factors into them; a length with a prime
 * factor above 5 (FFTPACK's general-radix pass) is refused at set-up.
 *
 * Indexing follows FFTPACK's Fortran: arrays are addressed 1-based through
 * the macros below, the work array CH and the data C have length N, and
 * the radix passes see CC/CH as (IDO, L1, IP) / (IDO, IP, L1) blocks
 * (forward) or the transpose (backward).
 */
#include "gdc_fftpack.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- set-up
 * lib/fft/rffti1.f:31-90: factor N by trying 4, 2, 3, 5, 7, 9, ... (a
 * factor 2 is moved to the front), then the twiddles cos/sin(2 pi l j/N)
 * of every pass but the last in factor order. */
int gdo_rfft_init(gdo_rfft* p, int n) {
  memset(p, 0, sizeof(*p));
  p->n = n;
  if (n < 1) return -1;
  p->wa = (double*)calloc((size_t)n + 1, sizeof(double));
  if (!p->wa) return -1;
  static const int ntryh[4] = {4, 2, 3, 5};
  int nl = n, nf = 0, j = 0, ntry = 0;
  while (nl != 1) {
    ++j;
    ntry = j <= 4 ? ntryh[j - 1] : ntry + 2;
    while (nl % ntry == 0) {
      ++nf;
      p->fac[nf + 2] = ntry;
      nl /= ntry;
      if (ntry == 2 && nf != 1) {
        for (int i = 2; i <= nf; ++i) {
          const int ib = nf - i + 2;
          p->fac[ib + 2] = p->fac[ib + 1];
        }
        p->fac[3] = 2;
      }
      if (nl == 1) break;
    }
  }
  p->fac[1] = n;
  p->fac[2] = nf;
  p->nf = nf;
  for (int k = 1; k <= nf; ++k)
    if (p->fac[k + 2] > 5) return -2; /* general radix: not restated */
  const double tpi = 8.0 * atan(1.0);
  const double argh = tpi / (double)n;
  int is = 0, l1 = 1;
  for (int k1 = 1; k1 <= nf - 1; ++k1) {
    const int ip = p->fac[k1 + 2];
    int ld = 0;
    const int l2 = l1 * ip, ido = n / l2;
    for (int jj = 1; jj <= ip - 1; ++jj) {
      ld += l1;
      int i = is;
      const double argld = (double)ld * argh;
      double fi = 0.0;
      for (int ii = 3; ii <= ido; ii += 2) {
        i += 2;
        fi = fi + 1.0;
        const double arg = fi * argld;
        p->wa[i - 1] = cos(arg);
        p->wa[i] = sin(arg);
      }
      is += ido;
    }
    l1 = l2;
  }
  p->ok = 1;
  return 0;
}

void gdo_rfft_free(gdo_rfft* p) {
  free(p->wa);
  p->wa = NULL;
  p->ok = 0;
}

/* Twiddle k (1-based) of the table that starts at WA(iw). */
#define TW(w, k) ((w)[(k)-1])

/* ------------------------------------------------------ forward passes
 * Input CC(i, k, j): IDO x L1 x IP; output CH(i, j, k): IDO x IP x L1. */
#define CCF(i, k, j) cc[((i)-1) + ido * (((k)-1) + l1 * ((j)-1))]
#define CHF(i, j, k) ch[((i)-1) + ido * (((j)-1) + IP * ((k)-1))]

/* lib/fft/r1f2kf.f */
static void fwd2(int ido, int l1, const double* cc, double* ch, const double* w1) {
  enum { IP = 2 };
  for (int k = 1; k <= l1; ++k) {
    CHF(1, 1, k) = CCF(1, k, 1) + CCF(1, k, 2);
    CHF(ido, 2, k) = CCF(1, k, 1) - CCF(1, k, 2);
  }
  if (ido < 2) return;
  if (ido > 2) {
    const int idp2 = ido + 2;
    for (int k = 1; k <= l1; ++k)
      for (int i = 3; i <= ido; i += 2) {
        const int ic = idp2 - i;
        const double ti2 = TW(w1, i - 2) * CCF(i, k, 2) - TW(w1, i - 1) * CCF(i - 1, k, 2);
        const double tr2 = TW(w1, i - 2) * CCF(i - 1, k, 2) + TW(w1, i - 1) * CCF(i, k, 2);
        CHF(i, 1, k) = CCF(i, k, 1) + ti2;
        CHF(ic, 2, k) = ti2 - CCF(i, k, 1);
        CHF(i - 1, 1, k) = CCF(i - 1, k, 1) + tr2;
        CHF(ic - 1, 2, k) = CCF(i - 1, k, 1) - tr2;
      }
    if (ido % 2 == 1) return;
  }
  for (int k = 1; k <= l1; ++k) {
    CHF(1, 2, k) = -CCF(ido, k, 2);
    CHF(ido, 1, k) = CCF(ido, k, 1);
  }
}

/* lib/fft/r1f3kf.f */
static void fwd3(int ido, int l1, const double* cc, double* ch, const double* w1, const double* w2) {
  enum { IP = 3 };
  const double arg = 2.0 * 4.0 * atan(1.0) / 3.0;
  const double taur = cos(arg), taui = sin(arg);
  for (int k = 1; k <= l1; ++k) {
    const double cr2 = CCF(1, k, 2) + CCF(1, k, 3);
    CHF(1, 1, k) = CCF(1, k, 1) + cr2;
    CHF(1, 3, k) = taui * (CCF(1, k, 3) - CCF(1, k, 2));
    CHF(ido, 2, k) = CCF(1, k, 1) + taur * cr2;
  }
  if (ido == 1) return;
  const int idp2 = ido + 2;
  for (int k = 1; k <= l1; ++k)
    for (int i = 3; i <= ido; i += 2) {
      const int ic = idp2 - i;
      const double dr2 = TW(w1, i - 2) * CCF(i - 1, k, 2) + TW(w1, i - 1) * CCF(i, k, 2);
      const double di2 = TW(w1, i - 2) * CCF(i, k, 2) - TW(w1, i - 1) * CCF(i - 1, k, 2);
      const double dr3 = TW(w2, i - 2) * CCF(i - 1, k, 3) + TW(w2, i - 1) * CCF(i, k, 3);
      const double di3 = TW(w2, i - 2) * CCF(i, k, 3) - TW(w2, i - 1) * CCF(i - 1, k, 3);
      const double cr2 = dr2 + dr3, ci2 = di2 + di3;
      CHF(i - 1, 1, k) = CCF(i - 1, k, 1) + cr2;
      CHF(i, 1, k) = CCF(i, k, 1) + ci2;
      const double tr2 = CCF(i - 1, k, 1) + taur * cr2;
      const double ti2 = CCF(i, k, 1) + taur * ci2;
      const double tr3 = taui * (di2 - di3);
      const double ti3 = taui * (dr3 - dr2);
      CHF(i - 1, 3, k) = tr2 + tr3;
      CHF(ic - 1, 2, k) = tr2 - tr3;
      CHF(i, 3, k) = ti2 + ti3;
      CHF(ic, 2, k) = ti3 - ti2;
    }
}

/* lib/fft/r1f4kf.f */
static void fwd4(int ido, int l1, const double* cc, double* ch, const double* w1, const double* w2,
                 const double* w3) {
  enum { IP = 4 };
  const double hsqt2 = sqrt(2.0) / 2.0;
  for (int k = 1; k <= l1; ++k) {
    const double tr1 = CCF(1, k, 2) + CCF(1, k, 4);
    const double tr2 = CCF(1, k, 1) + CCF(1, k, 3);
    CHF(1, 1, k) = tr1 + tr2;
    CHF(ido, 4, k) = tr2 - tr1;
    CHF(ido, 2, k) = CCF(1, k, 1) - CCF(1, k, 3);
    CHF(1, 3, k) = CCF(1, k, 4) - CCF(1, k, 2);
  }
  if (ido < 2) return;
  if (ido > 2) {
    const int idp2 = ido + 2;
    for (int k = 1; k <= l1; ++k)
      for (int i = 3; i <= ido; i += 2) {
        const int ic = idp2 - i;
        const double cr2 = TW(w1, i - 2) * CCF(i - 1, k, 2) + TW(w1, i - 1) * CCF(i, k, 2);
        const double ci2 = TW(w1, i - 2) * CCF(i, k, 2) - TW(w1, i - 1) * CCF(i - 1, k, 2);
        const double cr3 = TW(w2, i - 2) * CCF(i - 1, k, 3) + TW(w2, i - 1) * CCF(i, k, 3);
        const double ci3 = TW(w2, i - 2) * CCF(i, k, 3) - TW(w2, i - 1) * CCF(i - 1, k, 3);
        const double cr4 = TW(w3, i - 2) * CCF(i - 1, k, 4) + TW(w3, i - 1) * CCF(i, k, 4);
        const double ci4 = TW(w3, i - 2) * CCF(i, k, 4) - TW(w3, i - 1) * CCF(i - 1, k, 4);
        const double tr1 = cr2 + cr4, tr4 = cr4 - cr2;
        const double ti1 = ci2 + ci4, ti4 = ci2 - ci4;
        const double ti2 = CCF(i, k, 1) + ci3, ti3 = CCF(i, k, 1) - ci3;
        const double tr2 = CCF(i - 1, k, 1) + cr3, tr3 = CCF(i - 1, k, 1) - cr3;
        CHF(i - 1, 1, k) = tr1 + tr2;
        CHF(ic - 1, 4, k) = tr2 - tr1;
        CHF(i, 1, k) = ti1 + ti2;
        CHF(ic, 4, k) = ti1 - ti2;
        CHF(i - 1, 3, k) = ti4 + tr3;
        CHF(ic - 1, 2, k) = tr3 - ti4;
        CHF(i, 3, k) = tr4 + ti3;
        CHF(ic, 2, k) = tr4 - ti3;
      }
    if (ido % 2 == 1) return;
  }
  for (int k = 1; k <= l1; ++k) {
    const double ti1 = -(hsqt2 * (CCF(ido, k, 2) + CCF(ido, k, 4)));
    const double tr1 = hsqt2 * (CCF(ido, k, 2) - CCF(ido, k, 4));
    CHF(ido, 1, k) = tr1 + CCF(ido, k, 1);
    CHF(ido, 3, k) = CCF(ido, k, 1) - tr1;
    CHF(1, 2, k) = ti1 - CCF(ido, k, 3);
    CHF(1, 4, k) = ti1 + CCF(ido, k, 3);
  }
}

/* lib/fft/r1f5kf.f.  The real parts that feed the tr11/tr12 terms of
 * outputs (i-1, 3) and (ic-1, 2) are the four twiddled products added left
 * to right (x2, x3), not the paired sums dr2 + dr5 the other outputs use. */
static void fwd5(int ido, int l1, const double* cc, double* ch, const double* w1, const double* w2,
                 const double* w3, const double* w4) {
  enum { IP = 5 };
  const double arg = 2.0 * 4.0 * atan(1.0) / 5.0;
  const double tr11 = cos(arg), ti11 = sin(arg);
  const double tr12 = cos(2.0 * arg), ti12 = sin(2.0 * arg);
  for (int k = 1; k <= l1; ++k) {
    const double cr2 = CCF(1, k, 5) + CCF(1, k, 2), ci5 = CCF(1, k, 5) - CCF(1, k, 2);
    const double cr3 = CCF(1, k, 4) + CCF(1, k, 3), ci4 = CCF(1, k, 4) - CCF(1, k, 3);
    CHF(1, 1, k) = CCF(1, k, 1) + cr2 + cr3;
    CHF(ido, 2, k) = CCF(1, k, 1) + tr11 * cr2 + tr12 * cr3;
    CHF(1, 3, k) = ti11 * ci5 + ti12 * ci4;
    CHF(ido, 4, k) = CCF(1, k, 1) + tr12 * cr2 + tr11 * cr3;
    CHF(1, 5, k) = ti12 * ci5 - ti11 * ci4;
  }
  if (ido == 1) return;
  const int idp2 = ido + 2;
  for (int k = 1; k <= l1; ++k)
    for (int i = 3; i <= ido; i += 2) {
      const int ic = idp2 - i;
      const double dr2 = TW(w1, i - 2) * CCF(i - 1, k, 2) + TW(w1, i - 1) * CCF(i, k, 2);
      const double di2 = TW(w1, i - 2) * CCF(i, k, 2) - TW(w1, i - 1) * CCF(i - 1, k, 2);
      const double dr3 = TW(w2, i - 2) * CCF(i - 1, k, 3) + TW(w2, i - 1) * CCF(i, k, 3);
      const double di3 = TW(w2, i - 2) * CCF(i, k, 3) - TW(w2, i - 1) * CCF(i - 1, k, 3);
      const double dr4 = TW(w3, i - 2) * CCF(i - 1, k, 4) + TW(w3, i - 1) * CCF(i, k, 4);
      const double di4 = TW(w3, i - 2) * CCF(i, k, 4) - TW(w3, i - 1) * CCF(i - 1, k, 4);
      const double dr5 = TW(w4, i - 2) * CCF(i - 1, k, 5) + TW(w4, i - 1) * CCF(i, k, 5);
      const double di5 = TW(w4, i - 2) * CCF(i, k, 5) - TW(w4, i - 1) * CCF(i - 1, k, 5);
      const double cr2 = dr2 + dr5, ci5 = di2 - di5;   /* paired sums */
      const double cr3 = dr3 + dr4, ci4 = di3 - di4;
      const double ci2 = di2 + di5, cr5 = dr5 - dr2;
      const double ci3 = di3 + di4, cr4 = dr4 - dr3;
      /* the four products of x2, x3 added one at a time */
      const double x2 = dr2 + TW(w4, i - 2) * CCF(i - 1, k, 5) + TW(w4, i - 1) * CCF(i, k, 5);
      const double x3 = dr3 + TW(w3, i - 2) * CCF(i - 1, k, 4) + TW(w3, i - 1) * CCF(i, k, 4);
      CHF(i - 1, 1, k) = CCF(i - 1, k, 1) + cr2 + cr3;
      CHF(i, 1, k) = CCF(i, k, 1) + ci2 + ci3;
      const double base = CCF(i - 1, k, 1) + tr11 * x2 + tr12 * x3;
      CHF(i - 1, 3, k) = base + ti11 * ci5 + ti12 * ci4;
      CHF(ic - 1, 2, k) = base - (ti11 * ci5 + ti12 * ci4);
      const double ti2 = CCF(i, k, 1) + tr11 * ci2 + tr12 * ci3;
      const double ti5 = ti11 * cr5 + ti12 * cr4;
      CHF(i, 3, k) = ti2 + ti5;
      CHF(ic, 2, k) = ti5 - ti2;
      const double tr3 = CCF(i - 1, k, 1) + tr12 * cr2 + tr11 * cr3;
      const double tr4 = ti12 * ci5 - ti11 * ci4;
      CHF(i - 1, 5, k) = tr3 + tr4;
      CHF(ic - 1, 4, k) = tr3 - tr4;
      const double ti3 = CCF(i, k, 1) + tr12 * ci2 + tr11 * ci3;
      const double ti4 = ti12 * cr5 - ti11 * cr4;
      CHF(i, 5, k) = ti3 + ti4;
      CHF(ic, 4, k) = ti4 - ti3;
    }
}
#undef CCF
#undef CHF

/* ----------------------------------------------------- backward passes
 * Input CC(i, j, k): IDO x IP x L1; output CH(i, k, j): IDO x L1 x IP. */
#define CCB(i, j, k) cc[((i)-1) + ido * (((j)-1) + IP * ((k)-1))]
#define CHB(i, k, j) ch[((i)-1) + ido * (((k)-1) + l1 * ((j)-1))]

/* lib/fft/r1f2kb.f */
static void bwd2(int ido, int l1, const double* cc, double* ch, const double* w1) {
  enum { IP = 2 };
  for (int k = 1; k <= l1; ++k) {
    CHB(1, k, 1) = CCB(1, 1, k) + CCB(ido, 2, k);
    CHB(1, k, 2) = CCB(1, 1, k) - CCB(ido, 2, k);
  }
  if (ido < 2) return;
  if (ido > 2) {
    const int idp2 = ido + 2;
    for (int k = 1; k <= l1; ++k)
      for (int i = 3; i <= ido; i += 2) {
        const int ic = idp2 - i;
        CHB(i - 1, k, 1) = CCB(i - 1, 1, k) + CCB(ic - 1, 2, k);
        CHB(i, k, 1) = CCB(i, 1, k) - CCB(ic, 2, k);
        const double tr2 = CCB(i - 1, 1, k) - CCB(ic - 1, 2, k);
        const double ti2 = CCB(i, 1, k) + CCB(ic, 2, k);
        CHB(i - 1, k, 2) = TW(w1, i - 2) * tr2 - TW(w1, i - 1) * ti2;
        CHB(i, k, 2) = TW(w1, i - 2) * ti2 + TW(w1, i - 1) * tr2;
      }
    if (ido % 2 == 1) return;
  }
  for (int k = 1; k <= l1; ++k) {
    CHB(ido, k, 1) = CCB(ido, 1, k) + CCB(ido, 1, k);
    CHB(ido, k, 2) = -(CCB(1, 2, k) + CCB(1, 2, k));
  }
}

/* lib/fft/r1f3kb.f */
static void bwd3(int ido, int l1, const double* cc, double* ch, const double* w1, const double* w2) {
  enum { IP = 3 };
  const double arg = 2.0 * 4.0 * atan(1.0) / 3.0;
  const double taur = cos(arg), taui = sin(arg);
  for (int k = 1; k <= l1; ++k) {
    CHB(1, k, 1) = CCB(1, 1, k) + 2.0 * CCB(ido, 2, k);
    const double cr2 = CCB(1, 1, k) + (2.0 * taur) * CCB(ido, 2, k);
    CHB(1, k, 2) = cr2 - (2.0 * taui) * CCB(1, 3, k);
    CHB(1, k, 3) = cr2 + (2.0 * taui) * CCB(1, 3, k);
  }
  if (ido == 1) return;
  const int idp2 = ido + 2;
  for (int k = 1; k <= l1; ++k)
    for (int i = 3; i <= ido; i += 2) {
      const int ic = idp2 - i;
      const double tr2 = CCB(i - 1, 3, k) + CCB(ic - 1, 2, k);
      const double ti2 = CCB(i, 3, k) - CCB(ic, 2, k);
      CHB(i - 1, k, 1) = CCB(i - 1, 1, k) + tr2;
      CHB(i, k, 1) = CCB(i, 1, k) + ti2;
      const double cr2 = CCB(i - 1, 1, k) + taur * tr2;
      const double ci2 = CCB(i, 1, k) + taur * ti2;
      const double cr3 = taui * (CCB(i - 1, 3, k) - CCB(ic - 1, 2, k));
      const double ci3 = taui * (CCB(i, 3, k) + CCB(ic, 2, k));
      CHB(i - 1, k, 2) = TW(w1, i - 2) * (cr2 - ci3) - TW(w1, i - 1) * (ci2 + cr3);
      CHB(i, k, 2) = TW(w1, i - 2) * (ci2 + cr3) + TW(w1, i - 1) * (cr2 - ci3);
      CHB(i - 1, k, 3) = TW(w2, i - 2) * (cr2 + ci3) - TW(w2, i - 1) * (ci2 - cr3);
      CHB(i, k, 3) = TW(w2, i - 2) * (ci2 - cr3) + TW(w2, i - 1) * (cr2 + ci3);
    }
}

/* lib/fft/r1f4kb.f */
static void bwd4(int ido, int l1, const double* cc, double* ch, const double* w1, const double* w2,
                 const double* w3) {
  enum { IP = 4 };
  const double sqrt2 = sqrt(2.0);
  for (int k = 1; k <= l1; ++k) {
    const double tr1 = CCB(1, 1, k) - CCB(ido, 4, k);
    const double tr2 = CCB(1, 1, k) + CCB(ido, 4, k);
    const double tr3 = CCB(ido, 2, k) + CCB(ido, 2, k);
    const double tr4 = CCB(1, 3, k) + CCB(1, 3, k);
    CHB(1, k, 3) = tr2 - tr3;
    CHB(1, k, 1) = tr2 + tr3;
    CHB(1, k, 4) = tr1 + tr4;
    CHB(1, k, 2) = tr1 - tr4;
  }
  if (ido < 2) return;
  if (ido > 2) {
    const int idp2 = ido + 2;
    for (int k = 1; k <= l1; ++k)
      for (int i = 3; i <= ido; i += 2) {
        const int ic = idp2 - i;
        const double ti1 = CCB(i, 1, k) + CCB(ic, 4, k);
        const double ti2 = CCB(i, 1, k) - CCB(ic, 4, k);
        const double ti3 = CCB(i, 3, k) - CCB(ic, 2, k);
        const double tr4 = CCB(i, 3, k) + CCB(ic, 2, k);
        const double tr1 = CCB(i - 1, 1, k) - CCB(ic - 1, 4, k);
        const double tr2 = CCB(i - 1, 1, k) + CCB(ic - 1, 4, k);
        const double ti4 = CCB(i - 1, 3, k) - CCB(ic - 1, 2, k);
        const double tr3 = CCB(i - 1, 3, k) + CCB(ic - 1, 2, k);
        CHB(i - 1, k, 1) = tr2 + tr3;
        CHB(i, k, 1) = ti2 + ti3;
        const double cr3 = tr2 - tr3, ci3 = ti2 - ti3;
        const double cr2 = tr1 - tr4, cr4 = tr1 + tr4;
        const double ci2 = ti1 + ti4, ci4 = ti1 - ti4;
        CHB(i - 1, k, 2) = TW(w1, i - 2) * cr2 - TW(w1, i - 1) * ci2;
        CHB(i, k, 2) = TW(w1, i - 2) * ci2 + TW(w1, i - 1) * cr2;
        CHB(i - 1, k, 3) = TW(w2, i - 2) * cr3 - TW(w2, i - 1) * ci3;
        CHB(i, k, 3) = TW(w2, i - 2) * ci3 + TW(w2, i - 1) * cr3;
        CHB(i - 1, k, 4) = TW(w3, i - 2) * cr4 - TW(w3, i - 1) * ci4;
        CHB(i, k, 4) = TW(w3, i - 2) * ci4 + TW(w3, i - 1) * cr4;
      }
    if (ido % 2 == 1) return;
  }
  for (int k = 1; k <= l1; ++k) {
    const double a = CCB(ido, 1, k) + CCB(ido, 3, k);
    const double b = CCB(ido, 1, k) - CCB(ido, 3, k);
    const double c = CCB(1, 2, k) + CCB(1, 4, k);
    const double d = CCB(1, 4, k) - CCB(1, 2, k);
    CHB(ido, k, 1) = a + a;
    CHB(ido, k, 2) = sqrt2 * (b - c);
    CHB(ido, k, 3) = d + d;
    CHB(ido, k, 4) = -(sqrt2 * (b + c));
  }
}

/* lib/fft/r1f5kb.f */
static void bwd5(int ido, int l1, const double* cc, double* ch, const double* w1, const double* w2,
                 const double* w3, const double* w4) {
  enum { IP = 5 };
  const double arg = 2.0 * 4.0 * atan(1.0) / 5.0;
  const double tr11 = cos(arg), ti11 = sin(arg);
  const double tr12 = cos(2.0 * arg), ti12 = sin(2.0 * arg);
  for (int k = 1; k <= l1; ++k) {
    const double a = CCB(1, 1, k), r2 = CCB(ido, 2, k), r4 = CCB(ido, 4, k);
    const double i3 = CCB(1, 3, k), i5 = CCB(1, 5, k);
    CHB(1, k, 1) = a + 2.0 * r2 + 2.0 * r4;
    const double c2 = a + tr11 * 2.0 * r2 + tr12 * 2.0 * r4;
    const double c3 = a + tr12 * 2.0 * r2 + tr11 * 2.0 * r4;
    const double s2 = ti11 * 2.0 * i3 + ti12 * 2.0 * i5;
    const double s3 = ti12 * 2.0 * i3 - ti11 * 2.0 * i5;
    CHB(1, k, 2) = c2 - s2;
    CHB(1, k, 3) = c3 - s3;
    CHB(1, k, 4) = c3 + s3;
    CHB(1, k, 5) = c2 + s2;
  }
  if (ido == 1) return;
  const int idp2 = ido + 2;
  for (int k = 1; k <= l1; ++k)
    for (int i = 3; i <= ido; i += 2) {
      const int ic = idp2 - i;
      const double tr2 = CCB(i - 1, 3, k) + CCB(ic - 1, 2, k);
      const double tr3 = CCB(i - 1, 5, k) + CCB(ic - 1, 4, k);
      const double ti2 = CCB(i, 3, k) - CCB(ic, 2, k);
      const double ti3 = CCB(i, 5, k) - CCB(ic, 4, k);
      const double ti5 = CCB(i, 3, k) + CCB(ic, 2, k);
      const double ti4 = CCB(i, 5, k) + CCB(ic, 4, k);
      const double tr5 = CCB(i - 1, 3, k) - CCB(ic - 1, 2, k);
      const double tr4 = CCB(i - 1, 5, k) - CCB(ic - 1, 4, k);
      CHB(i - 1, k, 1) = CCB(i - 1, 1, k) + tr2 + tr3;
      CHB(i, k, 1) = CCB(i, 1, k) + ti2 + ti3;
      const double cr2 = CCB(i - 1, 1, k) + tr11 * tr2 + tr12 * tr3;
      const double ci2 = CCB(i, 1, k) + tr11 * ti2 + tr12 * ti3;
      const double cr3 = CCB(i - 1, 1, k) + tr12 * tr2 + tr11 * tr3;
      const double ci3 = CCB(i, 1, k) + tr12 * ti2 + tr11 * ti3;
      const double cr5 = ti11 * tr5 + ti12 * tr4;
      const double ci5 = ti11 * ti5 + ti12 * ti4;
      const double cr4 = ti12 * tr5 - ti11 * tr4;
      const double ci4 = ti12 * ti5 - ti11 * ti4;
      CHB(i - 1, k, 2) = TW(w1, i - 2) * (cr2 - ci5) - TW(w1, i - 1) * (ci2 + cr5);
      CHB(i, k, 2) = TW(w1, i - 2) * (ci2 + cr5) + TW(w1, i - 1) * (cr2 - ci5);
      CHB(i - 1, k, 3) = TW(w2, i - 2) * (cr3 - ci4) - TW(w2, i - 1) * (ci3 + cr4);
      CHB(i, k, 3) = TW(w2, i - 2) * (ci3 + cr4) + TW(w2, i - 1) * (cr3 - ci4);
      CHB(i - 1, k, 4) = TW(w3, i - 2) * (cr3 + ci4) - TW(w3, i - 1) * (ci3 - cr4);
      CHB(i, k, 4) = TW(w3, i - 2) * (ci3 - cr4) + TW(w3, i - 1) * (cr3 + ci4);
      CHB(i - 1, k, 5) = TW(w4, i - 2) * (cr2 + ci5) - TW(w4, i - 1) * (ci2 - cr5);
      CHB(i, k, 5) = TW(w4, i - 2) * (ci2 - cr5) + TW(w4, i - 1) * (cr2 + ci5);
    }
}
#undef CCB
#undef CHB

/* ---------------------------------------------------------- drivers
 * lib/fft/rfftf1.f:31-110.  c[0..n-1] is R(1..N), ch the work array.  The
 * passes run over the factors from last to first and alternate between c
 * and ch; the result is scaled into FFTPACK 5.1's packing: r(1) = a0,
 * (r(2k), r(2k+1)) = (a_k, b_k) with the sine term negated by the scaling
 * (-2/N), and r(N) the Nyquist term for even N. */
void gdo_rfft_forward(const gdo_rfft* p, double* c, double* ch) {
  const int n = p->n, nf = p->nf;
  if (n == 1) return;
  const double* wa = p->wa; /* wa[k] = WA(k), 1-based */
  int na = 1, l2 = n, iw = n;
  for (int k1 = 1; k1 <= nf; ++k1) {
    const int kh = nf - k1;
    const int ip = p->fac[kh + 3];
    const int l1 = l2 / ip, ido = n / l2;
    iw = iw - (ip - 1) * ido;
    na = 1 - na;
    const double* in = na == 0 ? c : ch;
    double* out = na == 0 ? ch : c;
    const double* w1 = wa + iw;
    if (ip == 4)
      fwd4(ido, l1, in, out, w1, w1 + ido, w1 + 2 * ido);
    else if (ip == 2)
      fwd2(ido, l1, in, out, w1);
    else if (ip == 3)
      fwd3(ido, l1, in, out, w1, w1 + ido);
    else
      fwd5(ido, l1, in, out, w1, w1 + ido, w1 + 2 * ido, w1 + 3 * ido);
    l2 = l1;
  }
  const double sn = 1.0 / n, tsn = 2.0 / n, tsnm = -tsn;
  const int modn = n % 2, nl = modn ? n - 1 : n - 2;
  const double* src = na == 0 ? ch : c;
  c[0] = sn * src[0];
  for (int j = 2; j <= nl; j += 2) {
    c[j - 1] = tsn * src[j - 1];
    c[j] = tsnm * src[j];
  }
  if (!modn) c[n - 1] = sn * src[n - 1];
}

/* lib/fft/rfftb1.f:31-112: undo the packing's scaling (halve the cosine
 * terms, negate and halve the sine terms), then the passes over the
 * factors from first to last; the pass count's parity decides whether the
 * data start in ch so that they end in c. */
void gdo_rfft_backward(const gdo_rfft* p, double* c, double* ch) {
  const int n = p->n, nf = p->nf;
  if (n == 1) return;
  const double* wa = p->wa;
  int na = 0;
  for (int k1 = 1; k1 <= nf; ++k1) na = 1 - na; /* radices <= 5 only */
  const double half = 0.5, halfm = -0.5;
  const int modn = n % 2, nl = modn ? n - 1 : n - 2;
  if (na != 0) {
    ch[0] = c[0];
    ch[n - 1] = c[n - 1];
    for (int j = 2; j <= nl; j += 2) {
      ch[j - 1] = half * c[j - 1];
      ch[j] = halfm * c[j];
    }
  } else {
    for (int j = 2; j <= nl; j += 2) {
      c[j - 1] = half * c[j - 1];
      c[j] = halfm * c[j];
    }
  }
  int l1 = 1, iw = 1;
  for (int k1 = 1; k1 <= nf; ++k1) {
    const int ip = p->fac[k1 + 2];
    const int l2 = ip * l1, ido = n / l2;
    const double* in = na == 0 ? c : ch;
    double* out = na == 0 ? ch : c;
    const double* w1 = wa + iw;
    if (ip == 4)
      bwd4(ido, l1, in, out, w1, w1 + ido, w1 + 2 * ido);
    else if (ip == 2)
      bwd2(ido, l1, in, out, w1);
    else if (ip == 3)
      bwd3(ido, l1, in, out, w1, w1 + ido);
    else
      bwd5(ido, l1, in, out, w1, w1 + ido, w1 + 2 * ido, w1 + 3 * ido);
    na = 1 - na;
    l1 = l2;
    iw = iw + (ip - 1) * ido;
  }
}
