/*
 * gdc_fftpack.h -- FFTPACK 5.1's real single transform (rfft1i, rfft1f,
 * rfft1b) restated for the oracle.  TEST INFRASTRUCTURE ONLY.
 */
#ifndef GDC_FFTPACK_H
#define GDC_FFTPACK_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int n, nf, ok;
  int fac[18];  /* fac[1] = n, fac[2] = nf, fac[3..nf+2] the factors */
  double* wa;   /* wa[1..n]: the twiddle table WA of rffti1 */
} gdo_rfft;

/* rffti1 (lib/fft/rffti1.f:31-90).  0 on success; -2 when n has a prime
 * factor above 5 (the general-radix pass is not restated). */
int gdo_rfft_init(gdo_rfft* p, int n);
void gdo_rfft_free(gdo_rfft* p);
/* rfft1f / rfftf1 (lib/fft/rfftf1.f:31-110): r[0..n-1] in place, work[n]. */
void gdo_rfft_forward(const gdo_rfft* p, double* r, double* work);
/* rfft1b / rfftb1 (lib/fft/rfftb1.f:31-112): r[0..n-1] in place, work[n]. */
void gdo_rfft_backward(const gdo_rfft* p, double* r, double* work);

#ifdef __cplusplus
}
#endif
#endif
