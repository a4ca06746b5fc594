/*
 * gdc_oracle.h -- CPU restatement of the gamil-dycore barotropic time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: a plain-C, FP64,
 * single-threaded restatement of the reference's hot path, used by tests/,
 * by __graft_entry__.smoke() and by bench.py's cpu_baseline / reference arm
 * to check the CUDA path.  The product library never links, loads or calls it.
 *
 * Parity status: unpinned by reference outputs.  The reference (Fortran 2003)
 * cannot be compiled in this environment (no Fortran compiler, empty
 * datetime/container submodules, no NetCDF) and ships no golden vectors, so
 * this restatement is pinned only by known-answer checks (FFT packing vs
 * numpy, antisymmetry identities, mass conservation) in tests/.
 *
 * Arrays use the reference's padded layout: a field with lon range
 * -1..N+2 and lat range -1..R+2 (R = num_lat for full rows, num_lat-1 for
 * half rows) is a contiguous C array of (R+4) rows of (N+4) doubles, lon
 * fastest; Fortran element (i,j) lives at [(j+1)*(N+4) + (i+1)].
 */
#ifndef GDC_ORACLE_H
#define GDC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gdo_model gdo_model;

/* split_scheme: 0 = none (also csp1, which the reference routes to the
 * no-split path), 2 = csp2, 3 = isp.  uv_adv_scheme: 0 = center_diff,
 * 1 = upwind, 2 = weno (weno_order 2).  cutoff: 20 entries of zonal_tend_filter_cutoff_wavenumber. */
gdo_model* gdo_create(int num_lon, int num_lat, double time_step_size,
                      int subcycles, int split_scheme, int qcon_modified,
                      int uv_adv_scheme, double upwind_lon_beta,
                      double upwind_lat_beta, int use_zonal_tend_filter,
                      const int* cutoff, int use_diffusion,
                      double diffusion_coef, int diffusion_order);
void gdo_destroy(gdo_model* m);
/* Extension guard of the filter rescale (0 = reference behaviour); the
 * CUDA path's gdc_params::filter_rescale_rtol. */
void gdo_set_rescale_rtol(gdo_model* m, double rtol);
/* Filter arithmetic: on = 0 projects onto the kept modes (default, the
 * CUDA path's), on = 1 runs FFTPACK 5.1's forward and backward transforms
 * as the reference does (src/filter_mod.F90:105-167).  Returns -1 when
 * num_lon has a prime factor above 5. */
int gdo_set_fft(gdo_model* m, int on);
/* FFTPACK's rfft1f (backward = 0) or rfft1b (backward = 1) of x[0..n-1] in
 * place (exposed for its self-test); -1 for an unsupported length. */
int gdo_rfft_row(int n, int backward, double* x);
/* Diagnostic: the worst conditioning sum|t w| / |s| of the filter's s1
 * (index 0) and s2 (index 1) since the last call, with the field (0 du,
 * 1 dv, 2 dgd) and Fortran row where it occurred; resets the record. */
void gdo_rescale_record(gdo_model* m, double* cond, int* field, int* row);
/* The benchmark's seeded state and its noise (gdc_oracle_ic.c): the
 * library's gdc_ic_seeded / gdc_ic_add_noise evaluated the same way, in
 * the padded layout with ld = num_lon + 4, without the library. */
int gdo_ic_seeded(int N, int M, unsigned long long seed, int lmax, double gd0, double gd_rms, double psi_rms,
                  double u0, int n_mountains, double mountain_height, double mountain_radius_deg, double* u,
                  double* v, double* gd, double* ghs);
int gdo_ic_add_noise(int N, int M, unsigned long long seed, double sigma, double* gd);
/* The oracle's correctly rounded sum (exposed for its self-test). */
double gdo_fsum(const double* x, int n);

/* Initial-condition hook: copies u, v, gd, ghs (padded layout) into
 * state(1) and static, as the reference's test-case modules do. */
void gdo_set_state(gdo_model* m, const double* u, const double* v,
                   const double* gd, const double* ghs);
/* dycore_run prologue: reset_cos_lat_at_poles, iap_transform, diag_run. */
void gdo_run_init(gdo_model* m);
/* nsteps iterations of the dycore_run loop body. Returns 0, or 1 when the
 * total mass or energy became NaN (the reference stops there). */
int gdo_step(gdo_model* m, int nsteps);

/* Copy state(old): u, v, gd, iap u, iap v, iap gd (any pointer may be NULL). */
void gdo_get_state(const gdo_model* m, double* u, double* v, double* gd,
                   double* iap_u, double* iap_v, double* iap_gd);
void gdo_diag(const gdo_model* m, double* total_mass, double* total_energy,
              double* last_beta);

/* Operator-level access used by the unit parity tests:
 * space_operators(state(old), tend(0), pass) and its du/dv/dgd. */
void gdo_tendency(gdo_model* m, int pass, double* du, double* dv, double* dgd);
/* History fields of state(old): A-grid u, v, gh = gd + ghs, div, vor
 * (padded layout; vor has num_lat - 1 rows). */
void gdo_history(const gdo_model* m, double* ua, double* va, double* gh, double* div, double* vor);
/* The four antisymmetry sums of check_antisymmetry for tend(0). */
void gdo_antisymmetry(const gdo_model* m, double* out4);
/* Filter one padded row x in place with the factors of a full (half=0) or
 * half (half=1) latitude row lat_idx (Fortran index). */
void gdo_filter_row(const gdo_model* m, int half, int lat_idx, double* x);
/* Flags: out_full[num_lat], out_half[num_lat-1] (0/1), and the cutoff in
 * effect for each row (-1 when the factor row is all zero). */
void gdo_filter_flags(const gdo_model* m, int* out_full, int* out_half,
                      int* cut_full, int* cut_half);

#ifdef __cplusplus
}
#endif
#endif
