/*
 * gdc.h -- C ABI of the GB300-native gamil-dycore barotropic time step.
 *
 * Plain C types only (ints, doubles, pointers, sizes): the reference's
 * Fortran host binds it through ISO_C_BINDING, Python through ctypes.
 * Every call returns GDC_OK (0) or a GDC_E_* code and never exits the
 * process; the message of the last failure is available from
 * gdc_last_error / gdc_batch_last_error.
 *
 * Host field layout ("padded layout"): the reference's own allocation,
 * src/parallel_mod.F90:302-310 -- a field with R latitude rows (R = num_lat
 * for u and gd, num_lat-1 for v) is (R+4) rows of `ld` doubles (ld >= N+4,
 * N = num_lon), longitude fastest, Fortran element (i,j) (i = -1..N+2,
 * j = -1..R+2) at index (j+1)*ld + (i+1).  Inputs are read from the
 * interior; outputs fill the interior, the periodic longitude halo, and
 * zero latitude-halo rows, exactly as the reference keeps them.
 */
#ifndef GDC_H
#define GDC_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define GDC_OK 0
#define GDC_E_CONFIG 1  /* invalid parameter / unsupported option          */
#define GDC_E_CUDA 2    /* CUDA runtime error                               */
#define GDC_E_OOM 3     /* device memory exhausted / admission refused      */
#define GDC_E_NAN 4     /* total mass or energy became NaN (diag_mod check) */
#define GDC_E_TIMEOUT 5 /* a bounded device wait gave up                    */
#define GDC_E_STATE 6   /* call out of order (e.g. step before set_state)   */

/* ---- option values (src/params_mod.F90:42-66, src/dycore_mod.F90:27-41) */
#define GDC_SPLIT_NONE 0
#define GDC_SPLIT_CSP1 1 /* routed to the no-split path, as the reference does */
#define GDC_SPLIT_CSP2 2
#define GDC_SPLIT_ISP 3
#define GDC_ADV_CENTER_DIFF 0
#define GDC_ADV_UPWIND 1
#define GDC_ADV_WENO 2 /* weno_order 2, src/weno_mod.F90 (8x32 tiles) */
#define GDC_FP64 0     /* plain path: everything in FP64                   */
#define GDC_FP32 1     /* FP32 state/tendencies, compensated time levels,
                          FP64 pole-cap sums and mass/energy integrals      */

/* Mirror of namelist /dycore_params/ (src/params_mod.F90:68-98) plus the
 * arithmetic precision and CUDA device.  Defaults as the reference. */
typedef struct gdc_params {
  int num_lon;
  int num_lat;
  double time_step_size;
  int subcycles;
  int split_scheme;
  int qcon_modified;
  int uv_adv_scheme;
  double uv_adv_upwind_lon_beta;
  double uv_adv_upwind_lat_beta;
  int use_zonal_tend_filter;
  int zonal_tend_filter_cutoff_wavenumber[20];
  int use_diffusion;
  double diffusion_coef;
  int diffusion_order;
  int run_days;
  int run_hours;
  int run_minutes;
  int run_seconds;
  int precision;
  int device; /* CUDA device; gdc_params_default takes the calling thread's current one */
  /* Extension, not in the reference (0 = the reference's behaviour): the
   * s1/s2 rescale of a filtered tendency row (src/dycore_mod.F90:212-219)
   * is skipped -- the row is filtered but not rescaled -- when
   * |s1| <= rtol * sum|t*w| or |s2| <= rtol * sum|t'*w|, i.e. when s1 or s2
   * is zero to within its own rounding and the ratio s1/s2 is noise.  The
   * reference rescales by that noise (e.g. zonal flows, whose gd+ghs is
   * constant along each row, give s1 ~ 1e-17 sum|t*w|). */
  double filter_rescale_rtol;
} gdc_params;

/* Reference defaults (src/params_mod.F90:13-66). */
void gdc_params_default(gdc_params* p);

/* params_read (src/params_mod.F90:102-115): parse namelist group
 * &dycore_params from `path`.  Unknown keys are an error (gfortran's
 * behaviour).  test_case/case_name are returned as strings (may be NULL). */
int gdc_params_read_namelist(const char* path, gdc_params* p, char* test_case,
                             int test_case_len, char* case_name,
                             int case_name_len, char* errbuf, int errbuf_len);

/* Number of dycore_run loop iterations for the configured run length:
 * time_is_finished (src/time_mod.F90:138-142) with end_time from
 * run_days/hours/minutes (src/time_mod.F90:59-64), i.e.
 * ceil(run_length / time_step_size). */
int gdc_steps_for_run(const gdc_params* p);

/* ---- single model (the dycore_mod public API) ------------------------ */
typedef struct gdc_handle gdc_handle;

/* dycore_init (src/dycore_mod.F90:60-111): mesh, coefficients, filter
 * masks, device buffers.  Reads no state.  num_lon must be a multiple of 4
 * (every grid of the reference's test suite is). */
int gdc_create(const gdc_params* p, gdc_handle** out);
/* dycore_final (src/dycore_mod.F90:144-157). */
void gdc_destroy(gdc_handle* h);
const char* gdc_last_error(const gdc_handle* h);

/* Initial-condition hook + dycore_run prologue: the test-case modules write
 * state(1)%u/v/gd and static%ghs (src/dycore_test.F90:26-43); then
 * reset_cos_lat_at_poles, iap_transform, diag_run
 * (src/dycore_mod.F90:121-129).  Pole-row u must be zero (every reference
 * initial condition has it so); otherwise GDC_E_CONFIG. */
int gdc_set_state(gdc_handle* h, const double* u, const double* v,
                  const double* gd, const double* ghs, int ld);

/* `nsteps` iterations of the dycore_run loop body (src/dycore_mod.F90:
 * 131-140): time_integrate, time_advance, diag_run.  Enqueued on the
 * handle's stream; returns without waiting. */
int gdc_step(gdc_handle* h, int nsteps);
/* Wait for enqueued work; GDC_E_NAN if a step produced NaN mass/energy
 * (the reference's log_error at src/diag_mod.F90:79-87). */
int gdc_sync(gdc_handle* h);
/* dycore_run's loop: gdc_step + gdc_sync. */
int gdc_run(gdc_handle* h, int nsteps);

/* state(old) in the padded layout (any pointer may be NULL). */
int gdc_get_state(gdc_handle* h, double* u, double* v, double* gd, int ld);
/* IAP fields of state(old): iap%u, iap%v, iap%gd (any may be NULL). */
int gdc_get_iap(gdc_handle* h, double* iap_u, double* iap_v, double* iap_gd,
                int ld);
/* diag%total_mass, diag%total_energy of state(old) and the last beta
 * logged by log_add_diag('beta') (src/dycore_mod.F90:787, :747). */
int gdc_diag(gdc_handle* h, double* total_mass, double* total_energy,
             double* beta);
/* Steps completed since set_state (or since the checkpointed run began). */
int gdc_steps_done(gdc_handle* h, long long* steps);
/* restart_write / restart_read + dycore_restart (src/restart_mod.F90:41-75,
 * src/dycore_mod.F90:113-117): the checkpoint format of
 * gdc_batch_checkpoint; reading replaces the current state and continues
 * the checkpointed run exactly. */
int gdc_write_restart(gdc_handle* h, const char* path);
int gdc_read_restart(gdc_handle* h, const char* path);
/* History output of state(old), computed on the device in FP64
 * (history_write_state, src/history_mod.F90:93-124, with diag_run's div and
 * vor, src/diag_mod.F90:49-68): u, v averaged to the A grid, gh = gd + ghs,
 * divergence (pole rows 0) and relative vorticity.  Padded layout, any
 * pointer may be NULL: u_a, v_a, gh, div num_lat rows, vor num_lat - 1. */
int gdc_history(gdc_handle* h, double* u_a, double* v_a, double* gh, double* div, double* vor, int ld);

/* space_operators(state(old), tend, pass) (src/dycore_mod.F90:184-365)
 * including the filter rescale; du/dv/dgd returned in the padded layout.
 * pass: 0 all, 1 fast, 2 slow. */
int gdc_debug_tendency(gdc_handle* h, int pass, double* du, double* dv,
                       double* dgd, int ld);

/* Run all device work of this handle on `cuda_stream` (a cudaStream_t;
 * NULL restores the handle's own stream). */
int gdc_set_stream(gdc_handle* h, void* cuda_stream);

/* No counterpart in the reference: space_operators (as gdc_debug_tendency)
 * for callers that cannot allocate device memory -- hosts whose allocator
 * owns every device allocation (a framework's caching pool, a memory
 * budget enforced per process), and plug-ins that must not grow the
 * device footprint once running.  FP64 only.  All pointers are the
 * CALLER's device buffers in the interior layout (rows x num_lon,
 * longitude fastest, no halo): gd, iap_u, ghs, du, dgd num_lat rows;
 * iap_v, dv num_lat-1 rows; given_u/given_v (both or neither) are u, v to
 * use as given (e.g. an initial condition's own u, v), NULL to derive them
 * from the iap fields.  The library keeps its descriptor, work list and
 * tables in one 2 MiB static device array (held by every GPU that loads the
 * library until exit), so grids are limited to 1440 x 721; larger grids
 * return GDC_E_CONFIG.  It calls no cudaMalloc / cudaFree.  The first call
 * on a device resolves the array's device address (set-up); make that
 * first call before any stream capture.  Each call uploads its tables from
 * host memory with cudaMemcpyAsync on `cuda_stream`.  All calls share the
 * array and each rewrites it: calls that overlap on the GPU race
 * (serialise them on one stream).  Enqueued on `cuda_stream`; returns
 * before the kernel finishes.  The message of the calling thread's last
 * failure is gdc_noalloc_last_error(). */
int gdc_tendency_noalloc(const gdc_params* p, int pass, const double* gd,
                         const double* iap_u, const double* iap_v,
                         const double* ghs, const double* given_u,
                         const double* given_v, double* du, double* dv,
                         double* dgd, void* cuda_stream);
const char* gdc_noalloc_last_error(void);

/* ---- initial conditions (host only, no GPU) ------------------------- */
/* src/test_cases/barotropic/rossby_haurwitz_wave_test_mod.F90:33-85
 * (R = 4, omg = 7.848e-6, gd0 = 8000 g). */
int gdc_ic_rossby_haurwitz(int num_lon, int num_lat, double* u, double* v,
                           double* gd, double* ghs, int ld);
/* src/test_cases/barotropic/steady_geostrophic_flow_test_mod.F90:20-62 */
int gdc_ic_steady_geostrophic(int num_lon, int num_lat, double* u, double* v,
                              double* gd, double* ghs, int ld);
/* src/test_cases/barotropic/mountain_zonal_flow_test_mod.F90:28-97
 * (smooth_mountain = .false.) */
int gdc_ic_mountain_zonal_flow(int num_lon, int num_lat, double* u,
                               double* v, double* gd, double* ghs, int ld);
/* Seeded state with no counterpart in the reference's test cases:
 * gd = gd0 + sum of real spherical harmonics of degree 1..lmax with N(0,1)
 * coefficients rescaled to gd_rms; a nondivergent u,v from a streamfunction
 * of the same family (independent draw) rescaled to psi_rms, differenced at
 * C-grid corners so the discrete divergence vanishes; when n_mountains > 0,
 * Gaussian mountains (height, e-folding radius in degrees, centres uniform
 * on the sphere) are added to ghs and subtracted from gd; u0 > 0 adds a
 * geostrophically balanced zonal flow u = u0 cos(lat). */
int gdc_ic_seeded(int num_lon, int num_lat, unsigned long long seed, int lmax,
                  double gd0, double gd_rms, double psi_rms, double u0,
                  int n_mountains, double mountain_height,
                  double mountain_radius_deg, double* u, double* v,
                  double* gd, double* ghs, int ld);
/* src/test_cases/barotropic/shallow_water_waves_test_mod.F90:97-135: the
 * linear Rossby wave (n = 5, k = 10, gH = 5e4) of Shamir and Paldor, gd =
 * g h + 5e4, ghs = 0.  As the reference, v's half row j takes the amplitude
 * of full row j; pole-row u (below 1e-100 there) is zero. */
int gdc_ic_shallow_water_waves(int num_lon, int num_lat, double* u, double* v,
                               double* gd, double* ghs, int ld);
/* getPhaseSpeed (same module, :139-183) in rad/s: wave_flag 0 Rossby, 1
 * eastward and -1 westward inertia-gravity wave. */
double gdc_sw_waves_phase_speed(int wave_flag);
/* Adds N(0, sigma) white noise to the interior of gd (per-member seed). */
int gdc_ic_add_noise(int num_lon, int num_lat, unsigned long long seed,
                     double sigma, double* gd, int ld);

/* ---- batched ensemble / serving engine ------------------------------ */
/* Many members of mixed grids, each with its own dt and length, advanced
 * together: every model step is one replay of a CUDA graph whose launches
 * cover the work items of all active members.  Scheme options (split,
 * subcycles, advection, filter cutoffs, diffusion, precision) are shared by
 * the batch; grid, dt and length are per member. */
typedef struct gdc_batch gdc_batch;

int gdc_batch_create(const gdc_params* scheme, gdc_batch** out);
void gdc_batch_destroy(gdc_batch* b);
const char* gdc_batch_last_error(const gdc_batch* b);
int gdc_batch_set_stream(gdc_batch* b, void* cuda_stream);

/* Device bytes one member of this grid needs in this batch's precision. */
size_t gdc_member_bytes(const gdc_params* scheme, int num_lon, int num_lat);
/* cudaMemGetInfo of the batch's device. */
int gdc_device_mem_info(int device, size_t* free_bytes, size_t* total_bytes);

/* Admit a member: allocate its device state, upload its initial condition
 * (padded layout) and run the dycore_run prologue for it.  It joins the
 * batched step at the next step boundary.  `cutoff` is the member's
 * zonal_tend_filter_cutoff_wavenumber (20 entries; NULL = the batch
 * scheme's): members of different resolutions filter different numbers of
 * polar rows; each entry 0 <= c <= num_lon/2 - 1 (the reference's factor
 * rows hold 2 (c+1) <= num_lon entries, src/filter_mod.F90:79-96), else
 * GDC_E_CONFIG.  GDC_E_OOM when free device memory minus `reserve_bytes`
 * cannot hold it.  Member state comes from the device's default
 * stream-ordered memory pool (cudaMallocAsync in the batch's stream); the
 * library raises that pool's release threshold so that retired members'
 * memory stays reserved for the next admission, and counts the pool's
 * unused reserve as free (as gdc_device_mem_info does). */
int gdc_batch_add(gdc_batch* b, int num_lon, int num_lat,
                  double time_step_size, long long nsteps, const int* cutoff,
                  const double* u, const double* v, const double* gd,
                  const double* ghs, int ld, size_t reserve_bytes,
                  int* member_id);
/* Initial conditions generated on the device, for gdc_batch_add_ic: the
 * same states as the gdc_ic_* functions, without building and uploading host
 * arrays (admission of large grids costs milliseconds of host time
 * otherwise).  Parameters of the seeded state as gdc_ic_seeded; a noise
 * sigma > 0 adds gdc_ic_add_noise's N(0, sigma) white noise (noise_seed). */
enum {
  GDC_IC_ROSSBY_HAURWITZ = 0,
  GDC_IC_STEADY_GEOSTROPHIC = 1,
  GDC_IC_MOUNTAIN_ZONAL_FLOW = 2,
  GDC_IC_SEEDED = 3,
  GDC_IC_SHALLOW_WATER_WAVES = 4
};
typedef struct gdc_ic_spec {
  int kind;
  int lmax;
  unsigned long long seed;
  double gd0, gd_rms, psi_rms, u0;
  int n_mountains;
  int reserved;
  double mountain_height, mountain_radius_deg;
  unsigned long long noise_seed;
  double noise_sigma;
} gdc_ic_spec;
/* Defaults of `kind` (seeded: the degree 1..6 state of gdc_ic_seeded's
 * documentation, seed 0, no mountains, no noise). */
void gdc_ic_spec_default(gdc_ic_spec* spec, int kind);
/* gdc_batch_add with the initial condition of `spec` generated in device
 * memory (FP64, then iap_transform into the member's precision). */
int gdc_batch_add_ic(gdc_batch* b, int num_lon, int num_lat, double time_step_size, long long nsteps,
                     const int* cutoff, const gdc_ic_spec* spec, size_t reserve_bytes, int* member_id);
/* Release a member's device memory (finished or evicted). */
int gdc_batch_remove(gdc_batch* b, int member_id);
/* Advance every active, unfinished member by `nsteps` model steps (members
 * stop at their own length).  Enqueue only. */
int gdc_batch_step(gdc_batch* b, int nsteps);
int gdc_batch_sync(gdc_batch* b);
/* Checkpoint of one member to `path` and its exact continuation: the file
 * holds the reference's restart fields u, v, gd, ghs (FP64; replaces
 * restart_write, src/restart_mod.F90:60-75) and the member's device state
 * (the current time level in the compute type with its FP32 compensation
 * words, ghs, the level's given u, v), so a restored member continues
 * bitwise as if never interrupted.  The batch's precision must match the
 * file's.  gdc_batch_restore admits the checkpoint as a new member
 * (admission by free memory as gdc_batch_add) with its steps done and
 * length. */
int gdc_batch_checkpoint(gdc_batch* b, int member_id, const char* path);
/* gdc_history for one member of a batch. */
int gdc_batch_history(gdc_batch* b, int member_id, double* u_a, double* v_a, double* gh, double* div,
                      double* vor, int ld);
int gdc_batch_restore(gdc_batch* b, const char* path, size_t reserve_bytes, int* member_id);
/* Per-member status: steps done, finished flag, NaN step (-1 if none). */
int gdc_batch_member_info(gdc_batch* b, int member_id, long long* steps_done,
                          int* finished, long long* nan_step);
int gdc_batch_get_state(gdc_batch* b, int member_id, double* u, double* v,
                        double* gd, int ld);
int gdc_batch_diag(gdc_batch* b, int member_id, double* total_mass,
                   double* total_energy, double* beta);
/* Number of active (admitted, unfinished) members. */
int gdc_batch_active(gdc_batch* b, int* n_active);

/* Work layout of the stage kernels: shared-memory tiles of rows x columns
 * (8x32, 8x64, 4x128, 16x64; 4x32 in FP64) or warp strips of rows x 30
 * columns (8x30, 16x30, 32x30, 64x30: one warp marches a 30-column strip
 * down a band of rows); 0,0 picks the default (16x64 tiles; 8x32 for
 * WENO).  gdc_batch_autotune times every supported shape under each
 * schedule of gdc_batch_set_schedule on the current members and keeps the
 * fastest; the members' states and step counts are saved before and
 * restored after, so tuning advances no forecast.  It returns the chosen
 * shape and its time per model step; gdc_batch_get_schedule reports the
 * whole choice. */
int gdc_batch_set_tile(gdc_batch* b, int tile_rows, int tile_cols);
/* Launch schedule of the stage kernels (a choice of how the work is
 * split, which gdc_batch_autotune also tunes):
 *   split_rows -1 picks automatically (one task per field in FP64 and in
 *     batches with few tiles per SM, one task per row otherwise), 0 one
 *     whole-row task per pole or filtered row, 1 one task per field of such
 *     a row;
 *   fuse_final 1 forms each predict_correct's final update
 *     (src/dycore_mod.F90:789-790) in the first stage of the next
 *     predict_correct of the same step instead of a launch of its own
 *     (tiles only; WENO batches and warp strips always launch it), 0
 *     (default) launches it;
 *   pair_rows 1 runs the FP64 stage launches as clusters of two blocks
 *     and splits each whole-row task over a pair (each block computes half
 *     of the row's columns into both blocks, forms half of the filter's
 *     coefficients and updates half of the row), 0 one block per task, -1
 *     (default) automatically: FP64 launches with at most two work items
 *     per SM (FP64 tiles only, not with fuse_final; FP32 batches never
 *     pair).
 * FP64 results are bitwise the same under every schedule; FP32 results
 * agree to rounding (the partial sums of beta group differently).
 * gdc_batch_get_schedule reports the tile shape and the schedule in effect
 * (pair_rows: whether rows are split over pairs now). */
int gdc_batch_set_schedule(gdc_batch* b, int split_rows, int fuse_final, int pair_rows);
int gdc_batch_get_schedule(gdc_batch* b, int* tile_rows, int* tile_cols, int* split_rows, int* fuse_final,
                           int* pair_rows);
int gdc_batch_autotune(gdc_batch* b, int* tile_rows, int* tile_cols,
                       double* best_ms_per_step);

/* Per-kernel-kind device time of `nsteps` steps run launch by launch with
 * CUDA events on the batch's stream (no graph).  Kinds: 0 stage (tendency
 * + update, including fused final updates), 1 final update, 2 diag, 3
 * diffusion, 4 beta.  ms[k] total, launches[k] count (5 entries each).
 * Advances the members like gdc_batch_step. */
int gdc_batch_profile(gdc_batch* b, int nsteps, double* ms, long long* launches);
/* Algorithmic bytes one grid-point-step moves (the roofline numerator
 * convention: prognostic words read+written per stage, summed over a
 * model step) for this batch's scheme and precision. */
double gdc_algorithmic_bytes_per_gpt_step(const gdc_params* scheme);

/* No counterpart in the reference: the device's FP64 fused multiply-add
 * rate in 1e9 FMA/s (an FMA-chain kernel on every SM, timed with CUDA
 * events), the roof of the FP64 path, which is bound by that unit and not
 * by memory. */
int gdc_fp64_fma_rate(int device, double* gfma_per_s);

#ifdef __cplusplus
}
#endif
#endif
