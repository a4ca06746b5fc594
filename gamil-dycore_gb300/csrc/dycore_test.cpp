// dycore_test -- the reference's driver program (src/dycore_test.F90:1-49)
// over the C ABI of libgdc: params_read -> dycore_init -> the test case's
// initial-condition hook (or dycore_restart) -> dycore_run -> dycore_final.
//
//   dycore_test <namelist_file_path> [--steps N] [--log-every K]
//               [--precision fp64|fp32] [--restart FILE] [--write-restart FILE]
//
// Without --steps the run length is the namelist's (run_days/hours/minutes/
// seconds, as time_is_finished).  Each logged step prints the model time and
// the diagnostics the reference logs (src/dycore_mod.F90:127-139): total
// mass, total energy and beta.  A NaN in mass or energy stops the run with
// the reference's message and exit status 1 (src/diag_mod.F90:79-87).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gdc.h"

namespace {

void log_step(long long step, double dt, double mass, double energy, double beta) {
  const long long secs = (long long)(step * dt + 0.5);
  std::printf(" => day %lld %02lld:%02lld:%02lld total_mass %.17g total_energy %.17g beta %.17g\n",
              secs / 86400, secs % 86400 / 3600, secs % 3600 / 60, secs % 60, mass, energy, beta);
}

int fail(const char* what, const char* msg) {
  std::printf(" [Error]: %s: %s\n", what, msg ? msg : "");
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::printf(" Usage: ./dycore_test.exe <namelist_file_path> [--steps N] [--log-every K] "
                "[--precision fp64|fp32] [--restart FILE] [--write-restart FILE]\n");
    return 1;
  }
  long long steps = -1, every = 1;
  int precision = GDC_FP64;
  const char* restart_in = nullptr;
  const char* restart_out = nullptr;
  for (int k = 2; k < argc; ++k) {
    const std::string a = argv[k];
    const char* v = k + 1 < argc ? argv[k + 1] : nullptr;
    if (a == "--steps" && v) {
      steps = std::atoll(v);
      ++k;
    } else if (a == "--log-every" && v) {
      every = std::atoll(v);
      ++k;
    } else if (a == "--precision" && v) {
      precision = std::strcmp(v, "fp32") == 0 ? GDC_FP32 : GDC_FP64;
      ++k;
    } else if (a == "--restart" && v) {
      restart_in = v;
      ++k;
    } else if (a == "--write-restart" && v) {
      restart_out = v;
      ++k;
    } else {
      std::printf(" [Error]: unknown argument %s\n", a.c_str());
      return 1;
    }
  }
  if (every < 1) every = 1;

  // params_read (src/params_mod.F90:102-115)
  gdc_params p;
  char test_case[256] = {0}, case_name[256] = {0}, err[512] = {0};
  if (gdc_params_read_namelist(argv[1], &p, test_case, sizeof(test_case), case_name, sizeof(case_name), err,
                               sizeof(err)) != GDC_OK)
    return fail("params_read", err);
  p.precision = precision;
  const int N = p.num_lon, M = p.num_lat, ld = N + 4;

  // dycore_init (src/dycore_mod.F90:60-111)
  gdc_handle* h = nullptr;
  if (gdc_create(&p, &h) != GDC_OK) return fail("dycore_init", "gdc_create failed");

  if (restart_in) {
    // dycore_restart (src/dycore_mod.F90:113-117)
    if (gdc_read_restart(h, restart_in) != GDC_OK) {
      const int rc = fail("dycore_restart", gdc_last_error(h));
      gdc_destroy(h);
      return rc;
    }
  } else {
    // The test cases' set_initial_condition hooks (src/dycore_test.F90:26-43)
    std::vector<double> u((size_t)ld * (M + 4)), v((size_t)ld * (M + 3)), gd(u.size()), ghs(u.size());
    int rc = GDC_E_CONFIG;
    const std::string tc = test_case;
    if (tc == "steady_geostrophic_flow")
      rc = gdc_ic_steady_geostrophic(N, M, u.data(), v.data(), gd.data(), ghs.data(), ld);
    else if (tc == "rossby_haurwitz_wave")
      rc = gdc_ic_rossby_haurwitz(N, M, u.data(), v.data(), gd.data(), ghs.data(), ld);
    else if (tc == "mountain_zonal_flow")
      rc = gdc_ic_mountain_zonal_flow(N, M, u.data(), v.data(), gd.data(), ghs.data(), ld);
    else if (tc == "shallow_water_waves")
      rc = gdc_ic_shallow_water_waves(N, M, u.data(), v.data(), gd.data(), ghs.data(), ld);
    else if (tc == "jet_zonal_flow") {
      gdc_destroy(h);
      return fail("dycore_test", "jet_zonal_flow needs QUADPACK's integrals, which this library does not provide");
    } else {
      gdc_destroy(h);
      std::printf(" [Error]: Unknown test case %s!\n", tc.c_str());
      return 1;
    }
    if (rc != GDC_OK || gdc_set_state(h, u.data(), v.data(), gd.data(), ghs.data(), ld) != GDC_OK) {
      rc = fail("set_initial_condition", gdc_last_error(h));
      gdc_destroy(h);
      return rc;
    }
  }

  // dycore_run (src/dycore_mod.F90:119-142)
  const long long total = steps >= 0 ? steps : gdc_steps_for_run(&p);
  long long done = 0;
  gdc_steps_done(h, &done);
  double mass = 0, energy = 0, beta = 0;
  gdc_diag(h, &mass, &energy, &beta);
  std::printf(" %s: %s %dx%d dt %g, %lld steps\n", case_name, test_case, N, M, p.time_step_size, total);
  log_step(done, p.time_step_size, mass, energy, beta);
  int status = 0;
  for (long long k = 0; k < total;) {
    const long long n = total - k < every ? total - k : every;
    const int rc = gdc_run(h, (int)n);
    k += n;
    gdc_steps_done(h, &done);
    gdc_diag(h, &mass, &energy, &beta);
    if (rc == GDC_E_NAN) {
      std::printf(" [Error]: %s\n", gdc_last_error(h));
      status = 1;
      break;
    }
    if (rc != GDC_OK) {
      status = fail("dycore_run", gdc_last_error(h));
      break;
    }
    log_step(done, p.time_step_size, mass, energy, beta);
  }
  if (status == 0 && restart_out && gdc_write_restart(h, restart_out) != GDC_OK)
    status = fail("restart_write", gdc_last_error(h));

  // dycore_final (src/dycore_mod.F90:144-157)
  gdc_destroy(h);
  return status;
}
