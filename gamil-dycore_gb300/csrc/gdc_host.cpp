// gdc_host.cpp -- host-side pieces of the gamil-dycore barotropic step:
// parameter defaults, the /dycore_params/ namelist reader, the run length,
// the mesh and coefficient tables (FP64, evaluated exactly as the reference
// evaluates them) and the initial-condition hooks.
#include <cuda_runtime.h>

#include "gdc_internal.h"

#include <cctype>
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace gdc {

// ------------------------------------------------------------------ mesh

// src/mesh_mod.F90:44-114 and src/data_mod.F90:26-59, 0-based rows:
// full row j (0..M-1) is the reference's j+1, half row jh (0..Mh-1) is jh+1.
Mesh make_mesh(int N, int M) {
  Mesh m;
  m.N = N;
  m.M = M;
  m.Mh = M - 1;
  const int Mh = m.Mh;
  m.dlon = 2 * kPi / N;
  m.dlat = kPi / Mh;
  m.full_lat.assign(M, 0.0);
  m.half_lat.assign(Mh, 0.0);
  for (int j = 0; j < Mh; ++j) {
    m.full_lat[j] = -0.5 * kPi + j * m.dlat;
    m.half_lat[j] = m.full_lat[j] + 0.5 * m.dlat;
  }
  m.full_lat[M - 1] = 0.5 * kPi;
  m.full_lon.resize(N);
  m.half_lon.resize(N);
  for (int i = 0; i < N; ++i) {
    m.full_lon[i] = i * m.dlon;
    m.half_lon[i] = m.full_lon[i] + 0.5 * m.dlon;
  }
  m.half_cos.resize(Mh);
  m.half_sin.resize(Mh);
  for (int j = 0; j < Mh; ++j) {
    m.half_cos[j] = std::cos(m.half_lat[j]);
    m.half_sin[j] = std::sin(m.half_lat[j]);
  }
  m.full_cos.resize(M);
  m.full_sin.resize(M);
  for (int j = 0; j < M; ++j) {
    m.full_cos[j] = std::cos(m.full_lat[j]);
    m.full_sin[j] = std::sin(m.full_lat[j]);
  }
  m.full_cos[0] = 0.0;
  m.full_cos[M - 1] = 0.0;
  m.full_sin[0] = -1.0;
  m.full_sin[M - 1] = 1.0;
  return m;
}

// Coefficients as the time loop sees them: data_init followed by
// reset_cos_lat_at_poles (src/dycore_mod.F90:159-173), which dycore_run
// applies after the initial condition has been set.
Coef make_coef(const Mesh& m) {
  Coef c;
  const int M = m.M, Mh = m.Mh;
  c.full_cos = m.full_cos;
  c.full_f.resize(M);
  c.full_c.resize(M);
  c.full_dlon.resize(M);
  c.full_dlat.resize(M);
  for (int j = 0; j < M; ++j) {
    c.full_f[j] = 2.0 * kOmega * m.full_sin[j];
    c.full_c[j] = (j == 0 || j == M - 1) ? 0.0 : m.full_sin[j] / m.full_cos[j] / kRadius;
    c.full_dlon[j] = kRadius * m.dlon * m.full_cos[j];
    c.full_dlat[j] = kRadius * m.dlat * m.full_cos[j];
  }
  c.half_cos = m.half_cos;
  c.half_dlon.resize(Mh);
  c.half_dlat.resize(Mh);
  for (int j = 0; j < Mh; ++j) {
    c.half_dlon[j] = kRadius * m.dlon * m.half_cos[j];
    c.half_dlat[j] = kRadius * m.dlat * m.half_cos[j];
  }
  for (int pole : {0, M - 1}) {
    const int adj = pole == 0 ? 0 : Mh - 1;
    c.full_cos[pole] = m.half_cos[adj] * 0.25;
    c.full_dlon[pole] = kRadius * m.dlon * c.full_cos[pole];
    c.full_dlat[pole] = kRadius * m.dlat * c.full_cos[pole];
  }
  return c;
}

// src/filter_mod.F90:35-103.  Returns, per full and half row, whether the
// row is filtered and how many packed FFTPACK coefficients its factor row
// keeps (2*(cutoff+1); 0 when the factor row is all zero).  The north half
// flag index (:56) is one row north of its factor index (:94-95); the flag
// for cutoff entry 1 falls past the last half row and is dropped.
void make_filter_rows(const Mesh& m, const gdc_params& p, std::vector<int>& flag_full,
                      std::vector<int>& keep_full, std::vector<int>& flag_half,
                      std::vector<int>& keep_half) {
  const int M = m.M, Mh = m.Mh;
  flag_full.assign(M, 0);
  keep_full.assign(M, 0);
  flag_half.assign(Mh, 0);
  keep_half.assign(Mh, 0);
  for (int k = 1; k <= 20; ++k) {
    const int c = p.zonal_tend_filter_cutoff_wavenumber[k - 1];
    if (c == 0) continue;
    // Fortran full_lat_start_idx+k -> 0-based k; half start+k-1 -> k-1;
    // north full end-k -> M-1-k; north half factor Mh-k+1 -> Mh-k;
    // north half flag (full_lat_end_idx-k+1) -> M-k.
    if (k < M) keep_full[k] = 2 * (c + 1);
    if (k - 1 < Mh) keep_half[k - 1] = 2 * (c + 1);
    if (M - 1 - k >= 0) keep_full[M - 1 - k] = 2 * (c + 1);
    if (Mh - k >= 0) keep_half[Mh - k] = 2 * (c + 1);
    if (p.use_zonal_tend_filter) {
      if (k < M) flag_full[k] = 1;
      if (k - 1 < Mh) flag_half[k - 1] = 1;
      if (M - 1 - k >= 0) flag_full[M - 1 - k] = 1;
      if (M - k <= Mh - 1) flag_half[M - k] = 1;
    }
  }
}

// ---------------------------------------------------------------- params

}  // namespace gdc

extern "C" void gdc_params_default(gdc_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->subcycles = 4;                // src/params_mod.F90:16
  p->use_diffusion = 0;            // :18
  p->diffusion_order = 2;          // :20
  p->split_scheme = GDC_SPLIT_NONE;
  p->qcon_modified = 0;
  p->uv_adv_scheme = GDC_ADV_CENTER_DIFF;  // :58
  p->uv_adv_upwind_lon_beta = 0.0;         // :59
  p->uv_adv_upwind_lat_beta = 0.5;         // :60
  p->use_zonal_tend_filter = 1;            // :65
  p->precision = GDC_FP64;
  // the calling thread's current CUDA device (0 where there is none), as a
  // process that runs one rank per device has selected it
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) {
    cudaGetLastError();
    d = 0;
  }
  p->device = d;
}

extern "C" int gdc_steps_for_run(const gdc_params* p) {
  // end_time = start + run_days/hours/minutes (run_seconds is not used by
  // time_init, src/time_mod.F90:59-64); the loop runs while curr < end.
  const double len = p->run_days * 86400.0 + p->run_hours * 3600.0 + p->run_minutes * 60.0;
  if (!(p->time_step_size > 0)) return 0;
  return (int)std::ceil(len / p->time_step_size - 1e-9);
}

namespace {

std::string lower(std::string s) {
  for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

// Split a namelist value list on commas outside quotes.
std::vector<std::string> split_values(const std::string& s) {
  std::vector<std::string> out;
  std::string cur;
  char q = 0;
  for (char ch : s) {
    if (q) {
      cur += ch;
      if (ch == q) q = 0;
    } else if (ch == '\'' || ch == '"') {
      q = ch;
      cur += ch;
    } else if (ch == ',') {
      out.push_back(trim(cur));
      cur.clear();
    } else {
      cur += ch;
    }
  }
  if (!trim(cur).empty()) out.push_back(trim(cur));
  return out;
}

bool parse_logical(const std::string& v, int* out) {
  std::string s = lower(trim(v));
  if (!s.empty() && s[0] == '.') s = s.substr(1);
  if (s.empty()) return false;
  if (s[0] == 't') { *out = 1; return true; }
  if (s[0] == 'f') { *out = 0; return true; }
  return false;
}

bool parse_real(const std::string& v, double* out) {
  std::string s = lower(trim(v));
  for (auto& ch : s)
    if (ch == 'd') ch = 'e';
  char* end = nullptr;
  *out = std::strtod(s.c_str(), &end);
  return end && *end == 0 && !s.empty();
}

bool parse_int(const std::string& v, int* out) {
  std::string s = trim(v);
  char* end = nullptr;
  long x = std::strtol(s.c_str(), &end, 10);
  if (!end || *end != 0 || s.empty()) return false;
  *out = (int)x;
  return true;
}

std::string parse_string(const std::string& v) {
  std::string s = trim(v);
  if (s.size() >= 2 && (s[0] == '\'' || s[0] == '"') && s.back() == s[0])
    return s.substr(1, s.size() - 2);
  return s;
}

void put(char* dst, int len, const std::string& s) {
  if (!dst || len <= 0) return;
  std::snprintf(dst, (size_t)len, "%s", s.c_str());
}

}  // namespace

// params_read (src/params_mod.F90:102-115) for namelist /dycore_params/
// (:68-98).  Other groups in the file are skipped.
extern "C" int gdc_params_read_namelist(const char* path, gdc_params* p, char* test_case,
                                        int test_case_len, char* case_name,
                                        int case_name_len, char* errbuf, int errbuf_len) {
  gdc_params_default(p);
  std::ifstream f(path);
  if (!f) {
    put(errbuf, errbuf_len, std::string("cannot open namelist ") + path);
    return GDC_E_CONFIG;
  }
  std::string body, line;
  bool in_group = false, found = false;
  while (std::getline(f, line)) {
    // Strip comments outside quotes.
    std::string clean;
    char q = 0;
    for (char ch : line) {
      if (q) {
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
      } else if (ch == '!') {
        break;
      }
      clean += ch;
    }
    std::string t = trim(clean);
    if (!in_group) {
      if (lower(t).rfind("&dycore_params", 0) == 0) {
        in_group = true;
        found = true;
        t = trim(t.substr(14));
      } else {
        continue;
      }
    }
    if (!t.empty() && t.back() == '/') {
      body += " " + t.substr(0, t.size() - 1) + "\n";
      in_group = false;
      break;
    }
    body += " " + t + "\n";
  }
  if (!found) {
    put(errbuf, errbuf_len, "namelist group &dycore_params not found");
    return GDC_E_CONFIG;
  }
  // Tokenise "key = values" pairs: a key starts where an identifier is
  // followed by '='.
  std::vector<std::pair<std::string, std::string>> kv;
  {
    size_t pos = 0;
    std::string key;
    std::string acc;
    auto flush = [&]() {
      if (!key.empty()) kv.emplace_back(lower(trim(key)), trim(acc));
      key.clear();
      acc.clear();
    };
    while (pos < body.size()) {
      // Find the next '=' outside quotes.
      size_t eq = std::string::npos;
      char q = 0;
      for (size_t k = pos; k < body.size(); ++k) {
        char ch = body[k];
        if (q) {
          if (ch == q) q = 0;
        } else if (ch == '\'' || ch == '"') {
          q = ch;
        } else if (ch == '=') {
          eq = k;
          break;
        }
      }
      if (eq == std::string::npos) {
        acc += body.substr(pos);
        break;
      }
      // The identifier immediately before '=' is the new key; text between
      // the previous key and it belongs to the previous value.
      size_t ke = eq;
      while (ke > pos && std::isspace((unsigned char)body[ke - 1])) --ke;
      size_t ks = ke;
      while (ks > pos && (std::isalnum((unsigned char)body[ks - 1]) || body[ks - 1] == '_' ||
                          body[ks - 1] == '(' || body[ks - 1] == ')'))
        --ks;
      acc += body.substr(pos, ks - pos);
      flush();
      key = body.substr(ks, ke - ks);
      pos = eq + 1;
    }
    flush();
  }
  std::string tc, cn, ts = "predict_correct";
  for (auto& [k, vraw] : kv) {
    std::string v = vraw;
    while (!v.empty() && (v.back() == ',' || std::isspace((unsigned char)v.back()))) v.pop_back();
    auto vals = split_values(v);
    auto bad = [&](const char* what) {
      put(errbuf, errbuf_len, "bad value for " + k + " (" + what + "): " + v);
      return GDC_E_CONFIG;
    };
    int iv;
    double dv;
    if (k == "num_lon") { if (!parse_int(v, &p->num_lon)) return bad("integer"); }
    else if (k == "num_lat") { if (!parse_int(v, &p->num_lat)) return bad("integer"); }
    else if (k == "subcycles") { if (!parse_int(v, &p->subcycles)) return bad("integer"); }
    else if (k == "run_days") { if (!parse_int(v, &p->run_days)) return bad("integer"); }
    else if (k == "run_hours") { if (!parse_int(v, &p->run_hours)) return bad("integer"); }
    else if (k == "run_minutes") { if (!parse_int(v, &p->run_minutes)) return bad("integer"); }
    else if (k == "run_seconds") { if (!parse_int(v, &p->run_seconds)) return bad("integer"); }
    else if (k == "time_step_size") { if (!parse_real(v, &p->time_step_size)) return bad("real"); }
    else if (k == "time_order") { if (!parse_int(v, &iv)) return bad("integer"); }
    else if (k == "qcon_modified") { if (!parse_logical(v, &p->qcon_modified)) return bad("logical"); }
    else if (k == "use_zonal_tend_filter") { if (!parse_logical(v, &p->use_zonal_tend_filter)) return bad("logical"); }
    else if (k == "use_diffusion") { if (!parse_logical(v, &p->use_diffusion)) return bad("logical"); }
    else if (k == "diffusion_order") { if (!parse_int(v, &p->diffusion_order)) return bad("integer"); }
    else if (k == "diffusion_coef") { if (!parse_real(v, &p->diffusion_coef)) return bad("real"); }
    else if (k == "uv_adv_upwind_lon_beta") { if (!parse_real(v, &p->uv_adv_upwind_lon_beta)) return bad("real"); }
    else if (k == "uv_adv_upwind_lat_beta") { if (!parse_real(v, &p->uv_adv_upwind_lat_beta)) return bad("real"); }
    else if (k == "zonal_tend_filter_cutoff_wavenumber") {
      if (vals.size() > 20) return bad("at most 20 integers");
      for (size_t q = 0; q < vals.size(); ++q)
        if (!parse_int(vals[q], &p->zonal_tend_filter_cutoff_wavenumber[q])) return bad("integer list");
    } else if (k == "start_time" || k == "end_time") {
      for (auto& s : vals)
        if (!parse_int(s, &iv)) return bad("integer list");
    } else if (k == "split_scheme") {
      std::string s = lower(parse_string(v));
      p->split_scheme = s == "csp1" ? GDC_SPLIT_CSP1 : s == "csp2" ? GDC_SPLIT_CSP2
                        : s == "isp" ? GDC_SPLIT_ISP : GDC_SPLIT_NONE;
    } else if (k == "uv_adv_scheme") {
      std::string s = lower(parse_string(v));
      if (s == "center_diff") p->uv_adv_scheme = GDC_ADV_CENTER_DIFF;
      else if (s == "upwind") p->uv_adv_scheme = GDC_ADV_UPWIND;
      else if (s == "weno") p->uv_adv_scheme = GDC_ADV_WENO;
      else return bad("Unknown uv_adv_scheme");
    } else if (k == "time_scheme") {
      ts = lower(parse_string(v));
    } else if (k == "test_case") {
      tc = parse_string(v);
    } else if (k == "case_name") {
      cn = parse_string(v);
    } else if (k == "case_desc" || k == "author" || k == "history_periods" ||
               k == "restart_period" || k == "restart_file" || k == "time_units") {
      // strings used only by output, restart and logging
    } else {
      put(errbuf, errbuf_len, "unknown namelist key " + k);
      return GDC_E_CONFIG;
    }
    (void)dv;
  }
  if (ts != "predict_correct") {
    put(errbuf, errbuf_len, "Unknown time_scheme " + ts + "!");
    return GDC_E_CONFIG;
  }
  put(test_case, test_case_len, tc);
  put(case_name, case_name_len, cn);
  return GDC_OK;
}

// ----------------------------------------------------- initial conditions

namespace {

using gdc::kOmega;
using gdc::kPi;
using gdc::kRadius;
constexpr double kG = gdc::kGrav;

// Padded-layout helpers: Fortran (i,j) = (i0+1, j0+1) for 0-based interior.
inline double& P(double* f, int ld, int i0, int j0) { return f[(size_t)(j0 + 2) * ld + (i0 + 2)]; }

void zero_field(double* f, int ld, int rows) {
  if (f) std::memset(f, 0, sizeof(double) * (size_t)ld * (rows + 4));
}

// parallel_fill_halo (src/parallel_mod.F90:466-524) on an interior-filled
// padded field of `rows` latitude rows.
void fill_lon_halo(double* f, int ld, int N, int rows) {
  for (int r = 0; r < rows + 4; ++r) {
    double* row = f + (size_t)r * ld;
    row[0] = row[N];
    row[1] = row[N + 1];
    row[N + 2] = row[2];
    row[N + 3] = row[3];
  }
}

bool check_grid(int N, int M, int ld) { return N >= 4 && M >= 5 && ld >= N + 4; }

// splitmix64 -> uniform (0,1) -> Box-Muller normals.
struct Rng {
  unsigned long long s;
  bool have = false;
  double spare = 0;
  explicit Rng(unsigned long long seed) : s(seed) {}
  unsigned long long next() {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double normal() {
    if (have) {
      have = false;
      return spare;
    }
    double u1 = uniform(), u2 = uniform();
    double r = std::sqrt(-2.0 * std::log(u1));
    spare = r * std::sin(2 * kPi * u2);
    have = true;
    return r * std::cos(2 * kPi * u2);
  }
};

// Real spherical-harmonic series sum_{l=1..L} sum_{m=0..l}
// Pbar_l^m(sin lat) (a_lm cos m lon + b_lm sin m lon) with orthonormal
// associated Legendre functions (standard three-term recurrence).
struct Harmonics {
  int L;
  std::vector<double> a, b;  // index l*(L+1)+m
  Harmonics(int L_, Rng& rng) : L(L_), a((L_ + 1) * (L_ + 1), 0.0), b((L_ + 1) * (L_ + 1), 0.0) {
    for (int l = 1; l <= L; ++l)
      for (int m = 0; m <= l; ++m) {
        a[l * (L + 1) + m] = rng.normal();
        if (m > 0) b[l * (L + 1) + m] = rng.normal();
      }
  }
  double eval(double lat, double lon) const {
    const double x = std::sin(lat), sx = std::cos(lat);
    std::vector<double> P((L + 1) * (L + 1), 0.0);
    P[0] = std::sqrt(1.0 / (4 * kPi));
    for (int m = 1; m <= L; ++m)
      P[m * (L + 1) + m] = std::sqrt((2.0 * m + 1) / (2.0 * m)) * sx * P[(m - 1) * (L + 1) + m - 1];
    for (int m = 0; m < L; ++m) P[(m + 1) * (L + 1) + m] = std::sqrt(2.0 * m + 3) * x * P[m * (L + 1) + m];
    for (int m = 0; m <= L; ++m)
      for (int l = m + 2; l <= L; ++l) {
        double al = std::sqrt((4.0 * l * l - 1) / ((double)l * l - (double)m * m));
        double bl = std::sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1));
        P[l * (L + 1) + m] = al * (x * P[(l - 1) * (L + 1) + m] - bl * P[(l - 2) * (L + 1) + m]);
      }
    double s = 0;
    for (int l = 1; l <= L; ++l)
      for (int m = 0; m <= l; ++m) {
        double w = (m == 0 ? 1.0 : std::sqrt(2.0)) * P[l * (L + 1) + m];
        s += w * (a[l * (L + 1) + m] * std::cos(m * lon) + b[l * (L + 1) + m] * std::sin(m * lon));
      }
    return s;
  }
};

}  // namespace

namespace gdc {
void rh_tables(const Mesh& m, std::vector<double>& t) {
  const int N = m.N, M = m.M, Mh = m.Mh;
  const double R = 4.0, omg = 7.848e-6;
  t.assign(rh_table_words(N, M), 0.0);
  for (int j = 0; j < M; ++j) {
    const double cl = m.full_cos[j], sl = m.full_sin[j];
    t[j] = cl;
    t[M + j] = R * std::pow(cl, R - 1) * (sl * sl);
    t[2 * M + j] = std::pow(cl, R + 1);
    t[4 * M + j] = 0.5 * omg * (2 * kOmega + omg) * (cl * cl) +
                   0.25 * omg * omg *
                       ((R + 1) * std::pow(cl, 2 * R + 2) + (2 * R * R - R - 2) * std::pow(cl, 2 * R) -
                        2 * R * R * std::pow(cl, 2 * R - 2));
    t[5 * M + j] = 2 * (kOmega + omg) * omg * std::pow(cl, R) *
                   (R * R + 2 * R + 2 - (R + 1) * (R + 1) * (cl * cl)) / (R + 1) / (R + 2);
    t[6 * M + j] = 0.25 * omg * omg * std::pow(cl, 2 * R) * ((R + 1) * (cl * cl) - R - 2);
  }
  for (int j = 0; j < Mh; ++j) t[3 * M + j] = R * std::pow(m.half_cos[j], R - 1) * m.half_sin[j];
  double* col = t.data() + 7 * (size_t)M;
  for (int i = 0; i < N; ++i) {
    col[i] = std::cos(R * m.half_lon[i]);
    col[N + i] = std::sin(R * m.full_lon[i]);
    col[2 * N + i] = std::cos(R * m.full_lon[i]);
    col[3 * N + i] = std::cos(2 * R * m.full_lon[i]);
  }
}
}  // namespace gdc

// src/test_cases/barotropic/rossby_haurwitz_wave_test_mod.F90:33-85: the
// factor tables of rh_tables and their products (rh_u, rh_v, rh_gd), which
// evaluate the reference's expressions in its order.
extern "C" int gdc_ic_rossby_haurwitz(int N, int M, double* u, double* v, double* gd,
                                      double* ghs, int ld) {
  if (!check_grid(N, M, ld) || !u || !v || !gd || !ghs) return GDC_E_CONFIG;
  const gdc::Mesh m = gdc::make_mesh(N, M);
  std::vector<double> t;
  gdc::rh_tables(m, t);
  zero_field(u, ld, M); zero_field(v, ld, M - 1); zero_field(gd, ld, M); zero_field(ghs, ld, M);
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < N; ++i) {
      P(u, ld, i, j) = gdc::rh_u(t.data(), N, M, i, j);
      P(gd, ld, i, j) = gdc::rh_gd(t.data(), N, M, i, j);
      if (j < M - 1) P(v, ld, i, j) = gdc::rh_v(t.data(), N, M, i, j);
    }
  fill_lon_halo(u, ld, N, M); fill_lon_halo(v, ld, N, M - 1); fill_lon_halo(gd, ld, N, M);
  return GDC_OK;
}

namespace {
// Shared body of steady_geostrophic_flow (alpha = 0) and
// mountain_zonal_flow: u = u0 cos(lat), v = -u0 sin(lon) sin(alpha),
// gd = gd0 - (a Omega u0 + u0^2/2) sin^2(lat) - ghs.
void zonal_flow(const gdc::Mesh& m, double u0, double gd0, double* u, double* v, double* gd,
                const double* ghs, int ld) {
  const int N = m.N, M = m.M;
  const double alpha = 0.0, ca = std::cos(alpha), sa = std::sin(alpha);
  for (int j = 1; j < M - 1; ++j)
    for (int i = 0; i < N; ++i)
      P(u, ld, i, j) = u0 * (m.full_cos[j] * ca + std::cos(m.half_lon[i]) * m.full_sin[j] * sa);
  for (int j = 0; j < M - 1; ++j)
    for (int i = 0; i < N; ++i) P(v, ld, i, j) = -u0 * std::cos(m.full_lon[i]) * sa;
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < N; ++i) {
      const double t = m.full_sin[j] * ca - std::cos(m.full_lon[i]) * m.full_cos[j] * sa;
      P(gd, ld, i, j) = gd0 - (kRadius * kOmega * u0 + u0 * u0 * 0.5) * (t * t) -
                        (ghs ? ghs[(size_t)(j + 2) * ld + (i + 2)] : 0.0);
    }
}
}  // namespace

// src/test_cases/barotropic/steady_geostrophic_flow_test_mod.F90:20-62
extern "C" int gdc_ic_steady_geostrophic(int N, int M, double* u, double* v, double* gd,
                                         double* ghs, int ld) {
  if (!check_grid(N, M, ld) || !u || !v || !gd || !ghs) return GDC_E_CONFIG;
  const gdc::Mesh m = gdc::make_mesh(N, M);
  zero_field(u, ld, M); zero_field(v, ld, M - 1); zero_field(gd, ld, M); zero_field(ghs, ld, M);
  zonal_flow(m, 2 * kPi * kRadius / (12 * 86400), 2.94e4, u, v, gd, nullptr, ld);
  fill_lon_halo(u, ld, N, M); fill_lon_halo(v, ld, N, M - 1); fill_lon_halo(gd, ld, N, M);
  return GDC_OK;
}

// src/test_cases/barotropic/mountain_zonal_flow_test_mod.F90:28-97
extern "C" int gdc_ic_mountain_zonal_flow(int N, int M, double* u, double* v, double* gd,
                                          double* ghs, int ld) {
  if (!check_grid(N, M, ld) || !u || !v || !gd || !ghs) return GDC_E_CONFIG;
  const gdc::Mesh m = gdc::make_mesh(N, M);
  zero_field(u, ld, M); zero_field(v, ld, M - 1); zero_field(gd, ld, M); zero_field(ghs, ld, M);
  const double lon0 = kPi * 1.5, lat0 = kPi / 6.0, R = kPi / 9.0, ghs0 = 2000.0 * kG;
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < N; ++i) {
      double dlon = std::fabs(m.full_lon[i] - lon0);
      dlon = std::fmin(dlon, 2 * kPi - dlon);
      const double dl = m.full_lat[j] - lat0;
      const double d = std::fmin(R, std::sqrt(dlon * dlon + dl * dl));
      P(ghs, ld, i, j) = ghs0 * (1.0 - d / R);
    }
  fill_lon_halo(ghs, ld, N, M);
  zonal_flow(m, 20.0, 5960.0 * kG, u, v, gd, ghs, ld);
  fill_lon_halo(u, ld, N, M); fill_lon_halo(v, ld, N, M - 1); fill_lon_halo(gd, ld, N, M);
  return GDC_OK;
}

namespace gdc {
namespace {
// Parameters of src/test_cases/barotropic/shallow_water_waves_test_mod.F90:
// 73-87 (the module's own Earth constants; its sigma and a3..a5 are
// compile-time constants there, rounded as double arithmetic).
constexpr double kSwOmega = 7.29212e-5, kSwG = 9.80616, kSwA = 6371220.0, kSwH0 = 5.0e3;
constexpr double kSwPi = 3.14159265358979323;
constexpr int kSwN = 5, kSwK = 10;
double sw_sigma() { return 0.5 + std::sqrt(0.25 + kSwK * kSwK); }

// Complex power as z**r evaluates it: exp(r log z).
std::complex<double> cpow_real(std::complex<double> z, double r) {
  return std::exp(std::complex<double>(r, 0.0) * std::log(z));
}
}  // namespace

// getPhaseSpeed (:139-183): the three roots of the cubic
// k^2 C^3 - En C - 2 g H0 omega / a^2 = 0 by Cardano's formula; Rossby is
// minus the smallest magnitude, EIG the largest, WIG the smallest.
double sw_waves_phase_speed(int wave_flag) {
  using cd = std::complex<double>;
  const double sigma = sw_sigma(), k = kSwK, n = kSwN;
  const double En = kSwG * kSwH0 / (kSwA * kSwA) * ((n + sigma) * (n + sigma));
  const double Delta0 = 3.0 * (k * k) * En;
  const double Delta4 = -(54.0 * (k * k * k * k) * kSwG * kSwH0 * kSwOmega / (kSwA * kSwA));
  const double r3 = 1.0 / 3.0;
  double Cj[3];
  for (int j = 1; j <= 3; ++j) {
    cd D = cpow_real(cd(1.0, 0.0) * (Delta4 * Delta4 - 4.0 * (Delta0 * Delta0 * Delta0)), 0.5);
    D = cpow_real(0.5 * (Delta4 + D), r3);
    D = D * std::exp(2.0 * kSwPi * cd(0.0, 1.0) * (double)j * r3);
    Cj[j - 1] = -(r3 / (k * k) * (D + Delta0 / D)).real();
  }
  if (wave_flag == 0) return -std::min({std::fabs(Cj[0]), std::fabs(Cj[1]), std::fabs(Cj[2])});
  if (wave_flag == 1) return std::max({Cj[0], Cj[1], Cj[2]});
  return std::min({Cj[0], Cj[1], Cj[2]});
}

// getPsi (:188-215) and getAmplitudes (:220-268) of the Rossby wave at the
// full latitudes; getFields' longitude factors (:272-318) at time 0.
void sw_waves_tables(const Mesh& m, std::vector<double>& t) {
  const int N = m.N, M = m.M;
  const double sigma = sw_sigma(), k = kSwK;
  const double a3 = sigma * (sigma + 1) * (sigma + 2), a4 = a3 * (sigma + 3), a5 = a4 * (sigma + 4);
  const double amp = 1.0e-8, r2 = 0.5, o2 = 2.0 * kSwOmega;
  const double C = sw_waves_phase_speed(0);
  t.assign(sw_table_words(N, M), 0.0);
  for (int j = 0; j < M; ++j) {
    const double lat = m.full_lat[j];
    const double s = std::sin(lat), c = std::cos(lat), tn = std::tan(lat);
    const double s2 = s * s, s4 = s2 * s2;
    const double C5 = (4.0 * a5 * s4 - 20.0 * a4 * s2 + 15.0 * a3) * s / 15.0;
    const double C5p = (4.0 * a5 * s4 - 12.0 * a4 * s2 + 3.0 * a3) * c / 3.0;
    const double psi = amp * std::pow(c, sigma) * C5;
    const double dpsi = amp * std::pow(c, sigma) * (-(sigma * tn * C5) + C5p);
    const double Kp = (kSwG * kSwH0 + kSwA * kSwA * (C * C) * (c * c)) / (C * c);
    const double Km = (kSwG * kSwH0 - kSwA * kSwA * (C * C) * (c * c)) / (C * c);
    const double vt = std::pow(o2 * std::fabs(Km) / (c * c), r2) * psi;
    const double ht = std::pow(o2 * std::fabs(Km) * (kSwA * kSwA) * (kSwH0 * kSwH0), r2) / Km *
                      (dpsi + tn * (r2 * Kp / Km - o2 / C) * psi);
    const double ut = (o2 * s / C) * vt + (kSwG / kSwA / c / C) * ht;
    t[j] = ut;
    t[M + j] = k * vt;
    t[2 * M + j] = ht;
  }
  double* col = t.data() + 3 * (size_t)M;
  for (int i = 0; i < N; ++i) {
    col[i] = std::cos(k * m.half_lon[i]);
    col[N + i] = std::cos(k * m.full_lon[i] - 0.5 * kSwPi);
    col[2 * N + i] = std::cos(k * m.full_lon[i]);
  }
}
}  // namespace gdc

// src/test_cases/barotropic/shallow_water_waves_test_mod.F90:97-135
extern "C" int gdc_ic_shallow_water_waves(int N, int M, double* u, double* v, double* gd, double* ghs,
                                          int ld) {
  if (!check_grid(N, M, ld) || !u || !v || !gd || !ghs) return GDC_E_CONFIG;
  const gdc::Mesh m = gdc::make_mesh(N, M);
  std::vector<double> t;
  gdc::sw_waves_tables(m, t);
  zero_field(u, ld, M); zero_field(v, ld, M - 1); zero_field(gd, ld, M); zero_field(ghs, ld, M);
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < N; ++i) {
      P(u, ld, i, j) = gdc::sw_u(t.data(), N, M, i, j);
      P(gd, ld, i, j) = gdc::sw_gd(t.data(), N, M, i, j);
      if (j < M - 1) P(v, ld, i, j) = gdc::sw_v(t.data(), N, M, i, j);
    }
  fill_lon_halo(u, ld, N, M); fill_lon_halo(v, ld, N, M - 1); fill_lon_halo(gd, ld, N, M);
  return GDC_OK;
}

extern "C" double gdc_sw_waves_phase_speed(int wave_flag) { return gdc::sw_waves_phase_speed(wave_flag); }

namespace gdc {
// The random draws of gdc_ic_seeded, in its order (mountain centres, then
// the gd and the streamfunction harmonics), for the device generator.
void seeded_draws(unsigned long long seed, int lmax, int n_mountains, std::vector<double>& clat,
                  std::vector<double>& clon, std::vector<double>& ag, std::vector<double>& bg,
                  std::vector<double>& ap, std::vector<double>& bp) {
  Rng rng(seed);
  clat.assign(n_mountains, 0.0);
  clon.assign(n_mountains, 0.0);
  for (int k = 0; k < n_mountains; ++k) {
    clon[k] = 2 * kPi * rng.uniform();
    clat[k] = std::asin(2 * rng.uniform() - 1);
  }
  Harmonics hg(lmax, rng), hp(lmax, rng);
  ag = hg.a;
  bg = hg.b;
  ap = hp.a;
  bp = hp.b;
}
}  // namespace gdc

extern "C" int gdc_ic_seeded(int N, int M, unsigned long long seed, int lmax, double gd0,
                             double gd_rms, double psi_rms, double u0, int n_mountains,
                             double mountain_height, double mountain_radius_deg, double* u,
                             double* v, double* gd, double* ghs, int ld) {
  if (!check_grid(N, M, ld) || !u || !v || !gd || !ghs || lmax < 0 || lmax > 64)
    return GDC_E_CONFIG;
  const gdc::Mesh m = gdc::make_mesh(N, M);
  const int Mh = M - 1;
  zero_field(u, ld, M); zero_field(v, ld, Mh); zero_field(gd, ld, M); zero_field(ghs, ld, M);
  Rng rng(seed);
  // Mountains first (fixed draw order: centres, then the two harmonic sets).
  std::vector<double> clat(n_mountains), clon(n_mountains);
  for (int k = 0; k < n_mountains; ++k) {
    clon[k] = 2 * kPi * rng.uniform();
    clat[k] = std::asin(2 * rng.uniform() - 1);
  }
  Harmonics hg(lmax, rng), hp(lmax, rng);
  // gd: harmonics at full points, rescaled to gd_rms over the interior.
  std::vector<double> f((size_t)M * N, 0.0);
  double ss = 0;
  if (lmax > 0 && gd_rms > 0) {
    for (int j = 0; j < M; ++j)
      for (int i = 0; i < N; ++i) {
        f[(size_t)j * N + i] = hg.eval(m.full_lat[j], m.full_lon[i]);
        ss += f[(size_t)j * N + i] * f[(size_t)j * N + i];
      }
  }
  const double gscale = ss > 0 ? gd_rms / std::sqrt(ss / ((double)M * N)) : 0.0;
  const double rr = mountain_radius_deg * kPi / 180.0;
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < N; ++i) {
      double h = 0;
      for (int k = 0; k < n_mountains; ++k) {
        // Great-circle angle (haversine form).
        const double dphi = m.full_lat[j] - clat[k], dlam = m.full_lon[i] - clon[k];
        const double s1 = std::sin(0.5 * dphi), s2 = std::sin(0.5 * dlam);
        const double hv = s1 * s1 + std::cos(m.full_lat[j]) * std::cos(clat[k]) * s2 * s2;
        const double d = 2 * std::asin(std::sqrt(std::fmin(1.0, hv)));
        h += mountain_height * kG * std::exp(-(d / rr) * (d / rr));
      }
      P(ghs, ld, i, j) = h;
      const double t = m.full_sin[j];
      P(gd, ld, i, j) = gd0 + gscale * f[(size_t)j * N + i] - (kRadius * kOmega * u0 + u0 * u0 * 0.5) * (t * t) - h;
    }
  // Streamfunction at C-grid corners (half lon, half lat).
  std::vector<double> psi((size_t)Mh * N, 0.0);
  ss = 0;
  if (lmax > 0 && psi_rms > 0) {
    for (int j = 0; j < Mh; ++j)
      for (int i = 0; i < N; ++i) {
        psi[(size_t)j * N + i] = hp.eval(m.half_lat[j], m.half_lon[i]);
        ss += psi[(size_t)j * N + i] * psi[(size_t)j * N + i];
      }
  }
  const double pscale = ss > 0 ? psi_rms / std::sqrt(ss / ((double)Mh * N)) : 0.0;
  for (auto& x : psi) x *= pscale;
  // u = -(1/a) dpsi/dlat at (half lon i, full row j), v = (1/(a cos)) dpsi/dlon
  // at (full lon i, half row j): the discrete C-grid divergence vanishes.
  for (int j = 1; j < M - 1; ++j)
    for (int i = 0; i < N; ++i)
      P(u, ld, i, j) = -(psi[(size_t)j * N + i] - psi[(size_t)(j - 1) * N + i]) / (kRadius * m.dlat) +
                       u0 * m.full_cos[j];
  for (int j = 0; j < Mh; ++j)
    for (int i = 0; i < N; ++i) {
      const int im = (i + N - 1) % N;
      P(v, ld, i, j) = (psi[(size_t)j * N + i] - psi[(size_t)j * N + im]) / (kRadius * m.half_cos[j] * m.dlon);
    }
  fill_lon_halo(u, ld, N, M); fill_lon_halo(v, ld, N, Mh);
  fill_lon_halo(gd, ld, N, M); fill_lon_halo(ghs, ld, N, M);
  return GDC_OK;
}

extern "C" void gdc_ic_spec_default(gdc_ic_spec* spec, int kind) {
  if (!spec) return;
  std::memset(spec, 0, sizeof(*spec));
  spec->kind = kind;
  spec->lmax = 6;
  spec->gd0 = 8000.0 * kG;
  spec->gd_rms = 100.0 * kG;
  spec->psi_rms = 1.0e7;
  spec->mountain_height = 2000.0;
  spec->mountain_radius_deg = 20.0;
}

extern "C" int gdc_ic_add_noise(int N, int M, unsigned long long seed, double sigma, double* gd,
                                int ld) {
  if (!check_grid(N, M, ld) || !gd) return GDC_E_CONFIG;
  Rng rng(seed);
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < N; ++i) P(gd, ld, i, j) += sigma * rng.normal();
  fill_lon_halo(gd, ld, N, M);
  return GDC_OK;
}
