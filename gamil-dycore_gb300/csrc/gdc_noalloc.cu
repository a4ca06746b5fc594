// gdc_noalloc.cu -- the space_operators tendency for callers that cannot
// allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: host frameworks that
// own every device allocation through their own pool and forbid others,
// processes that run under a fixed device-memory budget, and plug-ins that
// must not grow the process's device footprint once running.
// gdc_tendency_noalloc serves them: the caller passes its own device
// buffers for the state and for the tendencies, and everything else the
// stage kernel needs (member descriptor, work list, row coefficient
// tables, filter twiddles, the given-u/v marker) lives in one file-scope
// device array of fixed size, loaded with the library and held by every
// GPU that loads it until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gdc_internal.h"

namespace gdc {

// Scratch of the no-allocation entry point: 2 MiB, enough for grids up to
// 1440 x 721 (the largest configuration of the reference's test suite).
constexpr size_t kNoallocScratchBytes = 2u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
// Guards the per-device addresses and serialises the calls' uploads into
// the shared array.
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {nullptr};
// The calling thread's last failure (read without the lock).
thread_local std::string g_err;

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

}  // namespace gdc

extern "C" const char* gdc_noalloc_last_error(void) { return gdc::g_err.c_str(); }

// See include/gdc.h.
extern "C" int gdc_tendency_noalloc(const gdc_params* p, int pass, const double* gd, const double* iap_u,
                                    const double* iap_v, const double* ghs, const double* given_u,
                                    const double* given_v, double* du, double* dv, double* dgd,
                                    void* cuda_stream) {
  using namespace gdc;
  std::lock_guard<std::mutex> lock(g_mu);
  g_err.clear();
  auto fail = [](int code, const std::string& m) {
    g_err = m;
    return code;
  };
  if (!p || !gd || !iap_u || !iap_v || !ghs || !du || !dv || !dgd)
    return fail(GDC_E_CONFIG, "gdc_tendency_noalloc: null argument");
  if (pass < 0 || pass > 2) return fail(GDC_E_CONFIG, "gdc_tendency_noalloc: pass must be 0, 1 or 2");
  if ((given_u == nullptr) != (given_v == nullptr))
    return fail(GDC_E_CONFIG, "gdc_tendency_noalloc: give both u and v, or neither");
  if (p->uv_adv_scheme != GDC_ADV_CENTER_DIFF && p->uv_adv_scheme != GDC_ADV_UPWIND)
    return fail(GDC_E_CONFIG, "gdc_tendency_noalloc: uv_adv_scheme must be center_diff or upwind");
  const int N = p->num_lon, M = p->num_lat, Mh = M - 1;
  if (N < 8 || M < 5 || N > 1440 || M > 721 || N % 4 != 0)
    return fail(GDC_E_CONFIG,
                "gdc_tendency_noalloc: grid must be within 8..1440 x 5..721 with num_lon a multiple of 4 "
                "(scratch is 2 MiB)");
  for (int k = 0; k < 20; ++k) {
    const int c = p->zonal_tend_filter_cutoff_wavenumber[k];
    if (c < 0 || 2 * (c + 1) > N)
      return fail(GDC_E_CONFIG, "gdc_tendency_noalloc: zonal_tend_filter_cutoff_wavenumber out of range");
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(GDC_E_CUDA, "gdc_tendency_noalloc: no current CUDA device");
  // Once per device, with that device current: the device address of the
  // scratch array (its host-side name is only a stand-in).
  if (!g_scratch_addr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(GDC_E_CUDA, std::string("gdc_tendency_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_addr[dev] = ptr;
  }
  char* base = static_cast<char*>(g_scratch_addr[dev]);

  // Host tables, exactly as the batch engine builds them.
  const Mesh mesh = make_mesh(N, M);
  const Coef co = make_coef(mesh);
  std::vector<double> coef(coef_words(M), 0.0);
  for (int j = 0; j < M; ++j) {
    coef[cf_off(CF_COS, M) + j] = co.full_cos[j];
    coef[cf_off(CF_F, M) + j] = co.full_f[j];
    coef[cf_off(CF_C, M) + j] = co.full_c[j];
    coef[cf_off(CF_RADVLON, M) + j] = 0.25 / co.full_dlon[j];
    coef[cf_off(CF_RADVLAT, M) + j] = 0.25 / co.full_dlat[j];
    coef[cf_off(CF_DLON, M) + j] = co.full_dlon[j];
    coef[cf_off(CF_DLAT, M) + j] = co.full_dlat[j];
    if (j >= 1 && j <= M - 2) {
      coef[cf_off(CF_C1, M) + j] = co.half_cos[j - 1] / co.full_cos[j];
      coef[cf_off(CF_C2, M) + j] = co.half_cos[j] / co.full_cos[j];
    }
    coef[cf_off(CF_MASSW, M) + j] = co.full_cos[j] * mesh.dlon * mesh.dlat;
  }
  for (int j = 0; j < Mh; ++j) {
    coef[ch_off(CH_COS, M) + j + 1] = co.half_cos[j];
    coef[ch_off(CH_RADVLON, M) + j + 1] = 0.25 / co.half_dlon[j];
    coef[ch_off(CH_RADVLAT, M) + j + 1] = 0.25 / co.half_dlat[j];
    coef[ch_off(CH_DLON, M) + j + 1] = co.half_dlon[j];
    coef[ch_off(CH_DLAT, M) + j + 1] = co.half_dlat[j];
  }
  const std::vector<double> rowc = row_records(coef, M);
  std::vector<double> twid(2 * (size_t)N);
  for (int k = 0; k < N; ++k) {
    twid[k] = std::cos(2.0 * kPi * k / N);
    twid[N + k] = std::sin(2.0 * kPi * k / N);
  }
  std::vector<int> ff, kf, fh, kh;
  make_filter_rows(mesh, *p, ff, kf, fh, kh);
  std::vector<int> rowinfo(M, 0);
  for (int j = 0; j < M; ++j) {
    int bits = 0;
    if (ff[j]) bits |= RI_FLAG_FULL;
    if (j < Mh && fh[j]) bits |= RI_FLAG_HALF;
    if (j == 0 || j == M - 1 || bits) bits |= RI_SPECIAL;
    rowinfo[j] = bits | (kf[j] << 8) | ((j < Mh ? kh[j] : 0) << 20);
  }
  const int tile_r = 8, tile_c = 32;
  std::vector<WorkItem> wl;
  for (int j = 0; j < M; ++j)
    if (rowinfo[j] & RI_SPECIAL)
      for (int f : {F_GD, F_IU, F_IV})
        if (f != F_IV || j < M - 1) wl.push_back(WorkItem{0, 1, j, 0, 1, N, (int)wl.size(), f});
  for (int j = 0; j < M;) {
    if (rowinfo[j] & RI_SPECIAL) {
      ++j;
      continue;
    }
    int b = j;
    while (b + 1 < M && !(rowinfo[b + 1] & RI_SPECIAL)) ++b;
    for (int j0 = j; j0 <= b; j0 += tile_r)
      for (int i0 = 0; i0 < N; i0 += tile_c)
        wl.push_back(WorkItem{0, 0, j0, i0, std::min(tile_r, b - j0 + 1), std::min(tile_c, N - i0), (int)wl.size(), 0});
    j = b + 1;
  }
  // Scratch layout: descriptor, given-u/v marker, work list, tables.
  size_t off = 0;
  const size_t o_desc = off;
  off = up256(off + sizeof(MemberDev<double>));
  const size_t o_uvslot = off;
  off = up256(off + sizeof(int));
  const size_t o_wl = off;
  off = up256(off + wl.size() * sizeof(WorkItem));
  const size_t o_coef = off;
  off = up256(off + coef.size() * sizeof(double));
  const size_t o_rowc = off;
  off = up256(off + rowc.size() * sizeof(double));
  const size_t o_twid = off;
  off = up256(off + twid.size() * sizeof(double));
  const size_t o_row = off;
  off = up256(off + rowinfo.size() * sizeof(int));
  if (off > kNoallocScratchBytes)
    return fail(GDC_E_CONFIG, "gdc_tendency_noalloc: grid too large for the 2 MiB scratch");

  MemberDev<double> d;
  std::memset(&d, 0, sizeof(d));
  d.N = N;
  d.M = M;
  d.Mh = Mh;
  d.dt = p->time_step_size;
  d.pcdt[kAllPass] = p->time_step_size;
  d.pcdt[kFastPass] = p->subcycles > 0 ? p->time_step_size / p->subcycles : p->time_step_size;
  d.pcdt[kSlowPass] = 0.5 * p->time_step_size;
  d.st[SL_L0][F_GD] = const_cast<double*>(gd);
  d.st[SL_L0][F_IU] = const_cast<double*>(iap_u);
  d.st[SL_L0][F_IV] = const_cast<double*>(iap_v);
  d.td[TS_NEW][F_GD] = dgd;
  d.td[TS_NEW][F_IU] = du;
  d.td[TS_NEW][F_IV] = dv;
  d.ghs = const_cast<double*>(ghs);
  d.coef = reinterpret_cast<const double*>(base + o_coef);
  d.rowc = reinterpret_cast<const double*>(base + o_rowc);
  d.twid = reinterpret_cast<const double*>(base + o_twid);
  d.rowinfo = reinterpret_cast<const int*>(base + o_row);
  d.given_u = const_cast<double*>(given_u);
  d.given_v = const_cast<double*>(given_v);
  d.pbase = 0;
  d.pcount = (int)wl.size();
  // The array keeps the previous call's contents: every word this call
  // reads is rewritten here, the marker included.
  const int uvslot = given_u ? (int)SL_L0 : -1;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  cudaError_t e = cudaMemcpyAsync(base + o_desc, &d, sizeof(d), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(base + o_uvslot, &uvslot, sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(base + o_wl, wl.data(), wl.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(base + o_coef, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(base + o_rowc, rowc.data(), rowc.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(base + o_twid, twid.data(), twid.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(base + o_row, rowinfo.data(), rowinfo.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail(GDC_E_CUDA, std::string("gdc_tendency_noalloc: upload: ") + cudaGetErrorString(e));
  // The host tables above are pageable: each copy returns once its source
  // has been staged, so they may go out of scope after the calls.
  StageArgs a;
  std::memset(&a, 0, sizeof(a));
  a.pass = pass;
  a.in_slot = SL_L0;
  a.base_slot = a.out_slot = -1;
  a.tout = TS_NEW;
  a.tprev = a.tadd = a.tadd2 = a.taccum = -1;
  a.tadd_sign = 1;
  a.scale2 = 1.0;
  a.h_scale = 0.5;
  a.ip_slot = -1;
  a.qcon = p->qcon_modified;
  a.ub_lon = p->uv_adv_upwind_lon_beta;
  a.ub_lat = p->uv_adv_upwind_lat_beta;
  a.rescale_rtol = p->filter_rescale_rtol;
  a.uvslot = reinterpret_cast<int*>(base + o_uvslot);
  int rc = launch_stage<double>(reinterpret_cast<const MemberDev<double>*>(base + o_desc),
                                reinterpret_cast<const WorkItem*>(base + o_wl), (int)wl.size(), p->uv_adv_scheme,
                                tile_r, tile_c, N, a, s);
  if (rc) return fail(rc, "gdc_tendency_noalloc: kernel launch failed");
  return GDC_OK;
}
