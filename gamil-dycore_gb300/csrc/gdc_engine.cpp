// gdc_engine.cpp -- host engine behind the C ABI (include/gdc.h).
//
// A batch holds up to kSlots members, each with its own grid, time step and
// length, all advanced by one sequence of kernel launches per model step:
// the launches of the reference's time_integrate (src/dycore_mod.F90:
// 654-752) for the scheme of the batch, each covering the work items of
// every active member.  One model step is captured once into a CUDA graph
// per time-level parity and replayed.  A single model (gdc_handle) is a
// batch of one member.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "gdc_internal.h"

namespace gdc {

namespace {

constexpr int kSlots = 1024;
constexpr size_t kAlign = 256;

size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

bool uses_isp(const gdc_params& p) { return p.split_scheme == GDC_SPLIT_ISP; }

// Byte layout of one member's device allocation.
struct Layout {
  size_t st[SL_N][3], lo[SL_N][3], td[TS_N][3], ghs, coef, rowc, twid, rowinfo, dcoef, given_u, given_v, wadv[2],
      total;
};

template <typename T>
Layout make_layout(const gdc_params& p, int N, int M) {
  Layout L;
  const size_t full = (size_t)M * N, half = (size_t)(M - 1) * N;
  const size_t fsz[3] = {full, full, half};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  const bool isp = uses_isp(p), fp32 = sizeof(T) == 4;
  for (int s = 0; s < SL_N; ++s)
    for (int f = 0; f < 3; ++f) {
      const bool need = s != SL_SAVED || isp;
      L.st[s][f] = need ? take(fsz[f] * sizeof(T)) : (size_t)-1;
      const bool level = s <= SL_SAVED;
      L.lo[s][f] = (need && level && fp32) ? take(fsz[f] * sizeof(T)) : (size_t)-1;
    }
  for (int t = 0; t < TS_N; ++t)
    for (int f = 0; f < 3; ++f)
      L.td[t][f] = (t <= TS_NEW || isp) ? take(fsz[f] * sizeof(T)) : (size_t)-1;
  L.ghs = take(full * sizeof(T));
  L.coef = take(coef_words(M) * sizeof(T));
  L.rowc = take(rec_words(M) * sizeof(T));
  L.twid = take(2 * (size_t)N * sizeof(T));
  L.rowinfo = take((size_t)M * sizeof(int));
  L.dcoef = take((size_t)(3 * M) * sizeof(double));
  L.given_u = take(full * sizeof(T));
  L.given_v = take(half * sizeof(T));
  const bool weno = p.uv_adv_scheme == GDC_ADV_WENO;
  L.wadv[0] = weno ? take(full * sizeof(T)) : (size_t)-1;
  L.wadv[1] = weno ? take(half * sizeof(T)) : (size_t)-1;
  L.total = off;
  return L;
}

size_t member_bytes_for(const gdc_params& p, int N, int M) {
  return p.precision == GDC_FP32 ? make_layout<float>(p, N, M).total
                                 : make_layout<double>(p, N, M).total;
}

std::string cuda_msg(const char* what, cudaError_t e) {
  return std::string(what) + ": " + cudaGetErrorString(e);
}

// Host staging for uploads and read-backs: page-locked memory (copies run
// at the host link's full rate and asynchronously), grown on demand; plain
// host memory if page-locked memory cannot be had.
struct PinnedStage {
  char* p = nullptr;
  size_t cap = 0;
  bool pinned = false;
  std::vector<char> fallback;
  char* get(size_t n) {
    if (n <= cap) return p;
    if (pinned && p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    pinned = false;
    const size_t want = std::max(n, (size_t)1 << 20);
    if (cudaMallocHost((void**)&p, want) == cudaSuccess) {
      pinned = true;
      cap = want;
      return p;
    }
    cudaGetLastError();
    fallback.resize(n);
    p = fallback.data();
    cap = n;
    return p;
  }
  ~PinnedStage() {
    if (pinned && p) cudaFreeHost(p);
  }
};

// Host threads for the padded copies between the staging buffers and the
// caller's arrays (one core copies at a fraction of the host's memory
// bandwidth; a read-back of a 720x361 member is 6 MB).  One process-wide
// pool, started on first use; one parallel_for at a time, the caller taking
// items too.
class HostPool {
 public:
  static HostPool& get() {
    static HostPool pool;
    return pool;
  }
  // f(i) for i in [0, n); returns when every call has returned.
  void parallel_for(int n, const std::function<void(int)>& f) {
    if (n <= 0) return;
    if (workers_.empty() || n == 1) {
      for (int i = 0; i < n; ++i) f(i);
      return;
    }
    std::lock_guard<std::mutex> one(call_);
    std::unique_lock<std::mutex> g(m_);
    f_ = &f;
    n_ = n;
    next_ = 0;
    left_ = n;
    cv_.notify_all();
    while (next_ < n_) {
      const int i = next_++;
      g.unlock();
      f(i);
      g.lock();
      --left_;
    }
    done_.wait(g, [&] { return left_ == 0; });
    f_ = nullptr;
    n_ = next_ = 0;
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

 private:
  HostPool() {
    const unsigned hw = std::thread::hardware_concurrency();
    const int n = (int)std::min(hw > 1 ? hw - 1 : 0u, 7u);
    for (int k = 0; k < n; ++k) workers_.emplace_back([this] { loop(); });
  }
  void loop() {
    std::unique_lock<std::mutex> g(m_);
    for (;;) {
      cv_.wait(g, [&] { return stop_ || next_ < n_; });
      if (stop_) return;
      const int i = next_++;
      const std::function<void(int)>* f = f_;
      g.unlock();
      (*f)(i);
      g.lock();
      if (--left_ == 0) done_.notify_all();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex call_, m_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* f_ = nullptr;
  int n_ = 0, next_ = 0, left_ = 0;
  bool stop_ = false;
};

// Member state lives in the device's stream-ordered memory pool: a member's
// memory is taken and given back in its batch's stream (no device-wide
// synchronisation, as cudaFree makes), and freed memory stays reserved in
// the pool for the next admission instead of going back to the driver.
// The pool's reserve that is not in use counts as free device memory.
cudaMemPool_t member_pool(int device) {
  static std::mutex m;
  static std::vector<cudaMemPool_t> pools;
  if (device < 0) return nullptr;
  std::lock_guard<std::mutex> g(m);
  if ((int)pools.size() <= device) pools.resize(device + 1, nullptr);
  if (!pools[device]) {
    cudaMemPool_t p = nullptr;
    if (cudaDeviceGetDefaultMemPool(&p, device) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[device] = p;
  }
  return pools[device];
}

// Free device memory for admission: the driver's free memory plus the
// member pool's reserve not in use.
size_t free_device_memory(int device) {
  size_t f = 0, t = 0;
  cudaMemGetInfo(&f, &t);
  if (cudaMemPool_t p = member_pool(device)) {
    uint64_t reserved = 0, used = 0;
    if (cudaMemPoolGetAttribute(p, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
        cudaMemPoolGetAttribute(p, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
      f += (size_t)(reserved - used);
  }
  cudaGetLastError();
  return f;
}

struct MemberRec {
  bool used = false, active = false, finished = false, nan = false;
  int N = 0, M = 0;
  double dt = 0;
  long long nsteps = 0, steps_done = 0, nan_step = -1;
  int level = SL_L1;  // slot holding this member's state(old)
  void* dmem = nullptr;
  size_t bytes = 0;
  std::vector<int> rowinfo;
  std::vector<double> ic_u, ic_v;  // padded-layout u, v of the initial condition
  int ic_ld = 0;
  int cutoff[20] = {};             // this member's filter cutoffs
};

// Checkpoint file (little-endian): this header, then the reference's restart
// fields u (N x M), v (N x (M-1)), gd, ghs in FP64 (interior, lon fastest,
// src/restart_mod.F90:63-74), then the member's exact device state in the
// compute type: gd, iap u, iap v of its current time level, their FP32
// compensation words (FP32 only), ghs, and the level's given u, v when the
// level has them.
struct RestartHeader {
  char magic[8];  // "GDCRST01"
  int32_t version, precision, num_lon, num_lat;
  int64_t steps_done, nsteps;
  double dt;
  int32_t cutoff[20];
  int32_t has_given, reserved;
};
constexpr char kRestartMagic[8] = {'G', 'D', 'C', 'R', 'S', 'T', '0', '1'};

}  // namespace

// Interface shared by the FP64 and FP32 engines.
struct BatchIface {
  virtual ~BatchIface() = default;
  virtual int add(int N, int M, double dt, long long nsteps, const int* cutoff, const double* u,
                  const double* v, const double* gd, const double* ghs, int ld, size_t reserve,
                  int* id) = 0;
  virtual int add_ic(int N, int M, double dt, long long nsteps, const int* cutoff, const gdc_ic_spec& spec,
                     size_t reserve, int* id) = 0;
  virtual int remove(int id) = 0;
  virtual int step(int n) = 0;
  virtual int sync() = 0;
  virtual int member_info(int id, long long* steps, int* fin, long long* nan) = 0;
  virtual int get_state(int id, double* u, double* v, double* gd, double* iu, double* iv,
                        double* ig, int ld) = 0;
  virtual int diag(int id, double* m, double* e, double* b) = 0;
  virtual int active(int* n) = 0;
  virtual int set_tile(int r, int c) = 0;
  virtual int set_schedule(int split_rows, int fuse_final, int pair_rows) = 0;
  virtual int get_schedule(int* r, int* c, int* split, int* fuse, int* pair) = 0;
  virtual int autotune(int* r, int* c, double* ms) = 0;
  virtual int profile(int n, double* ms, long long* launches) = 0;
  virtual int set_stream(void* s) = 0;
  virtual int debug_tendency(int id, int pass, double* du, double* dv, double* dgd, int ld) = 0;
  virtual int checkpoint(int id, const char* path) = 0;
  virtual int history(int id, double* ua, double* va, double* gh, double* div, double* vor, int ld) = 0;
  virtual int restore(const char* path, size_t reserve, long long nsteps_override, int* id) = 0;
  std::string err;
};

template <typename T>
class Batch final : public BatchIface {
 public:
  explicit Batch(const gdc_params& p) : P(p) {}
  ~Batch() override { release(); }

  int init() {
    cudaError_t e = cudaSetDevice(P.device);
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("cudaSetDevice", e));
    e = cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("cudaStreamCreate", e));
    stream = own_stream;
    if (int rc = dalloc((void**)&d_mem, sizeof(MemberDev<T>) * kSlots)) return rc;
    if (int rc = dalloc((void**)&d_active, sizeof(int) * kSlots)) return rc;
    if (int rc = dalloc((void**)&d_uvslot, sizeof(int) * kSlots)) return rc;
    cudaMemset(d_uvslot, 0xff, sizeof(int) * kSlots);  // -1: no given u, v
    if (int rc = dalloc((void**)&d_beta, sizeof(double) * kSlots)) return rc;
    if (int rc = dalloc((void**)&d_diag, sizeof(double) * 3 * kSlots)) return rc;
    if (int rc = dalloc((void**)&d_steps, sizeof(long long) * kSlots)) return rc;
    if (int rc = dalloc((void**)&d_nan, sizeof(long long) * kSlots)) return rc;
    cudaMemset(d_beta, 0, sizeof(double) * kSlots);
    cudaMemset(d_diag, 0, sizeof(double) * 3 * kSlots);
    cudaMemset(d_steps, 0, sizeof(long long) * kSlots);
    cudaMemset(d_nan, 0xff, sizeof(long long) * kSlots);  // -1
    recs.resize(kSlots);
    hdesc.resize(kSlots);
    std::memset(hdesc.data(), 0, sizeof(MemberDev<T>) * kSlots);
    set_tile(0, 0);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, P.device);
    // Whether kernels may read pageable host memory through the host's page
    // tables (a coherent CPU-GPU link, as on Grace): admission then reads
    // the caller's arrays in place instead of staging them.
    int pma = 0, pma_host = 0;
    cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, P.device);
    cudaDeviceGetAttribute(&pma_host, cudaDevAttrPageableMemoryAccessUsesHostPageTables, P.device);
    host_direct = pma == 1 && pma_host == 1;
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("init", e));
    return GDC_OK;
  }

  // ------------------------------------------------------------ members
  // Admission shared by the host and the device initial conditions: checks,
  // a member slot, device memory (`extra` bytes more must stay free for the
  // caller's temporaries), the member's tables and its descriptor, all in
  // device memory; the state fields are left zero.
  int admit(int N, int M, double dt, long long nsteps, const int* cutoff, size_t reserve, size_t extra,
            int* out_slot) {
    if (N < 8 || M < 5 || !(dt > 0) || nsteps < 0)
      return fail(GDC_E_CONFIG, "add: invalid grid, time step or length");
    if (N % 4 != 0)
      return fail(GDC_E_CONFIG, "add: num_lon must be a multiple of 4 (tile rows are copied 16 bytes at a time)");
    gdc_params mp = P;  // this member's filter rows
    if (cutoff)
      for (int k = 0; k < 20; ++k) mp.zonal_tend_filter_cutoff_wavenumber[k] = cutoff[k];
    for (int k = 0; k < 20; ++k) {
      const int c = mp.zonal_tend_filter_cutoff_wavenumber[k];
      // the reference's factor rows hold 2 (c + 1) <= num_lon entries
      // (src/filter_mod.F90:79-96 writes past the row beyond that)
      if (c < 0 || 2 * (c + 1) > N)
        return fail(GDC_E_CONFIG, "zonal_tend_filter_cutoff_wavenumber out of range for this grid "
                                  "(0 <= c <= num_lon / 2 - 1)");
    }
    int slot = -1;
    for (int s = 0; s < kSlots; ++s)
      if (!recs[s].used) {
        slot = s;
        break;
      }
    if (slot < 0) return fail(GDC_E_OOM, "add: member table full");
    const Layout L = make_layout<T>(mp, N, M);
    const size_t free_b = free_device_memory(P.device);
    if (free_b < L.total + reserve + extra) return fail(GDC_E_OOM, "add: not enough free device memory");
    MemberRec& r = recs[slot];
    r = MemberRec();
    cudaError_t e = member_pool(P.device) ? cudaMallocAsync(&r.dmem, L.total, stream) : cudaMalloc(&r.dmem, L.total);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(GDC_E_OOM, cuda_msg("add: cudaMalloc", e));
    }
    r.used = true;
    r.level = old_;
    r.N = N;
    r.M = M;
    r.dt = dt;
    r.nsteps = nsteps;
    r.bytes = L.total;
    for (int k = 0; k < 20; ++k) r.cutoff[k] = mp.zonal_tend_filter_cutoff_wavenumber[k];
    // Host tables.
    const Mesh mesh = make_mesh(N, M);
    const Coef co = make_coef(mesh);
    const int Mh = M - 1;
    std::vector<T> coef(coef_words(M), T(0));
    for (int j = 0; j < M; ++j) {
      coef[cf_off(CF_COS, M) + j] = T(co.full_cos[j]);
      coef[cf_off(CF_F, M) + j] = T(co.full_f[j]);
      coef[cf_off(CF_C, M) + j] = T(co.full_c[j]);
      coef[cf_off(CF_RADVLON, M) + j] = T(0.25 / co.full_dlon[j]);
      coef[cf_off(CF_RADVLAT, M) + j] = T(0.25 / co.full_dlat[j]);
      coef[cf_off(CF_DLON, M) + j] = T(co.full_dlon[j]);
      coef[cf_off(CF_DLAT, M) + j] = T(co.full_dlat[j]);
      if (j >= 1 && j <= M - 2) {
        coef[cf_off(CF_C1, M) + j] = T(co.half_cos[j - 1] / co.full_cos[j]);
        coef[cf_off(CF_C2, M) + j] = T(co.half_cos[j] / co.full_cos[j]);
      }
      coef[cf_off(CF_MASSW, M) + j] = T(co.full_cos[j] * mesh.dlon * mesh.dlat);
    }
    for (int j = 0; j < Mh; ++j) {
      coef[ch_off(CH_COS, M) + j + 1] = T(co.half_cos[j]);
      coef[ch_off(CH_RADVLON, M) + j + 1] = T(0.25 / co.half_dlon[j]);
      coef[ch_off(CH_RADVLAT, M) + j + 1] = T(0.25 / co.half_dlat[j]);
      coef[ch_off(CH_DLON, M) + j + 1] = T(co.half_dlon[j]);
      coef[ch_off(CH_DLAT, M) + j + 1] = T(co.half_dlat[j]);
    }
    const std::vector<T> rowc = row_records(coef, M);
    std::vector<T> twid(2 * (size_t)N);
    for (int k = 0; k < N; ++k) {
      twid[k] = T(std::cos(2.0 * kPi * k / N));
      twid[N + k] = T(std::sin(2.0 * kPi * k / N));
    }
    std::vector<int> ff, kf, fh, kh;
    make_filter_rows(mesh, mp, ff, kf, fh, kh);
    r.rowinfo.assign(M, 0);
    for (int j = 0; j < M; ++j) {
      int bits = 0;
      if (ff[j]) bits |= RI_FLAG_FULL;
      if (j < Mh && fh[j]) bits |= RI_FLAG_HALF;
      if (j == 0 || j == M - 1 || bits) bits |= RI_SPECIAL;
      r.rowinfo[j] = bits | (kf[j] << 8) | ((j < Mh ? kh[j] : 0) << 20);
    }
    std::vector<double> dco(3 * (size_t)M, 0.0);
    for (int j = 0; j < M; ++j) {
      dco[j] = co.full_cos[j] * mesh.dlon * mesh.dlat;
      dco[M + j] = co.full_cos[j];
    }
    for (int j = 0; j < Mh; ++j) dco[2 * M + j] = co.half_cos[j];
    // Descriptor.
    MemberDev<T>& d = hdesc[slot];
    std::memset(&d, 0, sizeof(d));
    char* base = (char*)r.dmem;
    d.N = N;
    d.M = M;
    d.Mh = Mh;
    d.dt = dt;
    d.pcdt[kAllPass] = dt;                   // integrator(time_step_size, ...)
    d.pcdt[kFastPass] = dt / P.subcycles;    // fast_dt = time_step_size / subcycles
    d.pcdt[kSlowPass] = 0.5 * dt;            // integrator(0.5 * time_step_size, ...)
    for (int s = 0; s < SL_N; ++s)
      for (int f = 0; f < 3; ++f) {
        d.st[s][f] = L.st[s][f] == (size_t)-1 ? nullptr : (T*)(base + L.st[s][f]);
        d.lo[s][f] = L.lo[s][f] == (size_t)-1 ? nullptr : (T*)(base + L.lo[s][f]);
      }
    for (int t = 0; t < TS_N; ++t)
      for (int f = 0; f < 3; ++f) d.td[t][f] = L.td[t][f] == (size_t)-1 ? nullptr : (T*)(base + L.td[t][f]);
    d.ghs = (T*)(base + L.ghs);
    d.coef = (const T*)(base + L.coef);
    d.rowc = (const T*)(base + L.rowc);
    d.twid = (const T*)(base + L.twid);
    d.rowinfo = (const int*)(base + L.rowinfo);
    d.dcoef = (const double*)(base + L.dcoef);
    d.given_u = (T*)(base + L.given_u);
    d.given_v = (T*)(base + L.given_v);
    for (int k = 0; k < 2; ++k) d.wadv[k] = L.wadv[k] == (size_t)-1 ? nullptr : (T*)(base + L.wadv[k]);
    // Upload, on the stream from page-locked staging: the zeroed member, its
    // tables (contiguous in the layout: one image, one copy), the descriptor
    // and its step words.  The caller synchronises before it returns.
    sync_stream();  // the staging areas may still feed an earlier copy
    const size_t img = L.given_u - L.coef;
    const size_t dsz = (sizeof(d) + 15) & ~size_t(15);
    char* st = stage_tab.get(img + dsz + 2 * sizeof(long long));
    std::memset(st, 0, img);
    std::memcpy(st + (L.coef - L.coef), coef.data(), coef.size() * sizeof(T));
    std::memcpy(st + (L.rowc - L.coef), rowc.data(), rowc.size() * sizeof(T));
    std::memcpy(st + (L.twid - L.coef), twid.data(), twid.size() * sizeof(T));
    std::memcpy(st + (L.rowinfo - L.coef), r.rowinfo.data(), M * sizeof(int));
    std::memcpy(st + (L.dcoef - L.coef), dco.data(), dco.size() * sizeof(double));
    std::memcpy(st + img, &d, sizeof(d));
    long long* words = reinterpret_cast<long long*>(st + img + dsz);
    words[0] = -1;  // nan step
    words[1] = 0;   // steps done
    e = cudaMemsetAsync(r.dmem, 0, L.total, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + L.coef, st, img, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_mem + slot, st + img, sizeof(d), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_nan + slot, words, sizeof(long long), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_steps + slot, words + 1, sizeof(long long), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) {
      sync_stream();
      release(slot);
      return fail(GDC_E_CUDA, cuda_msg("add: upload", e));
    }
    *out_slot = slot;
    return GDC_OK;
  }

  // A slot that admit() gave out and whose state could not be written.
  void member_free(void* p) {
    if (!p) return;
    if (member_pool(P.device))
      cudaFreeAsync(p, stream);
    else
      cudaFree(p);
  }

  void release(int slot) {
    member_free(recs[slot].dmem);
    recs[slot] = MemberRec();
  }

  // Admission's end: the member joins the work lists and gets the
  // diagnostics of its initial state (diag_run, src/dycore_mod.F90:125).
  int finish(int slot, int* id) {
    MemberRec& r = recs[slot];
    r.active = r.nsteps > 0;
    r.finished = r.nsteps == 0;
    dirty = true;
    if (int rc = initial_diag(slot)) return rc;
    *id = slot;
    return GDC_OK;
  }

  int add(int N, int M, double dt, long long nsteps, const int* cutoff, const double* u,
          const double* v, const double* gd, const double* ghs, int ld, size_t reserve,
          int* id) override {
    if (ld < N + 4 || !u || !v || !gd || !ghs || N < 8 || M < 5)
      return fail(GDC_E_CONFIG, "add: invalid grid, leading dimension or buffers");
    // Pole-row u must vanish: u(:,1) and u(:,num_lat) are never updated by
    // the reference (update_state writes rows 2..num_lat-1 only), and every
    // reference initial condition sets them to zero.
    for (int jp : {0, M - 1})
      for (int i = 0; i < N; ++i)
        if (u[(size_t)(jp + 2) * ld + i + 2] != 0.0)
          return fail(GDC_E_CONFIG, "pole-row u must be zero in the initial condition");
    int slot = -1;
    if (int rc = admit(N, M, dt, nsteps, cutoff, reserve, 0, &slot)) return rc;
    MemberRec& r = recs[slot];
    const MemberDev<T>& d = hdesc[slot];
    const int Mh = M - 1;
    // The initial condition goes up as it is (FP64, compact rows: u, v, gd,
    // ghs); its iap_transform (src/types_mod.F90:399-426) runs on the device
    // in FP64 with the reference's operations and rounding (ic_iap_kernel),
    // and its own u, v become the level's given u, v: the first stage reads
    // them as given (state(1)%u, %v in the reference), not re-derived.
    const size_t full = (size_t)M * N, half = (size_t)Mh * N, words = 3 * full + half;
    r.ic_ld = ld;
    if (sizeof(T) == 8) {  // FP64 read-back of the initial level returns these as given
      r.ic_u.assign(u, u + (size_t)ld * (M + 4));
      r.ic_v.assign(v, v + (size_t)ld * (Mh + 4));
    }
    cudaError_t e = cudaSuccess;
    const int lvl = old_;
    if (host_direct) {
      // The device reads the caller's padded arrays in place (their
      // interior, rows ld apart) over the coherent host link.
      const size_t o = (size_t)2 * ld + 2;
      if (launch_ic_iap<T>(d_mem, slot, lvl, N, M, u + o, v + o, gd + o, ghs + o, ld, stream) != GDC_OK)
        e = cudaGetLastError();
    } else {
      double* hu = reinterpret_cast<double*>(stage_ic.get(words * sizeof(double)));
      double* hv = hu + full;
      double* hg = hv + half;
      double* hh = hg + full;
      for (int j = 0; j < M; ++j) {
        const size_t src = (size_t)(j + 2) * ld + 2, dst = (size_t)j * N;
        std::memcpy(hu + dst, u + src, N * sizeof(double));
        std::memcpy(hg + dst, gd + src, N * sizeof(double));
        std::memcpy(hh + dst, ghs + src, N * sizeof(double));
        if (j < Mh) std::memcpy(hv + dst, v + src, N * sizeof(double));
      }
      e = ensure_tmp(words);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_ictmp, hu, words * sizeof(double), cudaMemcpyHostToDevice, stream);
      if (e == cudaSuccess) {
        double* du = d_ictmp;
        double* dv = du + full;
        double* dg = dv + half;
        if (launch_ic_iap<T>(d_mem, slot, lvl, N, M, du, dv, dg, dg + full, N, stream) != GDC_OK)
          e = cudaGetLastError();
      }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_uvslot + slot, &lvl, sizeof(int), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(stream);
      release(slot);
      return fail(GDC_E_CUDA, cuda_msg("add: upload", e));
    }
    // The initial diagnostics follow in the same stream and end with its
    // synchronisation: the caller's arrays (read in place) and the staging
    // areas are free when this returns.
    if (int rc = finish(slot, id)) {
      cudaStreamSynchronize(stream);
      release(slot);
      return rc;
    }
    return GDC_OK;
  }

  // A member whose initial condition is generated in device memory
  // (gdc_batch_add_ic): the host sends only the mesh coordinates and, for
  // the seeded state, its random draws; the fields, their IAP transform and
  // the given u, v are computed on the device.
  int add_ic(int N, int M, double dt, long long nsteps, const int* cutoff, const gdc_ic_spec& spec,
             size_t reserve, int* id) override {
    if (spec.kind < GDC_IC_ROSSBY_HAURWITZ || spec.kind > GDC_IC_SHALLOW_WATER_WAVES)
      return fail(GDC_E_CONFIG, "add_ic: unknown initial condition kind");
    if (spec.kind == GDC_IC_SEEDED &&
        (spec.lmax < 0 || spec.lmax > 64 || spec.n_mountains < 0 || spec.n_mountains > 4096))
      return fail(GDC_E_CONFIG, "add_ic: lmax must be in 0..64 and n_mountains in 0..4096");
    if (!(spec.noise_sigma >= 0)) return fail(GDC_E_CONFIG, "add_ic: noise_sigma must be >= 0");
    if (N < 8 || M < 5) return fail(GDC_E_CONFIG, "add_ic: invalid grid");
    const Mesh mesh = make_mesh(N, M);
    const int Mh = M - 1;
    std::vector<double> tables;
    auto append = [&](const std::vector<double>& x, size_t n) { tables.insert(tables.end(), x.begin(), x.begin() + n); };
    append(mesh.full_lat, M);
    append(mesh.half_lat, Mh);
    append(mesh.full_lon, N);
    append(mesh.half_lon, N);
    append(mesh.full_cos, M);
    append(mesh.half_cos, Mh);
    append(mesh.full_sin, M);
    append(mesh.half_sin, Mh);
    if (spec.kind == GDC_IC_ROSSBY_HAURWITZ || spec.kind == GDC_IC_SHALLOW_WATER_WAVES) {
      std::vector<double> t;
      if (spec.kind == GDC_IC_ROSSBY_HAURWITZ)
        rh_tables(mesh, t);
      else
        sw_waves_tables(mesh, t);
      append(t, t.size());
    }
    if (spec.kind == GDC_IC_SEEDED) {
      std::vector<double> clat, clon, ag, bg, ap, bp;
      seeded_draws(spec.seed, spec.lmax, spec.n_mountains, clat, clon, ag, bg, ap, bp);
      for (const auto* x : {&clat, &clon, &ag, &bg, &ap, &bp}) append(*x, x->size());
    }
    const size_t n = (size_t)M * N;
    // u, v, gd, ghs, the generator's scratch, the tables.
    const size_t tmp_words = 4 * n + 2 * n + 2 + tables.size();
    int slot = -1;
    if (int rc = admit(N, M, dt, nsteps, cutoff, reserve, tmp_words * sizeof(double), &slot)) return rc;
    double* tmp = nullptr;
    cudaError_t e = member_pool(P.device) ? cudaMallocAsync((void**)&tmp, tmp_words * sizeof(double), stream)
                                          : cudaMalloc(&tmp, tmp_words * sizeof(double));
    if (e != cudaSuccess) {
      cudaGetLastError();
      release(slot);
      return fail(GDC_E_OOM, cuda_msg("add_ic: cudaMalloc", e));
    }
    double *du = tmp, *dv = du + n, *dg = dv + n, *dh = dg + n, *scratch = dh + n, *dt_tab = scratch + 2 * n + 2;
    const int lvl = old_;
    e = cudaMemcpyAsync(dt_tab, tables.data(), tables.size() * sizeof(double), cudaMemcpyHostToDevice, stream);
    int rc = e == cudaSuccess ? ic_generate(spec, N, M, dt_tab, scratch, du, dv, dg, dh, stream) : GDC_E_CUDA;
    if (rc == GDC_OK) rc = launch_ic_iap<T>(d_mem, slot, lvl, N, M, du, dv, dg, dh, N, stream);
    if (rc == GDC_OK)
      rc = cudaMemcpyAsync(d_uvslot + slot, &lvl, sizeof(int), cudaMemcpyHostToDevice, stream) == cudaSuccess
               ? GDC_OK
               : GDC_E_CUDA;
    member_free(tmp);
    e = cudaStreamSynchronize(stream);
    if (rc != GDC_OK || e != cudaSuccess) {
      if (e == cudaSuccess) e = cudaGetLastError();
      release(slot);
      return fail(GDC_E_CUDA, cuda_msg("add_ic: generate", e));
    }
    return finish(slot, id);
  }

  int checkpoint(int id, const char* path) override {
    if (!valid(id)) return fail(GDC_E_CONFIG, "checkpoint: unknown member");
    if (!path) return fail(GDC_E_CONFIG, "checkpoint: no path");
    const MemberRec& r = recs[id];
    const int N = r.N, M = r.M, Mh = M - 1, ld = N + 4;
    const size_t full = (size_t)N * M, half = (size_t)N * Mh;
    std::vector<double> pu((size_t)ld * (M + 4)), pv((size_t)ld * (Mh + 4)), pg((size_t)ld * (M + 4));
    if (int rc = get_state(id, pu.data(), pv.data(), pg.data(), nullptr, nullptr, nullptr, ld)) return rc;
    const MemberDev<T>& d = hdesc[id];
    const int lvl = r.level;
    int uvs = -1;
    cudaError_t e = cudaMemcpy(&uvs, d_uvslot + id, sizeof(int), cudaMemcpyDeviceToHost);
    const bool given = uvs == lvl;
    std::vector<std::vector<T>> raw;
    auto take = [&](const T* src, size_t n) {
      raw.emplace_back(n);
      if (e == cudaSuccess) e = cudaMemcpy(raw.back().data(), src, n * sizeof(T), cudaMemcpyDeviceToHost);
    };
    const size_t sz[3] = {full, full, half};
    for (int f = 0; f < 3; ++f) take(d.st[lvl][f], sz[f]);
    if (d.lo[lvl][0])
      for (int f = 0; f < 3; ++f) take(d.lo[lvl][f], sz[f]);
    take(d.ghs, full);
    if (given) {
      take(d.given_u, full);
      take(d.given_v, half);
    }
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("checkpoint: download", e));
    RestartHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kRestartMagic, 8);
    h.version = 1;
    h.precision = sizeof(T) == 4 ? GDC_FP32 : GDC_FP64;
    h.num_lon = N;
    h.num_lat = M;
    h.steps_done = r.steps_done;
    h.nsteps = r.nsteps;
    h.dt = r.dt;
    for (int k = 0; k < 20; ++k) h.cutoff[k] = r.cutoff[k];
    h.has_given = given ? 1 : 0;
    std::vector<double> ref;
    ref.reserve(3 * full + half);
    auto interior = [&](const std::vector<double>& a, int rows) {
      for (int j = 0; j < rows; ++j)
        for (int i = 0; i < N; ++i) ref.push_back(a[(size_t)(j + 2) * ld + i + 2]);
    };
    interior(pu, M);
    interior(pv, Mh);
    interior(pg, M);
    for (size_t q = 0; q < full; ++q) ref.push_back((double)raw[h.precision == GDC_FP32 ? 6 : 3][q]);
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(GDC_E_CONFIG, std::string("checkpoint: cannot open ") + path);
    bool ok = std::fwrite(&h, sizeof(h), 1, fp) == 1 && std::fwrite(ref.data(), sizeof(double), ref.size(), fp) == ref.size();
    for (auto& a : raw) ok = ok && std::fwrite(a.data(), sizeof(T), a.size(), fp) == a.size();
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? GDC_OK : fail(GDC_E_CONFIG, std::string("checkpoint: write failed: ") + path);
  }

  int history(int id, double* ua, double* va, double* gh, double* div, double* vor, int ld) override {
    if (!valid(id)) return fail(GDC_E_CONFIG, "history: unknown member");
    const MemberRec& r = recs[id];
    const int N = r.N, M = r.M, Mh = M - 1;
    if (ld < N + 4) return fail(GDC_E_CONFIG, "history: ld < num_lon + 4");
    sync_stream();
    const int lvl = level_of(id);
    int uvs = -1;
    cudaError_t e = cudaMemcpy(&uvs, d_uvslot + id, sizeof(int), cudaMemcpyDeviceToHost);
    const size_t full = (size_t)N * M;
    double* buf = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&buf, 5 * full * sizeof(double));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(GDC_E_OOM, cuda_msg("history: buffers", e));
    }
    int rc = launch_history<T>(d_mem, id, lvl, uvs == lvl ? 1 : 0, M, buf, buf + full, buf + 2 * full,
                               buf + 3 * full, buf + 4 * full, stream);
    std::vector<double> h(5 * full);
    if (rc == GDC_OK) e = cudaMemcpyAsync(h.data(), buf, h.size() * sizeof(double), cudaMemcpyDeviceToHost, stream);
    if (rc == GDC_OK && e == cudaSuccess) e = cudaStreamSynchronize(stream);
    cudaFree(buf);
    if (rc) return fail(rc, "history: launch failed");
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("history", e));
    auto put = [&](double* f, int k, int rows) {
      if (!f) return;
      std::memset(f, 0, sizeof(double) * (size_t)ld * (rows + 4));
      for (int j = 0; j < rows; ++j)
        for (int i = 0; i < N; ++i) f[(size_t)(j + 2) * ld + i + 2] = h[k * full + (size_t)j * N + i];
      for (int j = 0; j < rows + 4; ++j) {  // periodic longitude halo
        double* row = f + (size_t)j * ld;
        row[0] = row[N];
        row[1] = row[N + 1];
        row[N + 2] = row[2];
        row[N + 3] = row[3];
      }
    };
    put(ua, 0, M);
    put(va, 1, M);
    put(gh, 2, M);
    put(div, 3, M);
    put(vor, 4, Mh);
    return GDC_OK;
  }

  // Restores a checkpoint as a new member (nsteps_override >= 0 replaces the
  // member's length): exact continuation of the checkpointed run.
  int restore(const char* path, size_t reserve, long long nsteps_override, int* id) override {
    if (!path || !id) return fail(GDC_E_CONFIG, "restore: no path or id");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(GDC_E_CONFIG, std::string("restore: cannot open ") + path);
    RestartHeader h;
    auto bad = [&](const std::string& m) {
      std::fclose(fp);
      return fail(GDC_E_CONFIG, "restore: " + m);
    };
    if (std::fread(&h, sizeof(h), 1, fp) != 1 || std::memcmp(h.magic, kRestartMagic, 8) != 0 || h.version != 1)
      return bad("not a checkpoint file");
    if (h.precision != (sizeof(T) == 4 ? GDC_FP32 : GDC_FP64))
      return bad("checkpoint precision differs from the batch's");
    const int N = h.num_lon, M = h.num_lat;
    if (N < 8 || M < 5 || N % 4 != 0 || N > (1 << 16) || M > (1 << 16) || h.steps_done < 0)
      return bad("invalid grid in header");
    const int Mh = M - 1, ld = N + 4;
    const size_t full = (size_t)N * M, half = (size_t)N * Mh;
    std::vector<double> ref(3 * full + half);
    if (std::fread(ref.data(), sizeof(double), ref.size(), fp) != ref.size()) return bad("truncated file");
    const bool fp32 = sizeof(T) == 4;
    const size_t sz[3] = {full, full, half};
    std::vector<std::vector<T>> raw;
    auto take = [&](size_t n) {
      raw.emplace_back(n);
      return std::fread(raw.back().data(), sizeof(T), n, fp) == n;
    };
    bool ok = true;
    for (int f = 0; f < 3; ++f) ok = ok && take(sz[f]);
    if (fp32)
      for (int f = 0; f < 3; ++f) ok = ok && take(sz[f]);
    ok = ok && take(full);
    if (h.has_given) ok = ok && take(full) && take(half);
    if (!ok) return bad("truncated file");
    std::fclose(fp);
    // Admit with the reference fields, then put the exact state in place.
    std::vector<double> pu((size_t)ld * (M + 4), 0.0), pv((size_t)ld * (Mh + 4), 0.0), pg(pu.size(), 0.0),
        ph(pu.size(), 0.0);
    const double* src = ref.data();
    auto pad = [&](std::vector<double>& a, int rows) {
      for (int j = 0; j < rows; ++j)
        for (int i = 0; i < N; ++i) a[(size_t)(j + 2) * ld + i + 2] = *src++;
    };
    pad(pu, M);
    pad(pv, Mh);
    pad(pg, M);
    pad(ph, M);
    const long long nsteps = nsteps_override >= 0 ? nsteps_override : h.nsteps;
    if (int rc = add(N, M, h.dt, nsteps, h.cutoff, pu.data(), pv.data(), pg.data(), ph.data(), ld, reserve, id))
      return rc;
    MemberRec& r = recs[*id];
    const MemberDev<T>& d = hdesc[*id];
    const int lvl = r.level;
    cudaError_t e = cudaSuccess;
    auto put = [&](T* dst, const std::vector<T>& a) {
      if (e == cudaSuccess) e = cudaMemcpy(dst, a.data(), a.size() * sizeof(T), cudaMemcpyHostToDevice);
    };
    int q = 0;
    for (int f = 0; f < 3; ++f) put(d.st[lvl][f], raw[q++]);
    if (fp32)
      for (int f = 0; f < 3; ++f) put(d.lo[lvl][f], raw[q++]);
    put(d.ghs, raw[q++]);
    int uvs = -1;
    if (h.has_given) {
      put(d.given_u, raw[q++]);
      put(d.given_v, raw[q++]);
      uvs = lvl;
    }
    if (e == cudaSuccess) e = cudaMemcpy(d_uvslot + *id, &uvs, sizeof(int), cudaMemcpyHostToDevice);
    const long long done = h.steps_done;
    if (e == cudaSuccess) e = cudaMemcpy(d_steps + *id, &done, sizeof(done), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("restore: upload", e));
    r.steps_done = done;
    r.active = done < r.nsteps;
    r.finished = !r.active;
    dirty = true;
    return initial_diag(*id);  // the diagnostics of the restored state
  }

  int remove(int id) override {
    if (!valid(id)) return fail(GDC_E_CONFIG, "remove: unknown member");
    sync_stream();
    MemberRec& r = recs[id];
    member_free(r.dmem);
    r = MemberRec();
    std::memset(&hdesc[id], 0, sizeof(MemberDev<T>));
    dirty = true;
    return GDC_OK;
  }

  // --------------------------------------------------------------- steps
  int step(int n) override {
    for (int k = 0; k < n; ++k) {
      if (dirty)
        if (int rc = rebuild()) return rc;
      if (nwork == 0) return GDC_OK;
      int rc = GDC_OK;
      const int par = old_ == SL_L1 ? 0 : 1;
      if (use_graph && warm) {
        if (!gexec[par]) rc = capture(par);
        if (rc == GDC_OK && gexec[par]) {
          cudaError_t e = cudaGraphLaunch(gexec[par], stream);
          if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("cudaGraphLaunch", e));
        } else if (rc == GDC_OK) {
          rc = enqueue_step(nullptr);
        }
      } else {
        rc = enqueue_step(nullptr);
        warm = true;
      }
      if (rc) return rc;
      advance_bookkeeping();
    }
    return GDC_OK;
  }

  // time_advance (src/time_mod.F90:106-130) plus host-side step accounting
  // (deterministic, no device round trip).
  void advance_bookkeeping() {
    std::swap(old_, new_);
    bool changed = false;
    for (int s : active_slots) {
      MemberRec& r = recs[s];
      r.level = old_;
      ++r.steps_done;
      if (r.steps_done >= r.nsteps) {
        r.active = false;
        r.finished = true;
        changed = true;
      }
    }
    if (changed) dirty = true;
  }

  int sync() override {
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("sync", e));
    std::vector<long long> nan(kSlots);
    e = cudaMemcpy(nan.data(), d_nan, sizeof(long long) * kSlots, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("sync: nan flags", e));
    for (int s = 0; s < kSlots; ++s) {
      MemberRec& r = recs[s];
      if (!r.used || nan[s] < 0 || r.nan) continue;
      // A member whose mass or energy became NaN is evicted from the batch
      // (the reference stops the program, src/diag_mod.F90:79-87); the
      // others continue.
      r.nan = true;
      r.nan_step = nan[s];
      if (r.active) {
        r.active = false;
        r.finished = true;
        dirty = true;
      }
    }
    return GDC_OK;
  }

  int member_info(int id, long long* steps, int* fin, long long* nan) override {
    if (!valid(id)) return fail(GDC_E_CONFIG, "member_info: unknown member");
    const MemberRec& r = recs[id];
    if (steps) *steps = r.steps_done;
    if (fin) *fin = r.finished ? 1 : 0;
    if (nan) *nan = r.nan_step;
    return GDC_OK;
  }

  int active(int* n) override {
    int c = 0;
    for (auto& r : recs) c += (r.used && r.active) ? 1 : 0;
    *n = c;
    return GDC_OK;
  }

  int get_state(int id, double* u, double* v, double* gd, double* iu, double* iv, double* ig,
                int ld) override {
    if (!valid(id)) return fail(GDC_E_CONFIG, "get_state: unknown member");
    const MemberRec& r = recs[id];
    const int N = r.N, M = r.M, Mh = M - 1;
    if (ld < N + 4) return fail(GDC_E_CONFIG, "get_state: ld < num_lon + 4");
    sync_stream();
    // state(old) of this member: its last written level.
    const int lvl = level_of(id);
    int uvs = -1;
    cudaError_t e = cudaMemcpy(&uvs, d_uvslot + id, sizeof(int), cudaMemcpyDeviceToHost);
    const bool ic_uv = r.steps_done == 0 && std::is_same<T, double>::value && !r.ic_u.empty();
    const int uv_mode = (ic_uv || !(u || v)) ? 2 : (uvs == lvl ? 1 : 0);
    // The level in FP64 on the device (hi + lo, square roots, u and v as
    // update_state recovers them, src/dycore_mod.F90:636-645), one copy back.
    const size_t n = (size_t)M * N, nh = (size_t)Mh * N, words = 4 * n + 2 * nh;
    if (e == cudaSuccess) e = ensure_tmp(words);
    if (e == cudaSuccess && launch_state_out<T>(d_mem, id, lvl, uv_mode, N, M, d_ictmp, stream) != GDC_OK)
      e = cudaGetLastError();
    double* hbuf = reinterpret_cast<double*>(stage_ic.get(words * sizeof(double)));
    // gd, u, v first: the usual request copies only those
    const size_t back = (iu || iv || ig) ? words : 2 * n + nh;
    if (e == cudaSuccess) e = cudaMemcpyAsync(hbuf, d_ictmp, back * sizeof(double), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("get_state", e));
    const double* hg = hbuf;
    const double* ou = hg + n;
    const double* ov = ou + n;
    const double* hu = ov + nh;
    const double* hv = hu + n;
    const double* sg = hv + nh;
    // Each element of the padded array written once: zero latitude-halo
    // rows, then per interior row its values, periodic longitude halo and
    // zero padding past N + 4.
    // Bands of kBand rows of each requested field, over the host pool.
    constexpr int kBand = 16;
    struct Put {
      double* f;
      int rows;
      const double* src;
    };
    std::vector<Put> puts;
    auto want = [&](double* f, int rows, const double* src) {
      if (f) puts.push_back(Put{f, rows, src});
    };
    want(gd, M, hg);
    want(iu, M, hu);
    want(iv, Mh, hv);
    want(ig, M, sg);
    if (!ic_uv && uv_mode != 2) {
      want(u, M, ou);
      want(v, Mh, ov);
    }
    std::vector<std::pair<int, int>> bands;  // (put, first row)
    for (int k = 0; k < (int)puts.size(); ++k)
      for (int j = 0; j < puts[k].rows; j += kBand) bands.push_back({k, j});
    HostPool::get().parallel_for((int)bands.size(), [&](int b) {
      const Put& q = puts[bands[b].first];
      const int j0 = bands[b].second, j1 = std::min(q.rows, j0 + kBand);
      if (j0 == 0) std::memset(q.f, 0, sizeof(double) * (size_t)ld * 2);
      if (j1 == q.rows) std::memset(q.f + (size_t)(q.rows + 2) * ld, 0, sizeof(double) * (size_t)ld * 2);
      for (int j = j0; j < j1; ++j) {
        double* row = q.f + (size_t)(j + 2) * ld;
        const double* sr = q.src + (size_t)j * N;
        std::memcpy(row + 2, sr, N * sizeof(double));
        row[0] = sr[N - 2];
        row[1] = sr[N - 1];
        row[N + 2] = sr[0];
        row[N + 3] = sr[1];
        if (ld > N + 4) std::memset(row + N + 4, 0, sizeof(double) * (ld - N - 4));
      }
    });
    if (ic_uv) {
      // state(old) still holds the initial condition's own u and v.
      auto copy_ic = [&](double* f, const std::vector<double>& src, int rows) {
        if (!f) return;
        for (int j = 0; j < rows + 4; ++j)
          for (int i = 0; i < N + 4; ++i) f[(size_t)j * ld + i] = src[(size_t)j * r.ic_ld + i];
      };
      copy_ic(u, r.ic_u, M);
      copy_ic(v, r.ic_v, Mh);
    }
    return GDC_OK;
  }

  int diag(int id, double* m, double* e, double* b) override {
    if (!valid(id)) return fail(GDC_E_CONFIG, "diag: unknown member");
    sync_stream();
    double h[3];
    cudaError_t er = cudaMemcpy(h, d_diag + 3 * id, sizeof(h), cudaMemcpyDeviceToHost);
    if (er != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("diag", er));
    if (m) *m = h[0];
    if (e) *e = h[1];
    if (b) *b = h[2];
    return GDC_OK;
  }

  int set_tile(int r, int c) override {
    if (r == 0 && c == 0) {
      r = default_rows();
      c = default_cols();
    }
    const bool st = strip_shape_supported(r, c);
    if (weno() && (r != 8 || c != 32)) return fail(GDC_E_CONFIG, "set_tile: uv_adv_scheme weno runs on 8x32 tiles");
    if (!st && !tile_shape_supported(r, c, sizeof(T) == 8))
      return fail(GDC_E_CONFIG,
                  "set_tile: supported shapes are tiles 8x32, 8x64, 4x128, 16x64 (and 4x32 in FP64) and warp "
                  "strips 8x30, 16x30, 32x30, 64x30");
    tile_r = r;
    tile_c = c;
    strips = st;
    dirty = true;
    return GDC_OK;
  }

  int set_schedule(int split, int fuse, int pair) override {
    if (split < -1 || split > 1 || fuse < 0 || fuse > 1 || pair < -1 || pair > 1)
      return fail(GDC_E_CONFIG,
                  "set_schedule: split_rows and pair_rows must be -1, 0 or 1 and fuse_final 0 or 1");
    split_mode = split;
    fuse_final = fuse != 0;
    pair_mode = pair;
    dirty = true;
    return GDC_OK;
  }

  int set_stream(void* s) override {
    sync_stream();
    stream = s ? (cudaStream_t)s : own_stream;
    invalidate_graphs();
    return GDC_OK;
  }

  // Times each candidate launch schedule -- tile shape or warp strips, the
  // row-task split, the final update launched or fused -- on the current
  // members (CUDA graph replay, CUDA events, the median of `reps` timed
  // steps after warm steps) and keeps the fastest.  The members' states
  // and all step bookkeeping are saved first and restored afterwards, so
  // tuning advances no forecast: the members continue exactly as if it had
  // not run.
  int autotune(int* rr, int* cc, double* best_ms) override {
    if (dirty)
      if (int rc = rebuild()) return rc;
    sync_stream();
    if (active_slots.empty() || weno()) {  // nothing to time; WENO has one layout
      if (weno())
        if (int rc = set_tile(8, 32)) return rc;
      if (rr) *rr = tile_r;
      if (cc) *cc = tile_c;
      if (best_ms) *best_ms = 0.0;
      return GDC_OK;
    }
    // --- save: each active member's level (compute type, compensation
    // words), its given u, v, the per-member device words and the host
    // bookkeeping.
    struct Save {
      int slot;
      std::vector<std::pair<T*, size_t>> fields;  // device field, elements
      size_t off;                                  // into the scratch
    };
    std::vector<Save> saves;
    size_t total = 0;
    for (int sl : active_slots) {
      const MemberDev<T>& d = hdesc[sl];
      const int lvl = recs[sl].level;
      const size_t full = (size_t)recs[sl].N * recs[sl].M, half = (size_t)recs[sl].N * (recs[sl].M - 1);
      const size_t sz[3] = {full, full, half};
      Save sv{sl, {}, total};
      for (int f = 0; f < 3; ++f) {
        sv.fields.push_back({d.st[lvl][f], sz[f]});
        if (d.lo[lvl][f]) sv.fields.push_back({d.lo[lvl][f], sz[f]});
      }
      sv.fields.push_back({d.given_u, full});
      sv.fields.push_back({d.given_v, half});
      for (auto& f : sv.fields) total += f.second;
      saves.push_back(sv);
    }
    T* scratch = nullptr;
    if (cudaMalloc(&scratch, total * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return fail(GDC_E_OOM, "autotune: no device memory for the members' saved states");
    }
    cudaError_t e = cudaSuccess;
    for (auto& sv : saves) {
      size_t o = sv.off;
      for (auto& f : sv.fields) {
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(scratch + o, f.first, f.second * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        o += f.second;
      }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    std::vector<int> h_uv(kSlots);
    std::vector<long long> h_steps(kSlots), h_nan(kSlots);
    std::vector<double> h_beta(kSlots), h_diag(3 * kSlots);
    if (e == cudaSuccess) e = cudaMemcpy(h_uv.data(), d_uvslot, sizeof(int) * kSlots, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_steps.data(), d_steps, sizeof(long long) * kSlots, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_nan.data(), d_nan, sizeof(long long) * kSlots, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_beta.data(), d_beta, sizeof(double) * kSlots, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_diag.data(), d_diag, sizeof(double) * 3 * kSlots, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      cudaFree(scratch);
      return fail(GDC_E_CUDA, cuda_msg("autotune: save", e));
    }
    const std::vector<MemberRec> saved_recs = recs;
    const int saved_old = old_, saved_new = new_;
    std::array<int, 5> pick = {tile_r, tile_c, split_mode, fuse_final ? 1 : 0, pair_mode};
    // No member may finish while the candidates are timed.
    for (int sl : active_slots) recs[sl].nsteps = recs[sl].steps_done + (1LL << 40);

    // --- time the candidates
    std::vector<std::array<int, 5>> cand;  // rows, cols, split, fuse, pair
    const int shapes[][2] = {{16, 64}, {8, 64}, {8, 32}, {4, 128}, {4, 32}, {16, 30}};
    for (auto& sh : shapes) {
      const bool st = strip_shape_supported(sh[0], sh[1]);
      if (!st && !tile_shape_supported(sh[0], sh[1], sizeof(T) == 8)) continue;
      for (int split = 0; split <= 1; ++split)
        for (int fuse = 0; fuse <= (st ? 0 : 1); ++fuse)
          for (int pair = 0; pair <= (sizeof(T) == 4 || st || fuse || weno() ? 0 : 1); ++pair)
            cand.push_back({sh[0], sh[1], split, fuse, pair});
    }
    const int reps = 3;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 1e30;
    int rc = GDC_OK;
    for (auto& c : cand) {
      rc = set_tile(c[0], c[1]);
      if (rc == GDC_OK) rc = set_schedule(c[2], c[3], c[4]);
      if (rc == GDC_OK) rc = step(2);  // build, capture both time-level parities
      std::vector<float> t;
      for (int k = 0; k < reps && rc == GDC_OK; ++k) {
        cudaEventRecord(e0, stream);
        rc = step(1);
        cudaEventRecord(e1, stream);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        t.push_back(ms);
      }
      if (rc) break;
      std::sort(t.begin(), t.end());
      if (t[reps / 2] < best) {
        best = t[reps / 2];
        pick = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);

    // --- restore
    sync_stream();
    e = cudaSuccess;
    for (auto& sv : saves) {
      size_t o = sv.off;
      const MemberDev<T>& d = hdesc[sv.slot];
      const int lvl = saved_recs[sv.slot].level;
      // the level's fields go back to the slot that held them
      std::vector<T*> dst;
      for (int f = 0; f < 3; ++f) {
        dst.push_back(d.st[lvl][f]);
        if (d.lo[lvl][f]) dst.push_back(d.lo[lvl][f]);
      }
      dst.push_back(d.given_u);
      dst.push_back(d.given_v);
      for (size_t q = 0; q < sv.fields.size(); ++q) {
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(dst[q], scratch + o, sv.fields[q].second * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        o += sv.fields[q].second;
      }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess) e = cudaMemcpy(d_uvslot, h_uv.data(), sizeof(int) * kSlots, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_steps, h_steps.data(), sizeof(long long) * kSlots, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_nan, h_nan.data(), sizeof(long long) * kSlots, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_beta, h_beta.data(), sizeof(double) * kSlots, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_diag, h_diag.data(), sizeof(double) * 3 * kSlots, cudaMemcpyHostToDevice);
    cudaFree(scratch);
    recs = saved_recs;
    old_ = saved_old;
    new_ = saved_new;
    set_tile(pick[0], pick[1]);
    set_schedule(pick[2], pick[3], pick[4]);
    invalidate_graphs();
    dirty = true;
    if (rc) return rc;
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("autotune: restore", e));
    if (rr) *rr = pick[0];
    if (cc) *cc = pick[1];
    if (best_ms) *best_ms = best;
    return GDC_OK;
  }

  int get_schedule(int* r, int* c, int* split, int* fuse, int* pair) override {
    if (dirty)
      if (int rc = rebuild()) return rc;
    if (r) *r = tile_r;
    if (c) *c = tile_c;
    if (split) *split = split_mode;
    if (fuse) *fuse = fuse_final ? 1 : 0;
    if (pair) *pair = pair_rows ? 1 : 0;
    return GDC_OK;
  }

  int profile(int n, double* ms, long long* launches) override {
    for (int k = 0; k < 5; ++k) {
      ms[k] = 0;
      launches[k] = 0;
    }
    for (int s = 0; s < n; ++s) {
      if (dirty)
        if (int rc = rebuild()) return rc;
      if (nwork == 0) break;
      prof.clear();
      if (int rc = enqueue_step(&prof)) return rc;
      cudaError_t e = cudaStreamSynchronize(stream);
      if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("profile", e));
      for (auto& p : prof) {
        float t = 0;
        cudaEventElapsedTime(&t, p.e0, p.e1);
        ms[p.kind] += t;
        launches[p.kind] += 1;
        cudaEventDestroy(p.e0);
        cudaEventDestroy(p.e1);
      }
      prof.clear();
      advance_bookkeeping();
    }
    return GDC_OK;
  }

  int debug_tendency(int id, int pass, double* du, double* dv, double* dgd, int ld) override {
    if (!valid(id)) return fail(GDC_E_CONFIG, "debug_tendency: unknown member");
    if (pass < 0 || pass > 2) return fail(GDC_E_CONFIG, "debug_tendency: pass must be 0, 1 or 2");
    const MemberRec& r = recs[id];
    const int N = r.N, M = r.M, Mh = M - 1;
    if (ld < N + 4) return fail(GDC_E_CONFIG, "debug_tendency: ld < num_lon + 4");
    if (dirty)
      if (int rc = rebuild()) return rc;
    // One member's work items only.
    std::vector<WorkItem> wl;
    for (int q = 0; q < nwork; ++q)
      if (hwl[q].member == id) wl.push_back(hwl[q]);
    if (wl.empty()) {
      // A finished member is not in the work list; build its items.
      std::vector<WorkItem> all;
      int pc = 0;
      append_items(id, all, pc);
      wl = all;
    }
    WorkItem* dwl = nullptr;
    if (cudaMalloc(&dwl, sizeof(WorkItem) * wl.size()) != cudaSuccess) {
      cudaGetLastError();
      return fail(GDC_E_OOM, "debug_tendency: cudaMalloc");
    }
    sync_stream();
    cudaMemcpy(dwl, wl.data(), sizeof(WorkItem) * wl.size(), cudaMemcpyHostToDevice);
    StageArgs a = base_args(pass);
    a.in_slot = level_of(id);
    a.tout = TS_NEW;
    a.pair = 0;  // no clusters here: part 0 of a paired row task does it whole
    int nr = 0;
    for (const auto& w : wl) nr += w.kind == 1;
    int rc = GDC_OK;
    if (weno() && pass != kFastPass) {
      // the member's WENO terms first (its own flat items)
      std::vector<FlatItem> fl;
      const size_t n[3] = {(size_t)M * N, (size_t)M * N, (size_t)Mh * N};
      for (int f = 1; f < 3; ++f)
        for (size_t b = 0; b < n[f]; b += flat_chunk<T>())
          fl.push_back(FlatItem{id, f, (int)b, (int)std::min<size_t>(flat_chunk<T>(), n[f] - b)});
      FlatItem* dfl = nullptr;
      if (cudaMalloc(&dfl, sizeof(FlatItem) * fl.size()) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(dwl);
        return fail(GDC_E_OOM, "debug_tendency: cudaMalloc");
      }
      cudaMemcpy(dfl, fl.data(), sizeof(FlatItem) * fl.size(), cudaMemcpyHostToDevice);
      rc = launch_weno<T>(d_mem, dfl, (int)fl.size(), a.in_slot, d_uvslot, stream);
      cudaStreamSynchronize(stream);
      cudaFree(dfl);
    }
    if (rc) {
    } else if (!strips)
      rc = launch_stage<T>(d_mem, dwl, (int)wl.size(), P.uv_adv_scheme, tile_r, tile_c, std::max(max_n, N), a, stream);
    else {
      rc = launch_stage<T>(d_mem, dwl, nr, P.uv_adv_scheme, 8, 32, std::max(max_n, N), a, stream);
      if (!rc) rc = launch_stage_strips<T>(d_mem, dwl + nr, (int)wl.size() - nr, P.uv_adv_scheme, a, stream);
    }
    cudaError_t e = cudaStreamSynchronize(stream);
    cudaFree(dwl);
    if (rc) return fail(rc, "debug_tendency: launch failed");
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("debug_tendency", e));
    const MemberDev<T>& d = hdesc[id];
    std::vector<double> hg, hu, hv;
    e = download_field(d.td[TS_NEW][F_GD], nullptr, (size_t)M * N, hg);
    if (e == cudaSuccess) e = download_field(d.td[TS_NEW][F_IU], nullptr, (size_t)M * N, hu);
    if (e == cudaSuccess) e = download_field(d.td[TS_NEW][F_IV], nullptr, (size_t)Mh * N, hv);
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("debug_tendency: download", e));
    auto put = [&](double* f, int rows, const std::vector<double>& src) {
      if (!f) return;
      std::memset(f, 0, sizeof(double) * (size_t)ld * (rows + 4));
      for (int j = 0; j < rows; ++j)
        for (int i = 0; i < N; ++i) f[(size_t)(j + 2) * ld + i + 2] = src[(size_t)j * N + i];
    };
    put(dgd, M, hg);
    put(du, M, hu);
    put(dv, Mh, hv);
    return GDC_OK;
  }

 private:
  struct Prof {
    int kind;
    cudaEvent_t e0, e1;
  };

  gdc_params P;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  MemberDev<T>* d_mem = nullptr;
  int* d_active = nullptr;  // slots of the active members (beta / diag blocks)
  int* d_uvslot = nullptr;  // per member: level whose u, v are held as given (-1 none)
  double* d_beta = nullptr;
  double* d_ictmp = nullptr;  // FP64 scratch: an admitted initial condition, a read-back level
  size_t ictmp_cap = 0;       // its capacity in doubles
  PinnedStage stage_ic;       // host staging of the same
  PinnedStage stage_tab;      // host staging of an admitted member's tables
  PinnedStage stage_diag;     // host staging of its initial diagnostics' items
  // the initial diagnostics' work items, partials and member slot
  FlatItem* d_idl = nullptr;
  double* d_ipart = nullptr;
  int* d_islot = nullptr;
  size_t idl_cap = 0;
  double* d_diag = nullptr;
  long long* d_steps = nullptr;
  long long* d_nan = nullptr;
  WorkItem* d_wl = nullptr;
  size_t wl_cap = 0;
  FlatItem* d_flat = nullptr;
  size_t flat_cap = 0;
  std::vector<FlatItem> hflat;
  int nflat = 0;
  FlatItem* d_dl = nullptr;      // diag items: rows of a member, one warp per row
  double* d_dpart = nullptr;     // their partial sums
  size_t dl_cap = 0;
  std::vector<FlatItem> hdl;
  int ndl = 0;
  double* d_partials = nullptr;
  size_t part_cap = 0;
  std::vector<MemberRec> recs;
  std::vector<MemberDev<T>> hdesc;
  std::vector<WorkItem> hwl;
  std::vector<int> active_slots;
  int nwork = 0, max_n = 0;
  int nrow = 0;                  // whole-row tasks at the head of the work list
  int tile_r = 8, tile_c = 32;   // tile shape, or band rows x kStripCols
  bool strips = false;           // work list of warp strips instead of tiles
  // Whole-row tasks split by field: in FP64 (a row's filters are long FP64
  // work) or when the batch has few tiles per SM (the row tasks are then the
  // critical path); otherwise one task per row stages the row once.
  bool split_rows = sizeof(T) == 8;
  int split_mode = -1;     // -1 automatic (above), 0 whole rows, 1 split by field
  // Whole-row tasks split over the two blocks of a cluster (-1 automatic:
  // FP64 launches with at most two items per SM, where the filtered rows'
  // FP64 sums are the critical path; 0 off; 1 on).  FP64 tiles only, not
  // with a fused final update.
  int pair_mode = -1;
  bool pair_rows = false;
  // predict_correct's update formed in the next one's first stage: correct
  // and tested, but measured slower (the first stage is latency-bound and
  // the update's loads land on its critical path), so off by default.
  bool fuse_final = false;
  int num_sms = 152;
  bool host_direct = false;  // kernels read pageable host memory (see init)
  // With strips, the whole-row tasks run on a second stream, concurrently
  // with the strips over the ordinary rows.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // Tile work list (8x32) for the diffusion and copy kernels when the stage
  // kernels run on strips; otherwise the main list.
  WorkItem* d_twl = nullptr;
  size_t twl_cap = 0;
  int ntwork = 0;
  int old_ = SL_L1, new_ = SL_L2;  // src/time_mod.F90:68-69
  bool dirty = true, warm = false, use_graph = true;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  std::vector<Prof> prof;
  std::vector<void*> allocs;

  // Fastest measured: 16x64 tiles, in FP32 on the 64-member ensemble and in
  // FP64 on the single 360x181 member (one tile per SM: each tile has an
  // SM's FP64 pipe to itself).
  int default_rows() const { return weno() ? 8 : 16; }
  int default_cols() const { return weno() ? 32 : 64; }
  bool weno() const { return P.uv_adv_scheme == GDC_ADV_WENO; }

  // The diffusion and copy kernels run on 8x32, 8x64 or 4x128 tiles.
  bool own_tile_list() const {
    return strips || pair_rows ||
           !((tile_r == 8 && (tile_c == 32 || tile_c == 64)) || (tile_r == 4 && tile_c == 128));
  }
  const WorkItem* tile_list() const { return own_tile_list() ? d_twl : d_wl; }

  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  bool valid(int id) const { return id >= 0 && id < kSlots && recs[id].used; }
  // The slot holding state(old) of a member (frozen once it finishes).
  int level_of(int id) const { return recs[id].level; }

  int dalloc(void** p, size_t n) {
    cudaError_t e = cudaMalloc(p, n);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(GDC_E_OOM, cuda_msg("cudaMalloc", e));
    }
    allocs.push_back(*p);
    return GDC_OK;
  }

  void sync_stream() {
    if (stream) cudaStreamSynchronize(stream);
  }

  void invalidate_graphs() {
    for (auto& g : gexec)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    warm = false;
  }

  void release() {
    if (stream) cudaStreamSynchronize(stream);
    invalidate_graphs();
    for (auto& r : recs) member_free(r.dmem);
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : allocs) cudaFree(p);
    if (d_wl) cudaFree(d_wl);
    if (d_twl) cudaFree(d_twl);
    if (d_flat) cudaFree(d_flat);
    if (d_dl) cudaFree(d_dl);
    if (d_dpart) cudaFree(d_dpart);
    if (d_partials) cudaFree(d_partials);
    if (d_ictmp) cudaFree(d_ictmp);
    if (d_idl) cudaFree(d_idl);
    if (d_ipart) cudaFree(d_ipart);
    if (d_islot) cudaFree(d_islot);
    if (own_stream) cudaStreamDestroy(own_stream);
    if (side) cudaStreamDestroy(side);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
  }

  // The FP64 scratch for admissions and read-backs, grown on demand.
  cudaError_t ensure_tmp(size_t words) {
    if (ictmp_cap >= words) return cudaSuccess;
    if (d_ictmp) cudaFree(d_ictmp);
    d_ictmp = nullptr;
    ictmp_cap = 0;
    cudaError_t e = cudaMalloc(&d_ictmp, words * sizeof(double));
    if (e == cudaSuccess)
      ictmp_cap = words;
    else
      cudaGetLastError();
    return e;
  }

  cudaError_t download_field(const T* src, const T* lo, size_t n, std::vector<double>& out) {
    std::vector<T> hi(n), lw;
    cudaError_t e = cudaMemcpy(hi.data(), src, n * sizeof(T), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && lo) {
      lw.resize(n);
      e = cudaMemcpy(lw.data(), lo, n * sizeof(T), cudaMemcpyDeviceToHost);
    }
    out.resize(n);
    for (size_t q = 0; q < n; ++q) out[q] = (double)hi[q] + (lo ? (double)lw[q] : 0.0);
    return e;
  }

  // Diag items of member s: bands of diag_rows<T>() rows.
  void append_diag_items(int s, std::vector<FlatItem>& out) {
    hdesc[s].dbase = (int)out.size();
    constexpr int R = diag_rows<T>();
    for (int j = 0; j < recs[s].M; j += R) out.push_back(FlatItem{s, 0, j, std::min(R, recs[s].M - j)});
    hdesc[s].dcount = (int)out.size() - hdesc[s].dbase;
  }

  void append_items(int s, std::vector<WorkItem>& out, int& pcount) {
    append_items_as(s, out, pcount, strips, tile_r, tile_c, true, pair_rows);
  }

  // Work items of member s: its whole-row tasks, then tiles (tr x tc) or
  // warp strips (bands of tr rows, kStripCols columns) over its runs of
  // ordinary rows.
  void append_items_as(int s, std::vector<WorkItem>& out, int& pcount, bool as_strips, int tr, int tc,
                       bool own_partials, bool pairs = false) {
    const MemberRec& r = recs[s];
    const int N = r.N, M = r.M;
    int pbase = pcount;
    // Whole-row tasks first (they are the longest items).
    for (int j = 0; j < M; ++j)
      if (r.rowinfo[j] & RI_SPECIAL) {
        // a task as two items (parts 0, 1) when split over a block pair
        const int parts = pairs ? 2 : 1;
        if (split_rows) {
          // one task per field (no iap v on the north pole row): a row's
          // filters then run on three SMs
          for (int f : {F_GD, F_IU, F_IV})
            if (f != F_IV || j < M - 1)
              for (int q = 0; q < parts; ++q) out.push_back(WorkItem{s, 1, j, q, parts, N, pcount++, f});
        } else {
          // one task for the three fields (the row is staged once)
          for (int q = 0; q < parts; ++q) out.push_back(WorkItem{s, 1, j, q, parts, N, pcount++, -1});
        }
      }
    // Bulk tiles over runs of ordinary rows.
    int j = 0;
    while (j < M) {
      if (r.rowinfo[j] & RI_SPECIAL) {
        ++j;
        continue;
      }
      int b = j;
      while (b + 1 < M && !(r.rowinfo[b + 1] & RI_SPECIAL)) ++b;
      if (as_strips) {
        for (int i0 = 0; i0 < N; i0 += kStripCols)
          for (int j0 = j; j0 <= b; j0 += tr)
            out.push_back(WorkItem{s, 2, j0, i0, std::min(tr, b - j0 + 1), std::min(kStripCols, N - i0), pcount++, 0});
      } else {
        for (int j0 = j; j0 <= b; j0 += tr) {
          const int rows = std::min(tr, b - j0 + 1);
          for (int i0 = 0; i0 < N; i0 += tc)
            out.push_back(WorkItem{s, 0, j0, i0, rows, std::min(tc, N - i0), pcount++, 0});
        }
      }
      j = b + 1;
    }
    if (own_partials) {  // the stage list's partial slots of this member
      hdesc[s].pbase = pbase;
      hdesc[s].pcount = pcount - pbase;
    }
  }

  int rebuild() {
    sync_stream();
    invalidate_graphs();
    active_slots.clear();
    std::vector<WorkItem> rows_first, tiles;
    int pc = 0;
    max_n = 8;
    {
      long long ntiles = 0;  // bulk items of the layout, to pick the row-task form
      for (int s = 0; s < kSlots; ++s) {
        if (!recs[s].used || !recs[s].active) continue;
        const long long cols = strips ? (recs[s].N + kStripCols - 1) / kStripCols : (recs[s].N + tile_c - 1) / tile_c;
        ntiles += cols * ((recs[s].M + tile_r - 1) / tile_r);
      }
      split_rows = split_mode >= 0 ? split_mode == 1 : (sizeof(T) == 8 || ntiles < 8LL * num_sms);
      long long nrows = 0;  // whole-row tasks
      for (int s = 0; s < kSlots; ++s) {
        if (!recs[s].used || !recs[s].active) continue;
        for (int j = 0; j < recs[s].M; ++j) nrows += (recs[s].rowinfo[j] & RI_SPECIAL) ? (split_rows ? 3 : 1) : 0;
      }
      const bool can_pair = sizeof(T) == 8 && !strips && !weno() && !fuse_final;
      pair_rows = can_pair && (pair_mode >= 0 ? pair_mode == 1
                                              : (sizeof(T) == 8 && ntiles + nrows <= 2LL * num_sms));
    }
    for (int s = 0; s < kSlots; ++s) {
      if (!recs[s].used || !recs[s].active) continue;
      active_slots.push_back(s);
      std::vector<WorkItem> items;
      append_items(s, items, pc);
      for (auto& w : items) (w.kind == 1 ? rows_first : tiles).push_back(w);
      max_n = std::max(max_n, recs[s].N);
    }
    hwl = rows_first;
    hwl.insert(hwl.end(), tiles.begin(), tiles.end());
    // a paired launch runs clusters of two blocks: an even count (the pairs
    // of a row task are consecutive from an even index: row tasks first)
    if (pair_rows && hwl.size() % 2) hwl.push_back(WorkItem{active_slots.empty() ? 0 : active_slots[0], 3, 0, 0, 0, 0, -1, 0});
    nwork = (int)hwl.size();
    nrow = (int)rows_first.size();
    std::vector<WorkItem> htwl;
    if (own_tile_list()) {
      int pt = 0;
      std::vector<WorkItem> trows, ttiles;
      for (int s : active_slots) {
        std::vector<WorkItem> items;
        append_items_as(s, items, pt, false, 8, 32, false);
        for (auto& w : items) (w.kind == 1 ? trows : ttiles).push_back(w);
      }
      htwl = trows;
      htwl.insert(htwl.end(), ttiles.begin(), ttiles.end());
    }
    ntwork = own_tile_list() ? (int)htwl.size() : nwork;
    hflat.clear();
    for (int s : active_slots) {
      const int n[3] = {recs[s].N * recs[s].M, recs[s].N * recs[s].M, recs[s].N * (recs[s].M - 1)};
      for (int f = 0; f < 3; ++f)
        for (int b = 0; b < n[f]; b += flat_chunk<T>())
          hflat.push_back(FlatItem{s, f, b, std::min(flat_chunk<T>(), n[f] - b)});
    }
    nflat = (int)hflat.size();
    hdl.clear();
    for (int s : active_slots) append_diag_items(s, hdl);
    ndl = (int)hdl.size();
    if ((size_t)ndl > dl_cap) {
      if (d_dl) cudaFree(d_dl);
      if (d_dpart) cudaFree(d_dpart);
      d_dl = nullptr;
      d_dpart = nullptr;
      dl_cap = std::max<size_t>(ndl, 2 * dl_cap);
      cudaError_t e = cudaMalloc(&d_dl, dl_cap * sizeof(FlatItem));
      if (e == cudaSuccess) e = cudaMalloc(&d_dpart, dl_cap * 4 * sizeof(double));
      if (e != cudaSuccess) return fail(GDC_E_OOM, cuda_msg("rebuild: diag list", e));
    }
    if ((size_t)nflat > flat_cap) {
      if (d_flat) cudaFree(d_flat);
      d_flat = nullptr;
      flat_cap = std::max<size_t>(nflat, 2 * flat_cap);
      cudaError_t e = cudaMalloc(&d_flat, flat_cap * sizeof(FlatItem));
      if (e != cudaSuccess) return fail(GDC_E_OOM, cuda_msg("rebuild: flat list", e));
    }
    if (own_tile_list() && (size_t)ntwork > twl_cap) {
      if (d_twl) cudaFree(d_twl);
      d_twl = nullptr;
      twl_cap = std::max<size_t>(ntwork, 2 * twl_cap);
      cudaError_t e = cudaMalloc(&d_twl, twl_cap * sizeof(WorkItem));
      if (e != cudaSuccess) return fail(GDC_E_OOM, cuda_msg("rebuild: tile list", e));
    }
    if ((size_t)nwork > wl_cap) {
      if (d_wl) cudaFree(d_wl);
      d_wl = nullptr;
      wl_cap = std::max<size_t>(nwork, 2 * wl_cap);
      cudaError_t e = cudaMalloc(&d_wl, wl_cap * sizeof(WorkItem));
      if (e != cudaSuccess) return fail(GDC_E_OOM, cuda_msg("rebuild: work list", e));
    }
    if ((size_t)pc > part_cap) {
      if (d_partials) cudaFree(d_partials);
      d_partials = nullptr;
      part_cap = std::max<size_t>(pc, 2 * part_cap);
      cudaError_t e = cudaMalloc(&d_partials, part_cap * 4 * sizeof(double));
      if (e != cudaSuccess) return fail(GDC_E_OOM, cuda_msg("rebuild: partials", e));
    }
    cudaError_t e = cudaSuccess;
    if (nwork) e = cudaMemcpy(d_wl, hwl.data(), nwork * sizeof(WorkItem), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && own_tile_list() && ntwork)
      e = cudaMemcpy(d_twl, htwl.data(), ntwork * sizeof(WorkItem), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nflat)
      e = cudaMemcpy(d_flat, hflat.data(), nflat * sizeof(FlatItem), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && ndl) e = cudaMemcpy(d_dl, hdl.data(), ndl * sizeof(FlatItem), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !active_slots.empty())
      e = cudaMemcpy(d_active, active_slots.data(), active_slots.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_mem, hdesc.data(), sizeof(MemberDev<T>) * kSlots, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("rebuild: upload", e));
    dirty = false;
    return GDC_OK;
  }

  StageArgs base_args(int pass) const {
    StageArgs a;
    std::memset(&a, 0, sizeof(a));
    a.pass = pass;
    a.in_slot = a.base_slot = a.out_slot = -1;
    a.tout = a.tprev = a.tadd = a.tadd2 = a.taccum = -1;
    a.tadd_sign = 1;
    a.scale2 = 1.0;
    a.h_scale = 0.5;
    a.ip_slot = -1;
    a.partials = d_partials;
    a.beta = d_beta;
    a.qcon = P.qcon_modified;
    a.ub_lon = P.uv_adv_upwind_lon_beta;
    a.ub_lat = P.uv_adv_upwind_lat_beta;
    a.rescale_rtol = P.filter_rescale_rtol;
    a.uvslot = d_uvslot;
    a.pair = pair_rows ? 1 : 0;
    return a;
  }

  // Launch wrappers with optional per-launch CUDA events (profile mode).
  int run_stage(const StageArgs& a, std::vector<Prof>* pr) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (pr) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, stream);
    }
    int rc = GDC_OK;
    if (weno() && a.pass != kFastPass) rc = launch_weno<T>(d_mem, d_flat, nflat, a.in_slot, d_uvslot, stream);
    if (rc) {
    } else if (!strips) {
      rc = launch_stage<T>(d_mem, d_wl, nwork, P.uv_adv_scheme, tile_r, tile_c, max_n, a, stream);
    } else if (pr) {  // timed launch by launch: one stream
      rc = launch_stage<T>(d_mem, d_wl, nrow, P.uv_adv_scheme, 8, 32, max_n, a, stream);
      if (!rc) rc = launch_stage_strips<T>(d_mem, d_wl + nrow, nwork - nrow, P.uv_adv_scheme, a, stream);
    } else {
      // whole-row tasks on the side stream, strips on the main stream
      cudaEventRecord(ev_fork, stream);
      cudaStreamWaitEvent(side, ev_fork, 0);
      rc = launch_stage<T>(d_mem, d_wl, nrow, P.uv_adv_scheme, 8, 32, max_n, a, side);
      if (!rc) rc = launch_stage_strips<T>(d_mem, d_wl + nrow, nwork - nrow, P.uv_adv_scheme, a, stream);
      cudaEventRecord(ev_join, side);
      cudaStreamWaitEvent(stream, ev_join, 0);
    }
    if (pr) {
      cudaEventRecord(e1, stream);
      pr->push_back(Prof{0, e0, e1});
    }
    return rc ? fail(rc, "stage launch failed") : GDC_OK;
  }
  int run_beta(int beta_mode, std::vector<Prof>* pr) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (pr) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, stream);
    }
    int rc = launch_beta<T>(d_mem, d_active, (int)active_slots.size(), d_partials, d_beta, P.qcon_modified,
                            beta_mode, stream);
    if (pr) {
      cudaEventRecord(e1, stream);
      pr->push_back(Prof{4, e0, e1});
    }
    return rc ? fail(rc, "beta launch failed") : GDC_OK;
  }
  int run_final(const FinalArgs& a, std::vector<Prof>* pr) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (pr) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, stream);
    }
    int rc = launch_final<T>(d_mem, d_flat, nflat, a, stream);
    if (pr) {
      cudaEventRecord(e1, stream);
      pr->push_back(Prof{1, e0, e1});
    }
    return rc ? fail(rc, "final-update launch failed") : GDC_OK;
  }

  // A predict_correct's final update not yet launched: level `out` =
  // `base` + time_step_size(pass) * beta * T_new, left for the next
  // predict_correct's first stage to form (StageArgs::fuse).
  struct PendingFinal {
    bool valid = false;
    int base = -1, pass = 0;
  };
  bool fusable() const { return fuse_final && !strips && !weno(); }

  // One predict_correct call (src/dycore_mod.F90:754-792) from level o to n.
  // `in`: the previous call's pending final update, formed here by the
  // first stage (level o is its output); `out`: when given, this call's
  // final update is left pending instead of launched.
  int predict_correct(int pass, int o, int n, const PendingFinal* in, PendingFinal* out, std::vector<Prof>* pr) {
    const PendingFinal prev = in ? *in : PendingFinal();
    StageArgs a = base_args(pass);
    a.in_slot = o;
    a.base_slot = o;
    a.out_slot = SL_SA;
    if (prev.valid) {
      a.fuse = 1;
      a.fin_base = prev.base;
      a.fin_pass = prev.pass;
      a.fin_h_scale = 1.0;
    }
    if (int rc = run_stage(a, pr)) return rc;  // (final of the previous call +) predict 1
    a = base_args(pass);
    a.in_slot = SL_SA;
    a.base_slot = o;
    a.out_slot = SL_SB;
    a.tout = TS_OLD;
    if (int rc = run_stage(a, pr)) return rc;  // predict 2
    a = base_args(pass);
    a.in_slot = SL_SB;
    a.tout = TS_NEW;
    a.tprev = TS_OLD;
    a.do_ip = 1;
    if (int rc = run_stage(a, pr)) return rc;  // correct
    if (int rc = run_beta(0, pr)) return rc;   // beta
    if (out) {
      out->valid = true;
      out->base = o;
      out->pass = pass;
      return GDC_OK;
    }
    FinalArgs f;
    f.base_slot = o;
    f.out_slot = n;
    f.tslot = TS_NEW;
    f.pass = pass;
    f.use_lo = sizeof(T) == 4 ? 1 : 0;
    f.h_scale = 1.0;
    f.beta = d_beta;
    f.uvslot = d_uvslot;
    return run_final(f, pr);
  }

  // isp_splitting (src/dycore_mod.F90:689-752).
  int isp(std::vector<Prof>* pr) {
    const int m = P.subcycles;
    if (int rc = launch_copy_state<T>(d_mem, tile_list(), ntwork, old_, SL_SAVED, stream))
      return fail(rc, "copy launch failed");
    StageArgs a = base_args(kSlowPass);
    a.in_slot = old_;
    a.tout = TS_SLOW;
    if (int rc = run_stage(a, pr)) return rc;
    int t1 = old_, t2 = SL_L0;
    for (int k = 1; k <= m; ++k) {
      a = base_args(kFastPass);
      a.in_slot = t1;
      a.base_slot = t1;
      a.out_slot = SL_SA;
      a.tadd = TS_SLOW;
      if (int rc = run_stage(a, pr)) return rc;
      a.in_slot = SL_SA;
      a.out_slot = SL_SB;
      if (int rc = run_stage(a, pr)) return rc;
      a.in_slot = SL_SB;
      a.out_slot = t2;
      a.taccum = TS_ACCUM;
      a.accum_init = k == 1;
      a.h_scale = 1.0;
      if (int rc = run_stage(a, pr)) return rc;
      std::swap(t1, t2);
    }
    a = base_args(kSlowPass);
    a.in_slot = t1;
    a.base_slot = t1;
    a.out_slot = SL_SA;
    a.tadd = TS_SLOW;
    a.tadd_sign = -1;
    a.h_scale = 1.0;  // half_dt = pcdt[slow]
    if (int rc = run_stage(a, pr)) return rc;
    a.in_slot = SL_SA;
    a.out_slot = SL_SB;
    if (int rc = run_stage(a, pr)) return rc;
    a = base_args(kSlowPass);
    a.in_slot = SL_SB;
    a.tout = TS_NEW;
    a.tadd = TS_SLOW;
    a.tadd2 = TS_ACCUM;
    a.scale2 = 2.0 / m;
    a.do_ip = 1;
    a.beta_mode = 1;
    a.ip_slot = SL_SAVED;
    if (int rc = run_stage(a, pr)) return rc;
    if (int rc = run_beta(1, pr)) return rc;
    FinalArgs f;
    f.base_slot = SL_SAVED;
    f.out_slot = new_;
    f.tslot = TS_NEW;
    f.pass = kAllPass;
    f.use_lo = sizeof(T) == 4 ? 1 : 0;
    f.h_scale = 0.5;
    f.beta = d_beta;
    f.uvslot = d_uvslot;
    return run_final(f, pr);
  }

  int enqueue_step(std::vector<Prof>* pr) {
    int rc = GDC_OK;
    if (P.split_scheme == GDC_SPLIT_CSP2) {
      // csp2_splitting (src/dycore_mod.F90:671-687).  Every final update but
      // the step's last (diag_run reads the step's new level) is formed by
      // the next predict_correct's first stage when fusable.
      PendingFinal pend;
      PendingFinal* pp = fusable() ? &pend : nullptr;
      int t1 = SL_L0, t2 = old_;
      rc = predict_correct(kSlowPass, old_, t1, nullptr, pp, pr);
      for (int k = 0; k < P.subcycles && !rc; ++k) {
        rc = predict_correct(kFastPass, t1, t2, pp, pp, pr);
        std::swap(t1, t2);
      }
      if (!rc) rc = predict_correct(kSlowPass, t1, new_, pp, nullptr, pr);
    } else if (P.split_scheme == GDC_SPLIT_ISP) {
      rc = isp(pr);
    } else {
      rc = predict_correct(kAllPass, old_, new_, nullptr, nullptr, pr);
    }
    if (rc) return rc;
    if (P.use_diffusion) {
      // ordinary_diffusion(time_step_size, state(new)), order 2, sign +1.
      const double c = 1.0 * P.time_step_size * P.diffusion_coef;
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      if (pr) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, stream);
      }
      rc = launch_diffusion<T>(d_mem, tile_list(), ntwork, own_tile_list() ? 8 : tile_r, own_tile_list() ? 32 : tile_c,
                               max_n, new_, c,
                               d_uvslot, stream);
      if (pr) {
        cudaEventRecord(e1, stream);
        pr->push_back(Prof{3, e0, e1});
      }
      if (rc) return fail(rc, "diffusion launch failed");
    }
    // diag_run(state(old)) after time_advance (src/dycore_mod.F90:135).
    DiagArgs d;
    d.slot = new_;
    d.count_step = 1;
    d.partials = d_dpart;
    d.diag = d_diag;
    d.beta = d_beta;
    d.steps = d_steps;
    d.nan_step = d_nan;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (pr) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, stream);
    }
    rc = launch_diag<T>(d_mem, d_dl, ndl, d_active, (int)active_slots.size(), d, stream);
    if (pr) {
      cudaEventRecord(e1, stream);
      pr->push_back(Prof{2, e0, e1});
    }
    return rc ? fail(rc, "diag launch failed") : GDC_OK;
  }

  // diag_run of a freshly admitted member's initial state.
  int initial_diag(int slot) {
    std::vector<FlatItem> wl;
    const MemberDev<T> saved = hdesc[slot];
    append_diag_items(slot, wl);
    if (wl.size() > idl_cap) {
      if (d_idl) cudaFree(d_idl);
      if (d_ipart) cudaFree(d_ipart);
      d_idl = nullptr;
      d_ipart = nullptr;
      idl_cap = 0;
      if (cudaMalloc(&d_idl, sizeof(FlatItem) * wl.size()) != cudaSuccess ||
          cudaMalloc(&d_ipart, sizeof(double) * 4 * wl.size()) != cudaSuccess) {
        cudaGetLastError();
        return fail(GDC_E_OOM, "initial diag: cudaMalloc");
      }
      idl_cap = wl.size();
    }
    if (!d_islot && cudaMalloc(&d_islot, sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return fail(GDC_E_OOM, "initial diag: cudaMalloc");
    }
    // the items, the slot and the descriptor (its diag fields changed) from
    // a staging area of their own (the member's table upload from stage_tab
    // may still be in the stream; this call ends with the stream's
    // synchronisation)
    const size_t bytes = sizeof(FlatItem) * wl.size();
    char* st = stage_diag.get(bytes + sizeof(MemberDev<T>) + 16);
    std::memcpy(st, wl.data(), bytes);
    std::memcpy(st + bytes, &hdesc[slot], sizeof(MemberDev<T>));
    std::memcpy(st + bytes + sizeof(MemberDev<T>), &slot, sizeof(int));
    cudaError_t e = cudaMemcpyAsync(d_idl, st, bytes, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_mem + slot, st + bytes, sizeof(MemberDev<T>), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_islot, st + bytes + sizeof(MemberDev<T>), sizeof(int), cudaMemcpyHostToDevice, stream);
    DiagArgs d;
    d.slot = old_;
    d.count_step = 0;  // the initial diag is not a step
    d.partials = d_ipart;
    d.diag = d_diag;
    d.beta = nullptr;
    d.steps = d_steps;
    d.nan_step = d_nan;
    int rc = e == cudaSuccess ? launch_diag<T>(d_mem, d_idl, (int)wl.size(), d_islot, 1, d, stream) : GDC_E_CUDA;
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    hdesc[slot].dbase = saved.dbase;
    hdesc[slot].dcount = saved.dcount;
    if (e != cudaSuccess) return fail(GDC_E_CUDA, cuda_msg("initial diag", e));
    if (rc) return fail(rc, "initial diag: launch failed");
    return GDC_OK;
  }

  int capture(int par) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      use_graph = false;
      return GDC_OK;
    }
    int rc = enqueue_step(nullptr);
    e = cudaStreamEndCapture(stream, &g);
    if (rc || e != cudaSuccess || !g) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      use_graph = false;
      return rc;
    }
    e = cudaGraphInstantiate(&gexec[par], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      cudaGetLastError();
      gexec[par] = nullptr;
      use_graph = false;
    }
    return GDC_OK;
  }
};

}  // namespace gdc

// ------------------------------------------------------------------ C ABI

struct gdc_batch {
  std::unique_ptr<gdc::BatchIface> impl;
  gdc_params p;
  std::string err;
};

struct gdc_handle {
  gdc_batch* b = nullptr;
  int id = -1;
  gdc_params p;
  std::string err;
};

namespace {

int validate_scheme(const gdc_params* p, std::string& err) {
  if (!p) {
    err = "null params";
    return GDC_E_CONFIG;
  }
  if (p->uv_adv_scheme != GDC_ADV_CENTER_DIFF && p->uv_adv_scheme != GDC_ADV_UPWIND &&
      p->uv_adv_scheme != GDC_ADV_WENO) {
    err = "Unknown uv_adv_scheme";
    return GDC_E_CONFIG;
  }
  if (p->split_scheme < 0 || p->split_scheme > 3) {
    err = "Unknown split_scheme";
    return GDC_E_CONFIG;
  }
  if ((p->split_scheme == GDC_SPLIT_CSP2 || p->split_scheme == GDC_SPLIT_ISP) && p->subcycles < 1) {
    err = "subcycles must be >= 1";
    return GDC_E_CONFIG;
  }
  if (p->use_diffusion && p->diffusion_order != 2) {
    err = "only diffusion_order = 2 is supported";
    return GDC_E_CONFIG;
  }
  if (!(p->filter_rescale_rtol >= 0.0)) {
    err = "filter_rescale_rtol must be >= 0";
    return GDC_E_CONFIG;
  }
  if (p->precision != GDC_FP64 && p->precision != GDC_FP32) {
    err = "precision must be GDC_FP64 or GDC_FP32";
    return GDC_E_CONFIG;
  }
  return GDC_OK;
}

}  // namespace

extern "C" {

int gdc_batch_create(const gdc_params* scheme, gdc_batch** out) {
  if (!out) return GDC_E_CONFIG;
  *out = nullptr;
  std::string err;
  if (int rc = validate_scheme(scheme, err)) {
    std::fprintf(stderr, "gdc_batch_create: %s\n", err.c_str());
    return rc;
  }
  auto* b = new gdc_batch();
  b->p = *scheme;
  int rc;
  if (scheme->precision == GDC_FP32) {
    auto* impl = new gdc::Batch<float>(*scheme);
    b->impl.reset(impl);
    rc = impl->init();
  } else {
    auto* impl = new gdc::Batch<double>(*scheme);
    b->impl.reset(impl);
    rc = impl->init();
  }
  if (rc) {
    std::fprintf(stderr, "gdc_batch_create: %s\n", b->impl->err.c_str());
    delete b;
    return rc;
  }
  *out = b;
  return GDC_OK;
}

void gdc_batch_destroy(gdc_batch* b) { delete b; }
const char* gdc_batch_last_error(const gdc_batch* b) { return b ? b->impl->err.c_str() : "null batch"; }
int gdc_batch_set_stream(gdc_batch* b, void* s) { return b ? b->impl->set_stream(s) : GDC_E_CONFIG; }

size_t gdc_member_bytes(const gdc_params* scheme, int num_lon, int num_lat) {
  return scheme ? gdc::member_bytes_for(*scheme, num_lon, num_lat) : 0;
}

int gdc_device_mem_info(int device, size_t* free_bytes, size_t* total_bytes) {
  if (cudaSetDevice(device) != cudaSuccess) return GDC_E_CUDA;
  size_t f = 0, t = 0;
  if (cudaMemGetInfo(&f, &t) != cudaSuccess) return GDC_E_CUDA;
  f = gdc::free_device_memory(device);
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return GDC_OK;
}

int gdc_batch_add(gdc_batch* b, int num_lon, int num_lat, double time_step_size, long long nsteps,
                  const int* cutoff, const double* u, const double* v, const double* gd,
                  const double* ghs, int ld, size_t reserve_bytes, int* member_id) {
  if (!b || !member_id) return GDC_E_CONFIG;
  return b->impl->add(num_lon, num_lat, time_step_size, nsteps, cutoff, u, v, gd, ghs, ld,
                      reserve_bytes, member_id);
}
int gdc_batch_add_ic(gdc_batch* b, int num_lon, int num_lat, double time_step_size, long long nsteps,
                     const int* cutoff, const gdc_ic_spec* spec, size_t reserve_bytes, int* member_id) {
  if (!b || !spec || !member_id) return GDC_E_CONFIG;
  return b->impl->add_ic(num_lon, num_lat, time_step_size, nsteps, cutoff, *spec, reserve_bytes, member_id);
}
int gdc_batch_remove(gdc_batch* b, int id) { return b ? b->impl->remove(id) : GDC_E_CONFIG; }
int gdc_batch_step(gdc_batch* b, int nsteps) { return b ? b->impl->step(nsteps) : GDC_E_CONFIG; }
int gdc_batch_sync(gdc_batch* b) { return b ? b->impl->sync() : GDC_E_CONFIG; }
int gdc_batch_member_info(gdc_batch* b, int id, long long* steps, int* fin, long long* nan) {
  return b ? b->impl->member_info(id, steps, fin, nan) : GDC_E_CONFIG;
}
int gdc_batch_get_state(gdc_batch* b, int id, double* u, double* v, double* gd, int ld) {
  return b ? b->impl->get_state(id, u, v, gd, nullptr, nullptr, nullptr, ld) : GDC_E_CONFIG;
}
int gdc_batch_diag(gdc_batch* b, int id, double* m, double* e, double* beta) {
  return b ? b->impl->diag(id, m, e, beta) : GDC_E_CONFIG;
}
int gdc_batch_active(gdc_batch* b, int* n) { return (b && n) ? b->impl->active(n) : GDC_E_CONFIG; }
int gdc_batch_set_tile(gdc_batch* b, int r, int c) { return b ? b->impl->set_tile(r, c) : GDC_E_CONFIG; }
int gdc_batch_set_schedule(gdc_batch* b, int split_rows, int fuse_final, int pair_rows) {
  return b ? b->impl->set_schedule(split_rows, fuse_final, pair_rows) : GDC_E_CONFIG;
}
int gdc_batch_get_schedule(gdc_batch* b, int* tile_rows, int* tile_cols, int* split_rows, int* fuse_final,
                           int* pair_rows) {
  return b ? b->impl->get_schedule(tile_rows, tile_cols, split_rows, fuse_final, pair_rows) : GDC_E_CONFIG;
}
int gdc_batch_history(gdc_batch* b, int member_id, double* u_a, double* v_a, double* gh, double* div, double* vor,
                      int ld) {
  return b ? b->impl->history(member_id, u_a, v_a, gh, div, vor, ld) : GDC_E_CONFIG;
}
int gdc_batch_checkpoint(gdc_batch* b, int member_id, const char* path) {
  return b ? b->impl->checkpoint(member_id, path) : GDC_E_CONFIG;
}
int gdc_batch_restore(gdc_batch* b, const char* path, size_t reserve_bytes, int* member_id) {
  return b ? b->impl->restore(path, reserve_bytes, -1, member_id) : GDC_E_CONFIG;
}
int gdc_batch_autotune(gdc_batch* b, int* r, int* c, double* ms) {
  return b ? b->impl->autotune(r, c, ms) : GDC_E_CONFIG;
}
int gdc_batch_profile(gdc_batch* b, int nsteps, double* ms, long long* launches) {
  return (b && ms && launches) ? b->impl->profile(nsteps, ms, launches) : GDC_E_CONFIG;
}

double gdc_algorithmic_bytes_per_gpt_step(const gdc_params* p) {
  if (!p) return 0;
  // Words of {gd, iap u, iap v} (+ ghs) read and written per grid point by
  // one predict_correct call: stage 1 reads 4 writes 3, stage 2 reads 7
  // writes 6, stage 3 reads 7 writes 3, the final update reads 6 writes 3:
  // 39.  FP32 time levels carry a compensation word per field, which the
  // final update reads and writes too (+6).  The diagnostics read the new
  // level and ghs once per step (4 words, 7 with compensation words).
  const bool fp32 = p->precision == GDC_FP32;
  const double pc = 39.0 + (fp32 ? 6.0 : 0.0);
  double calls = 1;
  if (p->split_scheme == GDC_SPLIT_CSP2) calls = p->subcycles + 2;
  double words = pc * calls;
  if (p->split_scheme == GDC_SPLIT_ISP) {
    // copy 6, slow tendency 7, per subcycle 13 + 13 + 16, slow 13 + 13 + 13,
    // final update 9 (+6 compensation words).
    words = 6 + 7 + p->subcycles * 42.0 + 39 + 9 + (fp32 ? 6.0 : 0.0);
  }
  if (p->use_diffusion) words += 6;
  words += fp32 ? 7.0 : 4.0;
  return words * (fp32 ? 4.0 : 8.0);
}

// ---- single model

int gdc_create(const gdc_params* p, gdc_handle** out) {
  if (!out) return GDC_E_CONFIG;
  *out = nullptr;
  std::string err;
  if (int rc = validate_scheme(p, err)) {
    std::fprintf(stderr, "gdc_create: %s\n", err.c_str());
    return rc;
  }
  if (p->num_lon < 8 || p->num_lat < 5 || p->num_lon % 4 != 0 || !(p->time_step_size > 0)) {
    std::fprintf(stderr, "gdc_create: invalid num_lon (>= 8, multiple of 4), num_lat or time_step_size\n");
    return GDC_E_CONFIG;
  }
  auto* h = new gdc_handle();
  h->p = *p;
  int rc = gdc_batch_create(p, &h->b);
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return GDC_OK;
}

void gdc_destroy(gdc_handle* h) {
  if (!h) return;
  gdc_batch_destroy(h->b);
  delete h;
}

const char* gdc_last_error(const gdc_handle* h) {
  if (!h) return "null handle";
  if (!h->err.empty()) return h->err.c_str();
  return gdc_batch_last_error(h->b);
}

int gdc_set_state(gdc_handle* h, const double* u, const double* v, const double* gd,
                  const double* ghs, int ld) {
  if (!h) return GDC_E_CONFIG;
  h->err.clear();
  if (h->id >= 0) {
    gdc_batch_remove(h->b, h->id);
    h->id = -1;
  }
  // The single model runs until told otherwise: length is bounded by the
  // caller's gdc_step calls, not by the member's nsteps.
  return gdc_batch_add(h->b, h->p.num_lon, h->p.num_lat, h->p.time_step_size, (1LL << 62),
                       nullptr, u, v, gd, ghs, ld, 0, &h->id);
}

int gdc_step(gdc_handle* h, int nsteps) {
  if (!h) return GDC_E_CONFIG;
  if (h->id < 0) {
    h->err = "gdc_step before gdc_set_state";
    return GDC_E_STATE;
  }
  if (nsteps < 0) return GDC_E_CONFIG;
  return gdc_batch_step(h->b, nsteps);
}

int gdc_sync(gdc_handle* h) {
  if (!h) return GDC_E_CONFIG;
  int rc = gdc_batch_sync(h->b);
  if (rc || h->id < 0) return rc;
  long long nan = -1;
  gdc_batch_member_info(h->b, h->id, nullptr, nullptr, &nan);
  if (nan >= 0) {
    h->err = "Total mass or energy is NaN at step " + std::to_string(nan) + "!";
    return GDC_E_NAN;
  }
  return GDC_OK;
}

int gdc_run(gdc_handle* h, int nsteps) {
  int rc = gdc_step(h, nsteps);
  if (rc) return rc;
  return gdc_sync(h);
}

int gdc_get_state(gdc_handle* h, double* u, double* v, double* gd, int ld) {
  if (!h) return GDC_E_CONFIG;
  if (h->id < 0) {
    h->err = "gdc_get_state before gdc_set_state";
    return GDC_E_STATE;
  }
  return h->b->impl->get_state(h->id, u, v, gd, nullptr, nullptr, nullptr, ld);
}

int gdc_get_iap(gdc_handle* h, double* iu, double* iv, double* ig, int ld) {
  if (!h) return GDC_E_CONFIG;
  if (h->id < 0) {
    h->err = "gdc_get_iap before gdc_set_state";
    return GDC_E_STATE;
  }
  return h->b->impl->get_state(h->id, nullptr, nullptr, nullptr, iu, iv, ig, ld);
}

int gdc_diag(gdc_handle* h, double* m, double* e, double* beta) {
  if (!h) return GDC_E_CONFIG;
  if (h->id < 0) {
    h->err = "gdc_diag before gdc_set_state";
    return GDC_E_STATE;
  }
  return h->b->impl->diag(h->id, m, e, beta);
}

int gdc_history(gdc_handle* h, double* u_a, double* v_a, double* gh, double* div, double* vor, int ld) {
  if (!h) return GDC_E_CONFIG;
  h->err.clear();
  if (h->id < 0) {
    h->err = "gdc_history before gdc_set_state";
    return GDC_E_STATE;
  }
  return h->b->impl->history(h->id, u_a, v_a, gh, div, vor, ld);
}

int gdc_write_restart(gdc_handle* h, const char* path) {
  if (!h) return GDC_E_CONFIG;
  h->err.clear();
  if (h->id < 0) {
    h->err = "gdc_write_restart before gdc_set_state";
    return GDC_E_STATE;
  }
  return h->b->impl->checkpoint(h->id, path);
}

int gdc_read_restart(gdc_handle* h, const char* path) {
  if (!h) return GDC_E_CONFIG;
  h->err.clear();
  if (h->id >= 0) {
    gdc_batch_remove(h->b, h->id);
    h->id = -1;
  }
  int id = -1;
  const int rc = h->b->impl->restore(path, 0, (1LL << 62), &id);
  if (rc == GDC_OK) h->id = id;
  return rc;
}

int gdc_steps_done(gdc_handle* h, long long* steps) {
  if (!h || !steps) return GDC_E_CONFIG;
  if (h->id < 0) {
    *steps = 0;
    return GDC_OK;
  }
  return h->b->impl->member_info(h->id, steps, nullptr, nullptr);
}

int gdc_debug_tendency(gdc_handle* h, int pass, double* du, double* dv, double* dgd, int ld) {
  if (!h) return GDC_E_CONFIG;
  if (h->id < 0) {
    h->err = "gdc_debug_tendency before gdc_set_state";
    return GDC_E_STATE;
  }
  return h->b->impl->debug_tendency(h->id, pass, du, dv, dgd, ld);
}

int gdc_set_stream(gdc_handle* h, void* s) { return h ? gdc_batch_set_stream(h->b, s) : GDC_E_CONFIG; }

}  // extern "C"
