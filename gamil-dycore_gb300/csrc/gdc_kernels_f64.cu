// FP64 instantiation of the stage, update, diagnostic and diffusion kernels.
// Compiled with --fmad=false: every point-wise FP64 expression is then
// evaluated with the reference's own operations and rounding (no fused
// multiply-add), so the plain path differs from the reference's arithmetic
// only in the order of its parallel sums.
#include "gdc_kernels.cuh"

namespace gdc {

template size_t stage_smem_bytes<double>(int, int, int, int*);
template int launch_diffusion<double>(const MemberDev<double>*, const WorkItem*, int, int, int, int, int, double, int*, void*);
template int launch_copy_state<double>(const MemberDev<double>*, const WorkItem*, int, int, int, void*);
template int launch_stage<double>(const MemberDev<double>*, const WorkItem*, int, int, int, int, int,
                                  const StageArgs&, void*);
template int launch_stage_strips<double>(const MemberDev<double>*, const WorkItem*, int, int, const StageArgs&, void*);
template int launch_history<double>(const MemberDev<double>*, int, int, int, int, double*, double*, double*, double*,
                                   double*, void*);
template int launch_ic_iap<double>(const MemberDev<double>*, int, int, int, int, const double*, const double*,
                                 const double*, const double*, int, void*);
template int launch_weno<double>(const MemberDev<double>*, const FlatItem*, int, int, const int*, void*);
template int launch_state_out<double>(const MemberDev<double>*, int, int, int, int, int, double*, void*);
template int launch_final<double>(const MemberDev<double>*, const FlatItem*, int, const FinalArgs&, void*);
template int launch_diag<double>(const MemberDev<double>*, const FlatItem*, int, const int*, int, const DiagArgs&, void*);
template int launch_beta<double>(const MemberDev<double>*, const int*, int, const double*, double*, int, int, void*);

}  // namespace gdc

// ---------------------------------------------------------- FP64 roof
// The device's FP64 fused multiply-add rate, the roof of the FP64 path:
// every thread runs 8 independent chains of `iters` fused multiply-adds
// (explicit __fma_rn: the unit is built without contraction) on a grid of
// 4 blocks of 256 threads per SM; timed with CUDA events on a stream of its
// own after one untimed launch.
namespace {
__global__ void __launch_bounds__(256) fp64_fma_kernel(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = (double)(threadIdx.x + k);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = __fma_rn(x[k], a, b);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s = __dadd_rn(s, x[k]);
  if (s == 1.0e300) out[blockIdx.x] = s;  // never true: keeps the chains live
}
}  // namespace

extern "C" int gdc_fp64_fma_rate(int device, double* gfma_per_s) {
  if (!gfma_per_s) return GDC_E_CONFIG;
  if (cudaSetDevice(device) != cudaSuccess) return GDC_E_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = 4 * (sms > 0 ? sms : 1), iters = 1 << 14;
  double* out = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(double) * blocks);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float ms = 0.0f;
  if (e == cudaSuccess) {
    fp64_fma_kernel<<<blocks, 256, 0, s>>>(out, iters / 8, 0.999999, 1.0e-6);
    cudaEventRecord(e0, s);
    fp64_fma_kernel<<<blocks, 256, 0, s>>>(out, iters, 0.999999, 1.0e-6);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e1) cudaEventDestroy(e1);
  if (e0) cudaEventDestroy(e0);
  if (s) cudaStreamDestroy(s);
  if (out) cudaFree(out);
  if (e != cudaSuccess || !(ms > 0.0f)) {
    cudaGetLastError();
    return GDC_E_CUDA;
  }
  *gfma_per_s = (double)blocks * 256.0 * 8.0 * iters / (ms * 1.0e-3) / 1.0e9;
  return GDC_OK;
}

