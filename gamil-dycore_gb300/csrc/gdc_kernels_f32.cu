// FP32 instantiation of the stage, update, diagnostic and diffusion kernels
// (fused multiply-add allowed).
#include "gdc_kernels.cuh"

namespace gdc {

template size_t stage_smem_bytes<float>(int, int, int, int*);
template int launch_diffusion<float>(const MemberDev<float>*, const WorkItem*, int, int, int, int, int, double, int*, void*);
template int launch_copy_state<float>(const MemberDev<float>*, const WorkItem*, int, int, int, void*);
template int launch_stage<float>(const MemberDev<float>*, const WorkItem*, int, int, int, int, int,
                                 const StageArgs&, void*);
template int launch_stage_strips<float>(const MemberDev<float>*, const WorkItem*, int, int, const StageArgs&, void*);
template int launch_history<float>(const MemberDev<float>*, int, int, int, int, double*, double*, double*, double*,
                                   double*, void*);
template int launch_ic_iap<float>(const MemberDev<float>*, int, int, int, int, const double*, const double*,
                                 const double*, const double*, int, void*);
template int launch_weno<float>(const MemberDev<float>*, const FlatItem*, int, int, const int*, void*);
template int launch_state_out<float>(const MemberDev<float>*, int, int, int, int, int, double*, void*);
template int launch_final<float>(const MemberDev<float>*, const FlatItem*, int, const FinalArgs&, void*);
template int launch_diag<float>(const MemberDev<float>*, const FlatItem*, int, const int*, int, const DiagArgs&, void*);
template int launch_beta<float>(const MemberDev<float>*, const int*, int, const double*, double*, int, int, void*);

}  // namespace gdc
