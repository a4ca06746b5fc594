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
