// The stage kernels of one tile shape and real type, compiled once per pair
// with -DGDC_REAL=float|double -DGDC_TILE_R=rows -DGDC_TILE_W=cols (FP64
// without fused multiply-add, FP32 with fast division and square root, as
// the rest of each precision's kernels).
#define GDC_STAGE_SHAPE_UNIT
#include "gdc_kernels.cuh"

#if !defined(GDC_REAL) || !defined(GDC_TILE_R) || !defined(GDC_TILE_W)
#error "gdc_stage_shape.cu needs GDC_REAL, GDC_TILE_R and GDC_TILE_W"
#endif

namespace gdc {

template int launch_stage_shape<GDC_REAL, GDC_TILE_R, GDC_TILE_W>(const MemberDev<GDC_REAL>*, const WorkItem*, int,
                                                                  int, int, const StageArgs&, cudaStream_t);

}  // namespace gdc
