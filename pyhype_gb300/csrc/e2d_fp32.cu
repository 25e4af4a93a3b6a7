// e2d_fp32.cu - FP32 instantiation of the stage kernels: FP32 state, geometry, face
// arrays and flux arithmetic (contraction allowed), the step increment added to the
// state with Kahan compensation, FP64 time, dt reduction and positivity bookkeeping.
#include "e2d_fused.cuh"

namespace e2d {

E2D_EXTERN_RECON_LIM(float)
E2D_EXTERN_FUSED_LIM(float)
E2D_INSTANTIATE_FUSED_LAUNCHER(float)
E2D_INSTANTIATE_STAGE_LAUNCHERS(float)

}  // namespace e2d
