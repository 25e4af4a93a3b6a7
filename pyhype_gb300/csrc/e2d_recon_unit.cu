// e2d_recon_unit.cu - the reconstruction launchers of one (arithmetic type, limiter)
// pair: every tile-height / occupancy / persistent variant of k_reconstruct, the
// multi-point form and the fused stage kernel (every flux and reconstruction type).  Compiled once per pair with -DE2D_T=<double|float> and
// -DE2D_LIM=<0..3> (the FP64 objects with -fmad=false), so the eight pairs build in
// parallel; e2d_fp64.cu and e2d_fp32.cu dispatch to them.
#include "e2d_fused.cuh"

#if !defined(E2D_T) || !defined(E2D_LIM)
#error "compile with -DE2D_T=<double|float> -DE2D_LIM=<limiter code>"
#endif

namespace e2d {

E2D_RECON_LIM_DECL(, E2D_T, E2D_LIM)
E2D_FUSED_LIM_DECL(, E2D_T, E2D_LIM)

}  // namespace e2d
