/*
 * euler2d_bench.h - measurement aids used by the benchmark.  They have no
 * counterpart in the reference (which has no GPU code); they exist to put the
 * solver's kernels against the GPU's own measured FP64 rate.
 */
#ifndef EULER2D_BENCH_H
#define EULER2D_BENCH_H

#include "euler2d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Throughput of one FP64 instruction class on the current device, measured with
   CUDA events over a grid of independent dependency chains (8 per thread).
   op: 0 = DFMA (reported as 2 flops per instruction), 1 = DADD, 2 = DMUL.
   *tflops receives the best of three runs in TFLOP/s.                          */
E2D_API int e2d_bench_fp64_peak(int32_t op, double* tflops);

/* Kernel times of `steps` device-loop steps (as e2d_run issues them), each launch
   bracketed by CUDA events on the handle's stream.  ms[k] receives the average
   duration of one launch of kernel class k and launches[k] the launch count:
   0 = CFL dt, 1 = reconstruct, 2 = flux, 3 = update, 4 = step bookkeeping,
   5 = fused stage (stages run by the fused stage kernel).                      */
#define E2D_BENCH_NK 6
E2D_API int e2d_bench_kernels(E2DHandle h, int32_t steps, double* ms, int64_t* launches);

/* Cost of the halo: the reconstruction kernel (8-row tiles, default variant) forms
   ghost cells (inter-block neighbours and boundary conditions) and block-boundary
   face states on the fly in the tiles along block sides.  ms[0] receives the average
   duration of `reps` launches over the real tile table; ms[1] the same number of
   tiles with every tile touching an inter-block side replaced by an interior tile;
   ms[2] with every tile touching any block side replaced.  ntiles[0..2] = all tiles,
   tiles touching an inter-block side, tiles touching any side.  ms[0] - ms[1] is the
   inter-block halo cost of one stage.  Face arrays are stale after the call until
   the next reconstruction.                                                      */
E2D_API int e2d_bench_halo(E2DHandle h, int32_t reps, double* ms, int64_t* ntiles);

/* Tile loads of the reconstruction kernel: enable != 0 (the default) stages interior
   tiles (halo inside the block) with one TMA box load per tile where the block's
   layout allows it, 0 stages every tile with plain loads.  Both compute the same
   values.                                                                       */
E2D_API int e2d_bench_set_tma(E2DHandle h, int32_t enable);

/* Kernel-variant selection.  Every variant computes the same values; they differ in
   tile height, register/occupancy target and grid shape (one CTA per tile, or a
   persistent grid of resident CTAs striding over the tile table).
   kernel: 0 = reconstruct (variants 0..5: tile height x min CTAs per SM of (8,2),
   (8,1), (4,2), (4,4), (16,1), and (4,8) in the FP32 form, where the FP64 path
   runs variant 0), 1 = flux (variants 0..2: min CTAs per SM 4, 1, 6),
   2 = update (variant 0), 3 = stage form (variant 0: the three kernels above per
   stage; 1 and 2: one fused stage kernel per stage, with tiles of 28 x 32 cells and
   16 warps (1) or 13 x 32 cells and 8 warps (2), face states and fluxes in shared
   memory; stages whose updates overwrite their own input, and problems with several
   face quadrature points, stay split).  A handle starts at form 2 in the FP32 form
   and form 0 in FP64, the fastest of each on the benchmark problems.             */
E2D_API int e2d_set_kernel_choice(E2DHandle h, int32_t kernel, int32_t variant, int32_t persistent);
/* Autotuner: times every variant and grid shape of the reconstruct and flux kernels
   and the grid shape of the update kernel on the current state (`reps` launches each,
   CUDA events on the handle's stream), keeps the fastest, then compares one stage of
   those three against one fused stage of each tile shape and keeps the fastest form.  Returns the choices
   in chosen[0..7] = {reconstruct variant, persistent, flux variant, persistent,
   update variant, persistent, stage form, 0}.  Graphs captured before are dropped. */
E2D_API int e2d_autotune(E2DHandle h, int32_t reps, int32_t* chosen);

/* The bounded barrier wait of the reconstruction kernel's TMA tile staging, on its
   own: one warp waits on a shared-memory barrier phase for at most `limit` polls.
   complete != 0 completes the phase (*arrived = 1); complete == 0 announces a
   transfer that never comes, and the wait must run out and return (*arrived = 0)
   instead of spinning, leaving the context usable.                              */
E2D_API int e2d_check_wait_bound(int32_t complete, int32_t limit, int32_t* arrived);

/* The FP32 form's division routine applied elementwise: q[i] = a[i] / b[i] for n
   values in caller device buffers, on the default stream (synchronised).  For
   testing the routine against IEEE division.                                   */
E2D_API int e2d_check_div32(const float* a_dev, const float* b_dev, float* q_dev, int64_t n);
/* The FP32 form's division without div32's range test (rdiv, for the state algebra's
   positive divisors), elementwise as e2d_check_div32.                              */
E2D_API int e2d_check_rdiv32(const float* a_dev, const float* b_dev, float* q_dev, int64_t n);
/* The FP64 divergence's division by an area through its correctly rounded reciprocal
   (div_recip with y = 1/b): q[i] = x[i] / b[i] for b[i] > 0, elementwise.        */
E2D_API int e2d_check_div_recip(const double* x_dev, const double* b_dev, double* q_dev, int64_t n);
/* The FP32 form's paired limiter-function evaluation: pair_out[i] = the paired
   min(psi(sa[i]), psi(sb[i])), scalar_out[i] = the same from two scalar evaluations,
   for Venkatakrishnan or van Albada (the limiters with a maximum).                 */
E2D_API int e2d_check_psi_pair(int32_t limiter, const float* sa_dev, const float* sb_dev, float* pair_out_dev,
                               float* scalar_out_dev, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
