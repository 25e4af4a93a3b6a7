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
   0 = CFL dt, 1 = reconstruct, 2 = flux, 3 = update, 4 = step bookkeeping.     */
#define E2D_BENCH_NK 5
E2D_API int e2d_bench_kernels(E2DHandle h, int32_t steps, double* ms, int64_t* launches);

#ifdef __cplusplus
}
#endif
#endif
