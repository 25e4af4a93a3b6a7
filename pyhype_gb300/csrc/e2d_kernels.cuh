// e2d_kernels.cuh - launch interface between the C ABI (e2d_api.cu) and the stage
// kernels (e2d_fp64.cu).  Internal to the library.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/euler2d.h"

namespace e2d {

constexpr int TX = 32;        // cell tile width  (one warp along x)
constexpr int TY = 8;         // cell tile height
constexpr int MAX_STAGES = 8;

// Device view of the geometry planes.
struct DevGeometry {
  const double* cell[E2D_G_NCELL];
  const double* vface[E2D_F_NFACE];
  const double* hface[E2D_F_NFACE];
};

// Face-indexed left/right states (primitive, rotated into the face frame) and the
// integrated face fluxes L*(2F), 4 planes each.
struct FaceArrays {
  double* vL;
  double* vR;
  double* hL;
  double* hR;
  double* vI;
  double* hI;
};

// Per-instance time state, device resident so a whole step can be replayed from a
// CUDA graph.  One instance for a plain solver; one per problem in a batch.
struct InstanceState {
  double t;            // solver (non-dimensional) time at the start of the step
  double dt;           // current step
  double t_final;
  unsigned long long min_bits;  // min over cells of min(tx, ty) as IEEE bits (>= 0)
  int32_t active;      // 1 while this instance still steps
  int32_t steps;       // steps taken
  int32_t max_steps;
  int32_t halted;      // set when a step produced an unrealizable state
};

struct RealizState {
  unsigned long long first;  // (block << 40 | cell) of the first offending cell, or ~0
  unsigned long long nbad;
};

struct Params {
  const E2DBlock* blocks;   // device copy, side_coord patched to device pointers
  int nblocks;
  int64_t ncell, nvface, nhface;
  DevGeometry geo;
  double gamma, gm1, gm, k, cfl;
  int flux, limiter, recon;
};

// One update of the RK stage program: dst = src + (dt * a) * k (buffers by id).
struct StageUpdate {
  int dst;
  int src;
  double a;
};
struct StageProgram {
  int nupd;
  StageUpdate upd[MAX_STAGES];
  int final_stage;   // 1 on the last stage (realizability + step bookkeeping)
};

struct StateBuffers {
  double* buf[MAX_STAGES + 1];   // 0 = U^n, 1.. = row partial sums
};

struct DebugOut {
  double* gx;
  double* gy;
  double* phi;
  double* vflux_raw;
  double* hflux_raw;
  double* vflux;
  double* hflux;
};

// launchers (e2d_fp64.cu)
cudaError_t launch_reconstruct(const Params& P, const int4* cell_tiles, int ntiles, const double* U,
                               const InstanceState* inst, FaceArrays F, const DebugOut* dbg,
                               cudaStream_t st);
cudaError_t launch_flux(const Params& P, const int4* face_tiles, int ntiles, const InstanceState* inst,
                        FaceArrays F, const DebugOut* dbg, cudaStream_t st);
cudaError_t launch_update(const Params& P, const int4* cell_tiles, int ntiles, FaceArrays F,
                          StateBuffers S, const StageProgram& prog, InstanceState* inst,
                          RealizState* real, double* dudt_out, cudaStream_t st);
cudaError_t launch_dt(const Params& P, const int4* cell_tiles, int ntiles, const double* U,
                      InstanceState* inst, cudaStream_t st);
cudaError_t launch_begin_step(InstanceState* inst, int ninst, double cfl, int use_min, cudaStream_t st);
cudaError_t launch_end_step(InstanceState* inst, int ninst, const RealizState* real, cudaStream_t st);
cudaError_t launch_set_time(InstanceState* inst, int ninst, double t, double dt, cudaStream_t st);
cudaError_t launch_realizable(const Params& P, const int4* cell_tiles, int ntiles, const double* U,
                              RealizState* real, cudaStream_t st);

}  // namespace e2d
