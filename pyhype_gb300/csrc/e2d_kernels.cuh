// e2d_kernels.cuh - launch interface between the C ABI (e2d_api.cu) and the stage
// kernels (e2d_stage.cuh, instantiated by e2d_fp64.cu and e2d_fp32.cu).  Internal.
#pragma once
#include <cstdint>
#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>

#include "../../include/euler2d.h"

namespace e2d {

constexpr int TX = 32;        // cell tile width  (one warp along x)
constexpr int TY = 8;         // cell tile height
constexpr int MAX_STAGES = 8;
// tile heights of the fused stage kernel (e2d_fused.cuh): 28 rows for 16 warps and 13
// rows for 8 warps, where the tile rows and the ring tasks fill whole rounds of warps
constexpr int FUSED_TY[2] = {28, 13};
constexpr int FUSED_WARPS[2] = {16, 8};

// Device view of the geometry planes (in the arithmetic type of the path).
template <typename T>
struct DevGeometryT {
  const T* cell[E2D_G_NCELL];
  const T* vface[E2D_F_NFACE];
  const T* hface[E2D_F_NFACE];
  const T* qp[E2D_MAX_QP][8];  // with nqp > 1: point - centroid, x (E, W, N, S) then y
};

// Face-indexed left/right states (primitive, rotated into the face frame), 4 planes
// per face quadrature point (point q at plane offset 4q), and the integrated face
// fluxes L * sum_q w_q F_q, 4 planes.
template <typename T>
struct FaceArraysT {
  T* vL;
  T* vR;
  T* hL;
  T* hR;
  T* vI;
  T* hI;
};

// Per-instance time state, device resident so a whole step can be replayed from a
// CUDA graph.  One instance for a plain solver; one per problem in a batch.  Time,
// dt and the CFL minimum are FP64 on every path.
struct InstanceState {
  double t;            // solver (non-dimensional) time at the start of the step
  double dt;           // current step
  double t_final;
  unsigned long long min_bits;  // min over cells of min(tx, ty) as FP64 IEEE bits (>= 0)
  int32_t active;      // 1 while this instance still steps
  int32_t steps;       // steps taken
  int32_t max_steps;
  int32_t halted;      // set when a step produced an unrealizable state
  int32_t nbad;        // unrealizable cells found in this instance's last stage
  int32_t pad_;
};

struct RealizState {
  unsigned long long first;  // (block << 40 | cell) of the first offending cell, or ~0
  unsigned long long nbad;
};

template <typename T>
struct ParamsT {
  const E2DBlock* blocks;   // device copy, side_coord patched to device pointers
  int nblocks;
  int64_t ncell, nvface, nhface;
  DevGeometryT<T> geo;
  double gamma, gm1, gm, k, cfl;
  T gas[4];                 // gamma, gamma-1, gamma/(gamma-1), 1/(gamma-1) in the path's type
  int flux, limiter, recon;
  int nqp;                  // face quadrature points (1, 2, 3)
  T qw[E2D_MAX_QP];         // their weights (2; 1, 1; 5/9, 8/9, 5/9)
  const int* axis32;        // FP32 form: per block, 1 where every face frame is axis-aligned
                            // to FP32's resolution (null on the FP64 path)
};

// A block whose faces the kernels treat as axis-aligned (no rotations, no frame loads):
// the reference's test on its corner vertices (quad_block.py:96-113), or in the FP32
// form a block whose every vertical face has cos 1 and |sin| < 2^-24 and every
// horizontal face sin 1 and |cos| < 2^-24 in FP32.  A rotation by such a frame changes
// an FP32 velocity component only where it is below 2^-24 of the other component, a
// difference the FP32 state cannot hold.
template <typename T>
__device__ __forceinline__ bool block_cart(const ParamsT<T>& P, const E2DBlock* B, int b) {
  return B->is_cartesian != 0 || (sizeof(T) == 4 && P.axis32 != nullptr && P.axis32[b] != 0);
}

// One update of the RK stage program: dst = src + (dt * a) * k (buffers by id).
// src_zero: the partial sum starts here (src value 0, used for increments).
// kahan: the result is an increment added into buffer 0 with compensated (Kahan)
// summation; dst is unused.
struct StageUpdate {
  int dst;
  int src;
  double a;
  int src_zero;
  int kahan;
  // the buffers dst and src name, filled by resolve_program just before a launch (a
  // pointer per update instead of a run-time choice among the state buffers per cell)
  void* dstp;
  const void* srcp;
};
struct StageProgram {
  int nupd;
  StageUpdate upd[MAX_STAGES];
  int final_stage;   // 1 on the last stage (realizability + step bookkeeping)
};

template <typename T>
struct StateBuffersT {
  T* buf[MAX_STAGES + 1];   // 0 = U^n, 1.. = row partial sums
  T* comp;                  // Kahan compensation of U^n (FP32 path), else null
};

// The program with each update's buffers resolved to pointers (ids 0..MAX_STAGES,
// as build_program makes them).
template <typename T>
inline StageProgram resolve_program(const StageProgram& prog, const StateBuffersT<T>& S) {
  StageProgram r = prog;
  for (int u = 0; u < r.nupd; ++u) {
    r.upd[u].dstp = S.buf[r.upd[u].dst];
    r.upd[u].srcp = S.buf[r.upd[u].src];
  }
  return r;
}

template <typename T>
struct DebugOutT {
  T* gx;
  T* gy;
  T* phi;
  T* vflux_raw;
  T* hflux_raw;
  T* vflux;
  T* hflux;
};

using DevGeometry = DevGeometryT<double>;
using FaceArrays = FaceArraysT<double>;
using Params = ParamsT<double>;
using StateBuffers = StateBuffersT<double>;
using DebugOut = DebugOutT<double>;

// Tile tables: cell tiles for tile heights 4, 8 and 16 (index 0..2), the fused stage
// kernel's tiles (FUSED_TY), face-node tiles at height 8.  Each entry is (block, i0, j0, 0).
struct TileSet {
  const int4* cell[3];
  int ncell[3];
  const int4* fused[2];
  int nfused[2];
  const int4* face;
  int nface;
  bool all_cartesian;  // every block's faces are axis-aligned (the fused kernel's Cartesian variant)
};
// Tensor-memory-access (TMA) tile loads of one state buffer for the reconstruction
// kernel's interior tiles (tiles whose one-cell halo lies inside their block), at one
// tile height: one tensor map per block over its 4 planes (box: the tile and its halo,
// widened on both sides so that its first column is 16-byte aligned).  ok[b] = 0 where
// block b cannot use one (row stride, plane stride or base not 16-byte aligned); those
// blocks, edge tiles and maps == nullptr take plain loads.  timeouts counts bounded
// barrier waits that ran out (the kernel then drops that tile and reports through it).
struct TmaTiles {
  const CUtensorMap* maps;
  const int* ok;
  unsigned long long* timeouts;
};
// Columns of a staged tile: the box starts XO = 16 / sizeof(T) columns left of the tile
// (its first column is then 16-byte aligned: j0 is a multiple of 32) and is TXW columns
// wide; column j0 - 1 + lx of the block sits at shared-memory column C0 + lx.
template <typename T>
struct TileCols {
  static constexpr int XO = 16 / (int)sizeof(T);
  static constexpr int TXW = TX + 2 * XO;
  static constexpr int C0 = XO - 1;
};
// the three tile heights (4, 8, 16) of one state buffer, and the fused stage kernel's
// boxes (its tile rows and a 2-cell halo)
struct TmaSet {
  TmaTiles by_rty[3];
  TmaTiles fused[2];
};

// Kernel variant chosen by the autotuner (0 = default) and persistent-grid flag.
struct KernelChoice {
  int variant;
  bool persistent;
};
constexpr int N_RECON_VARIANTS = 6;  // (tile height, min CTAs/SM): (8,2) (8,1) (4,2) (4,4) (16,1), (4,8) FP32 only
constexpr int N_FLUX_VARIANTS = 3;   // min CTAs/SM: 4, 1, 6
constexpr int N_STAGE_FORMS = 3;     // 0: three kernels per stage; 1, 2: the fused stage kernel at
                                     // FUSED_TY[0] / FUSED_TY[1] rows

// launchers, instantiated for double (e2d_fp64.cu) and float (e2d_fp32.cu)
template <typename T>
cudaError_t launch_reconstruct(const ParamsT<T>& P, const TileSet& ts, KernelChoice kc, const T* U,
                               const InstanceState* inst, FaceArraysT<T> F, const DebugOutT<T>* dbg,
                               cudaStream_t st, const TmaSet* tma = nullptr);
template <typename T>
cudaError_t launch_flux(const ParamsT<T>& P, const TileSet& ts, KernelChoice kc, const InstanceState* inst,
                        FaceArraysT<T> F, const DebugOutT<T>* dbg, cudaStream_t st);
template <typename T>
cudaError_t launch_update(const ParamsT<T>& P, const TileSet& ts, KernelChoice kc, FaceArraysT<T> F,
                          StateBuffersT<T> S, const StageProgram& prog, InstanceState* inst,
                          RealizState* real, T* dudt_out, cudaStream_t st);
template <typename T>
cudaError_t launch_dt(const ParamsT<T>& P, const int4* cell_tiles, int ntiles, const T* U,
                      InstanceState* inst, cudaStream_t st);
template <typename T>
cudaError_t launch_realizable(const ParamsT<T>& P, const int4* cell_tiles, int ntiles, const T* U,
                              RealizState* real, cudaStream_t st);
template <typename T>
cudaError_t launch_totals(const ParamsT<T>& P, const int4* tiles, int n, const T* U, double* partial,
                          cudaStream_t st);
template <typename T>
cudaError_t launch_ghost_layer(const ParamsT<T>& P, const T* U, double t, const int64_t* base, double* out,
                               int64_t nghost, int maxlen, cudaStream_t st);
// What a fused stage records for the adjoint's reverse pass (null: nothing): its
// input state (4 planes, y) and its face states in the split reconstruction's face
// arrays (vL, vR, hL, hR)
template <typename T>
struct FusedRecordT {
  T* y;
  T* vL;
  T* vR;
  T* hL;
  T* hR;
};
// one RK stage in one launch (e2d_fused.cuh); prepare_only sets the kernel's shared
// memory limit on the current device and launches nothing
template <typename T>
cudaError_t launch_stage_fused(const ParamsT<T>& P, const TileSet& ts, int form, const T* U, InstanceState* inst,
                               StateBuffersT<T> S, const StageProgram& prog, RealizState* real, cudaStream_t st,
                               const TmaSet* tma, bool prepare_only, const FusedRecordT<T>& rec);
cudaError_t launch_begin_step(InstanceState* inst, int ninst, double cfl, int use_min, cudaStream_t st);
cudaError_t launch_end_step(InstanceState* inst, int ninst, const RealizState* real, cudaStream_t st);
cudaError_t launch_set_time(InstanceState* inst, int ninst, double t, double dt, cudaStream_t st);
// precision conversions between caller FP64 buffers and an FP32 state
cudaError_t launch_convert(const double* src, float* dst, int64_t n, cudaStream_t st);
cudaError_t launch_convert(const float* src, double* dst, int64_t n, cudaStream_t st);

}  // namespace e2d
