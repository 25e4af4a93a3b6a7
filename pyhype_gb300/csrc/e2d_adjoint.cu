// e2d_adjoint.cu - reverse mode of the time loop: the residual VJP, the RK step
// adjoint and the checkpointed forward/backward passes of a boundary-pressure
// objective (include/euler2d.h, "adjoint").  The reference has no counterpart; the
// forward steps are the plain path's own kernels, so a recomputed segment repeats
// the recorded forward pass value for value.
//
// Both paths are differentiated: FP64 (reverse kernels in FP64) and the FP32 form
// (FP32 state, face states and reverse kernels; the Kahan compensation planes are
// checkpointed with the state so recomputation is exact; J and dt stay FP64).
//
// Built with -fmad=false like the FP64 stage kernels: the reverse kernels recompute
// the forward reconstruction and must take the same min/max/branch selections.
#include <cmath>
#include <cstring>
#include <vector>

#include "e2d_adjoint.cuh"
#include "e2d_solver.cuh"

namespace e2d {
E2D_EXTERN_STAGE_LAUNCHERS(double)  // instantiated in e2d_fp64.cu
E2D_EXTERN_STAGE_LAUNCHERS(float)   // instantiated in e2d_fp32.cu
}

using namespace e2d;

// Storage of one recorded forward pass, in the arithmetic type of the handle's path
// (the void pointers hold T arrays).
struct E2DAdjoint {
  int nsteps = 0, K = 0, S = 0, prec = -1;
  E2DPressureObjective obj{};
  std::vector<double> dts, ts;  // per step: dt and the time at its start
  bool recorded = false;
  // device
  void* ckpt = nullptr;         // ceil(N/K) checkpoints: state (+ Kahan planes on FP32)
  void* final_state = nullptr;  // U^N (+ Kahan planes)
  void* stage = nullptr;        // K*S stage states of the segment being reversed
  void* face = nullptr;         // K*S face-state sets (vL, vR, hL, hR)
  void* lam = nullptr;          // adjoint of the state
  void* acc = nullptr;          // S stage-residual adjoints
  void* st = nullptr;           // 5 stencil slots x 4 planes
  void* io = nullptr;           // FP32 staging of FP64 caller buffers (2 x 4 planes)
  double* rec = nullptr;        // dts, ts recorded on the device (2N)
  double* J = nullptr;
  size_t cap_ckpt = 0, cap_seg = 0, cap_rec = 0, cap_acc = 0;
  std::vector<void*> allocs;
};

void destroy_adjoint(E2DAdjoint* a) {
  if (!a) return;
  for (void* p : a->allocs) cudaFree(p);
  delete a;
}

namespace {

int adj_alloc_bytes(E2DAdjoint* A, void** p, size_t bytes) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes ? bytes : 1);
  if (e != cudaSuccess)
    return fail(E2D_ERR_NOMEM, "adjoint storage: cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
  A->allocs.push_back(q);
  *p = q;
  return 0;
}

template <typename T>
T* as(void* p) { return static_cast<T*>(p); }

int64_t face_set_size(const E2DSolver* h) { return 8 * h->nvface + 8 * h->nhface; }

// values per checkpoint: the state, plus the Kahan compensation on the FP32 path
template <typename T>
size_t ckpt_size(const E2DSolver* h) { return (sizeof(T) == 4 ? 8 : 4) * (size_t)h->ncell; }

template <typename T>
FaceArraysT<T> face_slot(E2DSolver* h, T* base) {
  FaceArraysT<T> F = path<T>(h).F;  // vI, hI stay the path's own
  F.vL = base;
  F.vR = base + 4 * h->nvface;
  F.hL = base + 8 * h->nvface;
  F.hR = base + 8 * h->nvface + 4 * h->nhface;
  return F;
}

int check_supported(E2DSolver* h) {
  if (h->hinst.size() != 1) return fail(E2D_ERR_UNSUPPORTED, "the adjoint runs on single-instance problems");
  if (h->nstages < 1) return fail(E2D_ERR_INVALID, "no tableau set");
  if (h->cfg.nqp > 1) return fail(E2D_ERR_UNSUPPORTED, "the adjoint is built for one face quadrature point");
  return 0;
}

template <typename T>
int ensure_core(E2DSolver* h) {
  if (!h->adj) {
    h->adj = new E2DAdjoint();
    h->adj->prec = h->prec;
  }
  E2DAdjoint* A = h->adj;
  if (!A->st) {
    const size_t n = (size_t)4 * h->ncell;
    if (int e = adj_alloc_bytes(A, &A->st, sizeof(T) * ST_NSLOTS * n)) return e;
    if (int e = adj_alloc_bytes(A, &A->lam, sizeof(T) * n)) return e;
    if (int e = adj_alloc_bytes(A, reinterpret_cast<void**>(&A->J), sizeof(double))) return e;
    if (int e = adj_alloc_bytes(A, &A->final_state, sizeof(T) * ckpt_size<T>(h))) return e;
    if (sizeof(T) == 4)
      if (int e = adj_alloc_bytes(A, &A->io, sizeof(T) * 2 * n)) return e;
  }
  return 0;
}

// ---- launch helpers ---------------------------------------------------------------
template <typename T, int LIM>
cudaError_t recon_vjp_lim(E2DSolver* h, const T* Y, FaceArraysT<T> F, T* st) {
  const ParamsT<T>& P = path<T>(h).P;
  // tile table of height VTY = 4 (index 0 of the handle's tile set)
  static_assert(VTY == 4, "the reverse reconstruction runs on the height-4 tile table");
  const int4* tiles = h->ts.cell[0];
  const int n = h->ts.ncell[0];
  if (P.recon == E2D_RECON_PRIMITIVE)
    k_reconstruct_vjp<T, LIM, E2D_RECON_PRIMITIVE><<<n, TX * VTY, 0, h->stream>>>(P, tiles, Y, h->inst, F, st);
  else
    k_reconstruct_vjp<T, LIM, E2D_RECON_CONSERVATIVE><<<n, TX * VTY, 0, h->stream>>>(P, tiles, Y, h->inst, F, st);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reconstruct_vjp(E2DSolver* h, const T* Y, FaceArraysT<T> F, T* st) {
  switch (path<T>(h).P.limiter) {
    case E2D_LIM_BARTH_JESPERSEN: return recon_vjp_lim<T, E2D_LIM_BARTH_JESPERSEN>(h, Y, F, st);
    case E2D_LIM_VAN_ALBADA: return recon_vjp_lim<T, E2D_LIM_VAN_ALBADA>(h, Y, F, st);
    case E2D_LIM_VAN_LEER: return recon_vjp_lim<T, E2D_LIM_VAN_LEER>(h, Y, F, st);
    default: return recon_vjp_lim<T, E2D_LIM_VENKATAKRISHNAN>(h, Y, F, st);
  }
}

template <typename T>
cudaError_t launch_gather(E2DSolver* h, const T* Y, const T* st, T* lamU, const AdjProgramT<T>& prog) {
  const ParamsT<T>& P = path<T>(h).P;
  if (P.recon == E2D_RECON_PRIMITIVE)
    k_adjoint_gather<T, E2D_RECON_PRIMITIVE><<<h->ncell_tiles, TX * TY, 0, h->stream>>>(
        P, h->cell_tiles, Y, h->inst, st, lamU, prog);
  else
    k_adjoint_gather<T, E2D_RECON_CONSERVATIVE><<<h->ncell_tiles, TX * TY, 0, h->stream>>>(
        P, h->cell_tiles, Y, h->inst, st, lamU, prog);
  return cudaGetLastError();
}

// lamU += (dR/dY)^T lk, and acc[q] += coef[q] * (dR/dY)^T lk.  F holds the forward
// face states of R(Y) (overwritten).
template <typename T>
int residual_vjp(E2DSolver* h, const T* Y, FaceArraysT<T> F, const T* lk, T* lamU, const AdjProgramT<T>& prog) {
  E2DAdjoint* A = h->adj;
  const ParamsT<T>& P = path<T>(h).P;
  if (P.flux == E2D_FLUX_HLLL)
    k_flux_vjp<T, E2D_FLUX_HLLL><<<h->nface_tiles, TX * TY, 0, h->stream>>>(P, h->face_tiles, h->inst, F, lk);
  else if (P.flux == E2D_FLUX_HLLE)
    k_flux_vjp<T, E2D_FLUX_HLLE><<<h->nface_tiles, TX * TY, 0, h->stream>>>(P, h->face_tiles, h->inst, F, lk);
  else
    k_flux_vjp<T, E2D_FLUX_ROE><<<h->nface_tiles, TX * TY, 0, h->stream>>>(P, h->face_tiles, h->inst, F, lk);
  CK(cudaGetLastError());
  CK(launch_reconstruct_vjp<T>(h, Y, F, as<T>(A->st)));
  CK(launch_gather<T>(h, Y, as<T>(A->st), lamU, prog));
  return 0;
}

// One forward step of the plain path from buf[0] with the instance's dt; when
// stage_out/face_out are given, stage inputs and face states are kept there.
template <typename T>
int forward_step(E2DSolver* h, T* stage_out, T* face_out) {
  PathT<T>& p = path<T>(h);
  const size_t n = (size_t)4 * h->ncell;
  for (int s = 0; s < h->nstages; ++s) {
    const T* in = p.S.buf[h->stage_input[s]];
    FaceArraysT<T> F = p.F;
    if (sizeof(T) == 4 && h->use_fused(s)) {
      // FP32: one launch; kept for the reverse pass it records the stage's input and
      // face states, the same values the split kernels leave (FP64 recomputes split)
      FusedRecordT<T> rec{};
      if (stage_out) {
        F = face_slot<T>(h, face_out + (size_t)s * face_set_size(h));
        rec = FusedRecordT<T>{stage_out + (size_t)s * n, F.vL, F.vR, F.hL, F.hR};
      }
      CK(launch_stage_fused<T>(p.P, h->ts, h->ks.variant, in, h->inst, p.S, h->prog[s], h->real, h->stream,
                               h->tma_for(in), false, rec));
      continue;
    }
    if (stage_out) {
      T* Y = stage_out + (size_t)s * n;
      CK(cudaMemcpyAsync(Y, in, sizeof(T) * n, cudaMemcpyDeviceToDevice, h->stream));
      in = Y;
      F = face_slot<T>(h, face_out + (size_t)s * face_set_size(h));
    }
    CK(launch_reconstruct<T>(p.P, h->ts, h->kr, in, h->inst, F, nullptr, h->stream, h->tma_for(in)));
    CK(launch_flux<T>(p.P, h->ts, h->kf, h->inst, F, nullptr, h->stream));
    CK(launch_update<T>(p.P, h->ts, h->ku, F, p.S, h->prog[s], h->inst, h->real, nullptr, h->stream));
  }
  CK(launch_end_step(h->inst, 1, h->real, h->stream));
  return 0;
}

// state (+ Kahan planes) <-> a checkpoint slot
template <typename T>
int save_state(E2DSolver* h, T* dst) {
  PathT<T>& p = path<T>(h);
  const size_t n = (size_t)4 * h->ncell;
  CK(cudaMemcpyAsync(dst, p.S.buf[0], sizeof(T) * n, cudaMemcpyDeviceToDevice, h->stream));
  if (sizeof(T) == 4) CK(cudaMemcpyAsync(dst + n, p.S.comp, sizeof(T) * n, cudaMemcpyDeviceToDevice, h->stream));
  return 0;
}

template <typename T>
int load_state(E2DSolver* h, const T* src) {
  PathT<T>& p = path<T>(h);
  const size_t n = (size_t)4 * h->ncell;
  CK(cudaMemcpyAsync(p.S.buf[0], src, sizeof(T) * n, cudaMemcpyDeviceToDevice, h->stream));
  if (sizeof(T) == 4) CK(cudaMemcpyAsync(p.S.comp, src + n, sizeof(T) * n, cudaMemcpyDeviceToDevice, h->stream));
  return 0;
}

// Reverse of one RK step whose stage states and face states are stored:
// lam <- (dPhi/dU)^T lam.
template <typename T>
int adjoint_step(E2DSolver* h, const T* stages, T* faces, double dt) {
  E2DAdjoint* A = h->adj;
  const int S = h->nstages;
  const size_t n = (size_t)4 * h->ncell;
  const double* a = h->tableau.data();
  T* acc = as<T>(A->acc);
  T* lam = as<T>(A->lam);
  // acc[q] = dt * b_q * lam (b = last Butcher row)
  AdjProgramT<T> init{};
  init.n = S;
  for (int q = 0; q < S; ++q) {
    init.dst[q] = acc + (size_t)q * n;
    init.coef[q] = dt * a[(S - 1) * S + q];
  }
  k_adjoint_init<T><<<1024, 256, 0, h->stream>>>((int64_t)n, lam, init);
  CK(cudaGetLastError());
  for (int s = S - 1; s >= 0; --s) {
    // Y_s = U + dt * sum_{q<s} a[s-1][q] k_q: its adjoint feeds acc[q]
    AdjProgramT<T> prog{};
    prog.n = 0;
    if (s > 0)
      for (int q = 0; q < s; ++q) {
        const double c = a[(s - 1) * S + q];
        if (c == 0.0) continue;
        prog.dst[prog.n] = acc + (size_t)q * n;
        prog.coef[prog.n] = dt * c;
        ++prog.n;
      }
    FaceArraysT<T> F = face_slot<T>(h, faces + (size_t)s * face_set_size(h));
    if (int e = residual_vjp<T>(h, stages + (size_t)s * n, F, acc + (size_t)s * n, lam, prog)) return e;
  }
  return 0;
}

template <typename T>
int inject_objective(E2DSolver* h, const T* U, double coef) {
  E2DAdjoint* A = h->adj;
  const E2DBlock& B = h->hblocks[A->obj.block];
  const int n = (A->obj.side == E2D_E || A->obj.side == E2D_W) ? B.ny : B.nx;
  k_side_pressure_grad<T><<<(n + 127) / 128, 128, 0, h->stream>>>(path<T>(h).P, A->obj.block, A->obj.side, U, coef,
                                                                   as<T>(A->lam));
  CK(cudaGetLastError());
  return 0;
}

void reset_instance(E2DSolver* h, double t) {
  InstanceState& I = h->hinst[0];
  I.t = t;
  I.dt = 0.0;
  I.t_final = INFINITY;
  I.max_steps = 0x7fffffff;
  I.steps = 0;
  I.halted = 0;
  I.nbad = 0;
  I.active = 0;
  I.min_bits = 0x7ff0000000000000ULL;
}

__global__ void k_reset_realiz(RealizState* r) {
  r->first = ~0ULL;
  r->nbad = 0;
}

// FP64 caller buffer -> the path's type (FP32 staging slot 0 or 1) and back
const double* from_caller(E2DSolver*, const double* src, double*) { return src; }
const float* from_caller(E2DSolver* h, const double* src, float* stage) {
  launch_convert(src, stage, 4 * h->ncell, h->stream);
  return stage;
}

int to_caller(E2DSolver* h, const double* src, double* dst) {
  CK(cudaMemcpyAsync(dst, src, sizeof(double) * 4 * h->ncell, cudaMemcpyDeviceToDevice, h->stream));
  return 0;
}
int to_caller(E2DSolver* h, const float* src, double* dst) {
  CK(launch_convert(src, dst, 4 * h->ncell, h->stream));
  return 0;
}

template <typename T>
int residual_vjp_t(E2DSolver* h, double t, const double* lam_dev, double* out_dev) {
  if (int e = ensure_core<T>(h)) return e;
  PathT<T>& p = path<T>(h);
  const size_t n = (size_t)4 * h->ncell;
  CK(launch_set_time(h->inst, 1, t, 0.0, h->stream));
  T* io = as<T>(h->adj->io);  // null on the FP64 path
  const T* lk = from_caller(h, lam_dev, io);
  T* out = sizeof(T) == 8 ? reinterpret_cast<T*>(out_dev) : io + n;
  CK(cudaMemsetAsync(out, 0, sizeof(T) * n, h->stream));
  CK(launch_reconstruct<T>(p.P, h->ts, h->kr, p.S.buf[0], h->inst, p.F, nullptr, h->stream,
                           h->tma_for(p.S.buf[0])));
  AdjProgramT<T> none{};
  if (int e = residual_vjp<T>(h, p.S.buf[0], p.F, lk, out, none)) return e;
  if (sizeof(T) == 4)
    if (int e = to_caller(h, out, out_dev)) return e;
  CK(launch_end_step(h->inst, 1, h->real, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

template <typename T>
int adjoint_forward_t(E2DSolver* h, double t0, int32_t nsteps, int32_t ckpt_every, const E2DPressureObjective* obj,
                      const double* dts_in, double* dts_out, double* J_out) {
  if (int e = ensure_core<T>(h)) return e;
  E2DAdjoint* A = h->adj;
  PathT<T>& p = path<T>(h);
  const size_t n = (size_t)4 * h->ncell, nc = ckpt_size<T>(h);
  const int N = nsteps, K = ckpt_every < nsteps ? ckpt_every : nsteps, S = h->nstages;
  const size_t nck = (size_t)(N + K - 1) / K;
  if (nck > A->cap_ckpt) {
    if (int e = adj_alloc_bytes(A, &A->ckpt, sizeof(T) * nck * nc)) return e;
    A->cap_ckpt = nck;
  }
  if ((size_t)K * S > A->cap_seg) {
    if (int e = adj_alloc_bytes(A, &A->stage, sizeof(T) * (size_t)K * S * n)) return e;
    if (int e = adj_alloc_bytes(A, &A->face, sizeof(T) * (size_t)K * S * face_set_size(h))) return e;
    A->cap_seg = (size_t)K * S;
  }
  if ((size_t)S > A->cap_acc) {
    if (int e = adj_alloc_bytes(A, &A->acc, sizeof(T) * (size_t)S * n)) return e;
    A->cap_acc = S;
  }
  if ((size_t)N > A->cap_rec) {
    if (int e = adj_alloc_bytes(A, reinterpret_cast<void**>(&A->rec), sizeof(double) * 2 * (size_t)N)) return e;
    A->cap_rec = N;
  }
  A->nsteps = N;
  A->K = K;
  A->S = S;
  A->obj = *obj;
  A->recorded = false;
  h->drop_graphs();

  reset_instance(h, t0);
  CK(cudaMemcpyAsync(h->inst, h->hinst.data(), sizeof(InstanceState), cudaMemcpyHostToDevice, h->stream));
  k_reset_realiz<<<1, 1, 0, h->stream>>>(h->real);
  CK(cudaMemsetAsync(A->J, 0, sizeof(double), h->stream));
  double t = t0;
  for (int s = 0; s < N; ++s) {
    if (s % K == 0)
      if (int e = save_state<T>(h, as<T>(A->ckpt) + (size_t)(s / K) * nc)) return e;
    if (dts_in) {
      CK(launch_set_time(h->inst, 1, t, dts_in[s], h->stream));
      t = t + dts_in[s];
    } else {
      CK(launch_dt<T>(p.P, h->cell_tiles, h->ncell_tiles, p.S.buf[0], h->inst, h->stream));
      CK(launch_begin_step(h->inst, 1, p.P.cfl, 1, h->stream));
    }
    k_record_step<<<1, 1, 0, h->stream>>>(h->inst, A->rec, A->rec + N, s);
    CK(cudaGetLastError());
    if (int e = forward_step<T>(h, nullptr, nullptr)) return e;
    k_side_pressure<T><<<1, OBJ_THREADS, 0, h->stream>>>(p.P, obj->block, obj->side, p.S.buf[0], h->inst, A->J);
    CK(cudaGetLastError());
  }
  A->dts.resize(N);
  A->ts.resize(N);
  CK(cudaMemcpyAsync(A->dts.data(), A->rec, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(A->ts.data(), A->rec + N, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
  if (int e = save_state<T>(h, as<T>(A->final_state))) return e;
  double J = 0.0;
  CK(cudaMemcpyAsync(&J, A->J, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  RealizState r;
  CK(cudaMemcpyAsync(&r, h->real, sizeof r, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (r.nbad) return fail(E2D_ERR_UNREALIZABLE, "unrealizable state during the recorded forward pass");
  if (dts_out) std::memcpy(dts_out, A->dts.data(), sizeof(double) * N);
  if (J_out) *J_out = J;
  A->recorded = true;
  return 0;
}

template <typename T>
int adjoint_backward_t(E2DSolver* h, double* grad_dev) {
  E2DAdjoint* A = h->adj;
  const size_t n = (size_t)4 * h->ncell, nc = ckpt_size<T>(h);
  const int N = A->nsteps, K = A->K, S = A->S;
  if (S != h->nstages) return fail(E2D_ERR_INVALID, "tableau changed since the forward pass");
  T* lam = as<T>(A->lam);
  T* stage = as<T>(A->stage);
  T* face = as<T>(A->face);
  // lam = dt_{N-1} dP/dU (U^N)
  CK(cudaMemsetAsync(lam, 0, sizeof(T) * n, h->stream));
  if (int e = inject_objective<T>(h, as<T>(A->final_state), A->dts[N - 1])) return e;
  const int nseg = (N + K - 1) / K;
  for (int g = nseg - 1; g >= 0; --g) {
    const int n0 = g * K, n1 = (n0 + K < N) ? n0 + K : N;
    // recompute the segment from its checkpoint, keeping stage and face states
    if (int e = load_state<T>(h, as<T>(A->ckpt) + (size_t)g * nc)) return e;
    for (int s = n0; s < n1; ++s) {
      CK(launch_set_time(h->inst, 1, A->ts[s], A->dts[s], h->stream));
      const size_t slot = (size_t)(s - n0) * S;
      if (int e = forward_step<T>(h, stage + slot * n, face + slot * face_set_size(h))) return e;
    }
    for (int s = n1 - 1; s >= n0; --s) {
      CK(launch_set_time(h->inst, 1, A->ts[s], A->dts[s], h->stream));
      const size_t slot = (size_t)(s - n0) * S;
      const T* stages = stage + slot * n;
      if (int e = adjoint_step<T>(h, stages, face + slot * face_set_size(h), A->dts[s])) return e;
      // U^s = the first stage state of step s enters J through step s-1
      if (s >= 1)
        if (int e = inject_objective<T>(h, stages, A->dts[s - 1])) return e;
    }
  }
  CK(launch_end_step(h->inst, 1, h->real, h->stream));
  if (int e = to_caller(h, lam, grad_dev)) return e;
  if (int e = load_state<T>(h, as<T>(A->final_state))) return e;
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

}  // namespace

extern "C" {

int e2d_residual_vjp(E2DHandle h, double t, const double* lam_dev, double* out_dev) {
  if (!h || !lam_dev || !out_dev) return fail(E2D_ERR_INVALID, "null argument");
  if (int e = check_supported(h)) return e;
  return E2D_DISPATCH(h, residual_vjp_t, t, lam_dev, out_dev);
}

int e2d_adjoint_forward(E2DHandle h, double t0, int32_t nsteps, int32_t ckpt_every, const E2DPressureObjective* obj,
                        const double* dts_in, double* dts_out, double* J_out) {
  if (!h || !obj || nsteps < 1 || ckpt_every < 1) return fail(E2D_ERR_INVALID, "bad argument");
  if (int e = check_supported(h)) return e;
  if (obj->block < 0 || obj->block >= h->cfg.nblocks || obj->side < 0 || obj->side > 3)
    return fail(E2D_ERR_INVALID, "objective block %d side %d out of range", obj->block, obj->side);
  return E2D_DISPATCH(h, adjoint_forward_t, t0, nsteps, ckpt_every, obj, dts_in, dts_out, J_out);
}

int e2d_adjoint_backward(E2DHandle h, double* grad_dev) {
  if (!h || !grad_dev) return fail(E2D_ERR_INVALID, "null argument");
  if (!h->adj || !h->adj->recorded) return fail(E2D_ERR_INVALID, "no recorded forward pass");
  return E2D_DISPATCH(h, adjoint_backward_t, grad_dev);
}

}  // extern "C"
