// e2d_adjoint.cu - reverse mode of the time loop: the residual VJP, the RK step
// adjoint and the checkpointed forward/backward passes of a boundary-pressure
// objective (include/euler2d.h, "adjoint").  The reference has no counterpart; the
// forward steps are the plain path's own kernels, so a recomputed segment repeats
// the recorded forward pass value for value.
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
}

using namespace e2d;

// Storage of one recorded forward pass (FP64 path).
struct E2DAdjoint {
  int nsteps = 0, K = 0, S = 0;
  E2DPressureObjective obj{};
  std::vector<double> dts, ts;  // per step: dt and the time at its start
  bool recorded = false;
  // device
  double* ckpt = nullptr;    // ceil(N/K) states
  double* final_state = nullptr;
  double* stage = nullptr;   // K*S stage states of the segment being reversed
  double* face = nullptr;    // K*S face-state sets (vL, vR, hL, hR)
  double* lam = nullptr;     // adjoint of the state
  double* acc = nullptr;     // S stage-residual adjoints
  double* st = nullptr;      // 5 stencil slots x 4 planes
  double* rec = nullptr;     // dts, ts recorded on the device (2N)
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

template <typename T>
int adj_alloc(E2DAdjoint* A, T** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess)
    return fail(E2D_ERR_NOMEM, "adjoint storage: cudaMalloc(%zu bytes): %s", sizeof(T) * count, cudaGetErrorString(e));
  A->allocs.push_back(q);
  *p = static_cast<T*>(q);
  return 0;
}

int64_t face_set_size(const E2DSolver* h) { return 8 * h->nvface + 8 * h->nhface; }

FaceArraysT<double> face_slot(E2DSolver* h, double* base) {
  FaceArraysT<double> F = h->pd.F;  // vI, hI stay the path's own
  F.vL = base;
  F.vR = base + 4 * h->nvface;
  F.hL = base + 8 * h->nvface;
  F.hR = base + 8 * h->nvface + 4 * h->nhface;
  return F;
}

int check_supported(E2DSolver* h) {
  if (h->prec != E2D_FP64) return fail(E2D_ERR_UNSUPPORTED, "the adjoint runs on the FP64 path");
  if (h->cfg.flux != E2D_FLUX_ROE) return fail(E2D_ERR_UNSUPPORTED, "the adjoint supports the Roe flux");
  if (h->hinst.size() != 1) return fail(E2D_ERR_UNSUPPORTED, "the adjoint runs on single-instance problems");
  if (h->nstages < 1) return fail(E2D_ERR_INVALID, "no tableau set");
  return 0;
}

int ensure_core(E2DSolver* h) {
  if (!h->adj) h->adj = new E2DAdjoint();
  E2DAdjoint* A = h->adj;
  if (!A->st) {
    if (int e = adj_alloc(A, &A->st, (size_t)ST_NSLOTS * 4 * h->ncell)) return e;
    if (int e = adj_alloc(A, &A->lam, (size_t)4 * h->ncell)) return e;
    if (int e = adj_alloc(A, &A->J, 1)) return e;
    if (int e = adj_alloc(A, &A->final_state, (size_t)4 * h->ncell)) return e;
  }
  return 0;
}

// ---- launch helpers ---------------------------------------------------------------
template <int LIM>
cudaError_t recon_vjp_lim(E2DSolver* h, const double* Y, FaceArraysT<double> F, double* st) {
  const ParamsT<double>& P = h->pd.P;
  if (P.recon == E2D_RECON_PRIMITIVE)
    k_reconstruct_vjp<double, LIM, E2D_RECON_PRIMITIVE><<<h->ncell_tiles, TX * TY, 0, h->stream>>>(
        P, h->cell_tiles, Y, h->inst, F, st);
  else
    k_reconstruct_vjp<double, LIM, E2D_RECON_CONSERVATIVE><<<h->ncell_tiles, TX * TY, 0, h->stream>>>(
        P, h->cell_tiles, Y, h->inst, F, st);
  return cudaGetLastError();
}

cudaError_t launch_reconstruct_vjp(E2DSolver* h, const double* Y, FaceArraysT<double> F, double* st) {
  switch (h->pd.P.limiter) {
    case E2D_LIM_BARTH_JESPERSEN: return recon_vjp_lim<E2D_LIM_BARTH_JESPERSEN>(h, Y, F, st);
    case E2D_LIM_VAN_ALBADA: return recon_vjp_lim<E2D_LIM_VAN_ALBADA>(h, Y, F, st);
    case E2D_LIM_VAN_LEER: return recon_vjp_lim<E2D_LIM_VAN_LEER>(h, Y, F, st);
    default: return recon_vjp_lim<E2D_LIM_VENKATAKRISHNAN>(h, Y, F, st);
  }
}

cudaError_t launch_gather(E2DSolver* h, const double* Y, const double* st, double* lamU,
                          const AdjProgramT<double>& prog) {
  const ParamsT<double>& P = h->pd.P;
  if (P.recon == E2D_RECON_PRIMITIVE)
    k_adjoint_gather<double, E2D_RECON_PRIMITIVE><<<h->ncell_tiles, TX * TY, 0, h->stream>>>(
        P, h->cell_tiles, Y, h->inst, st, lamU, prog);
  else
    k_adjoint_gather<double, E2D_RECON_CONSERVATIVE><<<h->ncell_tiles, TX * TY, 0, h->stream>>>(
        P, h->cell_tiles, Y, h->inst, st, lamU, prog);
  return cudaGetLastError();
}

// lamU += (dR/dY)^T lk, and acc[q] += coef[q] * (dR/dY)^T lk.  F holds the forward
// face states of R(Y) (overwritten).
int residual_vjp(E2DSolver* h, const double* Y, FaceArraysT<double> F, const double* lk, double* lamU,
                 const AdjProgramT<double>& prog) {
  E2DAdjoint* A = h->adj;
  k_flux_vjp<double><<<h->nface_tiles, TX * TY, 0, h->stream>>>(h->pd.P, h->face_tiles, h->inst, F, lk);
  CK(cudaGetLastError());
  CK(launch_reconstruct_vjp(h, Y, F, A->st));
  CK(launch_gather(h, Y, A->st, lamU, prog));
  return 0;
}

// One forward step of the plain path from buf[0] with the instance's dt; when
// stage_out/face_out are given, stage inputs and face states are kept there.
int forward_step(E2DSolver* h, double* stage_out, double* face_out) {
  PathT<double>& p = h->pd;
  const size_t n = (size_t)4 * h->ncell;
  for (int s = 0; s < h->nstages; ++s) {
    const double* in = p.S.buf[h->stage_input[s]];
    FaceArraysT<double> F = p.F;
    if (stage_out) {
      double* Y = stage_out + (size_t)s * n;
      CK(cudaMemcpyAsync(Y, in, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
      in = Y;
      F = face_slot(h, face_out + (size_t)s * face_set_size(h));
    }
    CK(launch_reconstruct<double>(p.P, h->ts, h->kr, in, h->inst, F, nullptr, h->stream));
    CK(launch_flux<double>(p.P, h->ts, h->kf, h->inst, F, nullptr, h->stream));
    CK(launch_update<double>(p.P, h->ts, h->ku, F, p.S, h->prog[s], h->inst, h->real, nullptr, h->stream));
  }
  CK(launch_end_step(h->inst, 1, h->real, h->stream));
  return 0;
}

// Reverse of one RK step whose stage states and face states are stored:
// lam <- (dPhi/dU)^T lam.
int adjoint_step(E2DSolver* h, const double* stages, double* faces, double dt) {
  E2DAdjoint* A = h->adj;
  const int S = h->nstages;
  const size_t n = (size_t)4 * h->ncell;
  const double* a = h->tableau.data();
  // acc[q] = dt * b_q * lam (b = last Butcher row)
  AdjProgramT<double> init{};
  init.n = S;
  for (int q = 0; q < S; ++q) {
    init.dst[q] = A->acc + (size_t)q * n;
    init.coef[q] = dt * a[(S - 1) * S + q];
  }
  k_adjoint_init<double><<<1024, 256, 0, h->stream>>>((int64_t)n, A->lam, init);
  CK(cudaGetLastError());
  for (int s = S - 1; s >= 0; --s) {
    // Y_s = U + dt * sum_{q<s} a[s-1][q] k_q: its adjoint feeds acc[q]
    AdjProgramT<double> prog{};
    prog.n = 0;
    if (s > 0)
      for (int q = 0; q < s; ++q) {
        const double c = a[(s - 1) * S + q];
        if (c == 0.0) continue;
        prog.dst[prog.n] = A->acc + (size_t)q * n;
        prog.coef[prog.n] = dt * c;
        ++prog.n;
      }
    FaceArraysT<double> F = face_slot(h, faces + (size_t)s * face_set_size(h));
    if (int e = residual_vjp(h, stages + (size_t)s * n, F, A->acc + (size_t)s * n, A->lam, prog)) return e;
  }
  return 0;
}

int inject_objective(E2DSolver* h, const double* U, double coef) {
  E2DAdjoint* A = h->adj;
  const E2DBlock& B = h->hblocks[A->obj.block];
  const int n = (A->obj.side == E2D_E || A->obj.side == E2D_W) ? B.ny : B.nx;
  k_side_pressure_grad<double><<<(n + 127) / 128, 128, 0, h->stream>>>(h->pd.P, A->obj.block, A->obj.side, U, coef,
                                                                        A->lam);
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

}  // namespace

extern "C" {

int e2d_residual_vjp(E2DHandle h, double t, const double* lam_dev, double* out_dev) {
  if (!h || !lam_dev || !out_dev) return fail(E2D_ERR_INVALID, "null argument");
  if (int e = check_supported(h)) return e;
  if (int e = ensure_core(h)) return e;
  PathT<double>& p = h->pd;
  CK(launch_set_time(h->inst, 1, t, 0.0, h->stream));
  CK(cudaMemsetAsync(out_dev, 0, sizeof(double) * 4 * h->ncell, h->stream));
  CK(launch_reconstruct<double>(p.P, h->ts, h->kr, p.S.buf[0], h->inst, p.F, nullptr, h->stream));
  AdjProgramT<double> none{};
  if (int e = residual_vjp(h, p.S.buf[0], p.F, lam_dev, out_dev, none)) return e;
  CK(launch_end_step(h->inst, 1, h->real, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int e2d_adjoint_forward(E2DHandle h, double t0, int32_t nsteps, int32_t ckpt_every, const E2DPressureObjective* obj,
                        const double* dts_in, double* dts_out, double* J_out) {
  if (!h || !obj || nsteps < 1 || ckpt_every < 1) return fail(E2D_ERR_INVALID, "bad argument");
  if (int e = check_supported(h)) return e;
  if (obj->block < 0 || obj->block >= h->cfg.nblocks || obj->side < 0 || obj->side > 3)
    return fail(E2D_ERR_INVALID, "objective block %d side %d out of range", obj->block, obj->side);
  if (int e = ensure_core(h)) return e;
  E2DAdjoint* A = h->adj;
  PathT<double>& p = h->pd;
  const size_t n = (size_t)4 * h->ncell;
  const int N = nsteps, K = ckpt_every < nsteps ? ckpt_every : nsteps, S = h->nstages;
  const size_t nck = (size_t)(N + K - 1) / K;
  if (nck > A->cap_ckpt) {
    if (int e = adj_alloc(A, &A->ckpt, nck * n)) return e;
    A->cap_ckpt = nck;
  }
  if ((size_t)K * S > A->cap_seg) {
    if (int e = adj_alloc(A, &A->stage, (size_t)K * S * n)) return e;
    if (int e = adj_alloc(A, &A->face, (size_t)K * S * face_set_size(h))) return e;
    A->cap_seg = (size_t)K * S;
  }
  if ((size_t)S > A->cap_acc) {
    if (int e = adj_alloc(A, &A->acc, (size_t)S * n)) return e;
    A->cap_acc = S;
  }
  if ((size_t)N > A->cap_rec) {
    if (int e = adj_alloc(A, &A->rec, 2 * (size_t)N)) return e;
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
      CK(cudaMemcpyAsync(A->ckpt + (size_t)(s / K) * n, p.S.buf[0], sizeof(double) * n, cudaMemcpyDeviceToDevice,
                         h->stream));
    if (dts_in) {
      CK(launch_set_time(h->inst, 1, t, dts_in[s], h->stream));
      t = t + dts_in[s];
    } else {
      CK(launch_dt<double>(p.P, h->cell_tiles, h->ncell_tiles, p.S.buf[0], h->inst, h->stream));
      CK(launch_begin_step(h->inst, 1, p.P.cfl, 1, h->stream));
    }
    k_record_step<<<1, 1, 0, h->stream>>>(h->inst, A->rec, A->rec + N, s);
    CK(cudaGetLastError());
    if (int e = forward_step(h, nullptr, nullptr)) return e;
    k_side_pressure<double><<<1, OBJ_THREADS, 0, h->stream>>>(p.P, obj->block, obj->side, p.S.buf[0], h->inst, A->J);
    CK(cudaGetLastError());
  }
  A->dts.resize(N);
  A->ts.resize(N);
  CK(cudaMemcpyAsync(A->dts.data(), A->rec, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(A->ts.data(), A->rec + N, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(A->final_state, p.S.buf[0], sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
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

int e2d_adjoint_backward(E2DHandle h, double* grad_dev) {
  if (!h || !grad_dev) return fail(E2D_ERR_INVALID, "null argument");
  if (!h->adj || !h->adj->recorded) return fail(E2D_ERR_INVALID, "no recorded forward pass");
  E2DAdjoint* A = h->adj;
  PathT<double>& p = h->pd;
  const size_t n = (size_t)4 * h->ncell;
  const int N = A->nsteps, K = A->K, S = A->S;
  if (S != h->nstages) return fail(E2D_ERR_INVALID, "tableau changed since the forward pass");
  // lam = dt_{N-1} dP/dU (U^N)
  CK(cudaMemsetAsync(A->lam, 0, sizeof(double) * n, h->stream));
  if (int e = inject_objective(h, A->final_state, A->dts[N - 1])) return e;
  const int nseg = (N + K - 1) / K;
  for (int g = nseg - 1; g >= 0; --g) {
    const int n0 = g * K, n1 = (n0 + K < N) ? n0 + K : N;
    // recompute the segment from its checkpoint, keeping stage and face states
    CK(cudaMemcpyAsync(p.S.buf[0], A->ckpt + (size_t)g * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    for (int s = n0; s < n1; ++s) {
      CK(launch_set_time(h->inst, 1, A->ts[s], A->dts[s], h->stream));
      const size_t slot = (size_t)(s - n0) * S;
      if (int e = forward_step(h, A->stage + slot * n, A->face + slot * face_set_size(h))) return e;
    }
    for (int s = n1 - 1; s >= n0; --s) {
      CK(launch_set_time(h->inst, 1, A->ts[s], A->dts[s], h->stream));
      const size_t slot = (size_t)(s - n0) * S;
      const double* stages = A->stage + slot * n;
      if (int e = adjoint_step(h, stages, A->face + slot * face_set_size(h), A->dts[s])) return e;
      // U^s = the first stage state of step s enters J through step s-1
      if (s >= 1)
        if (int e = inject_objective(h, stages, A->dts[s - 1])) return e;
    }
  }
  CK(launch_end_step(h->inst, 1, h->real, h->stream));
  CK(cudaMemcpyAsync(grad_dev, A->lam, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(p.S.buf[0], A->final_state, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

}  // extern "C"
