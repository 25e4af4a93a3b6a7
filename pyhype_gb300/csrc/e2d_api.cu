// e2d_api.cu - the C ABI declared in include/euler2d.h.
//
// A handle owns, in one GPU's memory: the block table, the geometry planes, the
// tile tables that map CTAs to (block, tile), the state buffers of the RK stage
// program, the face-indexed L/R state and flux arrays, and the per-instance time
// state.  Host calls enqueue work on the handle's stream; a time loop can be
// replayed from a captured CUDA graph because dt and t live on the device.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

#include <mutex>

#include "e2d_solver.cuh"
#include "../../include/euler2d_bench.h"

using namespace e2d;

namespace {

thread_local std::string g_err;

__global__ void k_reset_min(InstanceState* inst, int n) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) inst[q].min_bits = 0x7ff0000000000000ULL;
}

__global__ void k_reset_real(RealizState* r) {
  r->first = ~0ULL;
  r->nbad = 0;
}

}  // namespace

namespace e2d {
int set_error(int code, const char* msg) {
  g_err = msg;
  return code;
}
}  // namespace e2d

// Stage program of a Butcher tableau (rows = stages; row s uses k_0..k_s).  Buffer 0
// holds U^n and, after the last stage, U^{n+1}; buffer r+1 holds row r's partial sum
// for r < S-1; buffer S holds the last row's partial sum until the last stage.  Each
// stage adds dt*a[r][s]*k_s to every row r >= s with a nonzero coefficient, in
// increasing s, which is the reference's summation order
// (explicit_runge_kutta.py:63-80).
// On the FP32 path the last row is formed as an increment (from zero) that the last
// stage adds to U^n with Kahan compensation, instead of as U^n + terms.
static int build_program(E2DSolver* h, int S, const double* a) {
  const bool kahan = h->prec == E2D_FP32;
  if (S < 1 || S > MAX_STAGES) return fail(E2D_ERR_INVALID, "nstages must be in [1, %d]", MAX_STAGES);
  h->prog.assign(S, StageProgram{});
  h->stage_input.assign(S, 0);
  auto row_buf = [&](int r) { return r == S - 1 ? S : r + 1; };
  std::vector<int> started(S, 0);
  for (int s = 0; s < S; ++s) {
    // input of stage s: row s-1's buffer if it has any term, else U^n
    if (s > 0) {
      bool any = false;
      for (int j = 0; j < s; ++j) any = any || a[(s - 1) * S + j] != 0.0;
      h->stage_input[s] = any ? row_buf(s - 1) : 0;
    }
    StageProgram& p = h->prog[s];
    p.nupd = 0;
    p.final_stage = (s == S - 1);
    for (int r = s; r < S; ++r) {
      double c = a[r * S + s];
      if (c == 0.0) continue;
      StageUpdate u{};
      u.a = c;
      u.src = started[r] ? row_buf(r) : 0;
      u.dst = (r == S - 1 && s == S - 1) ? 0 : row_buf(r);
      if (kahan && r == S - 1) {
        u.src_zero = !started[r];
        u.kahan = (s == S - 1);
        u.dst = row_buf(r);
      }
      started[r] = 1;
      p.upd[p.nupd++] = u;
    }
    if (s == S - 1) {
      // the final row's last term may sit in an earlier column: then U^{n+1} is the
      // finished partial sum (or U^n itself if the row is all zeros)
      bool wrote0 = false;
      for (int u = 0; u < p.nupd; ++u) wrote0 = wrote0 || p.upd[u].dst == 0 || p.upd[u].kahan;
      if (!wrote0 && started[S - 1]) {
        if (p.nupd >= MAX_STAGES) return fail(E2D_ERR_INVALID, "stage program overflow");
        StageUpdate u{};
        u.a = 0.0;
        u.src = row_buf(S - 1);
        u.dst = kahan ? row_buf(S - 1) : 0;
        u.kahan = kahan;
        p.upd[p.nupd++] = u;  // dta = 0: exact copy for finite k
      }
    }
  }
  // A stage may run fused when none of its updates writes the buffer it reads as input
  // (a fused tile would overwrite cells its neighbours still read as halo).  The FP32
  // Kahan update writes buffer 0 (and the compensation).
  h->fusable.assign(S, 1);
  for (int s = 0; s < S; ++s)
    for (int u = 0; u < h->prog[s].nupd; ++u) {
      const StageUpdate& up = h->prog[s].upd[u];
      if (up.dst == h->stage_input[s] || (up.kahan && h->stage_input[s] == 0)) h->fusable[s] = 0;
    }
  h->nstages = S;
  return 0;
}

// ---- TMA tensor maps ----------------------------------------------------------------
// cuTensorMapEncodeTiled from the driver, looked up once through the runtime (no link
// against libcuda); null when the driver does not offer it, and then every tile takes
// plain loads.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// Tensor maps of one state buffer for the reconstruction kernel's interior tiles, at
// the three tile heights: per block a 3-D map (x = column, y = row, z = the 4 planes)
// whose box is the tile, its one-cell halo and the alignment columns.  A block whose
// row stride, plane stride or base is not a multiple of 16 bytes gets ok = 0.
template <typename T>
static int build_tma_t(E2DSolver* h, const T* base) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return 0;
  const int nb = (int)h->hblocks.size();
  // box rows: tile height + the 1-cell halo for the reconstruction kernel's tiles, and
  // the fused stage kernel's tile rows + its 2-cell halo
  const int box_rows[5] = {4 + 2, 8 + 2, 16 + 2, FUSED_TY[0] + 4, FUSED_TY[1] + 4};
  E2DSolver::TmaEntry entry{base, {}};
  std::vector<CUtensorMap> maps(nb);
  std::vector<int> ok(nb);
  for (int r = 0; r < 5; ++r) {
    for (int b = 0; b < nb; ++b) {
      const E2DBlock& B = h->hblocks[b];
      const uint64_t row = (uint64_t)B.nx * sizeof(T), plane = (uint64_t)h->ncell * sizeof(T);
      const T* addr = base + B.cell_offset;
      bool good = row % 16 == 0 && plane % 16 == 0 && (reinterpret_cast<uintptr_t>(addr) % 16) == 0 &&
                  B.nx > TX && B.ny >= box_rows[r];
      std::memset(&maps[b], 0, sizeof(CUtensorMap));
      if (good) {
        const cuuint64_t dims[3] = {(cuuint64_t)B.nx, (cuuint64_t)B.ny, 4};
        const cuuint64_t strides[2] = {row, plane};
        const cuuint32_t box[3] = {(cuuint32_t)TileCols<T>::TXW, (cuuint32_t)box_rows[r], 4};
        const cuuint32_t estr[3] = {1, 1, 1};
        const CUresult cr = enc(&maps[b], sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                                3, const_cast<T*>(addr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        good = cr == CUDA_SUCCESS;
        if (!good) std::memset(&maps[b], 0, sizeof(CUtensorMap));
      }
      ok[b] = good ? 1 : 0;
    }
    CUtensorMap* dmaps = nullptr;
    int* dok = nullptr;
    if (int e = h->alloc(&dmaps, nb)) return e;
    if (int e = h->alloc(&dok, nb)) return e;
    CK(cudaMemcpy(dmaps, maps.data(), sizeof(CUtensorMap) * nb, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dok, ok.data(), sizeof(int) * nb, cudaMemcpyHostToDevice));
    (r < 3 ? entry.set.by_rty[r] : entry.set.fused[r - 3]) = TmaTiles{dmaps, dok, h->tma_timeouts};
  }
  h->tma_reg.push_back(entry);
  return 0;
}

// Bounded TMA waits that ran out since the last check (the kernel drops those tiles).
static int check_tma(E2DSolver* h) {
  if (!h->tma_timeouts) return 0;
  unsigned long long n = 0;
  CK(cudaMemcpyAsync(&n, h->tma_timeouts, sizeof n, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (!n) return 0;
  CK(cudaMemsetAsync(h->tma_timeouts, 0, sizeof n, h->stream));
  return fail(E2D_ERR_CUDA, "%llu TMA tile load(s) did not arrive within the wait bound", n);
}

template <typename T>
static int ensure_buffers_t(E2DSolver* h) {
  PathT<T>& p = path<T>(h);
  int need = h->nstages + 1;
  for (int b = h->nbuf; b < need; ++b) {
    if (int e = h->alloc(&p.S.buf[b], 4 * (size_t)h->ncell)) return e;
    if (b > 0) CK(cudaMemsetAsync(p.S.buf[b], 0, sizeof(T) * 4 * h->ncell, h->stream));
    if (int e = build_tma_t<T>(h, p.S.buf[b])) return e;
  }
  if (need > h->nbuf) h->nbuf = need;
  h->drop_graphs();
  return 0;
}

static int ensure_buffers(E2DSolver* h) { return E2D_DISPATCH(h, ensure_buffers_t); }

// Geometry planes in the path's type: one allocation, planes back to back.  The FP32
// path rounds the FP64 host planes once.
template <typename T>
static int upload_geometry(E2DSolver* h, const E2DGeometry* geo) {
  PathT<T>& p = path<T>(h);
  const int64_t ncell = h->ncell, nv = h->nvface, nh = h->nhface;
  const int nqp = h->cfg.nqp > 1 ? h->cfg.nqp : 1;
  const size_t nq = nqp > 1 ? (size_t)8 * nqp * ncell : 0;
  const size_t ngeo = (size_t)E2D_G_NCELL * ncell + (size_t)E2D_F_NFACE * (nv + nh) + nq;
  if (int e = h->alloc(&p.geo, ngeo)) return e;
  std::vector<T> tmp;
  auto put = [&](T* dst, const double* src, int64_t n) -> int {
    const void* from = src;
    if (sizeof(T) != sizeof(double)) {
      tmp.resize(n);
      for (int64_t i = 0; i < n; ++i) tmp[i] = (T)src[i];
      from = tmp.data();
    }
    CK(cudaMemcpy(dst, from, sizeof(T) * n, cudaMemcpyHostToDevice));
    return 0;
  };
  T* q = p.geo;
  for (int k = 0; k < E2D_G_NCELL; ++k, q += ncell) {
    if (int e = put(q, geo->cell[k], ncell)) return e;
    p.P.geo.cell[k] = q;
  }
  for (int k = 0; k < E2D_F_NFACE; ++k, q += nv) {
    if (int e = put(q, geo->vface[k], nv)) return e;
    p.P.geo.vface[k] = q;
  }
  for (int k = 0; k < E2D_F_NFACE; ++k, q += nh) {
    if (int e = put(q, geo->hface[k], nh)) return e;
    p.P.geo.hface[k] = q;
  }
  // FP32 form: blocks whose face frames are axis-aligned to FP32's resolution
  p.P.axis32 = nullptr;
  h->axis32.assign(h->hblocks.size(), 0);
  if (sizeof(T) == 4) {
    const float eps = 0x1p-24f;
    for (size_t b = 0; b < h->hblocks.size(); ++b) {
      const E2DBlock& B = h->hblocks[b];
      bool ok = true;
      for (int64_t f = B.vface_offset; ok && f < B.vface_offset + (int64_t)B.ny * (B.nx + 1); ++f)
        ok = (float)geo->vface[E2D_F_COS][f] == 1.0f && std::fabs((float)geo->vface[E2D_F_SIN][f]) < eps;
      for (int64_t f = B.hface_offset; ok && f < B.hface_offset + (int64_t)(B.ny + 1) * B.nx; ++f)
        ok = (float)geo->hface[E2D_F_SIN][f] == 1.0f && std::fabs((float)geo->hface[E2D_F_COS][f]) < eps;
      h->axis32[b] = ok ? 1 : 0;
    }
    int* d = nullptr;
    if (int e = h->alloc(&d, h->axis32.size())) return e;
    CK(cudaMemcpy(d, h->axis32.data(), sizeof(int) * h->axis32.size(), cudaMemcpyHostToDevice));
    p.P.axis32 = d;
  }
  for (int qi = 0; qi < E2D_MAX_QP; ++qi)
    for (int k = 0; k < 8; ++k) p.P.geo.qp[qi][k] = nullptr;
  if (nqp > 1)
    for (int qi = 0; qi < nqp; ++qi)
      for (int k = 0; k < 8; ++k, q += ncell) {
        if (!geo->qp[qi][k]) return fail(E2D_ERR_INVALID, "quadrature point %d plane %d missing", qi, k);
        if (int e = put(q, geo->qp[qi][k], ncell)) return e;
        p.P.geo.qp[qi][k] = q;
      }
  return 0;
}

// Face arrays, the Kahan compensation (FP32) and the scalar parameters of a path.
template <typename T>
static int init_path(E2DSolver* h) {
  PathT<T>& p = path<T>(h);
  const int64_t nv = h->nvface, nh = h->nhface;
  const int nqp = h->cfg.nqp > 1 ? h->cfg.nqp : 1;
  if (int e = h->alloc(&p.F.vL, 4 * (size_t)nqp * nv)) return e;
  if (int e = h->alloc(&p.F.vR, 4 * (size_t)nqp * nv)) return e;
  if (int e = h->alloc(&p.F.vI, 4 * (size_t)nv)) return e;
  if (int e = h->alloc(&p.F.hL, 4 * (size_t)nqp * nh)) return e;
  if (int e = h->alloc(&p.F.hR, 4 * (size_t)nqp * nh)) return e;
  if (int e = h->alloc(&p.F.hI, 4 * (size_t)nh)) return e;
  p.S.comp = nullptr;
  if (h->prec == E2D_FP32) {
    if (int e = h->alloc(&p.S.comp, 4 * (size_t)h->ncell)) return e;
    CK(cudaMemsetAsync(p.S.comp, 0, sizeof(T) * 4 * h->ncell, h->stream));
  }
  const E2DConfig* cfg = &h->cfg;
  p.P.blocks = h->dblocks;
  p.P.nblocks = cfg->nblocks;
  p.P.ncell = h->ncell;
  p.P.nvface = nv;
  p.P.nhface = nh;
  p.P.gamma = cfg->gamma;
  p.P.gm1 = cfg->gm1;
  p.P.gm = cfg->gamma / (cfg->gamma - 1.0);
  p.P.k = 1.0 / (cfg->gamma - 1.0);
  p.P.gas[0] = T(p.P.gamma);
  p.P.gas[1] = T(p.P.gm1);
  p.P.gas[2] = T(p.P.gm);
  p.P.gas[3] = T(p.P.k);
  p.P.cfl = cfg->cfl;
  p.P.flux = cfg->flux;
  p.P.limiter = cfg->limiter;
  p.P.recon = cfg->recon;
  // Gauss-Legendre weights as the reference's Python forms them (quadratures.py:33-37)
  const double w[3][3] = {{2.0, 0.0, 0.0}, {1.0, 1.0, 0.0}, {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0}};
  p.P.nqp = nqp;
  for (int k = 0; k < E2D_MAX_QP; ++k) p.P.qw[k] = T(w[nqp - 1][k]);
  return 0;
}

template <typename T>
static int bench_kernels_t(E2DHandle h, int32_t steps, double* ms, int64_t* launches) {
  PathT<T>& p = path<T>(h);
  const int ninst = (int)h->hinst.size();
  for (auto& I : h->hinst) {
    I.t_final = INFINITY;
    I.max_steps = 0x7fffffff;
    I.steps = 0;
    I.halted = 0;
    I.nbad = 0;
    I.min_bits = 0x7ff0000000000000ULL;
  }
  CK(cudaMemcpyAsync(h->inst, h->hinst.data(), sizeof(InstanceState) * ninst, cudaMemcpyHostToDevice, h->stream));
  k_reset_real<<<1, 1, 0, h->stream>>>(h->real);
  const int per_step = 3 + 3 * h->nstages;
  std::vector<cudaEvent_t> ev(2 * per_step * steps);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  std::vector<int> cls;
  int k = 0;
  auto rec = [&](int c) { cls.push_back(c); return cudaEventRecord(ev[k++], h->stream); };
  auto fin = [&]() { return cudaEventRecord(ev[k++], h->stream); };
  for (int st = 0; st < steps; ++st) {
    CK(rec(0));
    CK(launch_dt<T>(p.P, h->cell_tiles, h->ncell_tiles, p.S.buf[0], h->inst, h->stream));
    CK(fin());
    CK(rec(4));
    CK(launch_begin_step(h->inst, ninst, p.P.cfl, 1, h->stream));
    CK(fin());
    for (int s = 0; s < h->nstages; ++s) {
      const T* in = p.S.buf[h->stage_input[s]];
      if (h->use_fused(s)) {
        CK(rec(5));
        CK(launch_stage_fused<T>(p.P, h->ts, h->ks.variant, in, h->inst, p.S, h->prog[s], h->real, h->stream,
                                 h->tma_for(in), false, FusedRecordT<T>{}));
        CK(fin());
        continue;
      }
      CK(rec(1));
      CK(launch_reconstruct<T>(p.P, h->ts, h->kr, in, h->inst, p.F, nullptr, h->stream, h->tma_for(in)));
      CK(fin());
      CK(rec(2));
      CK(launch_flux<T>(p.P, h->ts, h->kf, h->inst, p.F, nullptr, h->stream));
      CK(fin());
      CK(rec(3));
      CK(launch_update<T>(p.P, h->ts, h->ku, p.F, p.S, h->prog[s], h->inst, h->real, nullptr,
                          h->stream));
      CK(fin());
    }
    CK(rec(4));
    CK(launch_end_step(h->inst, ninst, h->real, h->stream));
    CK(fin());
  }
  CK(cudaStreamSynchronize(h->stream));
  double tot[E2D_BENCH_NK] = {};
  int64_t cnt[E2D_BENCH_NK] = {};
  for (size_t q = 0; q < cls.size(); ++q) {
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, ev[2 * q], ev[2 * q + 1]));
    tot[cls[q]] += t;
    cnt[cls[q]] += 1;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  for (int c = 0; c < E2D_BENCH_NK; ++c) {
    ms[c] = cnt[c] ? tot[c] / cnt[c] : 0.0;
    if (launches) launches[c] = cnt[c];
  }
  CK(cudaMemcpyAsync(h->hinst.data(), h->inst, sizeof(InstanceState) * ninst, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}


// Cost of forming ghost cells and block-boundary face states inside the
// reconstruction kernel: the 8-row reconstruction launch over the real tile table,
// against launches of the same number of tiles in which the tiles touching an
// inter-block side (ms[1]) or any block side (ms[2]) are replaced by interior tiles.
// The replacement launches recompute interior tiles twice (same values written twice)
// and leave the replaced faces stale until the next reconstruction, which every
// stage runs before it reads face arrays.
template <typename T>
static int bench_halo_t(E2DHandle h, int32_t reps, double* ms, int64_t* ntiles) {
  PathT<T>& p = path<T>(h);
  const int n = h->ts.ncell[1];
  std::vector<int4> all(n);
  CK(cudaMemcpy(all.data(), h->ts.cell[1], sizeof(int4) * n, cudaMemcpyDeviceToHost));
  std::vector<int4> interior;
  std::vector<char> nb_edge(n, 0), edge(n, 0);
  for (int k = 0; k < n; ++k) {
    const int4 t = all[k];
    const E2DBlock& B = h->hblocks[t.x];
    const bool touch[4] = {t.z + TX >= B.nx, t.z == 0, t.y + 8 >= B.ny, t.y == 0};  // E, W, N, S
    for (int s = 0; s < 4; ++s) {
      if (!touch[s]) continue;
      edge[k] = 1;
      if (B.side_kind[s] == E2D_SIDE_NEIGHBOR) nb_edge[k] = 1;
    }
    if (!edge[k]) interior.push_back(t);
  }
  if (interior.empty()) return fail(E2D_ERR_UNSUPPORTED, "e2d_bench_halo: the problem has no interior tiles");
  std::vector<int4> lists[3] = {all, all, all};
  int64_t counts[3] = {n, 0, 0};
  size_t r1 = 0, r2 = 0;
  for (int k = 0; k < n; ++k) {
    if (nb_edge[k]) { lists[1][k] = interior[r1++ % interior.size()]; ++counts[1]; }
    if (edge[k]) { lists[2][k] = interior[r2++ % interior.size()]; ++counts[2]; }
  }
  // every instance active while timing (a finished run leaves them inactive, and an
  // inactive instance's tiles return at once); the instance table is put back after
  const int ninst = (int)h->hinst.size();
  std::vector<InstanceState> saved(ninst);
  CK(cudaMemcpyAsync(saved.data(), h->inst, sizeof(InstanceState) * ninst, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  int4* d = nullptr;
  CK(cudaMalloc(&d, sizeof(int4) * n));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t ce0 = launch_set_time(h->inst, ninst, saved[0].t, 0.0, h->stream);
  if (ce0 == cudaSuccess) ce0 = cudaEventCreate(&e0);
  if (ce0 == cudaSuccess) ce0 = cudaEventCreate(&e1);
  int err = ce0 == cudaSuccess ? 0 : fail(E2D_ERR_CUDA, "e2d_bench_halo: %s", cudaGetErrorString(ce0));
  for (int v = 0; v < 3 && !err; ++v) {
    TileSet ts = h->ts;
    ts.cell[1] = d;
    cudaError_t ce = cudaMemcpyAsync(d, lists[v].data(), sizeof(int4) * n, cudaMemcpyHostToDevice, h->stream);
    for (int r = -1; r < reps && ce == cudaSuccess; ++r) {  // r = -1 warms up
      if (r == 0) ce = cudaEventRecord(e0, h->stream);
      if (ce == cudaSuccess)
        ce = launch_reconstruct<T>(p.P, ts, KernelChoice{0, false}, p.S.buf[0], h->inst, p.F, nullptr, h->stream,
                                   h->tma_for(p.S.buf[0]));
    }
    float t = 0.f;
    if (ce == cudaSuccess) ce = cudaEventRecord(e1, h->stream);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&t, e0, e1);
    if (ce != cudaSuccess) err = fail(E2D_ERR_CUDA, "e2d_bench_halo: %s", cudaGetErrorString(ce));
    ms[v] = t / reps;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d);
  CK(cudaMemcpyAsync(h->inst, saved.data(), sizeof(InstanceState) * ninst, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (ntiles)
    for (int v = 0; v < 3; ++v) ntiles[v] = counts[v];
  return err;
}

// Times `reps` launches of one kernel class under the handle's current choice.
template <typename T>
static int time_kernel(E2DHandle h, int which, int reps, float* ms) {
  PathT<T>& p = path<T>(h);
  StageProgram none{};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (int r = -1; r < reps; ++r) {  // r = -1 warms up
    if (r == 0) CK(cudaEventRecord(e0, h->stream));
    if (which == 0)
      CK(launch_reconstruct<T>(p.P, h->ts, h->kr, p.S.buf[0], h->inst, p.F, nullptr, h->stream, h->tma_for(p.S.buf[0])));
    else if (which == 1) CK(launch_flux<T>(p.P, h->ts, h->kf, h->inst, p.F, nullptr, h->stream));
    else if (which == 2) CK(launch_update<T>(p.P, h->ts, h->ku, p.F, p.S, none, h->inst, h->real, nullptr, h->stream));
    else CK(launch_stage_fused<T>(p.P, h->ts, h->ks.variant, p.S.buf[0], h->inst, p.S, none, h->real, h->stream,
                                  h->tma_for(p.S.buf[0]), false, FusedRecordT<T>{}));
  }
  CK(cudaEventRecord(e1, h->stream));
  CK(cudaEventSynchronize(e1));
  CK(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms /= reps;
  return 0;
}

template <typename T>
static int autotune_t(E2DHandle h, int reps, int32_t* chosen) {
  const int ninst = (int)h->hinst.size();
  // every instance active with dt = 0 while timing; the instance table is put back after
  std::vector<InstanceState> saved(ninst);
  CK(cudaMemcpyAsync(saved.data(), h->inst, sizeof(InstanceState) * ninst, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  CK(launch_set_time(h->inst, ninst, 0.0, 0.0, h->stream));
  KernelChoice* ch[3] = {&h->kr, &h->kf, &h->ku};
  const int nvar[3] = {N_RECON_VARIANTS, N_FLUX_VARIANTS, 1};
  float split_ms = 0.f;
  for (int which = 0; which < 3; ++which) {
    KernelChoice best = *ch[which];
    float best_ms = 1e30f;
    for (int v = 0; v < nvar[which]; ++v)
      for (int pers = 0; pers < 2; ++pers) {
        *ch[which] = KernelChoice{v, pers != 0};
        float ms = 0.f;
        if (int e = time_kernel<T>(h, which, reps, &ms)) return e;
        if (ms < best_ms) {
          best_ms = ms;
          best = *ch[which];
        }
      }
    *ch[which] = best;
    if (chosen) {
      chosen[2 * which] = best.variant;
      chosen[2 * which + 1] = best.persistent ? 1 : 0;
    }
    split_ms += best_ms;
  }
  // the three tuned kernels of one stage against one fused stage of each tile height
  // (no updates either way)
  h->ks = KernelChoice{0, false};
  if (h->cfg.nqp <= 1) {
    float best_ms = split_ms;
    for (int form = 1; form < N_STAGE_FORMS; ++form) {
      const KernelChoice keep = h->ks;
      h->ks = KernelChoice{form, false};
      float fused_ms = 0.f;
      if (int e = time_kernel<T>(h, 3, reps, &fused_ms)) return e;
      h->ks = keep;
      if (fused_ms < best_ms) {
        best_ms = fused_ms;
        h->ks = KernelChoice{form, false};
      }
    }
  }
  if (chosen) {
    chosen[6] = h->ks.variant;
    chosen[7] = 0;
  }
  CK(cudaMemcpyAsync(h->inst, saved.data(), sizeof(InstanceState) * ninst, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->drop_graphs();
  return 0;
}

extern "C" {

int e2d_abi_version(void) { return E2D_ABI_VERSION; }
const char* e2d_last_error(void) { return g_err.c_str(); }

int e2d_create(const E2DConfig* cfg, const E2DBlock* blocks, const E2DGeometry* geo, E2DHandle* out) {
  if (!cfg || !blocks || !geo || !out) return fail(E2D_ERR_INVALID, "null argument");
  *out = nullptr;
  if (cfg->nblocks < 1) return fail(E2D_ERR_INVALID, "nblocks must be >= 1");
  if (cfg->precision != E2D_FP64 && cfg->precision != E2D_FP32) return fail(E2D_ERR_INVALID, "unknown precision");
  if (cfg->flux < 0 || cfg->flux > 2 || cfg->limiter < 0 || cfg->limiter > 3 || cfg->recon < 0 || cfg->recon > 1)
    return fail(E2D_ERR_INVALID, "unknown flux/limiter/reconstruction code");
  if (cfg->nqp < 0 || cfg->nqp > E2D_MAX_QP) return fail(E2D_ERR_INVALID, "nqp must be 1, 2 or 3");
  const int ninst = cfg->ninstances > 0 ? cfg->ninstances : 1;
  // validate the block table before anything touches the device
  int64_t ncell = 0, nv = 0, nh = 0;
  for (int b = 0; b < cfg->nblocks; ++b) {
    const E2DBlock& B = blocks[b];
    if (B.nx < 1 || B.ny < 1) return fail(E2D_ERR_INVALID, "block %d: nx, ny must be >= 1", b);
    if (B.instance < 0 || B.instance >= ninst) return fail(E2D_ERR_INVALID, "block %d: bad instance id", b);
    if (B.cell_offset < 0 || B.vface_offset < 0 || B.hface_offset < 0)
      return fail(E2D_ERR_INVALID, "block %d: negative offset", b);
    for (int s = 0; s < 4; ++s) {
      int k = B.side_kind[s];
      if (k < E2D_SIDE_NEIGHBOR || k > E2D_SIDE_MIXED) return fail(E2D_ERR_INVALID, "block %d side %d: bad kind", b, s);
      if (k == E2D_SIDE_NEIGHBOR) {
        int n = B.neighbor[s];
        if (n < 0 || n >= cfg->nblocks) return fail(E2D_ERR_INVALID, "block %d side %d: neighbour %d out of range", b, s, n);
        const E2DBlock& N = blocks[n];
        if ((s <= E2D_W && N.ny != B.ny) || (s >= E2D_N && N.nx != B.nx))
          return fail(E2D_ERR_INVALID, "block %d side %d: neighbour size mismatch", b, s);
        if (N.instance != B.instance) return fail(E2D_ERR_INVALID, "block %d side %d: neighbour in another instance", b, s);
      }
      if (k == E2D_SIDE_MIXED) {
        const E2DMixedSide& m = B.mixed[s];
        if (!B.side_coord[s]) return fail(E2D_ERR_INVALID, "block %d side %d: MIXED side without coordinates", b, s);
        for (int kk : {m.kind_below, m.kind_above})
          if (kk != E2D_SIDE_REFLECT && kk != E2D_SIDE_DIRICHLET)
            return fail(E2D_ERR_INVALID, "block %d side %d: MIXED sub-kind must be REFLECT or DIRICHLET", b, s);
      }
    }
    int64_t e1 = B.cell_offset + (int64_t)B.nx * B.ny;
    int64_t e2 = B.vface_offset + (int64_t)B.ny * (B.nx + 1);
    int64_t e3 = B.hface_offset + (int64_t)(B.ny + 1) * B.nx;
    ncell = e1 > ncell ? e1 : ncell;
    nv = e2 > nv ? e2 : nv;
    nh = e3 > nh ? e3 : nh;
  }
  for (int p = 0; p < E2D_G_NCELL; ++p)
    if (!geo->cell[p]) return fail(E2D_ERR_INVALID, "geometry cell plane %d missing", p);
  for (int p = 0; p < E2D_F_NFACE; ++p)
    if (!geo->vface[p] || !geo->hface[p]) return fail(E2D_ERR_INVALID, "geometry face plane %d missing", p);

  E2DSolver* h = new E2DSolver();
  auto bail = [&](int code) {
    delete h;
    return code;
  };
  cudaError_t ce = cudaGetDevice(&h->device);
  if (ce != cudaSuccess) return bail(fail(E2D_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(ce)));
  ce = cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking);
  if (ce != cudaSuccess) return bail(fail(E2D_ERR_CUDA, "stream: %s", cudaGetErrorString(ce)));
  h->stream = h->own;
  h->cfg = *cfg;
  h->ncell = ncell;
  h->nvface = nv;
  h->nhface = nh;
  h->hblocks.assign(blocks, blocks + cfg->nblocks);

  h->prec = cfg->precision;
  if (h->prec == E2D_FP32) {
    // FP32 defaults measured on GB300: 4-row reconstruction tiles at 8 CTAs/SM (the
    // autotuner's choice on the 512-instance ensemble) and the persistent flux grid at
    // 6 CTAs/SM (2x4x1024^2)
    h->kr = KernelChoice{5, false};
    h->kf = KernelChoice{2, true};
  }
  if (int e = (h->prec == E2D_FP32 ? upload_geometry<float>(h, geo) : upload_geometry<double>(h, geo)))
    return bail(e);
  // block table with MIXED side coordinates moved to the device
  std::vector<E2DBlock> dev_blocks = h->hblocks;
  for (int b = 0; b < cfg->nblocks; ++b)
    for (int s = 0; s < 4; ++s) {
      if (dev_blocks[b].side_kind[s] != E2D_SIDE_MIXED) {
        dev_blocks[b].side_coord[s] = nullptr;
        continue;
      }
      const int len = s <= E2D_W ? dev_blocks[b].ny : dev_blocks[b].nx;
      double* d = nullptr;
      if (int e = h->alloc(&d, len)) return bail(e);
      if ((ce = cudaMemcpy(d, blocks[b].side_coord[s], sizeof(double) * len, cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(fail(E2D_ERR_CUDA, "coord copy: %s", cudaGetErrorString(ce)));
      dev_blocks[b].side_coord[s] = d;
    }
  if (int e = h->alloc(&h->dblocks, cfg->nblocks)) return bail(e);
  if ((ce = cudaMemcpy(h->dblocks, dev_blocks.data(), sizeof(E2DBlock) * cfg->nblocks, cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(fail(E2D_ERR_CUDA, "block table copy: %s", cudaGetErrorString(ce)));

  // tile tables: cells (ny x nx) at tile heights 4, 8, 16 and face nodes ((ny+1) x (nx+1))
  {
    const int heights[3] = {4, 8, 16};
    for (int v = 0; v < 3; ++v) {
      std::vector<int4> ct;
      for (int b = 0; b < cfg->nblocks; ++b) {
        const E2DBlock& B = h->hblocks[b];
        for (int i0 = 0; i0 < B.ny; i0 += heights[v])
          for (int j0 = 0; j0 < B.nx; j0 += TX) ct.push_back(make_int4(b, i0, j0, 0));
      }
      int4* d = nullptr;
      if (int e = h->alloc(&d, ct.size())) return bail(e);
      if ((ce = cudaMemcpy(d, ct.data(), sizeof(int4) * ct.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(fail(E2D_ERR_CUDA, "tile copy: %s", cudaGetErrorString(ce)));
      h->ts.cell[v] = d;
      h->ts.ncell[v] = (int)ct.size();
    }
    h->ts.all_cartesian = true;  // as block_cart decides on the device
    for (int b = 0; b < cfg->nblocks; ++b)
      h->ts.all_cartesian = h->ts.all_cartesian && (h->hblocks[b].is_cartesian || h->axis32[b]);
    for (int v = 0; v < 2; ++v) {  // the fused stage kernel's tiles
      std::vector<int4> ct;
      for (int b = 0; b < cfg->nblocks; ++b) {
        const E2DBlock& B = h->hblocks[b];
        for (int i0 = 0; i0 < B.ny; i0 += FUSED_TY[v])
          for (int j0 = 0; j0 < B.nx; j0 += TX) ct.push_back(make_int4(b, i0, j0, 0));
      }
      int4* d = nullptr;
      if (int e = h->alloc(&d, ct.size())) return bail(e);
      if ((ce = cudaMemcpy(d, ct.data(), sizeof(int4) * ct.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(fail(E2D_ERR_CUDA, "tile copy: %s", cudaGetErrorString(ce)));
      h->ts.fused[v] = d;
      h->ts.nfused[v] = (int)ct.size();
    }
    std::vector<int4> ft;
    for (int b = 0; b < cfg->nblocks; ++b) {
      const E2DBlock& B = h->hblocks[b];
      for (int i0 = 0; i0 <= B.ny; i0 += TY)
        for (int j0 = 0; j0 <= B.nx; j0 += TX) ft.push_back(make_int4(b, i0, j0, 0));
    }
    if (int e = h->alloc(&h->face_tiles, ft.size())) return bail(e);
    if ((ce = cudaMemcpy(h->face_tiles, ft.data(), sizeof(int4) * ft.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
      return bail(fail(E2D_ERR_CUDA, "tile copy: %s", cudaGetErrorString(ce)));
    h->nface_tiles = (int)ft.size();
    h->ts.face = h->face_tiles;
    h->ts.nface = h->nface_tiles;
    h->cell_tiles = const_cast<int4*>(h->ts.cell[1]);
    h->ncell_tiles = h->ts.ncell[1];
  }

  // instance time state and realizability counters
  h->hinst.assign(ninst, InstanceState{});
  for (auto& I : h->hinst) {
    I.min_bits = 0x7ff0000000000000ULL;
    I.t_final = INFINITY;
    I.max_steps = 0x7fffffff;
  }
  if (int e = h->alloc(&h->inst, ninst)) return bail(e);
  if ((ce = cudaMemcpy(h->inst, h->hinst.data(), sizeof(InstanceState) * ninst, cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(fail(E2D_ERR_CUDA, "instance copy: %s", cudaGetErrorString(ce)));
  if (int e = h->alloc(&h->real, 1)) return bail(e);
  k_reset_real<<<1, 1, 0, h->stream>>>(h->real);
  if (int e = h->alloc(&h->tma_timeouts, 1)) return bail(e);
  if ((ce = cudaMemsetAsync(h->tma_timeouts, 0, sizeof(unsigned long long), h->stream)) != cudaSuccess)
    return bail(fail(E2D_ERR_CUDA, "counter init: %s", cudaGetErrorString(ce)));

  if (int e = E2D_DISPATCH(h, init_path)) return bail(e);
  for (int form = 1; form < N_STAGE_FORMS; ++form)
    if ((ce = (h->prec == E2D_FP32
                   ? launch_stage_fused<float>(h->pf.P, h->ts, form, nullptr, h->inst, h->pf.S, StageProgram{}, h->real,
                                               h->stream, nullptr, true, FusedRecordT<float>{})
                   : launch_stage_fused<double>(h->pd.P, h->ts, form, nullptr, h->inst, h->pd.S, StageProgram{},
                                                h->real, h->stream, nullptr, true, FusedRecordT<double>{}))) != cudaSuccess)
      return bail(fail(E2D_ERR_CUDA, "fused stage kernel set-up: %s", cudaGetErrorString(ce)));
  // the FP32 form starts with the fused stage kernel at 13-row tiles, its fastest form
  // on the benchmark problems (e2d_autotune chooses again per problem); FP64 keeps the
  // three kernels, its fastest
  if (h->prec == E2D_FP32 && h->cfg.nqp <= 1) h->ks = KernelChoice{2, false};

  // default integrator: the classical RK4 rows (explicit_runge_kutta.py:212-224)
  const double rk4[16] = {0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 1, 0, 1.0 / 6, 1.0 / 3, 1.0 / 3, 1.0 / 6};
  if (int e = build_program(h, 4, rk4)) return bail(e);
  if (int e = ensure_buffers(h)) return bail(e);
  if ((ce = cudaStreamSynchronize(h->stream)) != cudaSuccess)
    return bail(fail(E2D_ERR_CUDA, "create: %s", cudaGetErrorString(ce)));
  *out = h;
  return 0;
}

int e2d_destroy(E2DHandle h) {
  if (!h) return 0;
  cudaStreamSynchronize(h->stream);
  delete h;
  return 0;
}

int e2d_set_stream(E2DHandle h, void* stream) {
  if (!h) return fail(E2D_ERR_INVALID, "null handle");
  h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own;
  h->drop_graphs();
  return 0;
}

int64_t e2d_num_cells(E2DHandle h) { return h ? h->ncell : -1; }

int e2d_set_state(E2DHandle h, const double* host_soa) {
  if (!h || !host_soa) return fail(E2D_ERR_INVALID, "null argument");
  const size_t n = 4 * (size_t)h->ncell;
  if (h->prec == E2D_FP32) {
    std::vector<float> tmp(n);
    for (size_t i = 0; i < n; ++i) tmp[i] = (float)host_soa[i];
    CK(cudaMemcpyAsync(h->pf.S.buf[0], tmp.data(), sizeof(float) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->pf.S.comp, 0, sizeof(float) * n, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
  }
  CK(cudaMemcpyAsync(h->pd.S.buf[0], host_soa, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int e2d_get_state(E2DHandle h, double* host_soa) {
  if (!h || !host_soa) return fail(E2D_ERR_INVALID, "null argument");
  const size_t n = 4 * (size_t)h->ncell;
  if (h->prec == E2D_FP32) {
    std::vector<float> tmp(n);
    CK(cudaMemcpyAsync(tmp.data(), h->pf.S.buf[0], sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < n; ++i) host_soa[i] = (double)tmp[i];
    return 0;
  }
  CK(cudaMemcpyAsync(host_soa, h->pd.S.buf[0], sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int e2d_set_state_device(E2DHandle h, const double* dev_soa) {
  if (!h || !dev_soa) return fail(E2D_ERR_INVALID, "null argument");
  const int64_t n = 4 * h->ncell;
  if (h->prec == E2D_FP32) {
    CK(launch_convert(dev_soa, h->pf.S.buf[0], n, h->stream));
    CK(cudaMemsetAsync(h->pf.S.comp, 0, sizeof(float) * n, h->stream));
    return 0;
  }
  CK(cudaMemcpyAsync(h->pd.S.buf[0], dev_soa, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
  return 0;
}

int e2d_get_state_device(E2DHandle h, double* dev_soa) {
  if (!h || !dev_soa) return fail(E2D_ERR_INVALID, "null argument");
  const int64_t n = 4 * h->ncell;
  if (h->prec == E2D_FP32) {
    CK(launch_convert(h->pf.S.buf[0], dev_soa, n, h->stream));
    return 0;
  }
  CK(cudaMemcpyAsync(dev_soa, h->pd.S.buf[0], sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
  return 0;
}

int e2d_set_tableau(E2DHandle h, int32_t nstages, const double* a) {
  if (!h || !a) return fail(E2D_ERR_INVALID, "null argument");
  for (int r = 0; r < nstages; ++r)
    for (int c = r + 1; c < nstages; ++c)
      if (a[r * nstages + c] != 0.0) return fail(E2D_ERR_INVALID, "tableau must be lower triangular (explicit)");
  if (int e = build_program(h, nstages, a)) return e;
  h->tableau.assign(a, a + (size_t)nstages * nstages);
  return ensure_buffers(h);
}

}  // extern "C"

template <typename T>
static int enqueue_stages(E2DHandle h, T* dudt_out, const DebugOutT<T>* dbg) {
  PathT<T>& p = path<T>(h);
  for (int s = 0; s < h->nstages; ++s) {
    const T* in = p.S.buf[h->stage_input[s]];
    if (!dudt_out && !dbg && h->use_fused(s)) {
      CK(launch_stage_fused<T>(p.P, h->ts, h->ks.variant, in, h->inst, p.S, h->prog[s], h->real, h->stream,
                               h->tma_for(in), false, FusedRecordT<T>{}));
      continue;
    }
    CK(launch_reconstruct<T>(p.P, h->ts, h->kr, in, h->inst, p.F, dbg, h->stream, h->tma_for(in)));
    CK(launch_flux<T>(p.P, h->ts, h->kf, h->inst, p.F, dbg, h->stream));
    CK(launch_update<T>(p.P, h->ts, h->ku, p.F, p.S, h->prog[s], h->inst, h->real, dudt_out,
                        h->stream));
  }
  return 0;
}

template <typename T>
static int enqueue_run_step_t(E2DHandle h) {
  PathT<T>& p = path<T>(h);
  const int ninst = (int)h->hinst.size();
  CK(launch_dt<T>(p.P, h->cell_tiles, h->ncell_tiles, p.S.buf[0], h->inst, h->stream));
  CK(launch_begin_step(h->inst, ninst, p.P.cfl, 1, h->stream));
  if (int e = enqueue_stages<T>(h, nullptr, nullptr)) return e;
  CK(launch_end_step(h->inst, ninst, h->real, h->stream));
  return 0;
}

extern "C" {

static int enqueue_run_step(E2DHandle h) { return E2D_DISPATCH(h, enqueue_run_step_t); }

}  // extern "C"

template <typename T>
static int launch_dt_path(E2DHandle h) {
  PathT<T>& p = path<T>(h);
  CK(launch_dt<T>(p.P, h->cell_tiles, h->ncell_tiles, p.S.buf[0], h->inst, h->stream));
  return 0;
}

template <typename T>
static int totals_path(E2DHandle h, double* totals) {
  PathT<T>& p = path<T>(h);
  const int nt = h->ncell_tiles;
  std::vector<double> part(4 * (size_t)nt);
  std::vector<int4> tl(nt);
  double* dpart = nullptr;
  CK(cudaMalloc(&dpart, sizeof(double) * part.size()));
  cudaError_t e = launch_totals<T>(p.P, h->cell_tiles, nt, p.S.buf[0], dpart, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(part.data(), dpart, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(tl.data(), h->cell_tiles, sizeof(int4) * nt, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(dpart);
  CK(e);
  const size_t ninst = h->hinst.size();
  for (size_t q = 0; q < 4 * ninst; ++q) totals[q] = 0.0;
  for (int k = 0; k < nt; ++k) {  // tile order: reproducible
    const int q = h->hblocks[tl[k].x].instance;
    for (int v = 0; v < 4; ++v) totals[4 * q + v] += part[4 * (size_t)k + v];
  }
  return 0;
}

template <typename T>
static int ghost_layer_path(E2DHandle h, double t, double* out) {
  PathT<T>& p = path<T>(h);
  std::vector<int64_t> base(h->hblocks.size());
  int64_t n = 0;
  int maxlen = 0;
  for (size_t b = 0; b < h->hblocks.size(); ++b) {
    const int len = 2 * (h->hblocks[b].nx + h->hblocks[b].ny);
    base[b] = n;
    n += len;
    if (len > maxlen) maxlen = len;
  }
  int64_t* dbase = nullptr;
  CK(cudaMalloc(&dbase, sizeof(int64_t) * base.size()));
  cudaError_t e = cudaMemcpyAsync(dbase, base.data(), sizeof(int64_t) * base.size(), cudaMemcpyHostToDevice,
                                  h->stream);
  if (e == cudaSuccess) e = launch_ghost_layer<T>(p.P, p.S.buf[0], t, dbase, out, n, maxlen, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(dbase);
  CK(e);
  return 0;
}

extern "C" {

int e2d_compute_dt(E2DHandle h, double* dt_host) {
  if (!h || !dt_host) return fail(E2D_ERR_INVALID, "null argument");
  const int ninst = (int)h->hinst.size();
  k_reset_min<<<(ninst + 127) / 128, 128, 0, h->stream>>>(h->inst, ninst);
  CK(cudaGetLastError());
  if (int e = E2D_DISPATCH(h, launch_dt_path)) return e;
  CK(cudaMemcpyAsync(h->hinst.data(), h->inst, sizeof(InstanceState) * ninst, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int q = 0; q < ninst; ++q) {
    double m;
    unsigned long long b = h->hinst[q].min_bits;
    std::memcpy(&m, &b, sizeof m);
    dt_host[q] = h->cfg.cfl * m;
  }
  return 0;
}

int e2d_step(E2DHandle h, double dt, double t) {
  if (!h) return fail(E2D_ERR_INVALID, "null handle");
  const int ninst = (int)h->hinst.size();
  CK(launch_set_time(h->inst, ninst, t, dt, h->stream));
  if (int e = (h->prec == E2D_FP32 ? enqueue_stages<float>(h, nullptr, nullptr)
                                   : enqueue_stages<double>(h, nullptr, nullptr)))
    return e;
  CK(launch_end_step(h->inst, ninst, h->real, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return check_tma(h);
}

int e2d_residual(E2DHandle h, double t, double* dudt_dev, const E2DDebug* d) {
  if (!h || !dudt_dev) return fail(E2D_ERR_INVALID, "null argument");
  if (d && h->cfg.nqp > 1)
    return fail(E2D_ERR_UNSUPPORTED, "per-operator outputs are built for one face quadrature point");
  const int ninst = (int)h->hinst.size();
  CK(launch_set_time(h->inst, ninst, t, 0.0, h->stream));
  StageProgram none{};
  none.nupd = 0;
  none.final_stage = 0;
  if (h->prec == E2D_FP32) {
    if (d) return fail(E2D_ERR_UNSUPPORTED, "per-operator intermediates are produced by the FP64 path only");
    PathT<float>& p = h->pf;
    if (!p.dudt_tmp)
      if (int e = h->alloc(&p.dudt_tmp, 4 * (size_t)h->ncell)) return e;
    CK(launch_reconstruct<float>(p.P, h->ts, h->kr, p.S.buf[0], h->inst, p.F, nullptr, h->stream,
                                 h->tma_for(p.S.buf[0])));
    CK(launch_flux<float>(p.P, h->ts, h->kf, h->inst, p.F, nullptr, h->stream));
    CK(launch_update<float>(p.P, h->ts, h->ku, p.F, p.S, none, h->inst, h->real, p.dudt_tmp,
                            h->stream));
    CK(launch_convert(p.dudt_tmp, dudt_dev, 4 * h->ncell, h->stream));
  } else {
    PathT<double>& p = h->pd;
    DebugOut dbg{};
    const DebugOut* pdb = nullptr;
    if (d) {
      dbg.gx = d->gx; dbg.gy = d->gy; dbg.phi = d->phi;
      dbg.vflux_raw = d->vflux_raw; dbg.hflux_raw = d->hflux_raw;
      dbg.vflux = d->vflux; dbg.hflux = d->hflux;
      pdb = &dbg;
    }
    CK(launch_reconstruct<double>(p.P, h->ts, h->kr, p.S.buf[0], h->inst, p.F, pdb, h->stream,
                                  h->tma_for(p.S.buf[0])));
    CK(launch_flux<double>(p.P, h->ts, h->kf, h->inst, p.F, pdb, h->stream));
    CK(launch_update<double>(p.P, h->ts, h->ku, p.F, p.S, none, h->inst, h->real, dudt_dev,
                             h->stream));
    if (d) {
      const size_t bv = sizeof(double) * 4 * h->nvface, bh = sizeof(double) * 4 * h->nhface;
      if (d->vL) CK(cudaMemcpyAsync(d->vL, p.F.vL, bv, cudaMemcpyDeviceToDevice, h->stream));
      if (d->vR) CK(cudaMemcpyAsync(d->vR, p.F.vR, bv, cudaMemcpyDeviceToDevice, h->stream));
      if (d->hL) CK(cudaMemcpyAsync(d->hL, p.F.hL, bh, cudaMemcpyDeviceToDevice, h->stream));
      if (d->hR) CK(cudaMemcpyAsync(d->hR, p.F.hR, bh, cudaMemcpyDeviceToDevice, h->stream));
    }
  }
  CK(launch_end_step(h->inst, ninst, h->real, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int e2d_totals(E2DHandle h, double* totals) {
  if (!h || !totals) return fail(E2D_ERR_INVALID, "null argument");
  return E2D_DISPATCH(h, totals_path, totals);
}

int e2d_ghost_layer(E2DHandle h, double t, double* ghosts_dev) {
  if (!h || !ghosts_dev) return fail(E2D_ERR_INVALID, "null argument");
  return E2D_DISPATCH(h, ghost_layer_path, t, ghosts_dev);
}

int e2d_instance_times(E2DHandle h, double* t_out, int32_t* steps_out) {
  if (!h) return fail(E2D_ERR_INVALID, "null handle");
  const int ninst = (int)h->hinst.size();
  CK(cudaMemcpyAsync(h->hinst.data(), h->inst, sizeof(InstanceState) * ninst, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int q = 0; q < ninst; ++q) {
    if (t_out) t_out[q] = h->hinst[q].t;
    if (steps_out) steps_out[q] = h->hinst[q].steps;
  }
  return 0;
}

int e2d_check_realizable(E2DHandle h, E2DRealizability* out) {
  if (!h || !out) return fail(E2D_ERR_INVALID, "null argument");
  k_reset_real<<<1, 1, 0, h->stream>>>(h->real);
  CK(cudaGetLastError());
  if (h->prec == E2D_FP32)
    CK(launch_realizable<float>(h->pf.P, h->cell_tiles, h->ncell_tiles, h->pf.S.buf[0], h->real, h->stream));
  else
    CK(launch_realizable<double>(h->pd.P, h->cell_tiles, h->ncell_tiles, h->pd.S.buf[0], h->real, h->stream));
  RealizState r;
  CK(cudaMemcpyAsync(&r, h->real, sizeof r, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  out->ok = r.nbad == 0;
  out->nbad = (int64_t)r.nbad;
  out->block = r.nbad ? (int32_t)(r.first >> 40) : -1;
  out->cell = r.nbad ? (int64_t)(r.first & ((1ULL << 40) - 1)) : -1;
  return out->ok ? 0 : fail(E2D_ERR_UNREALIZABLE, "unrealizable state in block %d cell %lld", out->block, (long long)out->cell);
}

// Capture `steps` run-steps into one graph (replayed until the instances stop).
static int get_graph(E2DHandle h, int steps, cudaGraphExec_t* out) {
  for (auto& g : h->graphs)
    if (g.first == steps) {
      *out = g.second;
      return 0;
    }
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int err = 0;
  for (int k = 0; k < steps && !err; ++k) err = enqueue_run_step(h);
  cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
  if (err) {
    if (g) cudaGraphDestroy(g);
    return err;
  }
  if (ce != cudaSuccess) return fail(E2D_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
  cudaGraphExec_t ex = nullptr;
  ce = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) return fail(E2D_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
  h->graphs.emplace_back(steps, ex);
  *out = ex;
  return 0;
}

int e2d_run(E2DHandle h, double* t_inout, double t_final, int32_t max_steps, int32_t* steps_done,
            E2DRealizability* realo) {
  if (!h || !t_inout) return fail(E2D_ERR_INVALID, "null argument");
  const int ninst = (int)h->hinst.size();
  // one instance starts at *t_inout; a batch continues every instance from its own time
  if (ninst > 1) {
    CK(cudaMemcpyAsync(h->hinst.data(), h->inst, sizeof(InstanceState) * ninst, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  for (auto& I : h->hinst) {
    if (ninst == 1) I.t = *t_inout;
    I.t_final = t_final;
    I.max_steps = max_steps;
    I.steps = 0;
    I.halted = 0;
    I.nbad = 0;
    I.active = 0;
    I.min_bits = 0x7ff0000000000000ULL;
  }
  CK(cudaMemcpyAsync(h->inst, h->hinst.data(), sizeof(InstanceState) * ninst, cudaMemcpyHostToDevice, h->stream));
  k_reset_real<<<1, 1, 0, h->stream>>>(h->real);
  CK(cudaGetLastError());
  // steps per host check: enough to amortise the launch of a graph, few enough that
  // the inactive tail after t_final is cheap; the last chunk is cut to max_steps (every
  // active instance advances one step per replayed step, so none needs more)
  int64_t launched = 0;
  for (;;) {
    const int64_t left = (int64_t)max_steps - launched;
    const int chunk = left >= 8 ? 8 : (left > 0 ? (int)left : 1);
    cudaGraphExec_t gx = nullptr;
    if (int e = get_graph(h, chunk, &gx)) return e;
    CK(cudaGraphLaunch(gx, h->stream));
    launched += chunk;
    CK(cudaMemcpyAsync(h->hinst.data(), h->inst, sizeof(InstanceState) * ninst, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    bool any = false, halted = false;
    for (auto& I : h->hinst) {
      halted = halted || I.halted;
      any = any || (!I.halted && I.t < I.t_final && I.steps < I.max_steps);
    }
    // a batch keeps stepping its realizable instances; one instance stops
    if (!any || (ninst == 1 && halted)) break;
  }
  *t_inout = h->hinst[0].t;
  if (steps_done) *steps_done = h->hinst[0].steps;
  if (int e = check_tma(h)) return e;
  RealizState r;
  CK(cudaMemcpyAsync(&r, h->real, sizeof r, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (realo) {
    realo->ok = r.nbad == 0;
    realo->nbad = (int64_t)r.nbad;
    realo->block = r.nbad ? (int32_t)(r.first >> 40) : -1;
    realo->cell = r.nbad ? (int64_t)(r.first & ((1ULL << 40) - 1)) : -1;
  }
  if (r.nbad) return fail(E2D_ERR_UNREALIZABLE, "unrealizable state after step %d", h->hinst[0].steps);
  return 0;
}


// Per-kernel CUDA-event timing of `steps` device-loop steps (euler2d_bench.h).
int e2d_bench_kernels(E2DHandle h, int32_t steps, double* ms, int64_t* launches) {
  if (!h || !ms || steps < 1) return fail(E2D_ERR_INVALID, "bad argument");
  return E2D_DISPATCH(h, bench_kernels_t, steps, ms, launches);
}

int e2d_bench_set_tma(E2DHandle h, int32_t enable) {
  if (!h) return fail(E2D_ERR_INVALID, "null handle");
  h->tma_on = enable != 0;
  h->drop_graphs();
  return 0;
}

int e2d_bench_halo(E2DHandle h, int32_t reps, double* ms, int64_t* ntiles) {
  if (!h || !ms || reps < 1) return fail(E2D_ERR_INVALID, "bad argument");
  if (h->cfg.nqp > 1) return fail(E2D_ERR_UNSUPPORTED, "e2d_bench_halo: one-point face rule only");
  return E2D_DISPATCH(h, bench_halo_t, reps, ms, ntiles);
}

int e2d_set_kernel_choice(E2DHandle h, int32_t kernel, int32_t variant, int32_t persistent) {
  if (!h) return fail(E2D_ERR_INVALID, "null handle");
  const int nvar[4] = {N_RECON_VARIANTS, N_FLUX_VARIANTS, 1, N_STAGE_FORMS};
  if (kernel < 0 || kernel > 3 || variant < 0 || variant >= nvar[kernel])
    return fail(E2D_ERR_INVALID, "kernel %d has no variant %d", kernel, variant);
  if (kernel == 3 && variant >= 1 && h->cfg.nqp > 1)
    return fail(E2D_ERR_UNSUPPORTED, "the fused stage kernel has the one-point face rule only");
  KernelChoice* ch[4] = {&h->kr, &h->kf, &h->ku, &h->ks};
  *ch[kernel] = KernelChoice{variant, persistent != 0};
  h->drop_graphs();
  return 0;
}

int e2d_autotune(E2DHandle h, int32_t reps, int32_t* chosen) {
  if (!h || reps < 1) return fail(E2D_ERR_INVALID, "bad argument");
  return E2D_DISPATCH(h, autotune_t, reps, chosen);
}

}  // extern "C"
