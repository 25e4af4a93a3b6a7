// e2d_solver.cuh - the solver handle and the helpers shared by the host-side units
// (e2d_api.cu: the plain, FP32 and batched paths; e2d_adjoint.cu: the adjoint).
// Internal.
#pragma once
#include <cstdarg>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "e2d_kernels.cuh"

namespace e2d {
// records the thread-local message returned by e2d_last_error (e2d_api.cu)
int set_error(int code, const char* msg);

inline int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return set_error(code, buf);
}
}  // namespace e2d

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return e2d::fail(E2D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Everything that has the arithmetic type of a path: parameters (with the geometry
// plane pointers), face arrays and state buffers.
template <typename T>
struct PathT {
  e2d::ParamsT<T> P{};
  T* geo = nullptr;
  e2d::FaceArraysT<T> F{};
  e2d::StateBuffersT<T> S{};
  T* dudt_tmp = nullptr;  // FP32 residual staging for the FP64 caller buffer
};

struct E2DAdjoint;  // adjoint storage (e2d_adjoint.cu)
void destroy_adjoint(E2DAdjoint* a);

struct E2DSolver {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  E2DConfig cfg{};
  int prec = E2D_FP64;
  std::vector<E2DBlock> hblocks;
  PathT<double> pd;
  PathT<float> pf;
  E2DBlock* dblocks = nullptr;
  std::vector<void*> allocs;
  int4* cell_tiles = nullptr;   // tile height 8 (dt, update, default reconstruct)
  int ncell_tiles = 0;
  int4* face_tiles = nullptr;
  int nface_tiles = 0;
  e2d::TileSet ts{};                  // all tile tables (heights 4, 8, 16)
  e2d::KernelChoice kr{0, false};     // reconstruct variant (autotuned)
  e2d::KernelChoice kf{0, false};     // flux variant
  e2d::KernelChoice ku{0, false};     // update variant
  e2d::KernelChoice ks{0, false};     // stage form: 0 three kernels, 1 and 2 the fused stage kernel
  // per stage: its Butcher updates leave its input buffer alone, so it may be fused
  std::vector<int> fusable;
  std::vector<int> axis32;       // per block (FP32 form): face frames axis-aligned to FP32's resolution
  bool use_fused(int s) const { return ks.variant >= 1 && cfg.nqp <= 1 && fusable[s]; }
  int nbuf = 0;
  e2d::InstanceState* inst = nullptr;
  std::vector<e2d::InstanceState> hinst;
  e2d::RealizState* real = nullptr;
  int nstages = 0;
  std::vector<double> tableau;        // nstages x nstages Butcher rows
  std::vector<e2d::StageProgram> prog;
  std::vector<int> stage_input;
  // captured step graphs, keyed by the number of steps they replay
  std::vector<std::pair<int, cudaGraphExec_t>> graphs;
  int64_t ncell = 0, nvface = 0, nhface = 0;
  E2DAdjoint* adj = nullptr;
  // TMA tensor maps of each state buffer (interior reconstruction tiles), the device
  // counter of bounded TMA waits that ran out, and the switch between TMA and plain loads
  struct TmaEntry {
    const void* base;
    e2d::TmaSet set;
  };
  std::vector<TmaEntry> tma_reg;
  unsigned long long* tma_timeouts = nullptr;
  bool tma_on = true;
  const e2d::TmaSet* tma_for(const void* buf) const {
    if (!tma_on) return nullptr;
    for (const auto& e : tma_reg)
      if (e.base == buf) return &e.set;
    return nullptr;
  }

  void drop_graphs() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    graphs.clear();
  }
  ~E2DSolver() {
    drop_graphs();
    destroy_adjoint(adj);
    for (void* p : allocs) cudaFree(p);
    if (own) cudaStreamDestroy(own);
  }
  template <typename T>
  int alloc(T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess)
      return e2d::fail(E2D_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", sizeof(T) * count, cudaGetErrorString(e));
    allocs.push_back(q);
    *p = static_cast<T*>(q);
    return 0;
  }
};

template <typename T>
PathT<T>& path(E2DSolver* h);
template <>
inline PathT<double>& path<double>(E2DSolver* h) { return h->pd; }
template <>
inline PathT<float>& path<float>(E2DSolver* h) { return h->pf; }

// Run f<T>(h) for the handle's precision.
#define E2D_DISPATCH(h, f, ...) ((h)->prec == E2D_FP32 ? f<float>(h, ##__VA_ARGS__) : f<double>(h, ##__VA_ARGS__))
