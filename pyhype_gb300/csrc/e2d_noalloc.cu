// e2d_noalloc.cu - CFL time step for callers that may not allocate device memory.
//
// Same arithmetic as the solver's k_dt (u = rho*u/rho, p = (gamma-1)(E - rho*Ek),
// a = sqrt(gamma*p/rho), min over cells of min(dx/(|u|+a), dy/(|v|+a)), times CFL), but
// the per-tile partial minima live in a file-scope device array instead of memory a
// handle allocated.  Every GPU that loads the library holds the array until exit.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/euler2d.h"
#include "e2d_device.cuh"

namespace e2d {
int set_error(int code, const char* msg);
}

namespace {

constexpr int kTile = 256;  // cells per CTA, one partial minimum per CTA

// 65536 partial minima + 1 result word: 512 KiB + 8 B of device memory per GPU.
__device__ __align__(256) unsigned long long g_dt_scratch[E2D_NOALLOC_MAX_CELLS / kTile + 1];

// Device addresses of g_dt_scratch, resolved once per device at first use.
constexpr int kMaxDevices = 64;
unsigned long long* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mu;

__global__ void k_dt_partial(const double* __restrict__ U, int64_t ncell, const double* __restrict__ dx,
                             const double* __restrict__ dy, double gamma, double gm1,
                             unsigned long long* __restrict__ partial) {
  const int64_t c = (int64_t)blockIdx.x * kTile + threadIdx.x;
  double m = __longlong_as_double(0x7ff0000000000000LL);
  if (c < ncell) {
    const double q[4] = {U[c], U[ncell + c], U[2 * ncell + c], U[3 * ncell + c]};
    double w[4];
    const e2d::Gas<double> G{gamma, gm1, gamma / (gamma - 1.0), 1.0 / (gamma - 1.0)};
    e2d::cons_to_prim(q, G, w);
    const double a = sqrt(gamma * w[3] / w[0]);
    const double tx = dx[c] / (fabs(w[1]) + a);
    const double ty = dy[c] / (fabs(w[2]) + a);
    m = e2d::vmin(tx, ty);
  }
  unsigned long long bits = (unsigned long long)__double_as_longlong(m);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
    bits = other < bits ? other : bits;
  }
  __shared__ unsigned long long wmin[kTile / 32];
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = bits;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = wmin[0];
    for (int k = 1; k < kTile / 32; ++k) b = wmin[k] < b ? wmin[k] : b;
    partial[blockIdx.x] = b;  // every used slot is written before it is read
  }
}

__global__ void k_dt_final(unsigned long long* __restrict__ scratch, int nparts) {
  unsigned long long b = 0x7ff0000000000000ULL;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) b = scratch[k] < b ? scratch[k] : b;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long other = __shfl_xor_sync(0xffffffffu, b, o);
    b = other < b ? other : b;
  }
  __shared__ unsigned long long wmin[32];
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long r = wmin[0];
    for (int k = 1; k < (int)(blockDim.x / 32); ++k) r = wmin[k] < r ? wmin[k] : r;
    scratch[E2D_NOALLOC_MAX_CELLS / kTile] = r;  // result word after the partials
  }
}

int fail_cuda(const char* what, cudaError_t ce) {
  char buf[256];
  snprintf(buf, sizeof buf, "e2d_compute_dt_noalloc: %s: %s", what, cudaGetErrorString(ce));
  return e2d::set_error(E2D_ERR_CUDA, buf);
}

}  // namespace

extern "C" int e2d_compute_dt_noalloc(const double* dev_state, int64_t ncell, const double* dev_cfl_dx,
                                      const double* dev_cfl_dy, double gamma, double gm1, double cfl,
                                      void* stream, double* dt_host) {
  if (!dev_state || !dev_cfl_dx || !dev_cfl_dy || !dt_host || ncell < 1)
    return e2d::set_error(E2D_ERR_INVALID, "e2d_compute_dt_noalloc: null pointer or ncell < 1");
  if (ncell > (int64_t)E2D_NOALLOC_MAX_CELLS)  // the static scratch holds one slot per 256 cells
    return e2d::set_error(E2D_ERR_INVALID,
                          "e2d_compute_dt_noalloc: ncell exceeds E2D_NOALLOC_MAX_CELLS (16777216), the size of its "
                          "static scratch; use e2d_compute_dt on a handle for larger problems");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return e2d::set_error(E2D_ERR_CUDA, "e2d_compute_dt_noalloc: no usable CUDA device");
  unsigned long long* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_dt_scratch) != cudaSuccess || !p)
        return e2d::set_error(E2D_ERR_CUDA, "e2d_compute_dt_noalloc: cudaGetSymbolAddress of the scratch failed");
      g_scratch_ptr[dev] = static_cast<unsigned long long*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  // An error left by earlier, unrelated work on this thread is reported as such and
  // left in place for its owner: this call launches nothing on top of it.
  cudaError_t ce = cudaPeekAtLastError();
  if (ce != cudaSuccess) return fail_cuda("a CUDA error from earlier work is pending on this thread", ce);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nparts = (int)((ncell + kTile - 1) / kTile);
  k_dt_partial<<<nparts, kTile, 0, st>>>(dev_state, ncell, dev_cfl_dx, dev_cfl_dy, gamma, gm1, scratch);
  if ((ce = cudaGetLastError()) != cudaSuccess) return fail_cuda("launch of the per-tile minima", ce);
  k_dt_final<<<1, 1024, 0, st>>>(scratch, nparts);
  if ((ce = cudaGetLastError()) != cudaSuccess) return fail_cuda("launch of the final minimum", ce);
  unsigned long long bits = 0;
  if ((ce = cudaMemcpyAsync(&bits, scratch + E2D_NOALLOC_MAX_CELLS / kTile, sizeof bits, cudaMemcpyDeviceToHost,
                            st)) != cudaSuccess)
    return fail_cuda("result copy", ce);
  if ((ce = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda("stream synchronize", ce);
  double m;
  std::memcpy(&m, &bits, sizeof m);
  *dt_host = cfl * m;
  return 0;
}
