// e2d_bench.cu - FP64 instruction-throughput probe (see include/euler2d_bench.h).
#include <cuda_runtime.h>

#include <cstdio>

#include "../../include/euler2d_bench.h"
#include "e2d_device.cuh"
#include "e2d_tma.cuh"

namespace {

template <int OP>
__global__ void k_fp64_chain(double* out, int iters, double seed) {
  double a0 = seed + threadIdx.x, a1 = a0 + 1.0, a2 = a0 + 2.0, a3 = a0 + 3.0;
  double a4 = a0 + 4.0, a5 = a0 + 5.0, a6 = a0 + 6.0, a7 = a0 + 7.0;
  const double m = 1.0000000001, c = 1e-9;
  for (int i = 0; i < iters; ++i) {
    if (OP == 0) {
      a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
      a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    } else if (OP == 1) {
      a0 = a0 + c; a1 = a1 + c; a2 = a2 + c; a3 = a3 + c;
      a4 = a4 + c; a5 = a5 + c; a6 = a6 + c; a7 = a7 + c;
    } else {
      a0 = a0 * m; a1 = a1 * m; a2 = a2 * m; a3 = a3 * m;
      a4 = a4 * m; a5 = a5 * m; a6 = a6 * m; a7 = a7 * m;
    }
  }
  double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chains live, never true in practice
}

__global__ void k_div32(const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ q,
                        int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    q[i] = e2d::div32(a[i], b[i]);
}

__global__ void k_rdiv32(const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ q,
                         int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    q[i] = e2d::rdiv(a[i], b[i]);
}

// x / b by the geometry's route: div_recip with y = 1/b from IEEE division
__global__ void k_div_recip(const double* __restrict__ x, const double* __restrict__ b, double* __restrict__ q,
                            int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    q[i] = e2d::div_recip(x[i], b[i], 1.0 / b[i]);
}

// min(psi(s_a), psi(s_b)) by the paired evaluation and by two scalar psi_s
template <int LIM>
__global__ void k_psi_pair(const float* __restrict__ sa, const float* __restrict__ sb, float* __restrict__ pair_out,
                           float* __restrict__ scalar_out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    pair_out[i] = e2d::psi_min_pair<LIM>(sa[i], sb[i]);
    scalar_out[i] = e2d::vmin(e2d::psi_s<LIM>(sa[i]), e2d::psi_s<LIM>(sb[i]));
  }
}

// One warp waits on a shared-memory barrier phase with the reconstruction kernel's
// bounded wait.  complete != 0: thread 0 arrives (the phase completes); else thread 0
// announces 16 bytes of transfer that no copy delivers, so the phase cannot complete
// and the wait runs out after `limit` polls.  out[0] = 1 if the phase was seen
// complete, out[1] = 1 once the kernel got past the wait.
__global__ void k_wait_bound(int complete, int limit, int* out) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) e2d::mbar_init(&bar);
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned a = e2d::smem_u32(&bar);
    if (complete) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
    else asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], 16;" ::"r"(a) : "memory");
  }
  const bool arrived = __syncthreads_and(e2d::mbar_wait(&bar, 0u, limit));
  if (threadIdx.x == 0) {
    out[0] = arrived ? 1 : 0;
    out[1] = 1;
  }
}

}  // namespace

extern "C" int e2d_check_wait_bound(int32_t complete, int32_t limit, int32_t* arrived) {
  if (!arrived || limit < 1) return E2D_ERR_INVALID;
  int* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(int)) != cudaSuccess) return E2D_ERR_NOMEM;
  int h[2] = {0, 0};
  cudaMemset(d, 0, 2 * sizeof(int));
  k_wait_bound<<<1, 32>>>(complete, limit, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess || h[1] != 1) return E2D_ERR_CUDA;
  *arrived = h[0];
  return 0;
}

extern "C" int e2d_check_div32(const float* a, const float* b, float* q, int64_t n) {
  if (!a || !b || !q || n < 0) return E2D_ERR_INVALID;
  if (n == 0) return 0;
  k_div32<<<1024, 256>>>(a, b, q, n);
  if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) return E2D_ERR_CUDA;
  return 0;
}

extern "C" int e2d_check_rdiv32(const float* a, const float* b, float* q, int64_t n) {
  if (!a || !b || !q || n < 0) return E2D_ERR_INVALID;
  if (n == 0) return 0;
  k_rdiv32<<<1024, 256>>>(a, b, q, n);
  if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) return E2D_ERR_CUDA;
  return 0;
}

extern "C" int e2d_check_div_recip(const double* x, const double* b, double* q, int64_t n) {
  if (!x || !b || !q || n < 0) return E2D_ERR_INVALID;
  if (n == 0) return 0;
  k_div_recip<<<1024, 256>>>(x, b, q, n);
  if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) return E2D_ERR_CUDA;
  return 0;
}

extern "C" int e2d_check_psi_pair(int32_t limiter, const float* sa, const float* sb, float* pair_out,
                                  float* scalar_out, int64_t n) {
  if (!sa || !sb || !pair_out || !scalar_out || n < 0) return E2D_ERR_INVALID;
  if (limiter != E2D_LIM_VENKATAKRISHNAN && limiter != E2D_LIM_VAN_ALBADA) return E2D_ERR_INVALID;
  if (n == 0) return 0;
  if (limiter == E2D_LIM_VENKATAKRISHNAN)
    k_psi_pair<E2D_LIM_VENKATAKRISHNAN><<<1024, 256>>>(sa, sb, pair_out, scalar_out, n);
  else
    k_psi_pair<E2D_LIM_VAN_ALBADA><<<1024, 256>>>(sa, sb, pair_out, scalar_out, n);
  if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) return E2D_ERR_CUDA;
  return 0;
}

extern "C" int e2d_bench_fp64_peak(int32_t op, double* tflops) {
  if (!tflops || op < 0 || op > 2) return E2D_ERR_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return E2D_ERR_CUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * 65536) != cudaSuccess) return E2D_ERR_NOMEM;
  const int blocks = sms * 8, threads = 256, iters = 2048;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    if (op == 0) k_fp64_chain<0><<<blocks, threads>>>(out, iters, 1.0);
    else if (op == 1) k_fp64_chain<1><<<blocks, threads>>>(out, iters, 1.0);
    else k_fp64_chain<2><<<blocks, threads>>>(out, iters, 1.0);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double inst = (double)blocks * threads * iters * 8.0;
    const double fl = inst * (op == 0 ? 2.0 : 1.0) / (ms * 1e-3) / 1e12;
    if (rep > 0 && fl > best) best = fl;  // first launch is warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return E2D_ERR_CUDA;
  *tflops = best;
  return 0;
}
