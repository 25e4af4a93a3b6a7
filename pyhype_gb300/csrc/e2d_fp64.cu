// e2d_fp64.cu - FP64 instantiation of the stage kernels (the bit-exact path; this
// unit builds with -fmad=false so no multiply-add is contracted) and the
// precision-independent step bookkeeping kernels.
#include "e2d_fused.cuh"

namespace e2d {

E2D_EXTERN_RECON_LIM(double)
E2D_EXTERN_FUSED_LIM(double)
E2D_INSTANTIATE_FUSED_LAUNCHER(double)
E2D_INSTANTIATE_STAGE_LAUNCHERS(double)

// Step bookkeeping, one thread per instance.  begin: decide whether the instance
// still steps (t < t_final, steps < max_steps, not halted) and form
// dt = CFL*min, clamped to t_final - t (pyhype/solvers/base.py:114-136).
__global__ void k_begin_step(InstanceState* inst, int ninst, double cfl, int use_min) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ninst) return;
  InstanceState& I = inst[q];
  I.active = (!I.halted) && (I.t < I.t_final) && (I.steps < I.max_steps);
  if (use_min) {
    const double m = __longlong_as_double((long long)I.min_bits);
    double dt = cfl * m;
    if (I.t_final - I.t < dt) dt = I.t_final - I.t;
    I.dt = dt;
  }
  I.min_bits = 0x7ff0000000000000ULL;
}

__global__ void k_end_step(InstanceState* inst, int ninst, const RealizState*) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ninst) return;
  InstanceState& I = inst[q];
  if (I.active) {
    I.t = I.t + I.dt;
    I.steps += 1;
    if (I.nbad) I.halted = 1;
  }
  I.active = 0;
}

__global__ void k_set_time(InstanceState* inst, int ninst, double t, double dt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ninst) return;
  inst[q].t = t;
  inst[q].dt = dt;
  inst[q].active = 1;
  inst[q].nbad = 0;
}


__global__ void k_to_f32(const double* __restrict__ s, float* __restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (float)s[i];
}
__global__ void k_to_f64(const float* __restrict__ s, double* __restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (double)s[i];
}

cudaError_t launch_begin_step(InstanceState* inst, int ninst, double cfl, int use_min, cudaStream_t st) {
  k_begin_step<<<(ninst + 127) / 128, 128, 0, st>>>(inst, ninst, cfl, use_min);
  return cudaGetLastError();
}

cudaError_t launch_end_step(InstanceState* inst, int ninst, const RealizState* real, cudaStream_t st) {
  k_end_step<<<(ninst + 127) / 128, 128, 0, st>>>(inst, ninst, real);
  return cudaGetLastError();
}

cudaError_t launch_set_time(InstanceState* inst, int ninst, double t, double dt, cudaStream_t st) {
  k_set_time<<<(ninst + 127) / 128, 128, 0, st>>>(inst, ninst, t, dt);
  return cudaGetLastError();
}

cudaError_t launch_convert(const double* src, float* dst, int64_t n, cudaStream_t st) {
  k_to_f32<<<1024, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

cudaError_t launch_convert(const float* src, double* dst, int64_t n, cudaStream_t st) {
  k_to_f64<<<1024, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

}  // namespace e2d
