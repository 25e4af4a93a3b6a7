// e2d_tma.cuh - shared-memory mbarrier and TMA box-load helpers (inline PTX) of the
// reconstruction kernel's tile staging, and the bounded barrier wait it relies on.
#pragma once
#include <cuda.h>

namespace e2d {

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the barrier phase `parity`: at most `limit` polls (each may
// suspend the thread briefly in hardware); false when the bound ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int limit = 1 << 22) {
  const unsigned a = smem_u32(bar);
  for (int it = 0; it < limit; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// One thread: expect `bytes` on the barrier and load the 3-D box at (x, y, z) of the
// tensor map into shared memory.  The fence orders the CTA's earlier generic accesses
// of that shared memory (the previous tile) before the asynchronous write.
__device__ __forceinline__ void tma_load_box(void* dst, const CUtensorMap* map, int x, int y, int z,
                                             unsigned long long* bar, unsigned bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

}  // namespace e2d
