// tma.cuh — the Tensor Memory Accelerator and mbarrier operations the tile
// kernels stage their planes with (inline PTX, sm_90+ and so sm_103a).
//
// A block arms one mbarrier with the bytes it expects, one elected thread
// issues 2-D tensor loads (cp.async.bulk.tensor) of this GPU's own planes into
// shared memory, and every thread waits on the barrier's phase.  The wait is
// bounded: a block that does not see the bytes arrive within the limit counts
// a timeout in the film's stats, waits (bounded again) for its loads to land
// and leaves the tile, so a fault elsewhere cannot hang the GPU here.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace cfk {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// makes an initialised barrier visible to the tensor-load unit
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0u;
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// Waits for phase `phase` of the barrier for at most `limit` polls; returns
// whether it completed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t limit) {
  for (uint32_t k = 0; k < limit; ++k)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}
// 2-D tile load of a tensor map's box at element coordinates (x, y) (x of the
// box start a multiple of 16 bytes; coordinates outside the tensor read 0).
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

}  // namespace cfk
