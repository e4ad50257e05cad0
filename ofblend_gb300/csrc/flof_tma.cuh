// flof_tma.cuh -- device helpers for TMA-staged slab kernels: mbarrier
// waits with an iteration limit and the slab copy of a float4 grid viewed as
// a 4D float tensor (encode_slab_map).
#pragma once

#include <cuda.h>
#include <stdint.h>

#include "flof_common.cuh"

namespace flof {

constexpr int WAIT_LIMIT = 1 << 22;  // try_wait polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (int i = 0; i < WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// The slab buffers are reused: a copy lands (async proxy) in a buffer the
// block's threads read before (generic proxy).  The issuing thread passes the
// barrier that ends those reads and then fences the two proxies, so that no
// read still in flight sees the new slab.
__device__ __forceinline__ void tma_load_slab(void *dst, const CUtensorMap *map, int x, int y,
                                              int z, int t, uint64_t *bar) {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(smem_u32(dst)),
      "l"(map), "r"(4 * x), "r"(y), "r"(z), "r"(t), "r"(smem_u32(bar))
      : "memory");
}

// Tensor map of the float4 grid at base as a 4D float tensor (4X, Y, Z, T)
// with a (4W, H, D, 1) box (D consecutive z slabs per copy); false when the
// driver entry point is missing, base is not 16-byte aligned or 4W exceeds
// 256.
bool encode_slab_map(CUtensorMap *m, const float4 *base, Dims4 d, int W, int H, int D = 1);

}  // namespace flof
