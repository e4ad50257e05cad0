// flof_tcgen05.cuh -- the fifth-generation tensor-core instructions (tcgen05)
// used by the learned warm start's convolution kernels: tensor-memory
// allocation, the BF16 x BF16 -> FP32 MMA with both operands in shared
// memory, its completion on an mbarrier, and the tensor-memory loads of the
// epilogue.  Written from the PTX ISA's description of these instructions
// for sm_100a / sm_103a.
//
// Operand layouts in shared memory (K-major: each row's reduction entries
// are contiguous in 16-byte chunks of 8 BF16 values):
//  - no swizzle: a tile of R rows (R a multiple of 8) and 64 reduction
//    entries is a grid of 8-row x 16-byte core matrices; core matrix (row
//    group g, reduction group c) sits at byte (c * R / 8 + g) * 128, its row r
//    at + 16 r.  Leading-dimension offset R * 16 bytes (between core matrices
//    adjacent along the reduction), stride offset 128 bytes (between row
//    groups).
//  - 128-byte swizzle: row r's 64 entries form one 128-byte line at
//    (r / 8) * 1024 + (r % 8) * 128, its 16-byte chunk c stored at position
//    c ^ (r % 8).  Stride offset 1024 bytes (between 8-row groups); the tile
//    starts on a 1024-byte boundary; the K = 16 step kk starts at + 32 kk.
//    A warp writing the 8 chunks of a row, or one chunk of 8 rows, meets no
//    bank conflict.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace flof {
namespace tc {

constexpr int TC_WAIT_LIMIT = 1 << 22;  // mbarrier polls before a wait gives up

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of (row, reduction group kg) in a tile of `rows` rows
__device__ __forceinline__ uint32_t core_off(int row, int kg, int rows) {
  return (uint32_t)((kg * (rows >> 3) + (row >> 3)) * 128 + (row & 7) * 16);
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all >> 4), the fixed version bits 46-48 = 0b001, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Descriptor of a 128-byte-swizzled K-major tile (layout type 2 in bits
// 61-63, stride offset 1024 bytes; the leading offset is not used)
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) |
         (1ull << 46) | (2ull << 61);
}
__device__ __forceinline__ uint32_t swz128(int row, int chunk) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((chunk ^ (row & 7)) << 4));
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in
// bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// One warp allocates `ncols` tensor-memory columns (a power of two >= 32) and
// writes their address to *dst; the permit is released so that other blocks
// on the SM may allocate too.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                   smem_addr(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, M x N x 16, issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// The mbarrier receives one arrival when every MMA this thread issued so far
// has completed (and its shared-memory operands may be overwritten).
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// generic-proxy shared-memory writes made visible to the tensor core's reads
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane (the warp
// reads lanes 32 (warp % 4) .. + 31); the load and its wait form one
// statement, so no use of the registers can move above the wait.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (int i = 0; i < TC_WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// x = hi + lo with hi = bf16(x) and lo = bf16(x - hi): the pair carries about
// 16 significant bits (|x - hi - lo| <= 2^-18 |x|).  Eight values go to two
// 16-byte rows.
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&h);
}
__device__ __forceinline__ void split4(const float4 &x, uint2 &hi, uint2 &lo) {
  const float h0 = __bfloat162float(__float2bfloat16_rn(x.x));
  const float h1 = __bfloat162float(__float2bfloat16_rn(x.y));
  const float h2 = __bfloat162float(__float2bfloat16_rn(x.z));
  const float h3 = __bfloat162float(__float2bfloat16_rn(x.w));
  hi = make_uint2(pack_bf16(h0, h1), pack_bf16(h2, h3));
  lo = make_uint2(pack_bf16(__fsub_rn(x.x, h0), __fsub_rn(x.y, h1)),
                  pack_bf16(__fsub_rn(x.z, h2), __fsub_rn(x.w, h3)));
}
__device__ __forceinline__ void split8(const float (&x)[8], uint4 &hi, uint4 &lo) {
  float h[8], l[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    h[i] = __bfloat162float(__float2bfloat16_rn(x[i]));
    l[i] = __fsub_rn(x[i], h[i]);
  }
  hi = make_uint4(pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]),
                  pack_bf16(h[6], h[7]));
  lo = make_uint4(pack_bf16(l[0], l[1]), pack_bf16(l[2], l[3]), pack_bf16(l[4], l[5]),
                  pack_bf16(l[6], l[7]));
}

}  // namespace tc
}  // namespace flof
