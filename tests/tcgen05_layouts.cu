/*
 * tcgen05_layouts.cu -- GPU unit test of ofblend_gb300/csrc/flof_tcgen05.cuh:
 * one block computes C = A B^T (M = 128, N = 16..128, K = 128 in two chunks
 * of 64) from small-integer BF16 operands, whose products and sums are exact
 * in FP32, through the header's shared-memory layouts and descriptors (no
 * swizzle, or 128-byte swizzle), instruction descriptor, tensor-memory
 * allocation, MMA, commit and tensor-memory loads; the host compares every
 * entry exactly.  The shared memory has 96 KB of slack past the tiles.
 * Usage: tcgen05_layouts none|sw128; exit status 0 when every entry matches.
 */
#include <cuda_bf16.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "flof_tcgen05.cuh"

using namespace flof::tc;

constexpr int BM = 128, BK = 64, KCH = 2;

__global__ void k_layouts(const uint16_t *A, const uint16_t *B, float *C, int N, int sw, int *err) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  unsigned char *smem = smem_raw + ((1024u - (smem_addr(smem_raw) & 1023u)) & 1023u);
  const int tid = threadIdx.x, warp = tid / 32;
  unsigned char *At = smem;                      // KCH tiles of BM x BK
  unsigned char *Bt = smem + KCH * BM * BK * 2;  // KCH tiles of N x BK
  const uint32_t ncols = N <= 32 ? 32 : (N <= 64 ? 64 : 128);
  if (warp == 0) tmem_alloc(&tbase, ncols);
  if (tid == 0) mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t taddr = tbase;
  for (int c = 0; c < KCH; ++c) {
    for (int e = tid; e < BM * 8; e += blockDim.x) {
      const int row = e / 8, kg = e % 8;
      const uint4 v = *reinterpret_cast<const uint4 *>(A + row * (BK * KCH) + c * BK + kg * 8);
      *reinterpret_cast<uint4 *>(At + c * BM * BK * 2 + (sw ? swz128(row, kg) : core_off(row, kg, BM))) = v;
    }
    for (int e = tid; e < N * 8; e += blockDim.x) {
      const int row = e / 8, kg = e % 8;
      const uint4 v = *reinterpret_cast<const uint4 *>(B + row * (BK * KCH) + c * BK + kg * 8);
      *reinterpret_cast<uint4 *>(Bt + c * N * BK * 2 + (sw ? swz128(row, kg) : core_off(row, kg, N))) = v;
    }
  }
  fence_proxy_async_smem();
  __syncthreads();
  if (tid == 0) {
    fence_after_sync();
    const uint32_t idesc = idesc_bf16_f32(BM, N);
    for (int c = 0; c < KCH; ++c)
      for (int kk = 0; kk < BK / 16; ++kk) {
        const uint32_t a0 = smem_addr(At + c * BM * BK * 2), b0 = smem_addr(Bt + c * N * BK * 2);
        const uint64_t da = sw ? smem_desc_sw128(a0 + kk * 32) : smem_desc(a0 + kk * 2 * (BM * 16), BM * 16, 128);
        const uint64_t db = sw ? smem_desc_sw128(b0 + kk * 32) : smem_desc(b0 + kk * 2 * (N * 16), N * 16, 128);
        mma_bf16(taddr, da, db, idesc, (c | kk) != 0);
      }
    mma_commit(&bar);
  }
  const bool ok = mbar_wait_bounded(&bar, 0);
  if (!ok) atomicExch(err, 1);
  fence_after_sync();
  if (__syncthreads_and(ok)) {
    const int row = 32 * warp + (tid & 31);
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tmem_ld16(taddr + ((uint32_t)(32 * warp) << 16) + c0, v);
      for (int j = 0; j < 16; ++j) C[row * N + c0 + j] = v[j];
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(taddr, ncols);
  }
}

static uint16_t bf(float x) {  // small integers are exact in BF16
  unsigned u;
  memcpy(&u, &x, 4);
  return (uint16_t)(u >> 16);
}

int main(int argc, char **argv) {
  const int sw = argc > 1 && strcmp(argv[1], "sw128") == 0;
  const int K = BK * KCH;
  int fails = 0, *err = nullptr;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return 2;
  cudaMemset(err, 0, sizeof(int));
  const int smem = KCH * BM * BK * 2 + KCH * 128 * BK * 2 + 96 * 1024 + 1024;
  cudaFuncSetAttribute(k_layouts, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  for (int N : {16, 32, 48, 64, 96, 128}) {
    std::vector<float> a(BM * K), b(N * K);
    std::vector<uint16_t> ah(BM * K), bh(N * K);
    srand(N + 7 * sw);
    for (int i = 0; i < BM * K; ++i) a[i] = (float)(rand() % 9 - 4), ah[i] = bf(a[i]);
    for (int i = 0; i < N * K; ++i) b[i] = (float)(rand() % 9 - 4), bh[i] = bf(b[i]);
    uint16_t *dA = nullptr, *dB = nullptr;
    float *dC = nullptr;
    cudaMalloc(&dA, ah.size() * 2);
    cudaMalloc(&dB, bh.size() * 2);
    cudaMalloc(&dC, BM * N * 4);
    cudaMemcpy(dA, ah.data(), ah.size() * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, bh.data(), bh.size() * 2, cudaMemcpyHostToDevice);
    cudaMemset(dC, 0xFF, BM * N * 4);
    k_layouts<<<1, 128, smem>>>(dA, dB, dC, N, sw, err);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      printf("N=%d: %s\n", N, cudaGetErrorString(e));
      return 2;
    }
    std::vector<float> c(BM * N);
    cudaMemcpy(c.data(), dC, c.size() * 4, cudaMemcpyDeviceToHost);
    int bad = 0;
    for (int m = 0; m < BM; ++m)
      for (int n = 0; n < N; ++n) {
        float s = 0;
        for (int k = 0; k < K; ++k) s += a[m * K + k] * b[n * K + k];
        bad += s != c[m * N + n];
      }
    int he = 0;
    cudaMemcpy(&he, err, sizeof(int), cudaMemcpyDeviceToHost);
    printf("%s N=%d: %d mismatches of %d, wait error %d\n", sw ? "sw128" : "none", N, bad, BM * N, he);
    fails += bad != 0 || he != 0;
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
  }
  printf(fails ? "FAILED\n" : "OK\n");
  return fails ? 1 : 0;
}
