// flof_conv_tc.cu -- the learned warm start's 3^4 convolutions on the
// tcgen05 tensor cores: forward, input gradient and weight gradient as
// implicit GEMMs of 128-row tiles, accumulated in tensor memory.
//
// Operands: the weights are BF16 already (rounded from the FP32 master
// weights), so they enter as they are.  Activations and gradients are FP32;
// each value x enters as two BF16 parts hi = bf16(x), lo = bf16(x - hi)
// (about 16 significant bits), so the products carry FP32-like accuracy:
//   forward / input gradient: acc += A_hi W + A_lo W            (2 MMAs)
//   weight gradient:          acc += A_hi B_hi + A_lo B_hi + A_hi B_lo (3 MMAs)
// with FP32 accumulation in tensor memory.
//
// Per block: 256 threads gather a 128 x 64 reduction chunk of the operand
// (im2col on the fly: voxel rows x (tap, channel), or (tap, channel) rows x
// voxels for the weight gradient) through registers into shared memory in
// the 128-byte-swizzled K-major layout (flof_tcgen05.cuh), while the
// previous chunk's MMAs (issued by a ninth warp) run; two stages, each released by a
// tcgen05.commit on its mbarrier.  The forward and input-gradient gathers
// run along channels (16 lanes read 256 contiguous bytes of a row), the
// weight-gradient gather along the (tap, channel) rows.  The weight
// gradient carries one more row of ones, whose products are the bias
// gradient.  Layers with few row tiles split the reduction into slices
// written to a work buffer and summed in slice order (deterministic), with
// the bias and ReLU applied there.
//
// Every mbarrier wait is bounded: a block that gives up stores
// FLOF_DEV_ERR_TC_TIMEOUT in the context's device error word, waits (again
// bounded) for its issued MMAs, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>

#include "flof_internal.h"
#include "flof_tcgen05.cuh"

namespace flof {

namespace {

using namespace tc;

constexpr int TB_M = 128;  // rows per block (the MMA's M)
constexpr int TB_K = 64;   // reduction entries per chunk (four K = 16 MMAs)
constexpr int TB_T = 256;  // threads that stage operands
constexpr int TB_W = TB_T + 32;  // plus one warp that issues the MMAs
constexpr int KG_T = 8 * TB_M / TB_T;  // weight gradient: reduction groups (of 8) per thread
constexpr int A_TILE = TB_M * TB_K * 2;  // bytes of one BF16 A tile

struct TcArgs {
  const float *A;         // MODE 0: input; MODE 1: output gradient; MODE 2: input
  const float *B32;       // MODE 2: output gradient
  const uint16_t *Bw;     // MODE 0: WT[cout][Kpad]; MODE 1: WB[tap][cin][cout] (BF16 bits)
  const float *bias;      // MODE 0, unsplit only
  float *C;               // result rows x N, or slices of it
  int *err;
  int rin, rout, cin, cout, stride;
  int M, N, K, Kpad;      // rows, columns, reduction length, WT row length
  int relu, kslice, ncols;
  int bias_row;           // MODE 2: the last row is all ones (the bias gradient)
};

// A tap of the reduction: its source voxel is the row's voxel plus `off`
// (linear, in the grid the tap reads), and it falls off that grid for rows
// whose edge mask shares a bit with `need`.  For a forward tap with offsets
// o in 0..2 per axis, `need` has bit a where o_a = 0 and bit 4 + a where
// o_a = 2, and off = sum (o_a - 1) stride_a.  Bit 8 is always set, so an
// invalid row (edge mask 0x100) reads nothing.
struct TapEnt {
  int need, off;
};

__device__ const float kOne = 1.f;  // the weight gradient's bias row

__device__ __forceinline__ void tap_digits(int tap, int o[4]) {
  o[0] = tap % 3;
  o[1] = (tap / 3) % 3;
  o[2] = (tap / 9) % 3;
  o[3] = tap / 27;
}

// edge mask of a source position s (per axis, s = coordinate * stride): bit
// a when s_a = 0 (offset 0 falls off), bit 4 + a when s_a + 1 >= ext
__device__ __forceinline__ int edge_mask(const int s[4], int ext) {
  int m = 0;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    m |= (s[a] == 0) << a;
    m |= (s[a] + 1 >= ext) << (4 + a);
  }
  return m;
}

// weight gradient: voxel table of reduction chunk c (its 64 output voxels):
// (input voxel of v * stride times cin, edge mask), bit 8 set past the
// slice's end
__device__ __forceinline__ void fill_vtab(int2 *vt, int tid, int kbeg, int c, int nch, int kend,
                                          int rout, int rin, int stride, int cin) {
  if (tid >= TB_K) return;
  const int v = kbeg + c * TB_K + tid;
  int2 e = make_int2(0, 0x100);
  if (c < nch && v < kend) {
    int s[4], q = v;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      s[a] = (q % rout) * stride;
      q /= rout;
    }
    e = make_int2((s[0] + rin * (s[1] + rin * (s[2] + rin * s[3]))) * cin, edge_mask(s, rin));
  }
  vt[tid] = e;
}

// MODE 0/1 gather: this thread's four channels, starting at reduction index
// k (of K), of rows rsub, rsub + 16, ... of the tile: zero where the tap's
// `need` mask meets the row's edge mask or k is past the end
template <int VEC>
__device__ __forceinline__ void gather01(float4 (&xv)[TB_M / 16], const float *__restrict__ A,
                                         int k, int K, const TapEnt *taps, const int2 *rows_s,
                                         int rsub, int ch) {
#pragma unroll
  for (int it = 0; it < TB_M / 16; ++it) xv[it] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (VEC) {
    if (k >= K) return;
    const int tap = k / ch, c = k - tap * ch;
    const TapEnt t = taps[tap];
#pragma unroll
    for (int it = 0; it < TB_M / 16; ++it) {
      const int2 ri = rows_s[it * 16 + rsub];
      if (!(ri.y & t.need))
        xv[it] = __ldg(reinterpret_cast<const float4 *>(A + (size_t)(ri.x + t.off) * ch + c));
    }
  } else {  // a channel count that is not a multiple of 8 (the forward pass only)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int kj = k + j;
      if (kj < K) {
        const int tap = kj / ch, ci = kj - tap * ch;
        const TapEnt t = taps[tap];
#pragma unroll
        for (int it = 0; it < TB_M / 16; ++it) {
          const int2 ri = rows_s[it * 16 + rsub];
          if (!(ri.y & t.need)) {
            const float v = __ldg(A + (size_t)(ri.x + t.off) * ch + ci);
            if (j == 0) xv[it].x = v;
            if (j == 1) xv[it].y = v;
            if (j == 2) xv[it].z = v;
            if (j == 3) xv[it].w = v;
          }
        }
      }
    }
  }
}

// MODE 2 gather: this thread's row over the 8 voxels of each of its KG_T
// reduction groups (voxel table vt of the chunk)
__device__ __forceinline__ void gather2(float (&xw)[KG_T][8], const int2 *vt, int kgbase,
                                        int need_t, const float *src_t, int off_t, int xmask_t) {
#pragma unroll
  for (int g = 0; g < KG_T; ++g)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int2 e = vt[(kgbase + g) * 8 + j];
      xw[g][j] = (e.y & need_t) ? 0.f : __ldg(src_t + ((e.x + off_t) & xmask_t));
    }
}

template <int MODE, int VEC>
__global__ void __launch_bounds__(TB_W, 3) k_conv_tc(TcArgs p) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t bars[2];
  __shared__ uint32_t tbase;
  __shared__ TapEnt taps[81];     // MODE 0/1: the taps of the reduction
  __shared__ int ctap[16];        // MODE 1 at stride 2: the class's tap numbers
  __shared__ int2 rows_s[TB_M];   // MODE 0/1: row table (see below)
  __shared__ int2 vtab[3][TB_K];  // MODE 2: voxel tables of three chunks

  // tiles start on 1024-byte boundaries (128-byte swizzle)
  unsigned char *smem = smem_raw + ((1024u - (smem_addr(smem_raw) & 1023u)) & 1023u);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.x * TB_M;
  const int N = p.N;
  const int nb = MODE == 2 ? 2 : 1;  // B tiles per stage
  const int stage_bytes = 2 * A_TILE + nb * N * TB_K * 2;
  const int rin = p.rin, rout = p.rout;
  // MODE 1 at stride 1 reads the output gradient like a forward pass with
  // mirrored taps.  At stride 2 an input voxel u = 2 w + par (per axis)
  // receives only the taps o with u + 1 - o even: o = 1 where par_a = 0, o
  // in {0, 2} where par_a = 1.  Block row blockIdx.y is the parity class par;
  // its rows are the voxels w of the output-gradient grid and its reduction
  // runs over its 1 to 16 taps, each reading w + (par + 1 - o) / 2.
  const bool cls = MODE == 1 && p.stride == 2;
  const int par = cls ? (int)blockIdx.y : 0;
  int ntap_c = 0;
  if (cls) {
    ntap_c = 1;
#pragma unroll
    for (int a = 0; a < 4; ++a) ntap_c *= 1 + ((par >> a) & 1);
  }
  const int Kc = cls ? ntap_c * p.cout : p.K;  // this block's reduction length
  const int kbeg = blockIdx.z * p.kslice;
  const int kend = min(Kc, kbeg + p.kslice);
  const int kpad_end = MODE == 0 ? min(p.Kpad, kbeg + p.kslice) : kend;
  const int nch = (kpad_end - kbeg + TB_K - 1) / TB_K;

  if (warp == 0) tmem_alloc(&tbase, (uint32_t)p.ncols);
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
  }
  if (cls && tid < ntap_c) {
    // class tap tid: bit b of tid picks o = 0 or 2 on the b-th odd axis;
    // `need` marks the axes read at w + 1 (invalid where w + 1 = rout)
    int o[4], bit = 0, need = 0x100, off = 0, st = 1;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      if ((par >> a) & 1) {
        o[a] = ((tid >> bit) & 1) ? 2 : 0;
        ++bit;
      } else {
        o[a] = 1;
      }
      const int delta = (((par >> a) & 1) + 1 - o[a]) / 2;  // 0 or 1
      need |= delta << a;
      off += delta * st;
      st *= rout;
    }
    taps[tid] = TapEnt{need, off};
    ctap[tid] = o[0] + 3 * (o[1] + 3 * (o[2] + 3 * o[3]));
  }
  if ((MODE == 0 || (MODE == 1 && !cls)) && tid < 81) {
    // grid the taps read: the input (MODE 0) or the output gradient (MODE 1)
    const int e = MODE == 0 ? rin : rout;
    int o[4];
    tap_digits(tid, o);
    int need = 0x100, off = 0, st = 1;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int lo = MODE == 0 ? 0 : 2;  // the offset that falls off at coordinate 0
      need |= (o[a] == lo) << a;
      need |= (o[a] == 2 - lo) << (4 + a);
      off += (MODE == 0 ? o[a] - 1 : 1 - o[a]) * st;
      st *= e;
    }
    taps[tid] = TapEnt{need, off};
  }
  // row table: MODE 0: (input voxel of row * stride, edge mask);
  // MODE 1 at stride 1: (row's voxel, edge mask in the output-gradient grid);
  // MODE 1 at stride 2: (row's voxel w, bit a where w_a + 1 = rout)
  if ((MODE == 0 || MODE == 1) && tid < TB_M) {
    const int row = m0 + tid;
    int2 e = make_int2(0, 0x100);
    if (row < p.M) {
      const int ext = MODE == 0 || cls ? rout : rin;
      int c[4], v = row;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        c[a] = v % ext;
        v /= ext;
      }
      if (MODE == 0) {
        int s[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) s[a] = c[a] * p.stride;
        e = make_int2(s[0] + rin * (s[1] + rin * (s[2] + rin * s[3])), edge_mask(s, rin));
      } else if (!cls) {
        e = make_int2(row, edge_mask(c, rout));
      } else {
        int m = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) m |= (c[a] + 1 >= rout) << a;
        e = make_int2(row, m);
      }
    }
    rows_s[tid] = e;
  }
  // MODE 2: this thread's row (tap, ci) reads src_t[(e.x + off_t) & xmask_t]
  // for each voxel e of the table that its `need` mask admits.  The bias
  // row, and rows past the end (never stored), read the constant 1.
  const int lrow = tid & (TB_M - 1), kgbase = (tid / TB_M) * KG_T;
  const int row2 = m0 + lrow;
  const float *src_t = &kOne;
  int need_t = 0x100, off_t = 0, xmask_t = 0;
  if (MODE == 2 && row2 < p.M - p.bias_row) {
    const int tap = row2 / p.cin;
    int o[4];
    tap_digits(tap, o);
    int st = 1, tapoff = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      need_t |= (o[a] == 0) << a;
      need_t |= (o[a] == 2) << (4 + a);
      tapoff += (o[a] - 1) * st;
      st *= rin;
    }
    src_t = p.A;
    off_t = tapoff * p.cin + (row2 - tap * p.cin);
    xmask_t = -1;
  }
  if (MODE == 2) {
    fill_vtab(vtab[0], tid, kbeg, 0, nch, kend, rout, rin, p.stride, p.cin);
    fill_vtab(vtab[1], tid, kbeg, 1, nch, kend, rout, rin, p.stride, p.cin);
  }
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tacc = tbase;
  const uint32_t idesc = idesc_bf16_f32(TB_M, N);
  // MODE 0/1 staging: this thread loads 4 channels (half of reduction group
  // kgl) of rows rsub, rsub + 16, ..., so 16 lanes read 256 contiguous bytes
  // of a row when the chunk stays within one tap
  const int half = tid & 1, kgl = (tid >> 1) & 7, rsub = tid >> 4;
  const int ch = MODE == 0 ? p.cin : p.cout;

  // The next chunk's A values are loaded into registers right after this
  // chunk's are stored, so the loads are in flight across the barrier, the
  // MMA issue and the next stage's wait.
  float4 xv[TB_M / 16];  // MODE 0/1
  float xw[KG_T][8];     // MODE 2
  // warps 0-7 stage the operands; warp 8 only issues the MMAs, so that the
  // staging warps do not wait at the next barrier for the issuing thread
  const bool producer = tid < TB_T;
  if (producer) {
    if (MODE == 2)
      gather2(xw, vtab[0], kgbase, need_t, src_t, off_t, xmask_t);
    else
      gather01<VEC>(xv, p.A, kbeg + kgl * 8 + half * 4, Kc, taps, rows_s, rsub, ch);
  }

  int issued = 0;  // chunks whose MMAs were issued (block-uniform)
  bool bad = false;
  for (int i = 0; i < nch; ++i) {
    const int s = i & 1;
    const int k0 = kbeg + i * TB_K;
    unsigned char *st = smem + s * stage_bytes;
    unsigned char *Ahi = st, *Alo = st + A_TILE, *Bhi = st + 2 * A_TILE;
    unsigned char *Blo = Bhi + N * TB_K * 2;
    if (producer && i >= 2 && !mbar_wait_bounded(&bars[s], ((i - 2) >> 1) & 1)) bad = true;
    if (producer && !bad) {
      if (MODE == 2)
        fill_vtab(vtab[(i + 2) % 3], tid, kbeg, i + 2, nch, kend, rout, rin, p.stride, p.cin);
      // ---- A: store this chunk's registers
      if (MODE == 0 || MODE == 1) {
#pragma unroll
        for (int it = 0; it < TB_M / 16; ++it) {
          uint2 h, l;
          split4(xv[it], h, l);
          const uint32_t o = swz128(it * 16 + rsub, kgl) + half * 8;
          *reinterpret_cast<uint2 *>(Ahi + o) = h;
          *reinterpret_cast<uint2 *>(Alo + o) = l;
        }
      } else {
#pragma unroll
        for (int g = 0; g < KG_T; ++g) {
          uint4 h, l;
          split8(xw[g], h, l);
          const uint32_t o = swz128(lrow, kgbase + g);
          *reinterpret_cast<uint4 *>(Ahi + o) = h;
          *reinterpret_cast<uint4 *>(Alo + o) = l;
        }
      }
      // ---- B: N rows x 8 reduction groups
      for (int e = tid; e < N * 8; e += TB_T) {
        if (MODE == 2) {
          const int n = e % N, kg = e / N;
          float x[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int v = k0 + kg * 8 + j;
            x[j] = v < kend ? __ldg(p.B32 + (size_t)v * p.cout + n) : 0.f;
          }
          uint4 h, l;
          split8(x, h, l);
          const uint32_t o = swz128(n, kg);
          *reinterpret_cast<uint4 *>(Bhi + o) = h;
          *reinterpret_cast<uint4 *>(Blo + o) = l;
        } else {
          const int n = e >> 3, kg = e & 7;
          const int k = k0 + kg * 8;
          uint4 w = make_uint4(0, 0, 0, 0);
          if (MODE == 0) {
            w = __ldg(reinterpret_cast<const uint4 *>(p.Bw + (size_t)n * p.Kpad + k));
          } else if (k < Kc) {
            const int t = k / p.cout, c0 = k - t * p.cout;
            const int tap = cls ? ctap[t] : t;
            w = __ldg(reinterpret_cast<const uint4 *>(
                p.Bw + ((size_t)tap * p.cin + n) * p.cout + c0));
          }
          *reinterpret_cast<uint4 *>(Bhi + swz128(n, kg)) = w;
        }
      }
      // ---- A: the next chunk's loads
      if (i + 1 < nch) {
        if (MODE == 2)
          gather2(xw, vtab[(i + 1) % 3], kgbase, need_t, src_t, off_t, xmask_t);
        else
          gather01<VEC>(xv, p.A, k0 + TB_K + kgl * 8 + half * 4, Kc, taps, rows_s, rsub, ch);
      }
      fence_proxy_async_smem();
    }
    if (__syncthreads_or(bad)) break;
    if (tid == TB_T) {
      fence_after_sync();
      const uint32_t a_hi = smem_addr(Ahi), a_lo = smem_addr(Alo);
      const uint32_t b_hi = smem_addr(Bhi), b_lo = smem_addr(Blo);
#pragma unroll
      for (int kk = 0; kk < TB_K / 16; ++kk) {
        const uint64_t dah = smem_desc_sw128(a_hi + kk * 32);
        const uint64_t dal = smem_desc_sw128(a_lo + kk * 32);
        const uint64_t dbh = smem_desc_sw128(b_hi + kk * 32);
        mma_bf16(tacc, dah, dbh, idesc, (i | kk) != 0);
        mma_bf16(tacc, dal, dbh, idesc, 1);
        if (MODE == 2) mma_bf16(tacc, dah, smem_desc_sw128(b_lo + kk * 32), idesc, 1);
      }
      mma_commit(&bars[s]);
    }
    issued = i + 1;
  }

  // wait for the last issued chunk (its commit covers every earlier MMA)
  bool ok = !bad;
  if (issued > 0) {
    const int last = issued - 1;
    if (!mbar_wait_bounded(&bars[last & 1], (last >> 1) & 1)) ok = false;
  }
  if (!ok) atomicExch(p.err, FLOF_DEV_ERR_TC_TIMEOUT);
  ok = __syncthreads_and(ok);
  // a slice past this block's reduction (a parity class with fewer taps)
  // contributes zeros
  const bool empty = ok && issued == 0;
  ok = ok && issued > 0;
  fence_after_sync();
  if ((ok || empty) && producer) {
    // warp w reads tensor-memory lanes 32 (w % 4) .. + 31; warps 0-3 and
    // 4-7 take alternate 16-column groups
    const int q4 = warp & 3;
    const int r = m0 + 32 * q4 + (tid & 31);
    const bool split = MODE == 2 || gridDim.z > 1;
    // a slice holds every output row: M of them, or all rin^4 input voxels
    // of the parity classes
    const size_t rows_out = cls ? (size_t)rin * rin * rin * rin : (size_t)p.M;
    float *C = p.C + (split ? (size_t)blockIdx.z * rows_out * N : 0);
    // output row: the row itself, or for a parity class the input voxel
    // u = 2 w + par of the row's voxel w
    size_t orow = (size_t)r;
    if (cls && r < p.M) {
      int v = r, u = 0, mul = 1;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        u += (2 * (v % rout) + ((par >> a) & 1)) * mul;
        v /= rout;
        mul *= rin;
      }
      orow = (size_t)u;
    }
    for (int c0 = 16 * (warp >> 2); c0 < N; c0 += 32) {
      float v[16];
      if (ok) {
        tmem_ld16(tacc + ((uint32_t)(32 * q4) << 16) + (uint32_t)c0, v);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0.f;
      }
      if (r < p.M) {
        if (!split && MODE == 0) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float y = v[j] + (p.bias ? __ldg(p.bias + c0 + j) : 0.f);
            v[j] = p.relu && y < 0.f ? 0.f : y;
          }
        }
        float4 *dst = reinterpret_cast<float4 *>(C + orow * N + c0);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tacc, (uint32_t)p.ncols);
  }
}

// out[m][n] = sum over the slices (in order) + bias[n], then ReLU
__global__ void k_sum_slices_epi(const float *__restrict__ work, float *__restrict__ out,
                                 long long n, int nz, int N, const float *__restrict__ bias,
                                 int relu) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < nz; ++z) s += work[(size_t)z * n + q];
    if (bias) s += bias[q % N];
    if (relu && s < 0.f) s = 0.f;
    out[q] = s;
  }
}

// BF16 copies of one layer's weights W[tap][ci][co]: WB in the same order,
// WT[co][tap * cin + ci] with rows of length kpad (the tail stays zero).
// Both loops write consecutive entries from consecutive threads.
__global__ void k_weights_tc(const float *__restrict__ wq, uint16_t *__restrict__ wb,
                             uint16_t *__restrict__ wt, int taps, int cin, int cout, int kpad) {
  const long long K = (long long)taps * cin, n = K * cout;
  const long long step = (long long)gridDim.x * blockDim.x;
  auto bits = [](float x) {
    const __nv_bfloat16 b = __float2bfloat16_rn(x);
    return *reinterpret_cast<const uint16_t *>(&b);
  };
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += step)
    wb[q] = bits(wq[q]);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += step) {
    const long long co = q / K, k = q - co * K;
    wt[(size_t)co * kpad + k] = bits(wq[(size_t)k * cout + co]);
  }
}

// Weight and bias gradient of a 1^4 convolution with CI inputs and CO
// outputs: each thread accumulates its voxels' products, the block reduces
// them in a fixed order into part[block][CI CO + CO].
template <int CI, int CO>
__global__ void __launch_bounds__(256) k_wgrad_1x1(const float *__restrict__ in,
                                                   const float *__restrict__ dout, long long V,
                                                   float *__restrict__ part) {
  constexpr int NV = CI * CO + CO;
  __shared__ float red[8][NV];
  float acc[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) acc[j] = 0.f;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
       v += (long long)gridDim.x * blockDim.x) {
    float a[CI], d[CO];
#pragma unroll
    for (int c = 0; c < CI; ++c) a[c] = __ldg(in + v * CI + c);
#pragma unroll
    for (int c = 0; c < CO; ++c) d[c] = __ldg(dout + v * CO + c);
#pragma unroll
    for (int ci = 0; ci < CI; ++ci)
#pragma unroll
      for (int co = 0; co < CO; ++co) acc[ci * CO + co] += a[ci] * d[co];
#pragma unroll
    for (int co = 0; co < CO; ++co) acc[CI * CO + co] += d[co];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    float x = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][j] = x;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < NV; j += blockDim.x) {
    float x = 0.f;
    for (int w = 0; w < 8; ++w) x += red[w][j];
    part[(size_t)blockIdx.x * NV + j] = x;
  }
}

// out[j] = sum over the blocks' partials: one warp per entry, lane l adds
// blocks l, l + 32, ... in order, then a fixed butterfly (deterministic)
__global__ void k_sum_parts(const float *__restrict__ part, int nblocks, int nv,
                            float *__restrict__ out) {
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (j >= nv) return;
  float x = 0.f;
  for (int b = lane; b < nblocks; b += 32) x += part[(size_t)b * nv + j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if (lane == 0) out[j] = x;
}

struct TcPlan {
  int nz, kslice;
};

// Slices of the reduction.  With `slots` = resident blocks per SM x SMs, a
// split into nz slices takes ceil(tiles nz / slots) waves of ceil(chunks /
// nz) chunks each, plus the pass that sums the slices: a launch (about 1.5
// chunk times) and reading nz M N floats (about 1.1 M of them per chunk
// time).  The split with the lowest estimate wins (at least four chunks per
// slice).
TcPlan tc_plan(long long M, long long K, int N, int resident) {
  const long long tiles = (M + TB_M - 1) / TB_M;
  const long long chunks = (K + TB_K - 1) / TB_K;
  const long long slots = (long long)std::max(resident, 1) * sm_count();
  const long long maxz = std::max(chunks / 4, 1LL);
  long long best = 1;
  double best_t = 1e300;
  for (long long nz = 1; nz <= maxz; ++nz) {
    const long long per = (chunks + nz - 1) / nz;
    const long long z = (chunks + per - 1) / per;  // slices actually used
    const long long waves = (tiles * z + slots - 1) / slots;
    const double t = (double)(waves * per) + (z > 1 ? 1.5 + (double)z * M * N / 1.1e6 : 0.0);
    if (t < best_t) best_t = t, best = z;
  }
  const long long per = (chunks + best - 1) / best;
  return TcPlan{(int)((chunks + per - 1) / per), (int)(per * TB_K)};
}

int pow2_cols(int n) {
  int c = 32;
  while (c < n) c <<= 1;
  return c;
}

template <int MODE>
int tc_smem(int N) {
  return 2 * (2 * A_TILE + (MODE == 2 ? 2 : 1) * N * TB_K * 2) + 1024;
}

// once per kernel: room for the largest stage pair (N = 128, two B tiles)
template <int MODE, int VEC>
void tc_attr() {
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_conv_tc<MODE, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           tc_smem<2>(128));
  fh::cuda_check(attr, "cudaFuncSetAttribute(k_conv_tc)");
}

// resident blocks per SM for N columns (N a multiple of 16 up to 128),
// queried once per shape
template <int MODE, int VEC>
int tc_resident(int N) {
  static std::atomic<int> cache[128 / 16 + 1];
  std::atomic<int> &slot = cache[N / 16];
  const int known = slot.load(std::memory_order_relaxed);
  if (known > 0) return known;
  tc_attr<MODE, VEC>();
  int nb = 0;
  fh::cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_conv_tc<MODE, VEC>, TB_W,
                                                               tc_smem<MODE>(N)),
                 "cudaOccupancyMaxActiveBlocksPerMultiprocessor(k_conv_tc)");
  nb = std::max(nb, 1);
  slot.store(nb, std::memory_order_relaxed);
  return nb;
}

template <int MODE, int VEC>
TcPlan tc_plan_for(long long M, long long K, int N) {
  return tc_plan(M, K, N, tc_resident<MODE, VEC>(N));
}

template <int MODE, int VEC>
void launch_tc(const TcArgs &a0, int nz, cudaStream_t s, int gy = 1) {
  TcArgs a = a0;
  a.ncols = pow2_cols(a.N);
  tc_attr<MODE, VEC>();
  dim3 grid((a.M + TB_M - 1) / TB_M, gy, nz);
  k_conv_tc<MODE, VEC><<<grid, TB_W, tc_smem<MODE>(a.N), s>>>(a);
  // a refused launch (configuration) is reported here, not by a later sync
  fh::cuda_check(cudaGetLastError(), "k_conv_tc launch");
}

// Slices of a stride-2 input gradient (16 parity classes of M rows, at most K
// = 16 cout reduction entries): enough blocks for about three per SM, at
// least two chunks per slice.
int cls_slices(long long M, long long K) {
  const long long blocks = (M + TB_M - 1) / TB_M * 16;
  const long long chunks = (K + TB_K - 1) / TB_K;
  long long nz = (3LL * sm_count() + blocks - 1) / blocks;
  nz = std::min(nz, std::max(chunks / 2, 1LL));
  const long long per = (chunks + nz - 1) / nz;
  return (int)((chunks + per - 1) / per);
}

TcPlan plan_fwd(long long M, long long K, int cin, int cout) {
  return cin % 8 == 0 ? tc_plan_for<0, 1>(M, K, cout) : tc_plan_for<0, 0>(M, K, cout);
}

}  // namespace

// ---- launchers --------------------------------------------------------------

bool net_tc_fwd_ok(int cin, int cout, int ks) {
  (void)cin;
  return ks == 3 && cout % 16 == 0 && cout <= 128;
}
bool net_tc_bwd_data_ok(int cin, int cout, int ks) {
  return ks == 3 && cin % 16 == 0 && cin <= 128 && cout % 8 == 0;
}
bool net_tc_bwd_weight_ok(int cin, int cout, int ks) {
  (void)cin;
  return ks == 3 && cout % 16 == 0 && cout <= 128;
}
int net_tc_kpad(int cin, int ks) {
  const int K = (ks == 3 ? 81 : 1) * cin;
  return (K + TB_K - 1) / TB_K * TB_K;
}

size_t net_tc_work(int rin, int rout, int cin, int cout, int ks) {
  size_t w = 0;
  const long long Vi = (long long)rin * rin * rin * rin, Vo = (long long)rout * rout * rout * rout;
  if (net_tc_fwd_ok(cin, cout, ks)) {
    const TcPlan pl = plan_fwd(Vo, net_tc_kpad(cin, ks), cin, cout);
    if (pl.nz > 1) w = std::max(w, (size_t)pl.nz * (size_t)Vo * cout);
  }
  if (net_tc_bwd_data_ok(cin, cout, ks)) {
    const int nz = rin == rout ? tc_plan_for<1, 1>(Vi, 81LL * cout, cin).nz
                               : cls_slices(Vo, 16LL * cout);
    if (nz > 1) w = std::max(w, (size_t)nz * (size_t)Vi * cin);
  }
  if (net_tc_bwd_weight_ok(cin, cout, ks)) {
    const TcPlan pl = tc_plan_for<2, 0>(81LL * cin + 1, Vo, cout);
    w = std::max(w, (size_t)pl.nz * (81 * cin + 1) * cout);
  }
  return w;
}

bool net_wgrad_1x1_ok(int cin, int cout, int ks) { return ks == 1 && cin == 16 && cout == 4; }
size_t net_wgrad_1x1_work() { return (size_t)2 * 152 * (16 * 4 + 4) * 4; }

void net_wgrad_1x1(const float *in, const float *dout, float *dw, float *work, long long V,
                   cudaStream_t s) {
  const int nb = std::min(2 * sm_count(), 4 * 152);
  k_wgrad_1x1<16, 4><<<nb, 256, 0, s>>>(in, dout, V, work);
  k_sum_parts<<<(16 * 4 + 4 + 3) / 4, 128, 0, s>>>(work, nb, 16 * 4 + 4, dw);
}

void net_weights_tc(const float *wq, uint16_t *wb, uint16_t *wt, int cin, int cout, int ks,
                    cudaStream_t s) {
  const int taps = ks == 3 ? 81 : 1;
  const long long n = (long long)taps * cin * cout;
  k_weights_tc<<<grid_for(n, 256), 256, 0, s>>>(wq, wb, wt, taps, cin, cout,
                                                net_tc_kpad(cin, ks));
}

void net_tc_conv_fwd(const float *in, const uint16_t *wt, const float *b, float *out,
                     float *work, int rin, int rout, int cin, int cout, int stride, int relu,
                     int *err, cudaStream_t s) {
  TcArgs a{};
  a.A = in;
  a.Bw = wt;
  a.err = err;
  a.rin = rin, a.rout = rout, a.cin = cin, a.cout = cout, a.stride = stride;
  a.M = rout * rout * rout * rout;
  a.N = cout;
  a.K = 81 * cin;
  a.Kpad = net_tc_kpad(cin, 3);
  a.relu = relu;
  const TcPlan pl = plan_fwd(a.M, a.Kpad, cin, cout);
  a.kslice = pl.kslice;
  a.bias = pl.nz > 1 ? nullptr : b;
  a.C = pl.nz > 1 ? work : out;
  if (cin % 8 == 0)
    launch_tc<0, 1>(a, pl.nz, s);
  else
    launch_tc<0, 0>(a, pl.nz, s);
  if (pl.nz > 1) {
    const long long n = (long long)a.M * a.N;
    k_sum_slices_epi<<<grid_for(n, 256), 256, 0, s>>>(work, out, n, pl.nz, a.N, b, relu);
  }
}

void net_tc_conv_bwd_data(const float *dout, const uint16_t *wb, float *din, float *work,
                          int rin, int rout, int cin, int cout, int stride, int *err,
                          cudaStream_t s) {
  TcArgs a{};
  a.A = dout;
  a.Bw = wb;
  a.err = err;
  a.rin = rin, a.rout = rout, a.cin = cin, a.cout = cout, a.stride = stride;
  a.N = cin;
  if (stride == 2) {
    // 16 parity classes of rout^4 rows each, at most 16 taps
    a.M = rout * rout * rout * rout;
    a.K = 16 * cout;
    a.Kpad = a.K;
    const int nz = cls_slices(a.M, a.K);
    const int chunks = (a.K + TB_K - 1) / TB_K;
    a.kslice = (chunks + nz - 1) / nz * TB_K;
    a.C = nz > 1 ? work : din;
    launch_tc<1, 1>(a, nz, s, 16);
    if (nz > 1) {
      const long long n = (long long)rin * rin * rin * rin * cin;
      k_sum_slices_epi<<<grid_for(n, 256), 256, 0, s>>>(work, din, n, nz, cin, nullptr, 0);
    }
    return;
  }
  a.M = rin * rin * rin * rin;
  a.K = 81 * cout;
  a.Kpad = a.K;
  const TcPlan pl = tc_plan_for<1, 1>(a.M, a.K, a.N);
  a.kslice = pl.kslice;
  a.C = pl.nz > 1 ? work : din;
  launch_tc<1, 1>(a, pl.nz, s);
  if (pl.nz > 1) {
    const long long n = (long long)a.M * a.N;
    k_sum_slices_epi<<<grid_for(n, 256), 256, 0, s>>>(work, din, n, pl.nz, a.N, nullptr, 0);
  }
}

void net_tc_conv_bwd_weight(const float *in, const float *dout, float *dw, float *work, int rin,
                            int rout, int cin, int cout, int stride, int *err, cudaStream_t s) {
  TcArgs a{};
  a.A = in;
  a.B32 = dout;
  a.err = err;
  a.rin = rin, a.rout = rout, a.cin = cin, a.cout = cout, a.stride = stride;
  a.M = 81 * cin + 1;  // the (tap, ci) rows and the bias row
  a.bias_row = 1;
  a.N = cout;
  a.K = rout * rout * rout * rout;
  a.Kpad = a.K;
  const TcPlan pl = tc_plan_for<2, 0>(a.M, a.K, a.N);
  a.kslice = pl.kslice;
  a.C = work;
  launch_tc<2, 0>(a, pl.nz, s);
  const long long n = (long long)a.M * a.N;
  k_sum_slices_epi<<<grid_for(n, 256), 256, 0, s>>>(work, dw, n, pl.nz, a.N, nullptr, 0);
}

}  // namespace flof
