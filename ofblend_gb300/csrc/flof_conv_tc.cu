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
// Per block: 128 threads gather a 128 x 64 reduction chunk of the operand
// (im2col on the fly: voxel rows x (tap, channel), or (tap, channel) rows x
// voxels for the weight gradient) through registers into shared memory in
// the no-swizzle K-major layout (flof_tcgen05.cuh), while thread 0's MMAs of
// the previous chunk run; two stages, each released by a tcgen05.commit on
// its mbarrier.  Layers with few row tiles split the reduction into slices
// written to a work buffer and summed in slice order (deterministic), with
// the bias and ReLU applied there.
//
// Every mbarrier wait is bounded: a block that gives up stores
// FLOF_DEV_ERR_TC_TIMEOUT in the context's device error word, waits (again
// bounded) for its issued MMAs, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "flof_internal.h"
#include "flof_tcgen05.cuh"

namespace flof {

namespace {

using namespace tc;

constexpr int TB_M = 128;  // rows per block (the MMA's M)
constexpr int TB_K = 64;   // reduction entries per chunk (four K = 16 MMAs)
constexpr int TB_T = 128;  // threads
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
};

// (tap, channel) reduction entries of a 3^4 tap with offsets o in 0..2 per
// axis: `need` has bit a set when o_a = 0 and bit 4 + a when o_a = 2, plus
// bit 8 (never valid for an invalid row or voxel); `off` is the tap's
// linear voxel offset sum (o_a - 1) stride_a in the grid it reads.
struct TapEnt {
  int need, off;
};

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

template <int MODE, int VEC>
__global__ void __launch_bounds__(TB_T) k_conv_tc(TcArgs p) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bars[2];
  __shared__ uint32_t tbase;
  __shared__ TapEnt taps[81];          // MODE 0
  __shared__ int2 vtab[2][TB_K];       // MODE 2: (input voxel of v * stride, edge mask)

  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.x * TB_M;
  const int N = p.N;
  const int nb = MODE == 2 ? 2 : 1;  // B tiles per stage
  const int stage_bytes = 2 * A_TILE + nb * N * TB_K * 2;
  const int kbeg = blockIdx.z * p.kslice;
  const int kend = min(p.K, kbeg + p.kslice);
  const int kpad_end = MODE == 0 ? min(p.Kpad, kbeg + p.kslice) : kend;
  const int nch = (kpad_end - kbeg + TB_K - 1) / TB_K;
  const int rin = p.rin, rout = p.rout;
  const int is1 = rin, is2 = rin * rin, is3 = rin * rin * rin;  // input strides

  if (warp == 0) tmem_alloc(&tbase, (uint32_t)p.ncols);
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
  }
  if (MODE == 0 && tid < 81) {
    int o[4];
    tap_digits(tid, o);
    int need = 0x100, off = 0;
    const int st[4] = {1, is1, is2, is3};
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      need |= (o[a] == 0) << a;
      need |= (o[a] == 2) << (4 + a);
      off += (o[a] - 1) * st[a];
    }
    taps[tid] = TapEnt{need, off};
  }

  // this thread's row
  const int row = m0 + tid;
  const bool rowvalid = row < p.M;
  int rc[4] = {0, 0, 0, 0};     // MODE 0/1: voxel coordinates of the row
  int rowlin = 0, rowmask = 0x100;  // MODE 0
  int need_t = 0x100, tapoff_t = 0, ci_t = 0;  // MODE 2
  if (MODE == 0 || MODE == 1) {
    if (rowvalid) {
      int v = row;
      const int ext = MODE == 0 ? rout : rin;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        rc[a] = v % ext;
        v /= ext;
      }
    }
    if (MODE == 0 && rowvalid) {
      int s[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) s[a] = rc[a] * p.stride;
      rowlin = s[0] + s[1] * is1 + s[2] * is2 + s[3] * is3;
      rowmask = edge_mask(s, rin);
    }
  } else if (rowvalid) {
    const int tap = row / p.cin;
    ci_t = row - tap * p.cin;
    int o[4];
    tap_digits(tap, o);
    need_t = 0x100;
    const int st[4] = {1, is1, is2, is3};
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      need_t |= (o[a] == 0) << a;
      need_t |= (o[a] == 2) << (4 + a);
      tapoff_t += (o[a] - 1) * st[a];
    }
  }
  // MODE 2: voxel table of chunk c into vtab[c & 1]
  auto fill_vtab = [&](int c) {
    if (MODE == 2 && tid < TB_K) {
      const int v = kbeg + c * TB_K + tid;
      int2 e = make_int2(0, 0x100);
      if (c < nch && v < kend) {
        int s[4], q = v;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          s[a] = (q % rout) * p.stride;
          q /= rout;
        }
        e = make_int2(s[0] + s[1] * is1 + s[2] * is2 + s[3] * is3, edge_mask(s, rin));
      }
      vtab[c & 1][tid] = e;
    }
  };
  fill_vtab(0);
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tacc = tbase;
  const uint32_t idesc = idesc_bf16_f32(TB_M, N);

  int issued = 0;  // chunks whose MMAs were issued (block-uniform)
  bool bad = false;
  for (int i = 0; i < nch; ++i) {
    const int s = i & 1;
    const int k0 = kbeg + i * TB_K;
    unsigned char *st = smem + s * stage_bytes;
    unsigned char *Ahi = st, *Alo = st + A_TILE, *Bhi = st + 2 * A_TILE;
    unsigned char *Blo = Bhi + N * TB_K * 2;
    if (i >= 2 && !mbar_wait_bounded(&bars[s], ((i - 2) >> 1) & 1)) bad = true;
    if (!bad) {
      fill_vtab(i + 1);
      // ---- A: 8 reduction groups of this thread's row
      if (MODE == 0 || MODE == 1) {
        float x[8][8];
#pragma unroll
        for (int kg = 0; kg < 8; ++kg) {
          const int k = k0 + kg * 8;
#pragma unroll
          for (int j = 0; j < 8; ++j) x[kg][j] = 0.f;
          if (VEC) {
            const int ch = MODE == 0 ? p.cin : p.cout;
            if (rowvalid && k < p.K) {
              const int tap = k / ch, c0 = k - tap * ch;
              const float *src = nullptr;
              if (MODE == 0) {
                const TapEnt t = taps[tap];
                if (!(rowmask & t.need)) src = p.A + (size_t)(rowlin + t.off) * p.cin + c0;
              } else {
                int o[4];
                tap_digits(tap, o);
                bool ok = true;
                int lin = 0, mul = 1;
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                  const int num = rc[a] + 1 - o[a];
                  const int q = num / p.stride;
                  ok = ok && num >= 0 && q * p.stride == num && q < rout;
                  lin += q * mul;
                  mul *= rout;
                }
                if (ok) src = p.A + (size_t)lin * p.cout + c0;
              }
              if (src) {
                const float4 u = __ldg(reinterpret_cast<const float4 *>(src));
                const float4 w = __ldg(reinterpret_cast<const float4 *>(src) + 1);
                x[kg][0] = u.x, x[kg][1] = u.y, x[kg][2] = u.z, x[kg][3] = u.w;
                x[kg][4] = w.x, x[kg][5] = w.y, x[kg][6] = w.z, x[kg][7] = w.w;
              }
            }
          } else {  // MODE 0 with a channel count that is not a multiple of 8
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int kj = k + j;
              if (rowvalid && kj < p.K) {
                const int tap = kj / p.cin, ci = kj - tap * p.cin;
                const TapEnt t = taps[tap];
                if (!(rowmask & t.need))
                  x[kg][j] = __ldg(p.A + (size_t)(rowlin + t.off) * p.cin + ci);
              }
            }
          }
        }
#pragma unroll
        for (int kg = 0; kg < 8; ++kg) {
          uint4 h, l;
          split8(x[kg], h, l);
          const uint32_t o = core_off(tid, kg, TB_M);
          *reinterpret_cast<uint4 *>(Ahi + o) = h;
          *reinterpret_cast<uint4 *>(Alo + o) = l;
        }
      } else {  // MODE 2: row (tap, ci), reduction over voxels
#pragma unroll
        for (int kg = 0; kg < 8; ++kg) {
          float x[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int2 e = vtab[s][kg * 8 + j];
            x[j] = (rowvalid && !(e.y & need_t))
                       ? __ldg(p.A + (size_t)(e.x + tapoff_t) * p.cin + ci_t)
                       : 0.f;
          }
          uint4 h, l;
          split8(x, h, l);
          const uint32_t o = core_off(tid, kg, TB_M);
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
          const uint32_t o = core_off(n, kg, N);
          *reinterpret_cast<uint4 *>(Bhi + o) = h;
          *reinterpret_cast<uint4 *>(Blo + o) = l;
        } else {
          const int n = e >> 3, kg = e & 7;
          const int k = k0 + kg * 8;
          uint4 w = make_uint4(0, 0, 0, 0);
          if (MODE == 0) {
            w = __ldg(reinterpret_cast<const uint4 *>(p.Bw + (size_t)n * p.Kpad + k));
          } else if (k < p.K) {
            const int tap = k / p.cout, c0 = k - tap * p.cout;
            w = __ldg(reinterpret_cast<const uint4 *>(
                p.Bw + ((size_t)tap * p.cin + n) * p.cout + c0));
          }
          *reinterpret_cast<uint4 *>(Bhi + core_off(n, kg, N)) = w;
        }
      }
      fence_proxy_async_smem();
    }
    if (__syncthreads_or(bad)) break;
    if (tid == 0) {
      fence_after_sync();
      const uint32_t a_hi = smem_addr(Ahi), a_lo = smem_addr(Alo);
      const uint32_t b_hi = smem_addr(Bhi), b_lo = smem_addr(Blo);
#pragma unroll
      for (int kk = 0; kk < TB_K / 16; ++kk) {
        const uint32_t ao = kk * 2 * (TB_M * 16), bo = kk * 2 * (N * 16);
        const uint64_t dah = smem_desc(a_hi + ao, TB_M * 16, 128);
        const uint64_t dal = smem_desc(a_lo + ao, TB_M * 16, 128);
        const uint64_t dbh = smem_desc(b_hi + bo, N * 16, 128);
        mma_bf16(tacc, dah, dbh, idesc, (i | kk) != 0);
        mma_bf16(tacc, dal, dbh, idesc, 1);
        if (MODE == 2) mma_bf16(tacc, dah, smem_desc(b_lo + bo, N * 16, 128), idesc, 1);
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
  ok = __syncthreads_and(ok) && issued > 0;
  fence_after_sync();
  if (ok) {
    const int r = m0 + 32 * warp + (tid & 31);
    const bool split = MODE == 2 || gridDim.z > 1;
    float *C = p.C + (split ? (size_t)blockIdx.z * p.M * N : 0);
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tmem_ld16(tacc + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
      if (r < p.M) {
        if (!split && MODE == 0) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float y = v[j] + (p.bias ? __ldg(p.bias + c0 + j) : 0.f);
            v[j] = p.relu && y < 0.f ? 0.f : y;
          }
        }
        float4 *dst = reinterpret_cast<float4 *>(C + (size_t)r * N + c0);
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
// WT[co][tap * cin + ci] with rows of length kpad (the tail stays zero)
__global__ void k_weights_tc(const float *__restrict__ wq, uint16_t *__restrict__ wb,
                             uint16_t *__restrict__ wt, int taps, int cin, int cout, int kpad) {
  const long long n = (long long)taps * cin * cout;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const __nv_bfloat16 b = __float2bfloat16_rn(wq[q]);
    const uint16_t bits = *reinterpret_cast<const uint16_t *>(&b);
    const int co = (int)(q % cout);
    const long long k = q / cout;  // tap * cin + ci
    wb[q] = bits;
    wt[(size_t)co * kpad + k] = bits;
  }
}

struct TcPlan {
  int nz, kslice;
};

// Slices of the reduction: about two blocks per SM in total, at least four
// chunks per slice.
TcPlan tc_plan(long long M, long long K) {
  const long long tiles = (M + TB_M - 1) / TB_M;
  const long long chunks = (K + TB_K - 1) / TB_K;
  const long long target = 2LL * sm_count();
  long long nz = tiles >= target ? 1 : (target + tiles - 1) / tiles;
  const long long maxz = chunks / 4 > 1 ? chunks / 4 : 1;
  if (nz > maxz) nz = maxz;
  long long per = (chunks + nz - 1) / nz;
  nz = (chunks + per - 1) / per;
  return TcPlan{(int)nz, (int)(per * TB_K)};
}

int pow2_cols(int n) {
  int c = 32;
  while (c < n) c <<= 1;
  return c;
}

template <int MODE, int VEC>
void launch_tc(const TcArgs &a0, int nz, cudaStream_t s) {
  TcArgs a = a0;
  a.ncols = pow2_cols(a.N);
  const int smem = 2 * (2 * A_TILE + (MODE == 2 ? 2 : 1) * a.N * TB_K * 2);
  // once per kernel: room for the largest stage pair (N = 128, two B tiles)
  static const cudaError_t attr = cudaFuncSetAttribute(
      k_conv_tc<MODE, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      2 * (2 * A_TILE + 2 * 128 * TB_K * 2));
  fh::cuda_check(attr, "cudaFuncSetAttribute(k_conv_tc)");
  dim3 grid((a.M + TB_M - 1) / TB_M, 1, nz);
  k_conv_tc<MODE, VEC><<<grid, TB_T, smem, s>>>(a);
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
    const TcPlan pl = tc_plan(Vo, net_tc_kpad(cin, ks));
    if (pl.nz > 1) w = std::max(w, (size_t)pl.nz * (size_t)Vo * cout);
  }
  if (net_tc_bwd_data_ok(cin, cout, ks)) {
    const TcPlan pl = tc_plan(Vi, 81LL * cout);
    if (pl.nz > 1) w = std::max(w, (size_t)pl.nz * (size_t)Vi * cin);
  }
  if (net_tc_bwd_weight_ok(cin, cout, ks)) {
    const TcPlan pl = tc_plan(81LL * cin, Vo);
    w = std::max(w, (size_t)pl.nz * 81 * cin * cout);
  }
  return w;
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
  const TcPlan pl = tc_plan(a.M, a.Kpad);
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
  a.M = rin * rin * rin * rin;
  a.N = cin;
  a.K = 81 * cout;
  a.Kpad = a.K;
  const TcPlan pl = tc_plan(a.M, a.K);
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
  a.M = 81 * cin;
  a.N = cout;
  a.K = rout * rout * rout * rout;
  a.Kpad = a.K;
  const TcPlan pl = tc_plan(a.M, a.K);
  a.kslice = pl.kslice;
  a.C = work;
  launch_tc<2, 0>(a, pl.nz, s);
  const long long n = (long long)a.M * a.N;
  k_sum_slices_epi<<<grid_for(n, 256), 256, 0, s>>>(work, dw, n, pl.nz, a.N, nullptr, 0);
}

}  // namespace flof
