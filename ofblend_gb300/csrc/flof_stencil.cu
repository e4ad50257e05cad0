// flof_stencil.cu -- shared-memory slab kernels for the dense 4D stencils of
// the FlOF path: the Gaussian velocity blur (knGaussianBlur,
// optflow4d.cpp:132-158, radius 1 and 2) and the extrapolation sweep
// (knCvExpolBlur4d, :613-626).
//
// Both sum a (2S+1)^4 neighbourhood in the reference's loop order
// (t outermost, then z, y, x) with float adds in sequence, so the results are
// bitwise those of the reference.  A block owns a 32x32 (x,y) tile at one
// (z,t); it walks the (2S+1)^2 (t,z) offsets in that order, staging each
// (x,y) input slab with its S-cell halo in shared memory through cp.async
// (double buffered; cells outside the grid are zero-filled, which leaves a
// sum unchanged: adding w*0 = +0 to a running float sum never changes it).
// Each thread computes a 4 (x) by 2 (y) block of outputs, so every staged
// value it loads from shared memory feeds up to 8 outputs.
#include "flof_kernels.h"

namespace flof {

namespace {

constexpr int TX = 32, TY = 32, RX = 4, RY = 2;
constexpr int NTX = TX / RX, NTY = TY / RY, NTHREADS = NTX * NTY;  // 8 x 16

template <int S>
struct SlabGeom {
  static constexpr int W = TX + 2 * S;      // slab width in cells
  static constexpr int H = TY + 2 * S;      // slab height in cells
  static constexpr int PITCH = W + W / 8 + 1;
  static constexpr int SLOTS = H * PITCH;   // incl. skew padding
  // skewed column: one pad slot after every 8 cells keeps the 8 threads of a
  // 128-bit shared-memory phase on distinct banks
  __device__ static __forceinline__ int at(int row, int col) {
    return row * PITCH + col + (col >> 3);
  }
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes));
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem, int bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <int NC>
struct VT;
template <>
struct VT<4> {
  typedef float4 T;
  __device__ static __forceinline__ T zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
};
template <>
struct VT<1> {
  typedef float T;
  __device__ static __forceinline__ T zero() { return 0.f; }
};

__device__ __forceinline__ void mac(float4 &v, float w, const float4 &a) {
  v.x += w * a.x;
  v.y += w * a.y;
  v.z += w * a.z;
  v.w += w * a.w;
}
__device__ __forceinline__ void mac(float &v, float w, const float &a) { v += w * a; }
__device__ __forceinline__ void acc(float4 &v, const float4 &a) {
  v.x += a.x;
  v.y += a.y;
  v.z += a.z;
  v.w += a.w;
}
__device__ __forceinline__ void acc(float &v, const float &a) { v += a; }

// Issue the copies of the (x,y) slab at plane (zz, tt) into buffer `buf`.
// Warp w copies slab rows w, w+4, ...; lane l copies columns l and l+32 of
// each row, so the per-element work is one address add and one predicate.
template <int S, int NC>
__device__ __forceinline__ void issue_slab(typename VT<NC>::T *buf, const float *__restrict__ src,
                                           const Dims4 &d, int x0, int y0, int zz, int tt) {
  typedef SlabGeom<S> G;
  typedef typename VT<NC>::T T;
  static_assert(G::W <= 64, "slab wider than two warps of columns");
  const bool plane_ok = zz >= 0 && zz < d.z && tt >= 0 && tt < d.t;
  const T *base = (const T *)src;
  const T *plane = plane_ok ? base + ((idx_t)zz * d.sz() + (idx_t)tt * d.st()) : base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sx0 = lane, sx1 = lane + 32;
  const int gx0 = x0 - S + sx0, gx1 = x0 - S + sx1;
  const bool okx0 = gx0 >= 0 && gx0 < d.x;
  const bool okx1 = sx1 < G::W && gx1 >= 0 && gx1 < d.x;
  for (int sy = warp; sy < G::H; sy += NTHREADS / 32) {
    const int gy = y0 - S + sy;
    const bool oky = plane_ok && gy >= 0 && gy < d.y;
    const T *row = plane + (idx_t)(oky ? gy : 0) * d.x;
    {
      const bool ok = oky && okx0;
      T *s0 = buf + G::at(sy, sx0);
      if (NC == 4) cp_async16(s0, ok ? row + gx0 : base, ok ? 16 : 0);
      else cp_async4(s0, ok ? row + gx0 : base, ok ? 4 : 0);
    }
    if (sx1 < G::W) {
      const bool ok = oky && okx1;
      T *s1 = buf + G::at(sy, sx1);
      if (NC == 4) cp_async16(s1, ok ? row + gx1 : base, ok ? 16 : 0);
      else cp_async4(s1, ok ? row + gx1 : base, ok ? 4 : 0);
    }
  }
}

// Weight-sum table index of a cell: per axis, how many taps fall below 0 and
// above size-1 (knGaussianBlur skips those taps, optflow4d.cpp:143).
template <int S>
__device__ __forceinline__ int clip_code(int c, int ext) {
  int lo = S - c;
  lo = lo < 0 ? 0 : lo;
  int hi = c + S - (ext - 1);
  hi = hi < 0 ? 0 : hi;
  return lo * (S + 1) + hi;
}

}  // namespace

struct WTab2 {
  float w[40];  // exp weight by squared distance, S <= 2 (d^2 <= 16)
};

// MODE 0: Gaussian blur pass; MODE 1: extrapolation sweep (box sum of 81).
template <int S, int NC, int MODE>
__global__ void __launch_bounds__(NTHREADS)
k_slab_stencil(const float *__restrict__ src, float *__restrict__ dst, Dims4 d, int tiles_x,
               const float *__restrict__ wsum, const float *__restrict__ mark, WTab2 wt,
               int zero_border) {
  typedef SlabGeom<S> G;
  typedef typename VT<NC>::T T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *slab0 = (T *)smem_raw;
  T *slab1 = slab0 + G::SLOTS;
  __shared__ float wsh[40];
  if (MODE == 0 && threadIdx.x < 40) wsh[threadIdx.x] = wt.w[threadIdx.x];

  const int tile = blockIdx.x;
  const int x0 = (tile % tiles_x) * TX, y0 = (tile / tiles_x) * TY;
  const int z = blockIdx.y, t = blockIdx.z;
  const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;

  T val[RY][RX];
#pragma unroll
  for (int q = 0; q < RY; ++q)
#pragma unroll
    for (int r = 0; r < RX; ++r) val[q][r] = VT<NC>::zero();

  constexpr int K = 2 * S + 1;
  constexpr int NP = K * K;  // (t, z) offsets
  issue_slab<S, NC>(slab0, src, d, x0, y0, z - S, t - S);
  cp_async_commit();
  for (int p = 0; p < NP; ++p) {
    const int vt = p / K - S, zk = p % K - S;
    T *cur = (p & 1) ? slab1 : slab0;
    if (p + 1 < NP) {
      T *nxt = (p & 1) ? slab0 : slab1;
      issue_slab<S, NC>(nxt, src, d, x0, y0, z + ((p + 1) % K - S), t + ((p + 1) / K - S));
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    // rows 2ty .. 2ty+RY-1+2S of the slab feed output rows 2ty+q via yj = k-q-S
#pragma unroll
    for (int k = 0; k < RY + 2 * S; ++k) {
      T a[RX + 2 * S];
#pragma unroll
      for (int m = 0; m < RX + 2 * S; ++m) a[m] = cur[G::at(RY * ty + k, RX * tx + m)];
#pragma unroll
      for (int q = 0; q < RY; ++q) {
        const int yj = k - q - S;
        if (yj < -S || yj > S) continue;
        if (MODE == 0) {
          const int base = vt * vt + zk * zk + yj * yj;
          float wx[S + 1];  // weight by |xi|
#pragma unroll
          for (int e = 0; e <= S; ++e) wx[e] = wsh[base + e * e];
#pragma unroll
          for (int r = 0; r < RX; ++r)
#pragma unroll
            for (int xi = -S; xi <= S; ++xi) mac(val[q][r], wx[xi < 0 ? -xi : xi], a[r + S + xi]);
        } else {
#pragma unroll
          for (int r = 0; r < RX; ++r)
#pragma unroll
            for (int xi = -S; xi <= S; ++xi) acc(val[q][r], a[r + S + xi]);
        }
      }
    }
    __syncthreads();
  }

  const bool zt_inner = z >= 1 && z < d.z - 1 && t >= 1 && t < d.t - 1;
  int code_zt = 0;
  if (MODE == 0) {
    constexpr int P1 = (S + 1) * (S + 1);
    code_zt = (clip_code<S>(t, d.t) * P1 + clip_code<S>(z, d.z)) * P1;
  }
#pragma unroll
  for (int q = 0; q < RY; ++q) {
    const int y = y0 + RY * ty + q;
    if (y >= d.y) continue;
#pragma unroll
    for (int r = 0; r < RX; ++r) {
      const int x = x0 + RX * tx + r;
      if (x >= d.x) continue;
      const idx_t id = d.index(x, y, z, t);
      const bool inner = zt_inner && x >= 1 && x < d.x - 1 && y >= 1 && y < d.y - 1;
      T *out = (T *)dst;
      if (MODE == 0) {
        if (!inner) {
          if (zero_border) out[id] = VT<NC>::zero();
          continue;
        }
        constexpr int P1 = (S + 1) * (S + 1);
        const float wsum_c = __ldg(wsum + (code_zt + clip_code<S>(y, d.y)) * P1 + clip_code<S>(x, d.x));
        T v = val[q][r];
        if (NC == 4) {
          float4 &f = *(float4 *)&v;
          f.x = f.x / wsum_c;
          f.y = f.y / wsum_c;
          f.z = f.z / wsum_c;
          f.w = f.w / wsum_c;
        } else {
          *(float *)&v = *(float *)&v / wsum_c;
        }
        out[id] = v;
      } else {
        if (!inner || __ldg(mark + id) != 0.f) {
          out[id] = __ldg((const T *)src + id);
          continue;
        }
        T v = val[q][r];
        if (NC == 4) {
          float4 &f = *(float4 *)&v;
          f.x = mul_inv81(f.x);
          f.y = mul_inv81(f.y);
          f.z = mul_inv81(f.z);
          f.w = mul_inv81(f.w);
        } else {
          *(float *)&v = mul_inv81(*(float *)&v);
        }
        out[id] = v;
      }
    }
  }
}

template <int S, int NC, int MODE>
static void launch_slab(const float *src, float *dst, Dims4 d, const float *wsum, const float *mark,
                        const float *w, int zero_border, cudaStream_t st) {
  typedef SlabGeom<S> G;
  typedef typename VT<NC>::T T;
  const int tiles_x = (d.x + TX - 1) / TX, tiles_y = (d.y + TY - 1) / TY;
  dim3 grid(tiles_x * tiles_y, d.z, d.t);
  const size_t smem = 2 * G::SLOTS * sizeof(T);
  WTab2 wt;
  for (int i = 0; i < 40; ++i) wt.w[i] = (w && i <= 4 * S * S) ? w[i] : 0.f;
  static const bool attr_set = [] {
    cudaFuncSetAttribute(k_slab_stencil<S, NC, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(2 * SlabGeom<S>::SLOTS * sizeof(typename VT<NC>::T)));
    return true;
  }();
  (void)attr_set;
  k_slab_stencil<S, NC, MODE><<<grid, NTHREADS, smem, st>>>(src, dst, d, tiles_x, wsum, mark, wt,
                                                            zero_border);
}

bool gauss_slab_supported(int s, Dims4 d) {
  return (s == 1 || s == 2) && d.z <= 65535 && d.t <= 65535;
}

void launch_gauss_slab(const float *src, float *dst, Dims4 d, int nc, int s, const float *wtab,
                       const float *wsum_dev, int zero_border, cudaStream_t st) {
  if (s == 1) {
    if (nc == 4) launch_slab<1, 4, 0>(src, dst, d, wsum_dev, nullptr, wtab, zero_border, st);
    else launch_slab<1, 1, 0>(src, dst, d, wsum_dev, nullptr, wtab, zero_border, st);
  } else {
    if (nc == 4) launch_slab<2, 4, 0>(src, dst, d, wsum_dev, nullptr, wtab, zero_border, st);
    else launch_slab<2, 1, 0>(src, dst, d, wsum_dev, nullptr, wtab, zero_border, st);
  }
}

void launch_expol_slab(const float4 *in, float4 *out, const float *mark, Dims4 d,
                       cudaStream_t st) {
  launch_slab<1, 4, 1>((const float *)in, (float *)out, d, nullptr, mark, nullptr, 0, st);
}

}  // namespace flof
