// flof_tma.cu -- TMA-staged slab kernels for the dense 4D stencils on Vec4
// grids: the Gaussian velocity blur (knGaussianBlur, optflow4d.cpp:132-158,
// radius 1 and 2) and the extrapolation sweep (knCvExpolBlur4d, :613-626),
// direct and separable.
//
// Same arithmetic as flof_stencil.cu: every output of the blur and the direct
// sweep sums its (2S+1)^4 neighbourhood in the reference's order (t, z, y, x)
// with float adds in sequence.  A block owns a 32-column (x,y) tile and walks
// the input slabs its output planes need once, in (t, z) order: the blur one
// (z, t) plane per block, the sweeps two z planes walking t with the running
// sums of three t planes in registers.  Each (x,y) slab with its S-cell halo
// is brought into shared memory by one cp.async.bulk.tensor copy issued by a
// single thread, completion signalled on an mbarrier, a few slabs in flight.
// The tensor map views the float4 grid as a 4D float tensor (4X, Y, Z, T), so a
// slab row is one contiguous 16W-byte run, the innermost coordinate 4x is a
// multiple of 16 bytes for every x, and cells outside the grid arrive as
// zeros, which leave a running float sum unchanged (a 16-byte innermost box
// dimension, one float4 per row, made the copies several times slower).
// Lane l of a warp computes column x0+l for RY consecutive rows of
// each plane, so each 8-lane shared-memory phase reads 128 contiguous bytes
// of the dense TMA layout.
//
// Every wait on an mbarrier is bounded; a block that gives up records
// FLOF_DEV_ERR_TMA_TIMEOUT in the context's device error word, waits (again
// bounded) for its copies in flight and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <type_traits>

#include "flof_kernels.h"
#include "flof_tma.cuh"

namespace flof {

namespace {

constexpr int TX = 32;                // tile width: one column per lane

// Tile geometry: NW warps, RY rows per thread, DT consecutive t planes and DZ
// consecutive z planes per block, NSTAGE slab buffers in flight.
template <int S, int NW_, int RY_, int DT_, int DZ_, int NSTAGE_, int MINB_ = 1>
struct TG {
  static constexpr int NW = NW_, RY = RY_, DT = DT_, DZ = DZ_, NSTAGE = NSTAGE_, MINB = MINB_;
  static constexpr int NTHR = 32 * NW;
  static constexpr int TY = NW * RY;
  static constexpr int W = TX + 2 * S, H = TY + 2 * S, N = W * H;
  static constexpr int BYTES = N * 16;                   // one slab
  static constexpr int STRIDE = (BYTES + 127) / 128 * 128;  // slab start spacing
  static constexpr int SMEM = NSTAGE * STRIDE;
  static_assert(DZ * DT * RY <= 16, "the keep mask holds 16 cells per thread");
};
// The blur (S = 1, 2) is bound by its multiply-adds: one (z, t) plane per
// block, 32 rows.  ExpolGeom fixes the sweeps' keep-mask layout: a 16-bit
// word per thread for RY = 2 rows, DZ = 2 z planes and DT = 4 t planes.
template <int S> using BlurGeom = TG<S, 4, 8, 1, 1, 2>;
using ExpolGeom = TG<1, 8, 2, 4, 2, 4, 3>;

// The extrapolation sweeps and the blur add with sm_100-family packed
// `add.rn.f32x2`: a float4 is two float pairs (x,y), (z,w), each lane rounded
// like the scalar add, so the sums are bit for bit the scalar ones in the
// same order at half the instruction count (4M random pairs on GB300: no
// difference).  The blur's products stay scalar multiplies: the packed
// `mul.rn.f32x2` gave results different from the scalar multiply in about
// 15% of 4M random cases on GB300, and a blur built on it failed the bitwise
// comparisons with the reference's separately rounded products.
struct __align__(16) P4 {
  unsigned long long lo, hi;
};
__device__ __forceinline__ void add2(unsigned long long &acc, unsigned long long x) {
  asm("add.rn.f32x2 %0, %0, %1;" : "+l"(acc) : "l"(x));
}
__device__ __forceinline__ void acc4(P4 &v, const P4 &a) {
  add2(v.lo, a.lo);
  add2(v.hi, a.hi);
}
__device__ __forceinline__ float4 unpack4(const P4 &v) {
  float4 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v.lo));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.z), "=f"(r.w) : "l"(v.hi));
  return r;
}
// w times a float4 by scalar multiplies, the products packed as two float
// pairs for the packed adds
__device__ __forceinline__ P4 mulp4(float w, const float4 &a) {
  const float4 m = make_float4(__fmul_rn(w, a.x), __fmul_rn(w, a.y), __fmul_rn(w, a.z),
                               __fmul_rn(w, a.w));
  P4 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.lo) : "f"(m.x), "f"(m.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.hi) : "f"(m.z), "f"(m.w));
  return r;
}

template <int S>
__device__ __forceinline__ int clip_code_t(int c, int ext) {
  int lo = S - c;
  lo = lo < 0 ? 0 : lo;
  int hi = c + S - (ext - 1);
  hi = hi < 0 ? 0 : hi;
  return lo * (S + 1) + hi;
}

}  // namespace

struct WTabT {
  float w[40];
};

// The Gaussian blur pass.  A block computes the outputs of DZ x DT
// consecutive (z, t) planes.  It walks the input slabs (tt, zz) of the union
// of their neighbourhoods in lexicographic order; for a fixed output plane
// (z_o, t_o) that order is the reference's (vt, zk) order with
// vt = tt - t_o, zk = zz - z_o, so every output still adds its taps in the
// reference's sequence while each slab is fetched once for all planes.
template <int S, class G>
__global__ void __launch_bounds__(G::NTHR, G::MINB)
k_blur_tma(const __grid_constant__ CUtensorMap map, float4 *__restrict__ dst, Dims4 d,
           int tiles_x, const float *__restrict__ wsum, WTabT wt, int zero_border, int *err) {
  constexpr int RY = G::RY, DT = G::DT, DZ = G::DZ, NS = G::NSTAGE;
  extern __shared__ __align__(128) unsigned char raw[];
  __shared__ __align__(8) uint64_t bar[NS];
  __shared__ float wsh[40];

  const int tile = blockIdx.x;
  const int x0 = (tile % tiles_x) * TX, y0 = (tile / tiles_x) * G::TY;
  const int z0 = blockIdx.y * DZ, t0 = blockIdx.z * DT;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int x = x0 + tx;

  if (threadIdx.x == 0) {
#pragma unroll
    for (int b = 0; b < NS; ++b) mbar_init(&bar[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (threadIdx.x < 40) wsh[threadIdx.x] = wt.w[threadIdx.x];
  __syncthreads();

  constexpr int KZ = DZ + 2 * S;
  constexpr int NP = (DT + 2 * S) * KZ;  // slabs (tt, zz), tt-major
  // slab p lives in buffer p % NS; its barrier completes phase (p / NS) & 1
  auto issue = [&](int p) {
    uint64_t *b = &bar[p % NS];
    mbar_expect_tx(b, G::BYTES);
    tma_load_slab(raw + (p % NS) * G::STRIDE, &map, x0 - S, y0 - S, z0 - S + p % KZ,
                  t0 - S + p / KZ, b);
  };
  if (threadIdx.x == 0) {
#pragma unroll
    for (int p = 0; p < NS - 1; ++p)
      if (p < NP) issue(p);
  }

  typedef float4 V4;
  P4 val[DZ][DT][RY];  // running sums as two float pairs for the packed adds
#pragma unroll
  for (int oz = 0; oz < DZ; ++oz)
#pragma unroll
    for (int o = 0; o < DT; ++o)
#pragma unroll
      for (int q = 0; q < RY; ++q) memset(&val[oz][o][q], 0, sizeof(P4));

  for (int p = 0; p < NP; ++p) {
    const int vt0 = p / KZ - S, zk0 = p % KZ - S;  // offsets seen by plane (0, 0)
    // buffer (p - 1) % NS was released by the barrier that ended step p - 1
    if (threadIdx.x == 0 && p + NS - 1 < NP) issue(p + NS - 1);
    const bool ok = mbar_wait_bounded(&bar[p % NS], (p / NS) & 1);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(err, FLOF_DEV_ERR_TMA_TIMEOUT);
        // let the copies in flight land before the block's shared memory goes
        for (int r = p; r < NP && r < p + NS; ++r) mbar_wait_bounded(&bar[r % NS], (r / NS) & 1);
      }
      __syncthreads();
      return;
    }
    const V4 *cur = (const V4 *)(raw + (p % NS) * G::STRIDE);
    // slab rows RY*ty .. RY*ty+RY-1+2S feed output rows RY*ty+q via yj = k-q-S
#pragma unroll
    for (int k = 0; k < RY + 2 * S; ++k) {
      const V4 *row = cur + (RY * ty + k) * G::W + tx;
      V4 a[2 * S + 1];
#pragma unroll
      for (int m = 0; m <= 2 * S; ++m) a[m] = row[m];
#pragma unroll
      for (int oz = 0; oz < DZ; ++oz) {
        const int zk = zk0 - oz;
        if (zk < -S || zk > S) continue;
#pragma unroll
        for (int o = 0; o < DT; ++o) {
          const int vt = vt0 - o;
          if (vt < -S || vt > S) continue;
          // Output rows at y offsets +-ay use the same weights, so the
          // rounded products w * a are formed once per |yj| and added to
          // each of those rows in the usual xi order.
#pragma unroll
          for (int ay = 0; ay <= S; ++ay) {
            bool used = false;
#pragma unroll
            for (int q = 0; q < RY; ++q) used |= (k - q - S == ay) || (k - q - S == -ay);
            if (!used) continue;
            const int base = vt * vt + zk * zk + ay * ay;
            P4 prod[2 * S + 1];
#pragma unroll
            for (int xi = -S; xi <= S; ++xi) prod[xi + S] = mulp4(wsh[base + xi * xi], a[xi + S]);
#pragma unroll
            for (int q = 0; q < RY; ++q) {
              const int yj = k - q - S;
              if (yj != ay && yj != -ay) continue;
#pragma unroll
              for (int xi = -S; xi <= S; ++xi) acc4(val[oz][o][q], prod[xi + S]);
            }
          }
        }
      }
    }
    __syncthreads();
  }

  if (x >= d.x) return;
  constexpr int P1 = (S + 1) * (S + 1);
#pragma unroll
  for (int oz = 0; oz < DZ; ++oz) {
    const int z = z0 + oz;
    if (z >= d.z) break;
#pragma unroll
    for (int o = 0; o < DT; ++o) {
      const int t = t0 + o;
      if (t >= d.t) break;
      const bool zt_inner = z >= 1 && z < d.z - 1 && t >= 1 && t < d.t - 1;
      const int code_zt = (clip_code_t<S>(t, d.t) * P1 + clip_code_t<S>(z, d.z)) * P1;
#pragma unroll
      for (int q = 0; q < RY; ++q) {
        const int y = y0 + RY * ty + q;
        if (y >= d.y) continue;
        const idx_t id = d.index(x, y, z, t);
        const float4 v = unpack4(val[oz][o][q]);
        if (!(zt_inner && x >= 1 && x < d.x - 1 && y >= 1 && y < d.y - 1)) {
          if (zero_border) dst[id] = make_float4(0.f, 0.f, 0.f, 0.f);
          continue;
        }
        const float ws =
            __ldg(wsum + (code_zt + clip_code_t<S>(y, d.y)) * P1 + clip_code_t<S>(x, d.x));
        dst[id] = make_float4(v.x / ws, v.y / ws, v.z / ws, v.w / ws);
      }
    }
  }
}

// The extrapolation sweep walking t.  A block owns a 32 x 16 (x,y) tile
// and ETW_DZ consecutive z planes and walks ETW_TC + 2 t planes; for each
// t plane it takes the ETW_DZ + 2 (x,y) slabs (with their one-cell halo)
// that its outputs need, in z order, one TMA copy each, ETW_NS in flight.
// Each thread keeps the running sums of its cells for three output planes
// in registers: slab plane tt adds the taps vt = +1 of output tt - 1 (which
// is then complete and written), vt = 0 of output tt and vt = -1 of output
// tt + 1 (which starts there).  Every output thus adds its 81 taps in the
// reference's order (t, z, y, x) with float adds in sequence, and the loop
// body is the same for every plane: no run-time choice of outputs.
constexpr int ETW_NW = 8, ETW_RY = 2, ETW_DZ = 2, ETW_TC = 8, ETW_NS = 2;
constexpr int ETW_TY = ETW_NW * ETW_RY;
constexpr int ETW_W = TX + 2, ETW_H = ETW_TY + 2;
constexpr int ETW_BYTES = ETW_W * ETW_H * 16;
constexpr int ETW_SPC = 2;  // z slabs per copy of the direct sweep
constexpr int ETW_CBYTES = ETW_SPC * ETW_BYTES;
constexpr int ETW_CSTRIDE = (ETW_CBYTES + 127) / 128 * 128;
constexpr int ETW_SMEM = ETW_NS * ETW_CSTRIDE;
constexpr int ETW_KZ = ETW_DZ + 2;  // slabs per t plane
static_assert(ETW_RY == ExpolGeom::RY && ETW_DZ == ExpolGeom::DZ,
              "the keep mask groups rows and z planes as the sweep does");

// Four blocks per SM (64 registers, a few bytes spilled) beat three
// (80 registers): 0.221 against 0.229 ms per 64^4 sweep; copies of two z
// slabs, two copies in flight (one barrier per two slabs), 0.217 ms.
__global__ void __launch_bounds__(32 * ETW_NW, 4)
k_expol_tw(const __grid_constant__ CUtensorMap map, float4 *__restrict__ dst, Dims4 d,
           int tiles_x, const uint16_t *__restrict__ fixed, int *err) {
  extern __shared__ __align__(128) unsigned char raw[];
  __shared__ __align__(8) uint64_t bar[ETW_NS];
  constexpr int RY = ETW_RY, DZ = ETW_DZ, KZ = ETW_KZ, NS = ETW_NS;
  constexpr int DT = ExpolGeom::DT;  // t planes per keep-mask word
  const int tile = blockIdx.x;
  const int x0 = (tile % tiles_x) * TX, y0 = (tile / tiles_x) * ETW_TY;
  const int z0 = blockIdx.y * DZ, t0 = blockIdx.z * ETW_TC;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int x = x0 + tx;
  const int ygroups = (d.y + RY - 1) / RY, zgroups = (d.z + DZ - 1) / DZ;
  const int yg = y0 / RY + ty;
  const bool xy_ok = x < d.x && yg < ygroups;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int b = 0; b < NS; ++b) mbar_init(&bar[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  constexpr int CPP = KZ / ETW_SPC;   // copies per t plane
  // copy p: plane t0 - 1 + p / CPP, slabs from z0 - 1 + SPC (p % CPP)
  const int NP = (ETW_TC + 2) * CPP;
  auto issue = [&](int p) {
    uint64_t *b = &bar[p % NS];
    mbar_expect_tx(b, ETW_CBYTES);
    tma_load_slab(raw + (p % NS) * ETW_CSTRIDE, &map, x0 - 1, y0 - 1, z0 - 1 + ETW_SPC * (p % CPP),
                  t0 - 1 + p / CPP, b);
  };
  if (threadIdx.x == 0) {
#pragma unroll
    for (int p = 0; p < NS - 1; ++p) issue(p);
  }
  // running sums of outputs tt - 1 (A), tt (B) and tt + 1 (C)
  P4 A[DZ][RY], B[DZ][RY], C[DZ][RY];
  // One t plane j (tt = t0 - 1 + j).  SA, SB, SC say which of the three
  // outputs lie in the block's range t0 .. t0 + ETW_TC - 1: the first two and
  // the last two planes skip the sums of the others (a fifth of the adds).
  auto plane = [&](int j, auto SA, auto SB, auto SC) -> bool {
    constexpr bool DA = decltype(SA)::value, DB = decltype(SB)::value, DC = decltype(SC)::value;
    if (DC) {
#pragma unroll
      for (int oz = 0; oz < DZ; ++oz)
#pragma unroll
        for (int q = 0; q < RY; ++q) memset(&C[oz][q], 0, sizeof(P4));
    }
#pragma unroll
    for (int zc = 0; zc < CPP; ++zc) {
      const int p = j * CPP + zc;
      // buffer (p - 1) % NS was released by the barrier that ended copy p - 1
      if (threadIdx.x == 0 && p + NS - 1 < NP) issue(p + NS - 1);
      // A thread whose wait gave up still reads the buffer (stale values, in
      // bounds); the barrier that ends the copy's step then ends the block.
      const bool ok = mbar_wait_bounded(&bar[p % NS], (p / NS) & 1);
#pragma unroll
      for (int sl = 0; sl < ETW_SPC; ++sl) {
        const int zk = zc * ETW_SPC + sl;
        const P4 *cur = (const P4 *)(raw + (p % NS) * ETW_CSTRIDE + sl * ETW_BYTES);
#pragma unroll
        for (int k = 0; k < RY + 2; ++k) {
          const P4 *row = cur + (RY * ty + k) * ETW_W + tx;
          const P4 a0 = row[0], a1 = row[1], a2 = row[2];
#pragma unroll
          for (int oz = 0; oz < DZ; ++oz) {
            const int zrel = zk - 1 - oz;  // this slab's z offset from output plane z0 + oz
            if (zrel < -1 || zrel > 1) continue;
#pragma unroll
            for (int q = 0; q < RY; ++q) {
              const int yj = k - q - 1;
              if (yj < -1 || yj > 1) continue;
              // vt = -1 of output tt + 1, vt = 0 of output tt, vt = +1 of output tt - 1
              if (DC) {
                acc4(C[oz][q], a0);
                acc4(C[oz][q], a1);
                acc4(C[oz][q], a2);
              }
              if (DB) {
                acc4(B[oz][q], a0);
                acc4(B[oz][q], a1);
                acc4(B[oz][q], a2);
              }
              if (DA) {
                acc4(A[oz][q], a0);
                acc4(A[oz][q], a1);
                acc4(A[oz][q], a2);
              }
            }
          }
        }
      }
      if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
          atomicExch(err, FLOF_DEV_ERR_TMA_TIMEOUT);
          for (int r = p; r < NP && r < p + NS; ++r) mbar_wait_bounded(&bar[r % NS], (r / NS) & 1);
        }
        __syncthreads();
        return false;
      }
    }
    // output tt - 1 = t0 - 2 + j is complete
    const int t = t0 - 2 + j;
    if (DA && xy_ok && t < d.t) {
      const unsigned keep =
          __ldg(fixed + (((size_t)(t / DT) * zgroups + blockIdx.y) * ygroups + yg) * d.x + x);
#pragma unroll
      for (int oz = 0; oz < DZ; ++oz) {
        const int z = z0 + oz;
        if (z >= d.z) break;
#pragma unroll
        for (int q = 0; q < RY; ++q) {
          const int y = y0 + RY * ty + q;
          if (y >= d.y) continue;
          if (keep >> ((oz * DT + t % DT) * RY + q) & 1u) continue;
          const float4 v = unpack4(A[oz][q]);
          dst[d.index(x, y, z, t)] =
              make_float4(mul_inv81(v.x), mul_inv81(v.y), mul_inv81(v.z), mul_inv81(v.w));
        }
      }
    }
#pragma unroll
    for (int oz = 0; oz < DZ; ++oz)
#pragma unroll
      for (int q = 0; q < RY; ++q) {
        A[oz][q] = B[oz][q];
        B[oz][q] = C[oz][q];
      }
    return true;
  };
  using T_ = std::true_type;
  using F_ = std::false_type;
  static_assert(ETW_TC >= 2, "the peeled planes are distinct");
  if (!plane(0, F_(), F_(), T_())) return;
  if (!plane(1, F_(), T_(), T_())) return;
  for (int j = 2; j < ETW_TC; ++j)
    if (!plane(j, T_(), T_(), T_())) return;
  if (!plane(ETW_TC, T_(), T_(), F_())) return;
  plane(ETW_TC + 1, T_(), F_(), F_());
}

// The separable extrapolation sweep (blurType 2) walking t.  It takes
// k_expol_tw's slabs in k_expol_tw's order but forms each output's 3^4 sum as
// box sums: per slab the x sums of the rows a thread needs and the y sums of
// three of those, added over the three z slabs of each output plane as the
// slabs arrive, and over three consecutive t planes from a register ring.
// Each sum is taken in the two-pass separable sweep's order (x, then y, z, t,
// each (a-1 + a0) + a+1), so the two give the same bits; a cell costs about
// sixteen float4 adds instead of 81.  The kernel is bound by latency (few
// warps, two dependent shared-memory and add steps per slab) more than by
// shared-memory or DRAM bandwidth, so warps count most: at 64^4 on GB300,
// RY = 2 rows per thread (8 warps, three blocks per SM) took 0.168 ms a
// sweep against 0.178 ms for RY = 4 (4 warps), and TC = 4 or deeper slab
// pipelines did not help.  A copy brings two z slabs (one block barrier per
// two slabs): 0.165 ms.
constexpr int ESW_RY = 2, ESW_NW = ETW_TY / ESW_RY, ESW_TC = 8, ESW_NS = 3, ESW_MINB = 3;
constexpr int ESW_SPC = 2;  // z slabs per copy: one barrier step per two slabs
constexpr int ESW_CBYTES = ESW_SPC * ETW_BYTES;  // one copy, its slabs back to back
constexpr int ESW_CSTRIDE = (ESW_CBYTES + 127) / 128 * 128;
constexpr int ESW_SMEM = ESW_NS * ESW_CSTRIDE;
static_assert(ETW_KZ % ESW_SPC == 0, "whole copies per plane");

__global__ void __launch_bounds__(32 * ESW_NW, ESW_MINB)
k_expol_sep_tw(const __grid_constant__ CUtensorMap map, float4 *__restrict__ dst, Dims4 d,
               int tiles_x, const uint16_t *__restrict__ fixed, int *err) {
  extern __shared__ __align__(128) unsigned char raw[];
  __shared__ __align__(8) uint64_t bar[ESW_NS];
  constexpr int RY = ESW_RY, DZ = ETW_DZ, KZ = ETW_KZ, NS = ESW_NS;
  constexpr int MRY = ExpolGeom::RY, DT = ExpolGeom::DT;  // keep-mask word geometry
  static_assert(RY % MRY == 0, "a thread's rows cover whole keep-mask row groups");
  static_assert((DT & (DT - 1)) == 0, "t % DT as a mask");
  const int tile = blockIdx.x;
  const int x0 = (tile % tiles_x) * TX, y0 = (tile / tiles_x) * ETW_TY;
  const int z0 = blockIdx.y * DZ, t0 = blockIdx.z * ESW_TC;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int x = x0 + tx;
  const int ygroups = (d.y + MRY - 1) / MRY, zgroups = (d.z + DZ - 1) / DZ;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int b = 0; b < NS; ++b) mbar_init(&bar[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  constexpr int CPP = KZ / ESW_SPC;   // copies per t plane
  // copy p: plane t0 - 1 + p / CPP, slabs from z0 - 1 + SPC (p % CPP)
  const int NP = (ESW_TC + 2) * CPP;
  auto issue = [&](int p) {
    uint64_t *b = &bar[p % NS];
    mbar_expect_tx(b, ESW_CBYTES);
    tma_load_slab(raw + (p % NS) * ESW_CSTRIDE, &map, x0 - 1, y0 - 1, z0 - 1 + ESW_SPC * (p % CPP),
                  t0 - 1 + p / CPP, b);
  };
  if (threadIdx.x == 0) {
#pragma unroll
    for (int p = 0; p < NS - 1; ++p) issue(p);
  }
  // z sums of planes tt - 2 (Z0), tt - 1 (Z1) and tt (Zc, filled slab by slab)
  P4 Z0[DZ][RY], Z1[DZ][RY], Zc[DZ][RY];
  for (int j = 0; j < ESW_TC + 2; ++j) {
    // keep-mask words of output plane t = t0 - 2 + j, loaded before its slabs
    // are summed (all ones: nothing to write)
    const int t = t0 - 2 + j;
    unsigned keep[RY / MRY];
#pragma unroll
    for (int g = 0; g < RY / MRY; ++g) {
      const int yb = y0 + RY * ty + g * MRY;
      keep[g] = 0xffffu;
      if (j >= 2 && x < d.x && t < d.t && yb < d.y)
        keep[g] = __ldg(fixed + ((((size_t)(t / DT) * zgroups + blockIdx.y) * ygroups + yb / MRY) *
                                     d.x + x));
    }
#pragma unroll
    for (int zc = 0; zc < CPP; ++zc) {
      const int p = j * CPP + zc;
      if (threadIdx.x == 0 && p + NS - 1 < NP) issue(p + NS - 1);
      // A thread whose wait gave up still reads the buffer (stale values,
      // in bounds); the barrier that ends the copy's step then ends the block.
      const bool ok = mbar_wait_bounded(&bar[p % NS], (p / NS) & 1);
#pragma unroll
      for (int sl = 0; sl < ESW_SPC; ++sl) {
        const int zk = zc * ESW_SPC + sl;
        const P4 *cur =
            (const P4 *)(raw + (p % NS) * ESW_CSTRIDE + sl * ETW_BYTES) + RY * ty * ETW_W + tx;
        auto xsum = [&](int k) {
          const P4 *row = cur + k * ETW_W;
          P4 v = row[0];
          acc4(v, row[1]);
          acc4(v, row[2]);
          return v;
        };
        P4 r0 = xsum(0), r1 = xsum(1);
#pragma unroll
        for (int q = 0; q < RY; ++q) {
          const P4 r2 = xsum(q + 2);
          P4 xy = r0;
          acc4(xy, r1);
          acc4(xy, r2);
#pragma unroll
          for (int oz = 0; oz < DZ; ++oz) {
            const int zrel = zk - 1 - oz;  // this slab's z offset from output plane z0 + oz
            if (zrel == -1) Zc[oz][q] = xy;
            else if (zrel <= 1) acc4(Zc[oz][q], xy);
          }
          r0 = r1;
          r1 = r2;
        }
      }
      if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
          atomicExch(err, FLOF_DEV_ERR_TMA_TIMEOUT);
          for (int r = p; r < NP && r < p + NS; ++r) mbar_wait_bounded(&bar[r % NS], (r / NS) & 1);
        }
        __syncthreads();
        return;
      }
    }
    // output plane t: (Z(t - 1) + Z(t)) + Z(t + 1).  A clear bit means an
    // unmarked interior cell, so x, y, z and t are then inside the grid.
#pragma unroll
    for (int g = 0; g < RY / MRY; ++g) {
      const int yb = y0 + RY * ty + g * MRY;
#pragma unroll
      for (int oz = 0; oz < DZ; ++oz) {
#pragma unroll
        for (int m = 0; m < MRY; ++m) {
          if (keep[g] >> ((oz * DT + (t & (DT - 1))) * MRY + m) & 1u) continue;
          const int q = g * MRY + m;
          P4 v = Z0[oz][q];
          acc4(v, Z1[oz][q]);
          acc4(v, Zc[oz][q]);
          const float4 s = unpack4(v);
          dst[d.index(x, yb + m, z0 + oz, t)] =
              make_float4(mul_inv81(s.x), mul_inv81(s.y), mul_inv81(s.z), mul_inv81(s.w));
        }
      }
    }
#pragma unroll
    for (int oz = 0; oz < DZ; ++oz)
#pragma unroll
      for (int q = 0; q < RY; ++q) {
        Z0[oz][q] = Z1[oz][q];
        Z1[oz][q] = Zc[oz][q];
      }
  }
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // looked up once (thread-safe static init); null when the driver lacks it
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000)p;
    cudaGetLastError();
    return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
  }();
  return fn;
}

}  // namespace

// Tensor map of a float4 grid as a 4D float tensor (4X, Y, Z, T) with a
// (4W, H, 1, 1) box: each slab row is one contiguous run of 16W bytes.
bool encode_slab_map(CUtensorMap *m, const float4 *base, Dims4 d, int W, int H, int D) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn || ((uintptr_t)base & 15) || 4 * W > 256) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)4 * d.x, (cuuint64_t)d.y, (cuuint64_t)d.z,
                              (cuuint64_t)d.t};
  const cuuint64_t strides[3] = {(cuuint64_t)16 * d.x, (cuuint64_t)16 * d.x * d.y,
                                 (cuuint64_t)16 * d.x * d.y * d.z};
  const cuuint32_t box[4] = {(cuuint32_t)(4 * W), (cuuint32_t)H, (cuuint32_t)D, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (void *)base, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

namespace {

template <int S, class G>
bool launch_blur(const float4 *src, float4 *dst, Dims4 d, const float *wsum, const float *w,
                 int zero_border, int *err, cudaStream_t st) {
  const int tgroups = (d.t + G::DT - 1) / G::DT, zgroups = (d.z + G::DZ - 1) / G::DZ;
  if (zgroups > 65535 || tgroups > 65535) return false;
  CUtensorMap map;
  if (!encode_slab_map(&map, src, d, G::W, G::H)) return false;
  const int tiles_x = (d.x + TX - 1) / TX, tiles_y = (d.y + G::TY - 1) / G::TY;
  dim3 grid(tiles_x * tiles_y, zgroups, tgroups);
  static const bool attr = [] {
    if (cudaFuncSetAttribute(k_blur_tma<S, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)G::SMEM) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return true;
  }();
  if (!attr) return false;
  WTabT wt;
  for (int i = 0; i < 40; ++i) wt.w[i] = (w && i <= 4 * S * S) ? w[i] : 0.f;
  k_blur_tma<S, G><<<grid, G::NTHR, G::SMEM, st>>>(map, dst, d, tiles_x, wsum, wt, zero_border,
                                                   err);
  return true;
}

}  // namespace

bool launch_gauss_tma(const float4 *src, float4 *dst, Dims4 d, int s, const float *wtab,
                      const float *wsum_dev, int zero_border, int *err, cudaStream_t st) {
  if (s == 1) return launch_blur<1, BlurGeom<1>>(src, dst, d, wsum_dev, wtab, zero_border, err, st);
  if (s == 2) return launch_blur<2, BlurGeom<2>>(src, dst, d, wsum_dev, wtab, zero_border, err, st);
  return false;
}

namespace {

// One 16-bit word per sweep thread: (x, y group of RY rows, z group of DZ, t
// group of DT), x fastest.  A bit is set for each of the thread's cells that
// the sweep leaves alone: marked, outside the interior (knCvExpolBlur4d runs
// over bnd = 1), or past the grid's end.
__global__ void k_expol_mask(const float *__restrict__ mark, uint16_t *__restrict__ mask, Dims4 d,
                             int ygroups, int zgroups, long long nwords) {
  constexpr int RY = ExpolGeom::RY, DT = ExpolGeom::DT, DZ = ExpolGeom::DZ;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nwords;
       w += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(w % d.x);
    long long r = w / d.x;
    const int yg = (int)(r % ygroups);
    r /= ygroups;
    const int zg = (int)(r % zgroups);
    const int tg = (int)(r / zgroups);
    unsigned bits = 0;
    for (int oz = 0; oz < DZ; ++oz)
      for (int o = 0; o < DT; ++o)
        for (int q = 0; q < RY; ++q) {
          const int y = yg * RY + q, z = zg * DZ + oz, t = tg * DT + o;
          if (y >= d.y || z >= d.z || t >= d.t) {
            bits |= 1u << ((oz * DT + o) * RY + q);
            continue;
          }
          const bool inner = x >= 1 && x < d.x - 1 && y >= 1 && y < d.y - 1 && z >= 1 &&
                             z < d.z - 1 && t >= 1 && t < d.t - 1;
          if (!inner || __ldg(mark + d.index(x, y, z, t)) != 0.f)
            bits |= 1u << ((oz * DT + o) * RY + q);
        }
    mask[w] = (uint16_t)bits;
  }
}

}  // namespace

size_t expol_mask_words(Dims4 d) {
  return (size_t)d.x * ((d.y + ExpolGeom::RY - 1) / ExpolGeom::RY) *
         ((d.z + ExpolGeom::DZ - 1) / ExpolGeom::DZ) * ((d.t + ExpolGeom::DT - 1) / ExpolGeom::DT);
}

void launch_expol_mask(const float *mark, uint16_t *mask, Dims4 d, cudaStream_t st) {
  const long long n = (long long)expol_mask_words(d);
  const int ygroups = (d.y + ExpolGeom::RY - 1) / ExpolGeom::RY;
  const int zgroups = (d.z + ExpolGeom::DZ - 1) / ExpolGeom::DZ;
  k_expol_mask<<<grid_for(n, 256), 256, 0, st>>>(mark, mask, d, ygroups, zgroups, n);
}

bool launch_expol_tw(const float4 *in, float4 *out, const uint16_t *mask, Dims4 d, int *err,
                     cudaStream_t st) {
  const int zgroups = (d.z + ETW_DZ - 1) / ETW_DZ, tgroups = (d.t + ETW_TC - 1) / ETW_TC;
  if (zgroups > 65535 || tgroups > 65535) return false;
  CUtensorMap map;
  if (!encode_slab_map(&map, in, d, ETW_W, ETW_H, ETW_SPC)) return false;
  static const bool attr = [] {
    if (cudaFuncSetAttribute(k_expol_tw, cudaFuncAttributeMaxDynamicSharedMemorySize, ETW_SMEM) !=
        cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return true;
  }();
  if (!attr) return false;
  const int tiles_x = (d.x + TX - 1) / TX, tiles_y = (d.y + ETW_TY - 1) / ETW_TY;
  dim3 grid(tiles_x * tiles_y, zgroups, tgroups);
  k_expol_tw<<<grid, 32 * ETW_NW, ETW_SMEM, st>>>(map, out, d, tiles_x, mask, err);
  return true;
}

bool launch_expol_sep_tw(const float4 *in, float4 *out, const uint16_t *mask, Dims4 d, int *err,
                         cudaStream_t st) {
  const int zgroups = (d.z + ETW_DZ - 1) / ETW_DZ, tgroups = (d.t + ESW_TC - 1) / ESW_TC;
  if (zgroups > 65535 || tgroups > 65535) return false;
  CUtensorMap map;
  if (!encode_slab_map(&map, in, d, ETW_W, ETW_H, ESW_SPC)) return false;
  static const bool attr = [] {
    if (cudaFuncSetAttribute(k_expol_sep_tw, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             ESW_SMEM) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return true;
  }();
  if (!attr) return false;
  const int tiles_x = (d.x + TX - 1) / TX, tiles_y = (d.y + ETW_TY - 1) / ETW_TY;
  dim3 grid(tiles_x * tiles_y, zgroups, tgroups);
  k_expol_sep_tw<<<grid, 32 * ESW_NW, ESW_SMEM, st>>>(map, out, d, tiles_x, mask, err);
  return true;
}

}  // namespace flof
