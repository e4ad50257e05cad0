// flof_common.cuh -- device-side building blocks shared by the FlOF kernels.
//
// Layout (reference source/grid4d.h:92-97): a 4D grid (X,Y,Z,T) is stored
// x-fastest, idx = i + X*j + X*Y*k + X*Y*Z*t.  Real grids are float, Vec4
// grids are float4 (interleaved x,y,z,t), 16-byte aligned.
//
// Arithmetic: every translation unit is compiled with -fmad=false so that
// multiplies and adds are rounded separately, in the order written, like the
// reference's x86 build; fused multiply-adds appear only where a kernel asks
// for them explicitly (__fmaf_rn) and the reference has no bitwise claim.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace flof {

typedef long long idx_t;

struct Dims4 {
  int x, y, z, t;
  __host__ __device__ idx_t cells() const { return (idx_t)x * y * z * t; }
  __host__ __device__ idx_t sz() const { return (idx_t)x * y; }
  __host__ __device__ idx_t st() const { return (idx_t)x * y * z; }
  __host__ __device__ idx_t index(int i, int j, int k, int l) const {
    return (idx_t)i + (idx_t)x * j + (idx_t)x * y * k + (idx_t)x * y * z * l;
  }
};

// Unsigned division by an invariant divisor with a multiply-high
// (Granlund & Montgomery, PLDI 1994, "round-up" variant).  Valid for every
// 32-bit dividend.
struct FastDiv {
  uint32_t d, m, l;
  FastDiv() : d(1), m(0), l(0) {}
  explicit FastDiv(uint32_t div) : d(div) {
    l = 0;
    while ((1ull << l) < div) ++l;
    uint64_t mm = ((1ull << 32) * ((1ull << l) - div)) / div + 1;
    m = (uint32_t)mm;
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const {
    uint64_t hi = __umulhi(n, m);
    return (uint32_t)((hi + n) >> l);
  }
};

// Cell coordinates of a linear index over a box of extents (ex,ey,ez,*).
struct BoxDecoder {
  FastDiv fx, fy, fz;
  int ox, oy, oz, ot;  // coordinate offsets added after decoding
  uint32_t ex, ey, ez;
  __device__ __forceinline__ void decode(uint32_t n, int &i, int &j, int &k,
                                         int &l) const {
    uint32_t q = fx.div(n);
    i = (int)(n - q * ex) + ox;
    uint32_t q2 = fy.div(q);
    j = (int)(q - q2 * ey) + oy;
    uint32_t q3 = fz.div(q2);
    k = (int)(q2 - q3 * ez) + oz;
    l = (int)q3 + ot;
  }
};

inline BoxDecoder make_decoder(int ex, int ey, int ez, int ox, int oy, int oz,
                               int ot) {
  BoxDecoder b;
  b.fx = FastDiv((uint32_t)ex);
  b.fy = FastDiv((uint32_t)ey);
  b.fz = FastDiv((uint32_t)ez);
  b.ex = (uint32_t)ex;
  b.ey = (uint32_t)ey;
  b.ez = (uint32_t)ez;
  b.ox = ox;
  b.oy = oy;
  b.oz = oz;
  b.ot = ot;
  return b;
}

__device__ __forceinline__ bool in_bounds(const Dims4 &d, int i, int j, int k,
                                          int l, int b) {
  return i >= b && j >= b && i < d.x - b && j < d.y - b && k >= b &&
         k < d.z - b && l >= b && l < d.t - b;
}

// float -> int truncation (cvt.rzi.s32.f32: NaN gives 0, out of range
// saturates); equal to the reference's (int) cast for all in-range values.
__device__ __forceinline__ int trunc_i(float p) { return __float2int_rz(p); }

// Weights and base index of a quadrilinear sample, the reference's
// BUILD_INDEX_4D (source/util/vector4d.h:422-470).  `1. - s1` is evaluated
// in double by the reference; for a float s1 that equals 1.0f - s1.
struct IW4 {
  idx_t idx;
  float s0, s1, t0, t1, f0, f1, g0, g1;
};

// One axis of BUILD_INDEX_4D: base index b and the weights (w0, w1) of b and
// b + 1 for a sample at p on an axis of n cells.
struct AxisW {
  int b;
  float w0, w1;
};

__device__ __forceinline__ AxisW axis_index(float p, int n) {
  AxisW a;
  const float px = p - 0.5f;
  a.b = trunc_i(px);
  a.w1 = px - (float)a.b;
  a.w0 = 1.0f - a.w1;
  if (px < 0.f) { a.b = 0; a.w0 = 1.f; a.w1 = 0.f; }
  if (a.b >= n - 1) { a.b = n - 2; a.w0 = 0.f; a.w1 = 1.f; }
  return a;
}

__device__ __forceinline__ IW4 build_index4(const Dims4 &sz, float p0, float p1,
                                            float p2, float p3) {
  IW4 w;
  const AxisW ax = axis_index(p0, sz.x), ay = axis_index(p1, sz.y);
  const AxisW az = axis_index(p2, sz.z), at = axis_index(p3, sz.t);
  w.s0 = ax.w0;
  w.s1 = ax.w1;
  w.t0 = ay.w0;
  w.t1 = ay.w1;
  w.f0 = az.w0;
  w.f1 = az.w1;
  w.g0 = at.w0;
  w.g1 = at.w1;
  w.idx = sz.index(ax.b, ay.b, az.b, at.b);
  return w;
}

// interpol4d sum order (vector4d.h:497-512): pairs along y, then x, z, t.
template <class LD>
__device__ __forceinline__ float interp4_sum(const IW4 &w, idx_t sX, idx_t sY,
                                             idx_t sZ, idx_t sT, LD ld) {
  const idx_t i = w.idx;
  const float t0 = w.t0, t1 = w.t1, s0 = w.s0, s1 = w.s1, f0 = w.f0,
              f1 = w.f1, g0 = w.g0, g1 = w.g1;
  return (((ld(i) * t0 + ld(i + sY) * t1) * s0 +
           (ld(i + sX) * t0 + ld(i + sX + sY) * t1) * s1) *
              f0 +
          ((ld(i + sZ) * t0 + ld(i + sY + sZ) * t1) * s0 +
           (ld(i + sX + sZ) * t0 + ld(i + sX + sY + sZ) * t1) * s1) *
              f1) *
             g0 +
         (((ld(i + sT) * t0 + ld(i + sT + sY) * t1) * s0 +
           (ld(i + sT + sX) * t0 + ld(i + sT + sX + sY) * t1) * s1) *
              f0 +
          ((ld(i + sT + sZ) * t0 + ld(i + sT + sY + sZ) * t1) * s0 +
           (ld(i + sT + sX + sZ) * t0 + ld(i + sT + sX + sY + sZ) * t1) * s1) *
              f1) *
             g1;
}

__device__ __forceinline__ float interp4_real(const float *__restrict__ data,
                                              const Dims4 &sz, float p0,
                                              float p1, float p2, float p3) {
  IW4 w = build_index4(sz, p0, p1, p2, p3);
  return interp4_sum(w, 1, sz.x, sz.sz(), sz.st(),
                     [&](idx_t q) { return __ldg(data + q); });
}

__device__ __forceinline__ float4 interp4_vec(const float4 *__restrict__ data,
                                              const Dims4 &sz, float p0,
                                              float p1, float p2, float p3) {
  IW4 w = build_index4(sz, p0, p1, p2, p3);
  const idx_t sX = 1, sY = sz.x, sZ = sz.sz(), sT = sz.st();
  // Load the 16 corners once, then evaluate the sum per component.
  float4 c[16];
  const idx_t i = w.idx;
  c[0] = __ldg(data + i);
  c[1] = __ldg(data + i + sY);
  c[2] = __ldg(data + i + sX);
  c[3] = __ldg(data + i + sX + sY);
  c[4] = __ldg(data + i + sZ);
  c[5] = __ldg(data + i + sY + sZ);
  c[6] = __ldg(data + i + sX + sZ);
  c[7] = __ldg(data + i + sX + sY + sZ);
  c[8] = __ldg(data + i + sT);
  c[9] = __ldg(data + i + sT + sY);
  c[10] = __ldg(data + i + sT + sX);
  c[11] = __ldg(data + i + sT + sX + sY);
  c[12] = __ldg(data + i + sT + sZ);
  c[13] = __ldg(data + i + sT + sY + sZ);
  c[14] = __ldg(data + i + sT + sX + sZ);
  c[15] = __ldg(data + i + sT + sX + sY + sZ);
  const float t0 = w.t0, t1 = w.t1, s0 = w.s0, s1 = w.s1, f0 = w.f0,
              f1 = w.f1, g0 = w.g0, g1 = w.g1;
#define FLOF_IP4(C)                                                            \
  ((((c[0].C * t0 + c[1].C * t1) * s0 + (c[2].C * t0 + c[3].C * t1) * s1) *   \
        f0 +                                                                   \
    ((c[4].C * t0 + c[5].C * t1) * s0 + (c[6].C * t0 + c[7].C * t1) * s1) *   \
        f1) *                                                                  \
       g0 +                                                                    \
   (((c[8].C * t0 + c[9].C * t1) * s0 + (c[10].C * t0 + c[11].C * t1) * s1) * \
        f0 +                                                                   \
    ((c[12].C * t0 + c[13].C * t1) * s0 +                                      \
     (c[14].C * t0 + c[15].C * t1) * s1) *                                     \
        f1) *                                                                  \
       g1)
  float4 r;
  r.x = FLOF_IP4(x);
  r.y = FLOF_IP4(y);
  r.z = FLOF_IP4(z);
  r.w = FLOF_IP4(w);
#undef FLOF_IP4
  return r;
}

// Trilinear Vec4 sample of a 3D field (interpol<T>, source/util/interpol.h
// :57-116): z is clamped only when size.z > 1.
__device__ __forceinline__ float4 interp3_vec(const float4 *__restrict__ data,
                                              int sx, int sy, int sz, float q0,
                                              float q1, float q2) {
  const float px = q0 - 0.5f, py = q1 - 0.5f, pz = q2 - 0.5f;
  int xi = trunc_i(px), yi = trunc_i(py), zi = trunc_i(pz);
  float s1 = px - (float)xi, s0 = 1.0f - s1;
  float t1 = py - (float)yi, t0 = 1.0f - t1;
  float f1 = pz - (float)zi, f0 = 1.0f - f1;
  if (px < 0.f) { xi = 0; s0 = 1.f; s1 = 0.f; }
  if (py < 0.f) { yi = 0; t0 = 1.f; t1 = 0.f; }
  if (pz < 0.f) { zi = 0; f0 = 1.f; f1 = 0.f; }
  if (xi >= sx - 1) { xi = sx - 2; s0 = 0.f; s1 = 1.f; }
  if (yi >= sy - 1) { yi = sy - 2; t0 = 0.f; t1 = 1.f; }
  if (sz > 1) {
    if (zi >= sz - 1) { zi = sz - 2; f0 = 0.f; f1 = 1.f; }
  }
  const idx_t X = 1, Y = sx, Z = (idx_t)sx * sy;
  const idx_t i = (idx_t)xi + Y * yi + Z * zi;
  float4 c[8];
  c[0] = __ldg(data + i);
  c[1] = __ldg(data + i + Y);
  c[2] = __ldg(data + i + X);
  c[3] = __ldg(data + i + X + Y);
  c[4] = __ldg(data + i + Z);
  c[5] = __ldg(data + i + Y + Z);
  c[6] = __ldg(data + i + X + Z);
  c[7] = __ldg(data + i + X + Y + Z);
#define FLOF_IP3(C)                                                           \
  (((c[0].C * t0 + c[1].C * t1) * s0 + (c[2].C * t0 + c[3].C * t1) * s1) *   \
       f0 +                                                                   \
   ((c[4].C * t0 + c[5].C * t1) * s0 + (c[6].C * t0 + c[7].C * t1) * s1) *   \
       f1)
  float4 r;
  r.x = FLOF_IP3(x);
  r.y = FLOF_IP3(y);
  r.z = FLOF_IP3(z);
  r.w = FLOF_IP3(w);
#undef FLOF_IP3
  return r;
}

// interpol<Real> (source/util/interpol.h:57-95) on a 3D Real grid of extents
// size[0..2] with z stride sZ: same index build and sum order as
// interp3_vec.
__device__ __forceinline__ float interp3_real(const float *__restrict__ data, const int size[3],
                                              idx_t sZ, float q0, float q1, float q2) {
  const float px = q0 - 0.5f, py = q1 - 0.5f, pz = q2 - 0.5f;
  int xi = trunc_i(px), yi = trunc_i(py), zi = trunc_i(pz);
  float s1 = px - (float)xi, s0 = 1.0f - s1;
  float t1 = py - (float)yi, t0 = 1.0f - t1;
  float f1 = pz - (float)zi, f0 = 1.0f - f1;
  if (px < 0.f) { xi = 0; s0 = 1.f; s1 = 0.f; }
  if (py < 0.f) { yi = 0; t0 = 1.f; t1 = 0.f; }
  if (pz < 0.f) { zi = 0; f0 = 1.f; f1 = 0.f; }
  if (xi >= size[0] - 1) { xi = size[0] - 2; s0 = 0.f; s1 = 1.f; }
  if (yi >= size[1] - 1) { yi = size[1] - 2; t0 = 0.f; t1 = 1.f; }
  if (size[2] > 1) {
    if (zi >= size[2] - 1) { zi = size[2] - 2; f0 = 0.f; f1 = 1.f; }
  }
  const idx_t X = 1, Y = size[0], Z = sZ;
  const idx_t i = (idx_t)xi + Y * yi + Z * zi;
  return ((__ldg(data + i) * t0 + __ldg(data + i + Y) * t1) * s0 +
          (__ldg(data + i + X) * t0 + __ldg(data + i + X + Y) * t1) * s1) *
             f0 +
         ((__ldg(data + i + Z) * t0 + __ldg(data + i + Y + Z) * t1) * s0 +
          (__ldg(data + i + X + Z) * t0 + __ldg(data + i + X + Y + Z) * t1) * s1) *
             f1;
}

// ---- BF16 storage of Vec4 data ----------------------------------------------------

// Four bfloat16 values (x, y, z, w) in 8 bytes.  bf16 -> float is exact (the
// bf16 bits are the top half of the float); float -> bf16 rounds to nearest
// even (to_bf4).
struct __align__(8) BF4 {
  unsigned short x, y, z, w;
};
__device__ __forceinline__ float4 ld_g(const float4 *__restrict__ g, idx_t i) {
  return __ldg(g + i);
}
__device__ __forceinline__ float4 ld_g(const BF4 *__restrict__ g, idx_t i) {
  const uint2 u = __ldg((const uint2 *)(g + i));
  return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u),
                     __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xffff0000u));
}
// The same split in two: g_raw loads the stored value, g_value widens it.
__device__ __forceinline__ float4 g_raw(const float4 *__restrict__ g, idx_t i) {
  return __ldg(g + i);
}
__device__ __forceinline__ BF4 g_raw(const BF4 *__restrict__ g, idx_t i) {
  const uint2 u = __ldg((const uint2 *)(g + i));
  BF4 b;
  b.x = (unsigned short)(u.x & 0xffffu);
  b.y = (unsigned short)(u.x >> 16);
  b.z = (unsigned short)(u.y & 0xffffu);
  b.w = (unsigned short)(u.y >> 16);
  return b;
}
__device__ __forceinline__ float4 g_value(const float4 &v) { return v; }
__device__ __forceinline__ float4 g_value(const BF4 &b) {
  return make_float4(__uint_as_float((uint32_t)b.x << 16), __uint_as_float((uint32_t)b.y << 16),
                     __uint_as_float((uint32_t)b.z << 16), __uint_as_float((uint32_t)b.w << 16));
}

// ---- compensated accumulation ------------------------------------------------

// Float-float accumulator (Knuth's TwoSum): `hi` carries the running sum,
// `lo` the exact rounding errors of the adds.  Accumulating float products
// this way is about as accurate as the reference's double accumulator
// (optflow4d.cpp:234-241) and costs FP32 adds only; GB300's FP64 rate is a
// small fraction of its FP32 rate.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ void ff_add(FF &a, float p) {
  const float s = a.hi + p;
  const float bp = s - a.hi;
  const float e = (a.hi - (s - bp)) + (p - bp);
  a.hi = s;
  a.lo += e;
}
__device__ __forceinline__ double ff_value(const FF &a) { return (double)a.hi + (double)a.lo; }
// a + b in float-float: TwoSum of the high parts, then a renormalising
// Fast2Sum (Dekker 1971).
__device__ __forceinline__ FF ff_plus(const FF &a, const FF &b) {
  const float s = a.hi + b.hi;
  const float bp = s - a.hi;
  const float e = (a.hi - (s - bp)) + (b.hi - bp);
  const float lo = (a.lo + b.lo) + e;
  const float hi = s + lo;
  return {hi, lo - (hi - s)};
}
__device__ __forceinline__ FF warp_sum_ff(FF v) {
  for (int o = 16; o > 0; o >>= 1) {
    FF b;
    b.hi = __shfl_down_sync(0xffffffffu, v.hi, o);
    b.lo = __shfl_down_sync(0xffffffffu, v.lo, o);
    v = ff_plus(v, b);
  }
  return v;
}

// (float)((double)v * (1./81.)) as the reference computes it
// (knCvExpolBlur4d, optflow4d.cpp:625), mostly without FP64 work.  With
// c = c_hi + c_lo (+ a remainder below 2^-48 c), p + lo approximates v*c to
// about 2^-46 relative and f = RN(p + lo).  Rounding the exact product to
// double and then to float gives f unless the product lies within 2^-53 of
// a float rounding midpoint; products within 2^-40 of a midpoint, and tiny
// or non-finite values, take the double path.
__device__ __forceinline__ float mul_inv81(float v) {
  constexpr double c = 1. / 81.0;
  constexpr float c_hi = (float)c;
  constexpr float c_lo = (float)(c - (double)c_hi);
  const float p = v * c_hi;
  const float pe = __fmaf_rn(v, c_hi, -p);  // v*c_hi - p, exact
  const float lo = __fmaf_rn(v, c_lo, pe);
  const float f = p + lo;
  const unsigned E = (__float_as_uint(f) >> 23) & 0xffu;
  if (E > 41u && E < 255u) {
    const float rem = (p - f) + lo;                       // ~ v*c - f
    const float half_ulp = __uint_as_float((E - 24u) << 23);
    const float margin = __uint_as_float((E - 40u) << 23);
    if (fabsf(fabsf(rem) - half_ulp) > margin) return f;
  } else if (v == 0.f) {
    return f;
  }
  return (float)((double)v * c);
}

// ---- programmatic dependent launch (griddepcontrol, sm_90 and later) -------
// The image gradient g at an interior cell rebuilt from the level's target
// level set i1 with the assembly's own operations (central differences times
// 1/(2 mDx)): the stored g bit for bit, from 4 bytes per cell instead of 16
// (the neighbour loads hit L1 and L2).
struct GradFromI1 {
  const float *__restrict__ i1;
  idx_t sY, sZ, sT;
  float dxf;
  __device__ __forceinline__ float4 operator()(idx_t id) const {
    return make_float4((__ldg(i1 + id + 1) - __ldg(i1 + id - 1)) * dxf,
                       (__ldg(i1 + id + sY) - __ldg(i1 + id - sY)) * dxf,
                       (__ldg(i1 + id + sZ) - __ldg(i1 + id - sZ)) * dxf,
                       (__ldg(i1 + id + sT) - __ldg(i1 + id - sT)) * dxf);
  }
};

// pdl_wait returns once the grid this one depends on has completed and its
// writes are visible (at once for a grid launched without the attribute);
// pdl_launch_dependents lets the next grid of the stream be scheduled, whose
// blocks then wait in their own pdl_wait.  The next grid launches only after
// every block of this one has started or exited, so its waiting blocks never
// hold back this grid's.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---- reductions -----------------------------------------------------------

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_min(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum in a fixed tree order; the result is valid in thread 0.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *sh) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < NT / 32) ? sh[l] : 0.0;
    v = warp_sum(v);
  }
  __syncthreads();
  return v;
}
// Block sum of float-float values on the FP32 pipe (this part issues FP64
// at about 2 lanes per clock per SM); the result, as a double, is valid in
// thread 0.  sh holds NT / 32 entries.
template <int NT>
__device__ __forceinline__ double block_sum_ff(FF v, FF *sh) {
  v = warp_sum_ff(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    v = (l < NT / 32) ? sh[l] : FF{0.f, 0.f};
    v = warp_sum_ff(v);
    if (l == 0) r = ff_value(v);
  }
  __syncthreads();
  return r;
}
template <int NT>
__device__ __forceinline__ float block_max(float v, float *sh) {
  v = warp_max(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < NT / 32) ? sh[l] : -INFINITY;
    v = warp_max(v);
  }
  __syncthreads();
  return v;
}
template <int NT>
__device__ __forceinline__ float block_min(float v, float *sh) {
  v = warp_min(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < NT / 32) ? sh[l] : INFINITY;
    v = warp_min(v);
  }
  __syncthreads();
  return v;
}

// "Last block" completion: every block has published its partial result
// before it increments the counter; the block that sees gridDim.x-1 combines
// the partials in index order (deterministic) and resets the counter.  No
// block ever waits on another.
__device__ __forceinline__ bool last_block_arrives(unsigned int *counter) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int prev = atomicAdd(counter, 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}

}  // namespace flof
