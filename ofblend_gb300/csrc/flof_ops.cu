// flof_ops.cu -- Grid4d operations, reductions, resampling, semi-Lagrangian
// advection and the hi-res slice lookup of the FlOF path.
//
// Reference: source/grid4d.{h,cpp} (Grid4d ops, knSetBnd4d*, kn4dMax*,
// knInterpol4d), source/plugin/optflow4d.cpp (semiLagrange4d :1275,
// calcLsDiffTempl :895, knSemiLagrangeLookupSlice4d_WithVel :1648), and the
// mode-2/3 blends of scenes/flof.py (:603-610, :750-755).
#include <float.h>

#include "flof_kernels.h"

namespace flof {

// SM count of the current device, read once (thread-safe static init).
int sm_count() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

int grid_for(long long n, int nt, int per_sm) {
  long long b = (n + nt - 1) / nt;
  long long cap = (long long)sm_count() * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

constexpr int NT = 256;

// ---------------------------------------------------------------------------
// Elementwise
// ---------------------------------------------------------------------------

// op: 0 set, 1 add, 2 mult
template <int OP>
__global__ void k_const_vec4(float4 *a, long long n, float4 v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float4 x = a[i];
    if (OP == 0) x = v;
    if (OP == 1) { x.x += v.x; x.y += v.y; x.z += v.z; x.w += v.w; }
    if (OP == 2) { x.x *= v.x; x.y *= v.y; x.z *= v.z; x.w *= v.w; }
    a[i] = x;
  }
}
template <int OP>
__global__ void k_const_real(float *a, long long n, float v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float x = a[i];
    if (OP == 0) x = v;
    if (OP == 1) x += v;
    if (OP == 2) x *= v;
    a[i] = x;
  }
}

template <int OP>
static void const_op(float *a, long long ncell, int nc, float4 v, cudaStream_t s) {
  if (ncell <= 0) return;
  if (nc == 4) {
    k_const_vec4<OP><<<grid_for(ncell, NT), NT, 0, s>>>((float4 *)a, ncell, v);
  } else if (ncell % 4 == 0 && ((uintptr_t)a & 15) == 0) {
    float4 vv = make_float4(v.x, v.x, v.x, v.x);
    k_const_vec4<OP><<<grid_for(ncell / 4, NT), NT, 0, s>>>((float4 *)a, ncell / 4, vv);
  } else {
    k_const_real<OP><<<grid_for(ncell, NT), NT, 0, s>>>(a, ncell, v.x);
  }
}
void launch_set_const(float *a, long long ncell, int nc, float4 v, cudaStream_t s) {
  const_op<0>(a, ncell, nc, v, s);
}
void launch_add_const(float *a, long long ncell, int nc, float4 v, cudaStream_t s) {
  const_op<1>(a, ncell, nc, v, s);
}
void launch_mult_const(float *a, long long ncell, int nc, float4 v, cudaStream_t s) {
  const_op<2>(a, ncell, nc, v, s);
}

// op: 0 add, 1 sub, 2 scaled add with per-component factor
template <int OP>
__global__ void k_binary_vec4(float4 *a, const float4 *__restrict__ b, long long n,
                              float4 f) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float4 x = a[i];
    const float4 y = __ldg(b + i);
    if (OP == 0) { x.x += y.x; x.y += y.y; x.z += y.z; x.w += y.w; }
    if (OP == 1) { x.x -= y.x; x.y -= y.y; x.z -= y.z; x.w -= y.w; }
    if (OP == 2) {
      x.x += f.x * y.x; x.y += f.y * y.y; x.z += f.z * y.z; x.w += f.w * y.w;
    }
    a[i] = x;
  }
}
template <int OP>
__global__ void k_binary_real(float *a, const float *__restrict__ b, long long n,
                              float f) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float x = a[i];
    const float y = __ldg(b + i);
    if (OP == 0) x += y;
    if (OP == 1) x -= y;
    if (OP == 2) x += f * y;
    a[i] = x;
  }
}
template <int OP>
static void binary_op(float *a, const float *b, long long nfloat, float4 f,
                      bool per_comp, cudaStream_t s) {
  if (nfloat <= 0) return;
  const bool vec = nfloat % 4 == 0 && ((uintptr_t)a & 15) == 0 && ((uintptr_t)b & 15) == 0;
  if (vec) {
    float4 ff = per_comp ? f : make_float4(f.x, f.x, f.x, f.x);
    k_binary_vec4<OP><<<grid_for(nfloat / 4, NT), NT, 0, s>>>((float4 *)a, (const float4 *)b,
                                                             nfloat / 4, ff);
  } else {
    k_binary_real<OP><<<grid_for(nfloat, NT), NT, 0, s>>>(a, b, nfloat, f.x);
  }
}
void launch_add(float *a, const float *b, long long n, cudaStream_t s) {
  binary_op<0>(a, b, n, make_float4(0, 0, 0, 0), false, s);
}
void launch_sub(float *a, const float *b, long long n, cudaStream_t s) {
  binary_op<1>(a, b, n, make_float4(0, 0, 0, 0), false, s);
}
void launch_add_scaled(float *a, const float *b, long long ncell, int nc, float4 f,
                       cudaStream_t s) {
  binary_op<2>(a, b, ncell * nc, f, nc == 4, s);
}

// ---------------------------------------------------------------------------
// Borders (grid4d.cpp:355-407)
// ---------------------------------------------------------------------------

__global__ void k_set_bound(float *a, Dims4 d, BoxDecoder bx, int nc, float4 v,
                            int w) {
  const uint32_t n = (uint32_t)d.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    const bool b = (i <= w || i >= d.x - 1 - w || j <= w || j >= d.y - 1 - w ||
                    k <= w || k >= d.z - 1 - w || l <= w || l >= d.t - 1 - w);
    if (!b) continue;
    if (nc == 4) ((float4 *)a)[q] = v;
    else a[q] = v.x;
  }
}
void launch_set_bound(float *a, Dims4 d, int nc, float4 v, int w, cudaStream_t s) {
  BoxDecoder bx = make_decoder(d.x, d.y, d.z, 0, 0, 0, 0);
  k_set_bound<<<grid_for(d.cells(), NT), NT, 0, s>>>(a, d, bx, nc, v, w);
}

__global__ void k_set_bound_neumann(float *a, Dims4 d, BoxDecoder bx, int nc, int w) {
  const uint32_t n = (uint32_t)d.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    bool set = false;
    int si = i, sj = j, sk = k, sl = l;
    if (i <= w) { si = w + 1; set = true; }
    if (i >= d.x - 1 - w) { si = d.x - 1 - w - 1; set = true; }
    if (j <= w) { sj = w + 1; set = true; }
    if (j >= d.y - 1 - w) { sj = d.y - 1 - w - 1; set = true; }
    if (k <= w) { sk = w + 1; set = true; }
    if (k >= d.z - 1 - w) { sk = d.z - 1 - w - 1; set = true; }
    if (l <= w) { sl = w + 1; set = true; }
    if (l >= d.t - 1 - w) { sl = d.t - 1 - w - 1; set = true; }
    if (!set) continue;
    // Source cells lie strictly inside the written ring, so the in-place
    // update does not depend on the visiting order.
    const idx_t src = d.index(si, sj, sk, sl);
    if (nc == 4) ((float4 *)a)[q] = ((const float4 *)a)[src];
    else a[q] = a[src];
  }
}
void launch_set_bound_neumann(float *a, Dims4 d, int nc, int w, cudaStream_t s) {
  BoxDecoder bx = make_decoder(d.x, d.y, d.z, 0, 0, 0, 0);
  k_set_bound_neumann<<<grid_for(d.cells(), NT), NT, 0, s>>>(a, d, bx, nc, w);
}

__global__ void k_reset_outside(float4 *a, Dims4 d, BoxDecoder bx, int rb) {
  const uint32_t n = (uint32_t)d.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    if (in_bounds(d, i, j, k, l, rb)) continue;
    a[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}
void launch_reset_outside(float4 *a, Dims4 d, int resetBnd, cudaStream_t s) {
  BoxDecoder bx = make_decoder(d.x, d.y, d.z, 0, 0, 0, 0);
  k_reset_outside<<<grid_for(d.cells(), NT), NT, 0, s>>>(a, d, bx, resetBnd);
}

// ---------------------------------------------------------------------------
// Reductions (grid4d.cpp:142-172, :263-285)
// ---------------------------------------------------------------------------

template <int WHICH>
__global__ void k_reduce_minmax(const float *__restrict__ a, long long n, int nc,
                                float *partials, unsigned int *counter,
                                float *result) {
  __shared__ float sh[NT / 32];
  float acc = WHICH == 0 ? -FLT_MAX : FLT_MAX;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float v;
    if (nc == 4) {
      const float4 x = __ldg((const float4 *)a + i);
      v = x.x * x.x + x.y * x.y + x.z * x.z + x.w * x.w;  // normSquare
    } else {
      v = __ldg(a + i);
    }
    if (WHICH == 0) { if (v > acc) acc = v; }
    else { if (v < acc) acc = v; }
  }
  float b = WHICH == 0 ? block_max<NT>(acc, sh) : block_min<NT>(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
  if (last_block_arrives(counter)) {
    float m = WHICH == 0 ? -FLT_MAX : FLT_MAX;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
      float v = __ldcg(partials + q);
      if (WHICH == 0) { if (v > m) m = v; }
      else { if (v < m) m = v; }
    }
    m = WHICH == 0 ? block_max<NT>(m, sh) : block_min<NT>(m, sh);
    if (threadIdx.x == 0) {
      *result = m;
      *counter = 0;
    }
  }
}
void launch_reduce_minmax(const float *a, long long ncell, int nc, int which,
                          float *partials, unsigned int *counter, float *result,
                          cudaStream_t s) {
  const int nb = grid_for(ncell, NT, 4);
  if (which == 0)
    k_reduce_minmax<0><<<nb, NT, 0, s>>>(a, ncell, nc, partials, counter, result);
  else
    k_reduce_minmax<1><<<nb, NT, 0, s>>>(a, ncell, nc, partials, counter, result);
}

// calcLsDiffTempl (optflow4d.cpp:895-927)
__global__ void k_ls_diff(const float *__restrict__ i0, const float *__restrict__ i1,
                          float *out, Dims4 d, BoxDecoder bx, uint32_t nbox,
                          float correction, double scale, double *partials,
                          unsigned int *counter, double *result_d,
                          float *result_f) {
  __shared__ double sh[NT / 32];
  double acc = 0.0;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nbox;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float a = __ldg(i0 + id), b = __ldg(i1 + id);
    if ((a < 0.f && b < 0.f) || (a >= 0.f && b >= 0.f)) {
      if (out) out[id] = 0.f;
    } else {
      float dd = fabsf(a - b) * correction;
      if (dd > 1.f) dd = 1.f;
      acc += (double)dd;
      if (out) out[id] = dd;
    }
  }
  double b = block_sum<NT>(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
  if (last_block_arrives(counter)) {
    double m = 0.0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) m += __ldcg(partials + q);
    m = block_sum<NT>(m, sh);
    if (threadIdx.x == 0) {
      double accu = m * 1000.;
      if (d.t > 1) accu *= 1000.;
      accu *= scale;
      *result_d = accu;
      *result_f = (float)accu;
      *counter = 0;
    }
  }
}
int ls_diff_blocks(Dims4 d, int bnd) {
  const long long ex = d.x - 2 * bnd, ey = d.y - 2 * bnd, ez = d.z - 2 * bnd, et = d.t - 2 * bnd;
  const long long nb = (ex > 0 && ey > 0 && ez > 0 && et > 0) ? ex * ey * ez * et : 1;
  return grid_for(nb, NT, 4);
}
void launch_ls_diff(const float *i0, const float *i1, float *out, Dims4 d,
                    float correction, int bnd, double *partials,
                    unsigned int *counter, double *result_d, float *result_f,
                    cudaStream_t s) {
  const int ex = d.x - 2 * bnd, ey = d.y - 2 * bnd, ez = d.z - 2 * bnd, et = d.t - 2 * bnd;
  long long nbox = (ex > 0 && ey > 0 && ez > 0 && et > 0) ? (long long)ex * ey * ez * et : 0;
  BoxDecoder bx = make_decoder(ex > 0 ? ex : 1, ey > 0 ? ey : 1, ez > 0 ? ez : 1, bnd, bnd, bnd, bnd);
  // accu *= 1. / double(sx*sy*sz*st) with int arithmetic for the count.
  // Grid4d's is3D() and is4D() are constant true (grid4d.h:82-83), so
  // FOR_IJKT_BND (kernel.h:62-68) and this count shrink every axis, T == 1
  // included.  When bnd leaves no cells the loop adds nothing and the
  // reference returns 0 * (1 / cnt): -0 for a negative count, NaN for 0.
  const int cnt = ex * ey * ez * et;
  const double scale = 1. / (double)cnt;
  k_ls_diff<<<ls_diff_blocks(d, bnd), NT, 0, s>>>(i0, i1, out, d, bx, (uint32_t)nbox,
                                                  correction, scale, partials, counter,
                                                  result_d, result_f);
}

// ---------------------------------------------------------------------------
// Resampling: knInterpol4d / KnInterpolateGrid4dTempl (grid4d.cpp:531-538,
// grid4d.h:463-471)
// ---------------------------------------------------------------------------

template <int NC>
__global__ void k_resample(float *__restrict__ target, Dims4 td, BoxDecoder bx,
                           const float *__restrict__ source, Dims4 sd, float4 fac,
                           float4 off) {
  const uint32_t n = (uint32_t)td.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    const float p0 = (float)i * fac.x + off.x;
    const float p1 = (float)j * fac.y + off.y;
    const float p2 = (float)k * fac.z + off.z;
    const float p3 = (float)l * fac.w + off.w;
    if (NC == 4)
      ((float4 *)target)[q] = interp4_vec((const float4 *)source, sd, p0, p1, p2, p3);
    else
      target[q] = interp4_real(source, sd, p0, p1, p2, p3);
  }
}
void launch_resample(float *target, Dims4 td, const float *source, Dims4 sd,
                     int nc, float4 fac, float4 off, cudaStream_t s) {
  BoxDecoder bx = make_decoder(td.x, td.y, td.z, 0, 0, 0, 0);
  const int nb = grid_for(td.cells(), NT);
  if (nc == 4)
    k_resample<4><<<nb, NT, 0, s>>>(target, td, bx, source, sd, fac, off);
  else
    k_resample<1><<<nb, NT, 0, s>>>(target, td, bx, source, sd, fac, off);
}

// ---------------------------------------------------------------------------
// semiLagrange4d (optflow4d.cpp:1275-1290): dst = src(ijkt+0.5 - vel*dt) over
// bnd=1 cells of a fresh (zeroed) grid.
// ---------------------------------------------------------------------------

// With `maxn2` set, the launch is the single substep of advectCflHelper4d
// (optflow4d.cpp:1309-1321): the substep count int(maxVel/cfl)+1 is
// evaluated here from the device-resident max |v|^2, and a count other than
// one is reported through `flag` so that the host can redo the call with
// host-side substeps.
template <int NC>
__global__ void k_advect(const float4 *__restrict__ vel, const float *__restrict__ src,
                         float *__restrict__ dst, Dims4 d, BoxDecoder bx, float dt,
                         const float *maxn2, float cfl, int *flag) {
  if (maxn2 && blockIdx.x == 0 && threadIdx.x == 0) {
    const float maxVel = sqrtf(*maxn2) * 1.0f;
    const int steps = trunc_i(maxVel / cfl) + 1;
    if (steps != 1) *flag = 1;
  }
  const uint32_t n = (uint32_t)d.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    if (!in_bounds(d, i, j, k, l, 1)) {
      if (NC == 4) ((float4 *)dst)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      else dst[q] = 0.f;
      continue;
    }
    const float4 v = __ldg(vel + q);
    const float p0 = (float)(i + 0.5f) - v.x * dt;
    const float p1 = (float)(j + 0.5f) - v.y * dt;
    const float p2 = (float)(k + 0.5f) - v.z * dt;
    const float p3 = (float)(l + 0.5f) - v.w * dt;
    if (NC == 4)
      ((float4 *)dst)[q] = interp4_vec((const float4 *)src, d, p0, p1, p2, p3);
    else
      dst[q] = interp4_real(src, d, p0, p1, p2, p3);
  }
}
void launch_advect(const float4 *vel, const float *src, float *dst, Dims4 d,
                   int nc, float dt, cudaStream_t s) {
  BoxDecoder bx = make_decoder(d.x, d.y, d.z, 0, 0, 0, 0);
  const int nb = grid_for(d.cells(), NT);
  if (nc == 4)
    k_advect<4><<<nb, NT, 0, s>>>(vel, src, dst, d, bx, dt, nullptr, 0.f, nullptr);
  else
    k_advect<1><<<nb, NT, 0, s>>>(vel, src, dst, d, bx, dt, nullptr, 0.f, nullptr);
}

void launch_advect_cfl1(const float4 *vel, const float *src, float *dst, Dims4 d, int nc,
                        const float *maxn2, float cfl, int *flag, cudaStream_t s) {
  BoxDecoder bx = make_decoder(d.x, d.y, d.z, 0, 0, 0, 0);
  const int nb = grid_for(d.cells(), NT);
  const float dt = (1.0f / (float)1) * 1.0f;
  if (nc == 4)
    k_advect<4><<<nb, NT, 0, s>>>(vel, src, dst, d, bx, dt, maxn2, cfl, flag);
  else
    k_advect<1><<<nb, NT, 0, s>>>(vel, src, dst, d, bx, dt, maxn2, cfl, flag);
}

__global__ void k_deform_twoway(const float4 *__restrict__ vel,
                                const float4 *__restrict__ velInv,
                                const float *__restrict__ i0,
                                const float *__restrict__ i1, float *__restrict__ out,
                                Dims4 d, BoxDecoder bx, float alpha, float alphaInv) {
  const uint32_t n = (uint32_t)d.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    float a0 = 0.f, a1 = 0.f;
    if (in_bounds(d, i, j, k, l, 1)) {
      const float4 v = __ldg(vel + q);
      const float4 w = __ldg(velInv + q);
      a0 = interp4_real(i0, d, (float)(i + 0.5f) - v.x * alpha,
                        (float)(j + 0.5f) - v.y * alpha,
                        (float)(k + 0.5f) - v.z * alpha,
                        (float)(l + 0.5f) - v.w * alpha);
      a1 = interp4_real(i1, d, (float)(i + 0.5f) - w.x * alphaInv,
                        (float)(j + 0.5f) - w.y * alphaInv,
                        (float)(k + 0.5f) - w.z * alphaInv,
                        (float)(l + 0.5f) - w.w * alphaInv);
    }
    out[q] = a0 * alphaInv + alpha * a1;
  }
}
void launch_deform_twoway(const float4 *vel, const float4 *velInv,
                          const float *i0, const float *i1, float *out, Dims4 d,
                          float alpha, float alphaInv, cudaStream_t s) {
  BoxDecoder bx = make_decoder(d.x, d.y, d.z, 0, 0, 0, 0);
  k_deform_twoway<<<grid_for(d.cells(), NT), NT, 0, s>>>(vel, velInv, i0, i1, out, d, bx,
                                                         alpha, alphaInv);
}

// ---------------------------------------------------------------------------
// Mode-3 hi-res slice lookup (optflow4d.cpp:1648-1665, :2009-2013)
// ---------------------------------------------------------------------------

__global__ void k_blend_slices(const float4 *__restrict__ v1, const float4 *__restrict__ v2,
                               float4 *__restrict__ vt, long long n, float f1, float f2) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float4 a = __ldg(v1 + q), b = __ldg(v2 + q);
    float4 r;
    r.x = 0.f + f1 * a.x; r.x += f2 * b.x;
    r.y = 0.f + f1 * a.y; r.y += f2 * b.y;
    r.z = 0.f + f1 * a.z; r.z += f2 * b.z;
    r.w = 0.f + f1 * a.w; r.w += f2 * b.w;
    vt[q] = r;
  }
}
void launch_blend_slices(const float4 *v1, const float4 *v2, float4 *vt,
                         long long cells, float f1, float f2, cudaStream_t s) {
  k_blend_slices<<<grid_for(cells, NT), NT, 0, s>>>(v1, v2, vt, cells, f1, f2);
}

// The blends of both directions of a two-way frame in one launch: cells of
// the first set, then of the second, each blended as k_blend_slices does.
struct BlendSet {
  const float4 *v1, *v2;
  float4 *vt;
  float f1, f2;
};
__global__ void k_blend_slices2(BlendSet a, BlendSet b, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < 2 * n;
       q += (long long)gridDim.x * blockDim.x) {
    const BlendSet &S = q < n ? a : b;
    const long long e = q < n ? q : q - n;
    const float4 x = __ldg(S.v1 + e), y = __ldg(S.v2 + e);
    float4 r;
    r.x = 0.f + S.f1 * x.x; r.x += S.f2 * y.x;
    r.y = 0.f + S.f1 * x.y; r.y += S.f2 * y.y;
    r.z = 0.f + S.f1 * x.z; r.z += S.f2 * y.z;
    r.w = 0.f + S.f1 * x.w; r.w += S.f2 * y.w;
    S.vt[e] = r;
  }
}
void launch_blend_slices2(const float4 *v1a, const float4 *v2a, float4 *vta, float fa1, float fa2,
                          const float4 *v1b, const float4 *v2b, float4 *vtb, float fb1, float fb2,
                          long long cells, cudaStream_t s) {
  k_blend_slices2<<<grid_for(2 * cells, NT), NT, 0, s>>>(BlendSet{v1a, v2a, vta, fa1, fa2},
                                                         BlendSet{v1b, v2b, vtb, fb1, fb2}, cells);
}

__device__ __forceinline__ float lookup_one(const float *__restrict__ phi, const Dims4 &pd,
                                            float time, float dt,
                                            const float4 *__restrict__ vt, int vx,
                                            int vy, int vz, float4 sf3, float4 off3,
                                            float4 df, int i, int j, int k) {
  const float q0 = (float)i * sf3.x + off3.x;
  const float q1 = (float)j * sf3.y + off3.y;
  const float q2 = (float)k * sf3.z + off3.z;
  float4 v = interp3_vec(vt, vx, vy, vz, q0, q1, q2);
  v.x *= df.x;
  v.y *= df.y;
  v.z *= df.z;
  v.w *= df.w;
  return interp4_real(phi, pd, (float)(i + 0.5f) - v.x * dt,
                      (float)(j + 0.5f) - v.y * dt,
                      (float)(k + 0.5f) - v.z * dt, (time + 0.5f) - v.w * dt);
}

__global__ void k_lookup_slice(float *__restrict__ dst, int dx, int dy, BoxDecoder bx,
                               uint32_t nbox, const float *__restrict__ phi, Dims4 pd,
                               float time, float dt, const float4 *__restrict__ vt,
                               int vx, int vy, int vz, float4 sf3, float4 off3,
                               float4 df) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nbox;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    dst[(idx_t)i + (idx_t)dx * j + (idx_t)dx * dy * k] =
        lookup_one(phi, pd, time, dt, vt, vx, vy, vz, sf3, off3, df, i, j, k);
  }
}

static void lookup_box(int dx, int dy, int dz, int bordSkip, int &lo, int &ex,
                       int &ey, int &ez, int minBnd = 10) {
  lo = bordSkip > minBnd ? bordSkip : minBnd;
  ex = dx - 2 * lo;
  ey = dy - 2 * lo;
  ez = dz - 2 * lo;
}

void launch_lookup_slice(float *dst, int dx, int dy, int dz, const float *phi,
                         Dims4 pd, float time, float dt, const float4 *vt,
                         int vx, int vy, int vz, float4 sf3, float4 off3,
                         float4 defoFactor, int bordSkip, cudaStream_t s, int minBnd) {
  int lo, ex, ey, ez;
  lookup_box(dx, dy, dz, bordSkip, lo, ex, ey, ez, minBnd);
  if (ex <= 0 || ey <= 0 || ez <= 0) return;
  BoxDecoder bx = make_decoder(ex, ey, ez, lo, lo, lo, 0);
  const long long nbox = (long long)ex * ey * ez;
  k_lookup_slice<<<grid_for(nbox, NT), NT, 0, s>>>(dst, dx, dy, bx, (uint32_t)nbox, phi, pd,
                                                   time, dt, vt, vx, vy, vz, sf3, off3,
                                                   defoFactor);
}

__global__ void k_lookup_slice_twoway(float *__restrict__ dst, int dx, int dy,
                                      BoxDecoder bx, uint32_t nbox,
                                      const float *__restrict__ phi0,
                                      const float *__restrict__ phi1, Dims4 pd,
                                      float time, float alpha, float alphaInv,
                                      const float4 *__restrict__ vt0,
                                      const float4 *__restrict__ vt1, int vx, int vy,
                                      int vz, float4 sf3, float4 off3, float4 df) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nbox;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    const float a = lookup_one(phi0, pd, time, alpha, vt0, vx, vy, vz, sf3, off3, df, i, j, k);
    const float b = lookup_one(phi1, pd, time, alphaInv, vt1, vx, vy, vz, sf3, off3, df, i, j, k);
    // dst.multConst(1-alpha); dst.addScaled(dst1, alpha)
    dst[(idx_t)i + (idx_t)dx * j + (idx_t)dx * dy * k] = a * alphaInv + alpha * b;
  }
}
void launch_lookup_slice_twoway(float *dst, int dx, int dy, int dz,
                                const float *phi0, const float *phi1, Dims4 pd,
                                float time, float alpha, float alphaInv,
                                const float4 *vt0, const float4 *vt1, int vx,
                                int vy, int vz, float4 sf3, float4 off3,
                                float4 defoFactor, int bordSkip, cudaStream_t s) {
  int lo, ex, ey, ez;
  lookup_box(dx, dy, dz, bordSkip, lo, ex, ey, ez);
  if (ex <= 0 || ey <= 0 || ez <= 0) return;
  BoxDecoder bx = make_decoder(ex, ey, ez, lo, lo, lo, 0);
  const long long nbox = (long long)ex * ey * ez;
  k_lookup_slice_twoway<<<grid_for(nbox, NT), NT, 0, s>>>(
      dst, dx, dy, bx, (uint32_t)nbox, phi0, phi1, pd, time, alpha, alphaInv, vt0, vt1, vx,
      vy, vz, sf3, off3, defoFactor);
}

}  // namespace flof
