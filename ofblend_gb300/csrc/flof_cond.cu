// flof_cond.cu -- the steps either side of the solve: input conditioning of
// the 4D level sets (flof.py postProcessPhiData) and the output stage of the
// hi-res frames (flof.py time-SDF merge, blend union and writeResults
// smoothing).
//
// Reference:
//   repeatFrame4d          source/plugin/optflow4d.cpp:1254-1266
//   extrap4dLsSimple       source/plugin/optflow4d.cpp:1332-1406
//   knSimpleBlurSpecial    source/test.cpp:94-131
//   LevelsetGrid::join     source/levelset.cpp:114-118
//   Grid<T>::setBound      source/grid.cpp:462-473
//   Grid<T>::setBoundNeumann source/grid.cpp:475-511
//   knLoadPlaceGridIpol / knLoadPlaceGridRescale, shiftForwGrid4d
//                          source/plugin/optflow4d.cpp:1443-1458, 1596-1616
#include "flof_kernels.h"

namespace flof {

namespace {

constexpr int NT = 256;

// 3D cell of a linear index over an (X, Y, Z) box.
struct Box3 {
  FastDiv fx, fy;
  int ex, ey;
  __device__ __forceinline__ void decode(uint32_t n, int &i, int &j, int &k) const {
    const uint32_t q = fx.div(n);
    i = (int)(n - q * (uint32_t)ex);
    const uint32_t q2 = fy.div(q);
    j = (int)(q - q2 * (uint32_t)ey);
    k = (int)q2;
  }
};
Box3 box3(int ex, int ey) {
  Box3 b;
  b.fx = FastDiv((uint32_t)ex);
  b.fy = FastDiv((uint32_t)ey);
  b.ex = ex;
  b.ey = ey;
  return b;
}

// ---------------------------------------------------------------------------
// repeatFrame4d: every slice t in [t0, t1] of the bnd box gets the value
// interpolated at (i+.5, j+.5, k+.5, srct+.5).  The x, y, z coordinates
// land on cell centres, so each value depends on the cell itself at the two
// time slices around srct (the other corners carry weight zero).  The values
// are computed into a 3D buffer first and then written, so no thread reads a
// slice another thread is writing.
// ---------------------------------------------------------------------------
__global__ void k_repeat_frame_eval(const float *__restrict__ phi, Dims4 d, float srct,
                                    float *__restrict__ slice, Box3 bx, uint32_t n, int bnd) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k;
    bx.decode(q, i, j, k);
    i += bnd;
    j += bnd;
    k += bnd;
    slice[(idx_t)i + (idx_t)d.x * j + (idx_t)d.x * d.y * k] =
        interp4_real(phi, d, (float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f, srct + 0.5f);
  }
}

__global__ void k_repeat_frame_store(float *__restrict__ phi, Dims4 d,
                                     const float *__restrict__ slice, Box3 bx, uint32_t n,
                                     int bnd, int t0, int nt) {
  const idx_t sT = d.st();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k;
    bx.decode(q, i, j, k);
    i += bnd;
    j += bnd;
    k += bnd;
    const idx_t id3 = (idx_t)i + (idx_t)d.x * j + (idx_t)d.x * d.y * k;
    const float v = slice[id3];
    for (int t = 0; t < nt; ++t) phi[id3 + (idx_t)(t0 + t) * sT] = v;
  }
}

// ---------------------------------------------------------------------------
// extrap4dLsSimple.  tmp holds the reference's Grid4d<int> marks: 1 = inside
// the front, 2 = first layer, d+1 = filled by sweep d.  Each sweep reads only
// cells marked d (final since the previous launch) and writes only cells
// still marked 0, so sweeping in place has no read/write overlap.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool inner1(const Dims4 &d, int i, int j, int k, int t) {
  return i >= 1 && j >= 1 && k >= 1 && t >= 1 && i < d.x - 1 && j < d.y - 1 && k < d.z - 1 &&
         t < d.t - 1;
}

__global__ void k_extrap_mark(const float *__restrict__ phi, int *__restrict__ tmp, Dims4 d,
                              BoxDecoder bx, uint32_t n, int inside) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k, t;
    bx.decode(q, i, j, k, t);
    int m = 0;
    if (inner1(d, i, j, k, t)) {
      const float v = phi[q];
      m = (inside ? v > 0.f : v < 0.f) ? 1 : 0;
    }
    tmp[q] = m;
  }
}

// neighbour order of nbs4d (optflow4d.cpp:1323-1326): -x,+x,-y,+y,-z,+z,-t,+t
__global__ void k_extrap_layer(int *__restrict__ tmp, Dims4 d, BoxDecoder bx, uint32_t n) {
  const idx_t off[8] = {-1, 1, -(idx_t)d.x, (idx_t)d.x, -d.sz(), d.sz(), -d.st(), d.st()};
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k, t;
    bx.decode(q, i, j, k, t);
    const idx_t id = d.index(i, j, k, t);
    if (tmp[id]) continue;
    bool hit = false;
#pragma unroll
    for (int m = 0; m < 8; ++m) hit |= (tmp[id + off[m]] == 1);
    if (hit) tmp[id] = 2;
  }
}

__global__ void k_extrap_step(float *__restrict__ phi, int *__restrict__ tmp, Dims4 d,
                              BoxDecoder bx, uint32_t n, int dd, float direction) {
  const idx_t off[8] = {-1, 1, -(idx_t)d.x, (idx_t)d.x, -d.sz(), d.sz(), -d.st(), d.st()};
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k, t;
    bx.decode(q, i, j, k, t);
    const idx_t id = d.index(i, j, k, t);
    if (tmp[id] != 0) continue;
    int nbs = 0;
    float avg = 0.f;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      if (tmp[id + off[m]] == dd) {
        avg += phi[id + off[m]];
        nbs++;
      }
    }
    if (nbs > 0) {
      tmp[id] = dd + 1;
      phi[id] = avg / (float)nbs + direction;
    }
  }
}

__global__ void k_extrap_remaining(float *__restrict__ phi, const int *__restrict__ tmp, Dims4 d,
                                   BoxDecoder bx, uint32_t n, float value) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k, t;
    bx.decode(q, i, j, k, t);
    const idx_t id = d.index(i, j, k, t);
    if (tmp[id] == 0) phi[id] = value;
  }
}

// ---------------------------------------------------------------------------
// knSimpleBlurSpecial over the bnd = 1 box of a 3D grid (k = 0 only for a 2D
// grid): cells outside isInBounds(bord) or below thresh are copied, the rest
// get the mean of their 6 (3D) or 4 (2D) face neighbours, added in the
// reference's order and scaled by the double constant 1/6 (1/4).  The ring
// outside the box is not written.
// ---------------------------------------------------------------------------
__global__ void k_simple_blur_special(const float *__restrict__ a, float *__restrict__ tmp,
                                      int X, int Y, int Z, Box3 bx, uint32_t n, float thresh,
                                      int bord) {
  const bool is3d = Z > 1;
  const idx_t sY = X, sZ = (idx_t)X * Y;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k;
    bx.decode(q, i, j, k);
    i += 1;
    j += 1;
    if (is3d) k += 1;
    const idx_t id = (idx_t)i + sY * j + sZ * k;
    bool inb = i >= bord && j >= bord && i < X - bord && j < Y - bord;
    inb = inb && (is3d ? (k >= bord && k < Z - bord) : (k == 0));
    const float v = a[id];
    if (!inb || v < thresh) {
      tmp[id] = v;
      continue;
    }
    float s = a[id + 1] + a[id - 1];
    s = s + a[id + sY];
    s = s + a[id - sY];
    if (is3d) {
      s += a[id + sZ] + a[id - sZ];
      tmp[id] = (float)((double)s * (1. / 6.));
    } else {
      tmp[id] = (float)((double)s * (1. / 4.));
    }
  }
}

// LevelsetGrid::join: a = std::min(a, b), i.e. b only where b < a.
__global__ void k_join(float *__restrict__ a, const float *__restrict__ b, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float x = a[q], y = b[q];
    a[q] = (y < x) ? y : x;
  }
}

// Grid<T>::setBound for a 3D (or 2D, Z == 1) grid: every cell with
// i <= w, i >= X-1-w, j <= w, j >= Y-1-w or, in 3D, the same in k.
__global__ void k_set_bound3(float *__restrict__ a, int X, int Y, int Z, int nc, float4 v,
                             int w, Box3 bx, uint32_t n) {
  const bool is3d = Z > 1;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k;
    bx.decode(q, i, j, k);
    const bool b = i <= w || i >= X - 1 - w || j <= w || j >= Y - 1 - w ||
                   (is3d && (k <= w || k >= Z - 1 - w));
    if (!b) continue;
    if (nc == 4)
      ((float4 *)a)[q] = v;
    else
      a[q] = v.x;
  }
}

// Grid<T>::setBoundNeumann for a 3D (or 2D) grid: boundary cells copy the
// nearest cell just inside the w+1 wide ring.  The cells read are never
// boundary cells, so the kernel runs in place.
__global__ void k_set_bound_neumann3(float *__restrict__ a, int X, int Y, int Z, int nc, int w,
                                     Box3 bx, uint32_t n) {
  const bool is3d = Z > 1;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k;
    bx.decode(q, i, j, k);
    bool set = false;
    int si = i, sj = j, sk = k;
    if (i <= w) { si = w + 1; set = true; }
    if (i >= X - 1 - w) { si = X - 1 - w - 1; set = true; }
    if (j <= w) { sj = w + 1; set = true; }
    if (j >= Y - 1 - w) { sj = Y - 1 - w - 1; set = true; }
    if (is3d) {
      if (k <= w) { sk = w + 1; set = true; }
      if (k >= Z - 1 - w) { sk = Z - 1 - w - 1; set = true; }
    }
    if (!set) continue;
    const idx_t src = (idx_t)si + (idx_t)X * sj + (idx_t)X * Y * sk;
    if (nc == 4)
      ((float4 *)a)[q] = ((const float4 *)a)[src];
    else
      a[q] = a[src];
  }
}

// knLoadPlaceGridIpol: phi(i,j,k,slice) += wc * trilinear(src3, ijk * sf + off)
// over the bnd = 1 box of phi's (x,y,z) extent.
__global__ void k_place_slice(float *__restrict__ phi, Dims4 d, int slice,
                              const float *__restrict__ src, int sx, int sy, int sz, float3 sf,
                              float3 off, float wc, Box3 bx, uint32_t n) {
  const int size[3] = {sx, sy, sz};
  const idx_t sZs = sz > 1 ? (idx_t)sx * sy : 0;  // a 2D grid has no z stride
  const idx_t base = (idx_t)slice * d.st();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k;
    bx.decode(q, i, j, k);
    i += 1;
    j += 1;
    k += 1;
    const float p0 = (float)i * sf.x + off.x;
    const float p1 = (float)j * sf.y + off.y;
    const float p2 = (float)k * sf.z + off.z;
    const float v = interp3_real(src, size, sZs, p0, p1, p2);
    const idx_t id = base + (idx_t)i + (idx_t)d.x * j + d.sz() * k;
    phi[id] += wc * v;
  }
}

// tmp(i,j,k) += v over the bnd = 1 box of a 3D grid (the sdfIsoOff fix-up of
// loadPlaceGrid4d, optflow4d.cpp:1566-1572).
__global__ void k_add_inner3(float *__restrict__ a, int X, int Y, int Z, float v, Box3 bx,
                             uint32_t n) {
  const bool is3d = Z > 1;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k;
    bx.decode(q, i, j, k);
    i += 1;
    j += 1;
    if (is3d) k += 1;
    a[(idx_t)i + (idx_t)X * j + (idx_t)X * Y * k] += v;
  }
}

// knLoadPlaceGridRescale: phi(i,j,k,t) *= w[t] where w[t] > 0, bnd = 1 box.
__global__ void k_rescale_slices(float *__restrict__ phi, Dims4 d, const float *__restrict__ w,
                                 BoxDecoder bx, uint32_t n) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k, t;
    bx.decode(q, i, j, k, t);
    const float wt = w[t];
    if (wt <= 0.f) continue;
    const idx_t id = d.index(i, j, k, t);
    phi[id] *= wt;
  }
}

}  // namespace

void launch_repeat_frame(float *phi, Dims4 d, float srct, int t0, int t1, int bnd, float *slice,
                         cudaStream_t s) {
  const int ex = d.x - 2 * bnd, ey = d.y - 2 * bnd, ez = d.z - 2 * bnd;
  if (ex <= 0 || ey <= 0 || ez <= 0 || t1 < t0) return;
  const uint32_t n = (uint32_t)((long long)ex * ey * ez);
  const Box3 bx = box3(ex, ey);
  k_repeat_frame_eval<<<grid_for(n, NT), NT, 0, s>>>(phi, d, srct, slice, bx, n, bnd);
  k_repeat_frame_store<<<grid_for(n, NT), NT, 0, s>>>(phi, d, slice, bx, n, bnd, t0,
                                                      t1 - t0 + 1);
}

void launch_extrap_mark(const float *phi, int *tmp, Dims4 d, int inside, cudaStream_t s) {
  const uint32_t n = (uint32_t)d.cells();
  k_extrap_mark<<<grid_for(n, NT), NT, 0, s>>>(phi, tmp, d, make_decoder(d.x, d.y, d.z, 0, 0, 0, 0),
                                               n, inside);
}

void launch_extrap_layer(int *tmp, Dims4 d, cudaStream_t s) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return;
  const uint32_t n = (uint32_t)((long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2));
  k_extrap_layer<<<grid_for(n, NT), NT, 0, s>>>(
      tmp, d, make_decoder(d.x - 2, d.y - 2, d.z - 2, 1, 1, 1, 1), n);
}

void launch_extrap_step(float *phi, int *tmp, Dims4 d, int dd, float direction, cudaStream_t s) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return;
  const uint32_t n = (uint32_t)((long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2));
  k_extrap_step<<<grid_for(n, NT), NT, 0, s>>>(
      phi, tmp, d, make_decoder(d.x - 2, d.y - 2, d.z - 2, 1, 1, 1, 1), n, dd, direction);
}

void launch_extrap_remaining(float *phi, const int *tmp, Dims4 d, float value, cudaStream_t s) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return;
  const uint32_t n = (uint32_t)((long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2));
  k_extrap_remaining<<<grid_for(n, NT), NT, 0, s>>>(
      phi, tmp, d, make_decoder(d.x - 2, d.y - 2, d.z - 2, 1, 1, 1, 1), n, value);
}

void launch_simple_blur_special(const float *a, float *tmp, int X, int Y, int Z, float thresh,
                                int bord, cudaStream_t s) {
  const int ex = X - 2, ey = Y - 2, ez = Z > 1 ? Z - 2 : 1;
  if (ex <= 0 || ey <= 0 || ez <= 0) return;
  const uint32_t n = (uint32_t)((long long)ex * ey * ez);
  k_simple_blur_special<<<grid_for(n, NT), NT, 0, s>>>(a, tmp, X, Y, Z, box3(ex, ey), n, thresh,
                                                       bord);
}

void launch_join(float *a, const float *b, long long n, cudaStream_t s) {
  k_join<<<grid_for(n, NT), NT, 0, s>>>(a, b, n);
}

void launch_set_bound3(float *a, int X, int Y, int Z, int nc, float4 v, int w, cudaStream_t s) {
  const uint32_t n = (uint32_t)((long long)X * Y * Z);
  k_set_bound3<<<grid_for(n, NT), NT, 0, s>>>(a, X, Y, Z, nc, v, w, box3(X, Y), n);
}

void launch_set_bound_neumann3(float *a, int X, int Y, int Z, int nc, int w, cudaStream_t s) {
  const uint32_t n = (uint32_t)((long long)X * Y * Z);
  k_set_bound_neumann3<<<grid_for(n, NT), NT, 0, s>>>(a, X, Y, Z, nc, w, box3(X, Y), n);
}

void launch_place_slice(float *phi, Dims4 d, int slice, const float *src, const int sdims[3],
                        const float sf[3], const float off[3], float wc, cudaStream_t s) {
  const int ex = d.x - 2, ey = d.y - 2, ez = d.z - 2;
  if (ex <= 0 || ey <= 0 || ez <= 0) return;
  const uint32_t n = (uint32_t)((long long)ex * ey * ez);
  k_place_slice<<<grid_for(n, NT), NT, 0, s>>>(phi, d, slice, src, sdims[0], sdims[1], sdims[2],
                                               make_float3(sf[0], sf[1], sf[2]),
                                               make_float3(off[0], off[1], off[2]), wc,
                                               box3(ex, ey), n);
}

void launch_add_inner3(float *a, int X, int Y, int Z, float v, cudaStream_t s) {
  const int ex = X - 2, ey = Y - 2, ez = Z > 1 ? Z - 2 : 1;
  if (ex <= 0 || ey <= 0 || ez <= 0) return;
  const uint32_t n = (uint32_t)((long long)ex * ey * ez);
  k_add_inner3<<<grid_for(n, NT), NT, 0, s>>>(a, X, Y, Z, v, box3(ex, ey), n);
}

void launch_rescale_slices(float *phi, Dims4 d, const float *w, cudaStream_t s) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return;
  const uint32_t n = (uint32_t)((long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2));
  k_rescale_slices<<<grid_for(n, NT), NT, 0, s>>>(
      phi, d, w, make_decoder(d.x - 2, d.y - 2, d.z - 2, 1, 1, 1, 1), n);
}

}  // namespace flof
