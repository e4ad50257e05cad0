// flof_net.cu -- kernels of the learned warm start: a small 4D convolutional
// encoder-decoder that predicts the coarsest-level deformation of the
// multiscale solve from the two coarse inputs.  It has no counterpart in
// the reference; the plain solve stays the drop-in and judges its output.
//
// Tensors are channels-last: element (v, c) of a tensor with C channels over
// a cubic 4D grid of extent R sits at v * C + c, v = x + R(y + R(z + R t)).
// Convolutions are 3^4 (padding 1, stride 1 or 2) or 1^4, written as
// implicit GEMMs: output voxels x output channels, reduced over (tap, input
// channel).  The weights are the BF16-rounded copy of the FP32 master
// weights (stored as floats); products are accumulated in FP32 with fused
// multiply-adds.  The backward kernels (input gradient, weight gradient)
// share the tiled GEMM core with the forward one.
#include <cuda_bf16.h>
#include <float.h>

#include "flof_kernels.h"

namespace flof {

namespace {

constexpr int GT_M = 64;   // GEMM tile rows
constexpr int GT_N = 32;   // GEMM tile columns
constexpr int GT_K = 16;   // reduction chunk
constexpr int GT_T = 128;  // threads: 16 x 8, each 4 rows x 4 columns

struct ConvGeom {
  int rin, rout;       // cubic extents of input and output
  int cin, cout;       // channels
  int ks, stride, pad;  // kernel 3 (pad 1) or 1 (pad 0)
  int taps;            // ks^4
};

__device__ __forceinline__ void vox_coords(int v, int R, int c[4]) {
  c[0] = v % R;
  v /= R;
  c[1] = v % R;
  v /= R;
  c[2] = v % R;
  c[3] = v / R;
}

// MODE 0 forward:   C[v][co]  = sum_{tap,ci} in[src(v,tap)][ci] * W[tap][ci][co]
// MODE 1 bwd data:  C[u][ci]  = sum_{tap,co} dout[dst(u,tap)][co] * W[tap][ci][co]
// MODE 2 bwd weight: C[(tap,ci)][co] = sum_v in[src(v,tap)][ci] * dout[v][co]
// src(v, tap) = v * stride + off(tap) - pad per axis (zero outside); dst is
// its inverse.  Voxel coordinates of the tile's rows and the (tap, channel)
// split of each reduction chunk are decoded once into shared memory.  MODE 2
// reduces over output voxels and is split along that reduction into
// gridDim.z slices written to C + z * M * N (summed by k_sum_slices).
template <int MODE>
__global__ void __launch_bounds__(GT_T)
k_conv_gemm(const float *__restrict__ A, const float *__restrict__ Bsrc,
            const float *__restrict__ bias, float *__restrict__ C, ConvGeom g, int M, int N,
            int K, int relu, int kslice) {
  __shared__ float As[GT_K][GT_M + 4];
  __shared__ float Bs[GT_K][GT_N + 4];
  __shared__ int rowc[GT_M][4];   // MODE 0/1: voxel coordinates of the rows
  __shared__ int rowx[GT_M][2];   // MODE 2: (tap, ci) of the rows
  __shared__ int kc[GT_K][5];     // MODE 0/1: (tap offsets x,y,z,t, channel); MODE 2: voxel
  const int m0 = blockIdx.x * GT_M, n0 = blockIdx.y * GT_N;
  const int kbeg = MODE == 2 ? blockIdx.z * kslice : 0;
  const int kend = MODE == 2 ? min(K, kbeg + kslice) : K;
  const int tid = threadIdx.x;
  const int tr = tid / 8, tc = tid % 8;  // 16 x 8 threads
  const int ch = MODE == 0 ? g.cin : g.cout;  // channels of the reduction (MODE 0/1)
  if (tid < GT_M) {
    const int m = m0 + tid;
    if (MODE == 2) {
      rowx[tid][0] = m < M ? m / g.cin : 0;
      rowx[tid][1] = m < M ? m % g.cin : 0;
    } else {
      int c[4] = {0, 0, 0, 0};
      if (m < M) vox_coords(m, MODE == 0 ? g.rout : g.rin, c);
#pragma unroll
      for (int a = 0; a < 4; ++a) rowc[tid][a] = c[a];
    }
  }
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;

  for (int k0 = kbeg; k0 < kend; k0 += GT_K) {
    if (tid < GT_K) {
      const int k = k0 + tid;
      if (MODE == 2) {
        int c[4] = {0, 0, 0, 0};
        if (k < kend) vox_coords(k, g.rout, c);
        kc[tid][0] = c[0];
        kc[tid][1] = c[1];
        kc[tid][2] = c[2];
        kc[tid][3] = c[3];
        kc[tid][4] = k < kend ? 1 : 0;
      } else {
        const int tap = k < kend ? k / ch : 0;
        kc[tid][4] = k < kend ? k % ch : -1;
        int tq = tap;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          kc[tid][a] = tq % g.ks;
          tq /= g.ks;
        }
      }
    }
    __syncthreads();
    // A tile: GT_M rows x GT_K reduction entries
    for (int e = tid; e < GT_M * GT_K; e += GT_T) {
      const int mm = e / GT_K, kk = e % GT_K;
      const int m = m0 + mm;
      float val = 0.f;
      if (m < M && (MODE == 2 ? kc[kk][4] != 0 : kc[kk][4] >= 0)) {
        if (MODE == 0) {
          int s = 0, ok = 1, mul = 1;
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const int q = rowc[mm][a] * g.stride + kc[kk][a] - g.pad;
            ok &= (q >= 0) & (q < g.rin);
            s += q * mul;
            mul *= g.rin;
          }
          if (ok) val = __ldg(A + (size_t)s * g.cin + kc[kk][4]);
        } else if (MODE == 1) {
          int s = 0, ok = 1, mul = 1;
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const int num = rowc[mm][a] + g.pad - kc[kk][a];
            const int o = num / g.stride;
            ok &= (num >= 0) & (o * g.stride == num) & (o < g.rout);
            s += o * mul;
            mul *= g.rout;
          }
          if (ok) val = __ldg(A + (size_t)s * g.cout + kc[kk][4]);
        } else {
          const int tap = rowx[mm][0], ci = rowx[mm][1];
          int s = 0, ok = 1, mul = 1, tq = tap;
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const int off = tq % g.ks;
            tq /= g.ks;
            const int q = kc[kk][a] * g.stride + off - g.pad;
            ok &= (q >= 0) & (q < g.rin);
            s += q * mul;
            mul *= g.rin;
          }
          if (ok) val = __ldg(A + (size_t)s * g.cin + ci);
        }
      }
      As[kk][mm] = val;
    }
    // B tile: GT_K reduction entries x GT_N columns
    for (int e = tid; e < GT_K * GT_N; e += GT_T) {
      const int kk = e / GT_N, nn = e % GT_N;
      const int k = k0 + kk, n = n0 + nn;
      float val = 0.f;
      if (k < kend && n < N) {
        if (MODE == 0) {
          val = __ldg(Bsrc + (size_t)k * g.cout + n);  // W[(tap, ci)][co]
        } else if (MODE == 1) {
          const int tap = k / g.cout, co = k % g.cout;  // W[tap][ci = n][co]
          val = __ldg(Bsrc + ((size_t)tap * g.cin + n) * g.cout + co);
        } else {
          val = __ldg(Bsrc + (size_t)k * g.cout + n);  // dout[v][co]
        }
      }
      Bs[kk][nn] = val;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GT_K; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tr * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tc * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = __fmaf_rn(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  float *Cz = MODE == 2 ? C + (size_t)blockIdx.z * M * N : C;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + tr * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tc * 4 + j;
      if (n >= N) continue;
      float v = acc[i][j];
      if (MODE == 0) {
        if (bias) v += __ldg(bias + n);
        if (relu) v = v > 0.f ? v : 0.f;
      }
      Cz[(size_t)m * N + n] = v;
    }
  }
}

// out[i] = sum over the z slices of in (in order)
__global__ void k_sum_slices(const float *__restrict__ in, float *__restrict__ out, long long n,
                             int nz) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < nz; ++z) s += in[(size_t)z * n + q];
    out[q] = s;
  }
}

// dX *= (Y > 0): ReLU backward through the stored output Y
__global__ void k_relu_bwd(float *__restrict__ dy, const float *__restrict__ y, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    if (!(y[q] > 0.f)) dy[q] = 0.f;
}

// out[v][0:c1] = lo[parent(v)][.], out[v][c1:c1+c2] = skip[v][.]
__global__ void k_upcat(const float *__restrict__ lo, const float *__restrict__ skip,
                        float *__restrict__ out, int R, int c1, int c2) {
  const long long V = (long long)R * R * R * R;
  const int C = c1 + c2;
  const int Rl = R / 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < V * C;
       e += (long long)gridDim.x * blockDim.x) {
    const long long v = e / C;
    const int c = (int)(e % C);
    if (c < c1) {
      const int x = (int)(v % R), y = (int)((v / R) % R), z = (int)((v / R / R) % R),
                t = (int)(v / R / R / R);
      const long long p = (x / 2) + (long long)Rl * ((y / 2) + (long long)Rl * ((z / 2) + (long long)Rl * (t / 2)));
      out[e] = __ldg(lo + p * c1 + c);
    } else {
      out[e] = __ldg(skip + v * c2 + (c - c1));
    }
  }
}

// backward of k_upcat: dlo[p][c] = sum over the 16 children, dskip[v][c] += d
__global__ void k_upcat_bwd(const float *__restrict__ dout, float *__restrict__ dlo,
                            float *__restrict__ dskip, int R, int c1, int c2) {
  const int Rl = R / 2;
  const long long Vl = (long long)Rl * Rl * Rl * Rl;
  const int C = c1 + c2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < Vl * c1;
       e += (long long)gridDim.x * blockDim.x) {
    const long long p = e / c1;
    const int c = (int)(e % c1);
    const int x = (int)(p % Rl), y = (int)((p / Rl) % Rl), z = (int)((p / Rl / Rl) % Rl),
              t = (int)(p / Rl / Rl / Rl);
    float s = 0.f;
    for (int q = 0; q < 16; ++q) {
      const long long v = (2 * x + (q & 1)) +
                          (long long)R * ((2 * y + ((q >> 1) & 1)) +
                                          (long long)R * ((2 * z + ((q >> 2) & 1)) +
                                                          (long long)R * (2 * t + ((q >> 3) & 1))));
      s += dout[v * C + c];
    }
    dlo[e] = s;
  }
  const long long V = (long long)R * R * R * R;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < V * c2;
       e += (long long)gridDim.x * blockDim.x) {
    const long long v = e / c2;
    const int c = (int)(e % c2);
    dskip[e] += dout[v * C + c1 + c];
  }
}

// per-channel bias gradient: db[c] = sum_v d[v][c] (one block per channel)
__global__ void k_bias_grad(const float *__restrict__ d, float *__restrict__ db, long long V,
                            int C) {
  __shared__ double sh[8];
  const int c = blockIdx.x;
  double s = 0.0;
  for (long long v = threadIdx.x; v < V; v += blockDim.x) s += d[v * C + c];
  s = block_sum<256>(s, sh);
  if (threadIdx.x == 0) db[c] = (float)s;
}

// loss = mean (pred - target)^2 over n values; dpred = 2 (pred - target) / n
__global__ void k_mse(const float *__restrict__ pred, const float *__restrict__ target,
                      float *__restrict__ dpred, long long n, double *partial, unsigned *counter,
                      double *loss) {
  __shared__ double sh[8];
  double s = 0.0;
  const float inv = (float)(2.0 / (double)n);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float e = pred[q] - target[q];
    s += (double)e * e;
    if (dpred) dpred[q] = e * inv;
  }
  s = block_sum<256>(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (last_block_arrives(counter)) {
    double t = 0.0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) t += __ldcg(partial + q);
    t = block_sum<256>(t, sh);
    if (threadIdx.x == 0) {
      *loss += t / (double)n;
      *counter = 0;
    }
  }
}

// Adam on FP32 master weights, then the BF16-rounded working copy
__global__ void k_adam(float *__restrict__ w, float *__restrict__ wq, const float *__restrict__ gsum,
                       float *__restrict__ m, float *__restrict__ v, long long n, float lr,
                       float b1, float b2, float eps, float c1, float c2, float gscale) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float gr = gsum[q] * gscale;
    const float mm = b1 * m[q] + (1.f - b1) * gr;
    const float vv = b2 * v[q] + (1.f - b2) * gr * gr;
    m[q] = mm;
    v[q] = vv;
    const float upd = (mm / c1) / (sqrtf(vv / c2) + eps);
    const float nw = w[q] - lr * upd;
    w[q] = nw;
    wq[q] = __bfloat162float(__float2bfloat16_rn(nw));
  }
}

__global__ void k_round_bf16(const float *__restrict__ w, float *__restrict__ wq, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    wq[q] = __bfloat162float(__float2bfloat16_rn(w[q]));
}

// Network input from the coarse level: channels (i0, i1) scaled by `scale`
__global__ void k_net_input(const float *__restrict__ i0, const float *__restrict__ i1,
                            float *__restrict__ x, long long V, float scale) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
       v += (long long)gridDim.x * blockDim.x) {
    x[2 * v] = __ldg(i0 + v) * scale;
    x[2 * v + 1] = __ldg(i1 + v) * scale;
  }
}

__global__ void k_add_into(float *__restrict__ a, const float *__restrict__ b, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    a[q] += b[q];
}

}  // namespace

// ---- launchers --------------------------------------------------------------

static ConvGeom geom(int rin, int rout, int cin, int cout, int ks, int stride) {
  ConvGeom g;
  g.rin = rin;
  g.rout = rout;
  g.cin = cin;
  g.cout = cout;
  g.ks = ks;
  g.stride = stride;
  g.pad = ks == 3 ? 1 : 0;
  g.taps = ks == 3 ? 81 : 1;
  return g;
}

void net_conv_fwd(const float *in, const float *w, const float *b, float *out, int rin, int rout,
                  int cin, int cout, int ks, int stride, int relu, cudaStream_t s) {
  const ConvGeom g = geom(rin, rout, cin, cout, ks, stride);
  const int M = rout * rout * rout * rout, N = cout, K = g.taps * cin;
  dim3 grid((M + GT_M - 1) / GT_M, (N + GT_N - 1) / GT_N);
  k_conv_gemm<0><<<grid, GT_T, 0, s>>>(in, w, b, out, g, M, N, K, relu, K);
}

void net_conv_bwd_data(const float *dout, const float *w, float *din, int rin, int rout,
                       int cin, int cout, int ks, int stride, cudaStream_t s) {
  const ConvGeom g = geom(rin, rout, cin, cout, ks, stride);
  const int M = rin * rin * rin * rin, N = cin, K = g.taps * cout;
  dim3 grid((M + GT_M - 1) / GT_M, (N + GT_N - 1) / GT_N);
  k_conv_gemm<1><<<grid, GT_T, 0, s>>>(dout, w, nullptr, din, g, M, N, K, 0, K);
}

// The weight gradient reduces over all output voxels: the reduction is split
// into slices (about four blocks per SM in total) whose partial products go
// to `work` (slices x M x N floats) and are summed in slice order.
size_t net_conv_bwd_weight_work(int rout, int cin, int cout, int ks) {
  const int taps = ks == 3 ? 81 : 1;
  const long long M = (long long)taps * cin, N = cout, K = (long long)rout * rout * rout * rout;
  const long long tiles = ((M + GT_M - 1) / GT_M) * ((N + GT_N - 1) / GT_N);
  long long slices = (4LL * sm_count() + tiles - 1) / tiles;
  const long long maxs = (K + 255) / 256;
  if (slices > maxs) slices = maxs;
  if (slices < 1) slices = 1;
  return (size_t)(slices * M * N);
}

void net_conv_bwd_weight(const float *in, const float *dout, float *dw, float *work, int rin,
                         int rout, int cin, int cout, int ks, int stride, cudaStream_t s) {
  const ConvGeom g = geom(rin, rout, cin, cout, ks, stride);
  const int M = g.taps * cin, N = cout, K = rout * rout * rout * rout;
  const long long slices = (long long)net_conv_bwd_weight_work(rout, cin, cout, ks) / ((long long)M * N);
  int kslice = (int)((K + slices - 1) / slices);
  kslice = (kslice + GT_K - 1) / GT_K * GT_K;
  const int nz = (K + kslice - 1) / kslice;
  dim3 grid((M + GT_M - 1) / GT_M, (N + GT_N - 1) / GT_N, nz);
  k_conv_gemm<2><<<grid, GT_T, 0, s>>>(in, dout, nullptr, work, g, M, N, K, 0, kslice);
  const long long n = (long long)M * N;
  k_sum_slices<<<grid_for(n, 256), 256, 0, s>>>(work, dw, n, nz);
}

void net_relu_bwd(float *dy, const float *y, long long n, cudaStream_t s) {
  k_relu_bwd<<<grid_for(n, 256), 256, 0, s>>>(dy, y, n);
}
void net_upcat(const float *lo, const float *skip, float *out, int R, int c1, int c2,
               cudaStream_t s) {
  const long long n = (long long)R * R * R * R * (c1 + c2);
  k_upcat<<<grid_for(n, 256), 256, 0, s>>>(lo, skip, out, R, c1, c2);
}
void net_upcat_bwd(const float *dout, float *dlo, float *dskip, int R, int c1, int c2,
                   cudaStream_t s) {
  const long long n = (long long)R * R * R * R * (c1 + c2);
  k_upcat_bwd<<<grid_for(n, 256), 256, 0, s>>>(dout, dlo, dskip, R, c1, c2);
}
void net_bias_grad(const float *d, float *db, long long V, int C, cudaStream_t s) {
  k_bias_grad<<<C, 256, 0, s>>>(d, db, V, C);
}
void net_mse(const float *pred, const float *target, float *dpred, long long n, double *partial,
             unsigned *counter, double *loss, cudaStream_t s) {
  k_mse<<<grid_for(n, 256, 2), 256, 0, s>>>(pred, target, dpred, n, partial, counter, loss);
}
void net_adam(float *w, float *wq, const float *g, float *m, float *v, long long n, float lr,
              int step, float gscale, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<grid_for(n, 256), 256, 0, s>>>(w, wq, g, m, v, n, lr, b1, b2, eps, c1, c2, gscale);
}
void net_round_bf16(const float *w, float *wq, long long n, cudaStream_t s) {
  k_round_bf16<<<grid_for(n, 256), 256, 0, s>>>(w, wq, n);
}
void net_input(const float *i0, const float *i1, float *x, long long V, float scale,
               cudaStream_t s) {
  k_net_input<<<grid_for(V, 256), 256, 0, s>>>(i0, i1, x, V, scale);
}
void net_add_into(float *a, const float *b, long long n, cudaStream_t s) {
  k_add_into<<<grid_for(n, 256), 256, 0, s>>>(a, b, n);
}

}  // namespace flof
