// flof_mixed.cu -- the mixed-precision solve's own kernels.
//
// In mixed precision the PCG iterates on a matrix built from the image
// gradient stored in BF16 (8 bytes per cell instead of 16, read by all three
// PCG kernels), with FP32 vectors and float-float dot products.  Mixed-
// precision iterative refinement then restores the FP32 system: the
// residual r = b - A x of the FP32 matrix is formed with FP64 row sums, the
// BF16 solver solves for the correction, and x += e is added in FP64 before
// rounding.  The reference solves in one precision throughout
// (GridCGOptflow4d, optflow4d.cpp:268-355).
#include <cuda_bf16.h>
#include <float.h>

#include "flof_kernels.h"

namespace flof {

namespace {

constexpr int NT = 256;

__device__ __forceinline__ unsigned short bf16_bits(float v) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

__global__ void k_to_bf4(const float4 *__restrict__ g, BF4 *__restrict__ o, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float4 v = __ldg(g + q);
    BF4 b;
    b.x = bf16_bits(v.x);
    b.y = bf16_bits(v.y);
    b.z = bf16_bits(v.z);
    b.w = bf16_bits(v.w);
    o[q] = b;
  }
}

// r = b - A x, A the FP32 system (applyMat order, optflow4d.cpp:211-232),
// each row summed in FP64.  Also ||r||^2, ||b||^2 and the signed max of r.
__global__ void __launch_bounds__(NT)
k_residual64(const float4 *__restrict__ x, const float4 *__restrict__ b,
             const float4 *__restrict__ g, float4 *__restrict__ r, Dims4 d, BoxDecoder bx,
             uint32_t nint, OFConsts c, double *dpart, unsigned int *counter, double *res,
             float *fres) {
  __shared__ double shd[NT / 32];
  __shared__ float shf[NT / 32];
  double rr2 = 0.0, bb2 = 0.0;
  float mx = -FLT_MAX;
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  const double o = (double)c.offd;
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint;
       n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float4 xc = __ldg(x + id), gg = __ldg(g + id), bc = __ldg(b + id);
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if (c.offd != 0.f) {
      const idx_t off[8] = {-sT, -sZ, -sY, -1, 1, sY, sZ, sT};
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const float4 xn = __ldg(x + id + off[m]);
        v[0] += o * xn.x;
        v[1] += o * xn.y;
        v[2] += o * xn.z;
        v[3] += o * xn.w;
      }
    }
    const double gv[4] = {gg.x, gg.y, gg.z, gg.w};
    const double xv[4] = {xc.x, xc.y, xc.z, xc.w};
    const double bv[4] = {bc.x, bc.y, bc.z, bc.w};
    float rv[4];
#pragma unroll
    for (int dd = 0; dd < 4; ++dd) {
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        double a = gv[dd] * gv[m];
        if (dd == m) a += (double)c.diag;
        v[dd] += a * xv[m];
      }
      const double rd = bv[dd] - v[dd];
      rv[dd] = (float)rd;
      rr2 += rd * rd;
      bb2 += bv[dd] * bv[dd];
      mx = fmaxf(mx, rv[dd]);
    }
    r[id] = make_float4(rv[0], rv[1], rv[2], rv[3]);
  }
  const double s1 = block_sum<NT>(rr2, shd);
  const double s2 = block_sum<NT>(bb2, shd);
  const float bm = block_max<NT>(mx, shf);
  if (threadIdx.x == 0) {
    dpart[2 * blockIdx.x] = s1;
    dpart[2 * blockIdx.x + 1] = s2;
    ((float *)(dpart + 2 * gridDim.x))[blockIdx.x] = bm;
  }
  if (last_block_arrives(counter)) {
    double a = 0.0, bsum = 0.0;
    float m = 0.0f;  // border rows: r = 0
    for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
      a += __ldcg(dpart + 2 * q);
      bsum += __ldcg(dpart + 2 * q + 1);
      m = fmaxf(m, __ldcg((const float *)(dpart + 2 * gridDim.x) + q));
    }
    a = block_sum<NT>(a, shd);
    bsum = block_sum<NT>(bsum, shd);
    m = block_max<NT>(m, shf);
    if (threadIdx.x == 0) {
      res[0] = a;
      res[1] = bsum;
      fres[0] = m;
      *counter = 0;
    }
  }
}

// PCG start from residual r with x0 = 0 (x zeroed by the caller): p = z on
// the interior; the state logic of k_of_assemble_init.
template <class GT>
__global__ void __launch_bounds__(NT)
k_cg_init_r(const float4 *__restrict__ r, const GT *__restrict__ g, float4 *__restrict__ p,
            Dims4 d, BoxDecoder bx, uint32_t nint, OFConsts c, float accuracy, CGState *st,
            double *dpart, float *fpart) {
  __shared__ double shd[NT / 32];
  __shared__ FF shff[NT / 32];
  __shared__ float shf[NT / 32];
  FF dot = {0.f, 0.f};
  float mx = -FLT_MAX;
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint;
       n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float4 rr = __ldg(r + id), gg = ld_g(g, id);
    float4 pre;
    pre.x = __frcp_rn(gg.x * gg.x + c.diag);
    pre.y = __frcp_rn(gg.y * gg.y + c.diag);
    pre.z = __frcp_rn(gg.z * gg.z + c.diag);
    pre.w = __frcp_rn(gg.w * gg.w + c.diag);
    const float4 z = make_float4(rr.x * pre.x, rr.y * pre.y, rr.z * pre.z, rr.w * pre.w);
    p[id] = z;
    ff_add(dot, z.x * rr.x);
    ff_add(dot, z.y * rr.y);
    ff_add(dot, z.z * rr.z);
    ff_add(dot, z.w * rr.w);
    mx = fmaxf(mx, fmaxf(fmaxf(rr.x, rr.y), fmaxf(rr.z, rr.w)));
  }
  const double bd = block_sum_ff<NT>(dot, shff);
  const float bm = block_max<NT>(mx, shf);
  if (threadIdx.x == 0) {
    dpart[blockIdx.x] = bd;
    fpart[blockIdx.x] = bm;
  }
  if (last_block_arrives(&st->counter[0])) {
    double s = 0.0;
    float m = 0.0f;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
      s += __ldcg(dpart + q);
      m = fmaxf(m, __ldcg(fpart + q));
    }
    s = block_sum<NT>(s, shd);
    m = block_max<NT>(m, shf);
    if (threadIdx.x == 0) {
      const double residual = (double)m;
      st->resIni = residual;
      st->resMax = m;
      st->iters = 0;
      st->xpend = 0;
      st->counter[0] = 0;
      if (residual < (double)1e-6f) {
        st->retResidual = 0.f;
        st->done = CG_EARLY;
      } else {
        st->acc = (double)accuracy * residual;
        st->sigma = s;
        if (s == 0.0 || s != s) {
          st->retResidual = 1e10f;
          st->done = CG_FAILED_SIGMA;
        } else {
          st->retResidual = 1.0f;
          st->done = CG_RUNNING;
        }
      }
    }
  }
}

__global__ void k_add_correction(float4 *__restrict__ x, const float4 *__restrict__ e,
                                 long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float4 a = x[q], b = __ldg(e + q);
    x[q] = make_float4((float)((double)a.x + (double)b.x), (float)((double)a.y + (double)b.y),
                       (float)((double)a.z + (double)b.z), (float)((double)a.w + (double)b.w));
  }
}

BoxDecoder interior_decoder(Dims4 d) {
  return make_decoder(d.x - 2 > 0 ? d.x - 2 : 1, d.y - 2 > 0 ? d.y - 2 : 1,
                      d.z - 2 > 0 ? d.z - 2 : 1, 1, 1, 1, 1);
}
uint32_t interior_count(Dims4 d) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return 0;
  return (uint32_t)((long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2));
}

}  // namespace

void launch_to_bf4(const float4 *g, BF4 *g16, long long n, cudaStream_t s) {
  k_to_bf4<<<grid_for(n, NT), NT, 0, s>>>(g, g16, n);
}

void launch_residual64(const float4 *x, const float4 *b, const float4 *g, float4 *r, Dims4 d,
                       OFConsts c, double *dpart, unsigned int *counter, double *res,
                       float *fres, cudaStream_t s) {
  const uint32_t n = interior_count(d);
  // partials: 2 doubles + 1 float per block, within the 65536-double buffer
  k_residual64<<<grid_for(n > 0 ? n : 1, NT, 8), NT, 0, s>>>(
      x, b, g, r, d, interior_decoder(d), n, c, dpart, counter, res, fres);
}

void launch_cg_init_r(const float4 *r, const BF4 *g, float4 *p, Dims4 d, OFConsts c,
                      float accuracy, CGState *st, double *dpart, float *fpart, cudaStream_t s) {
  const uint32_t n = interior_count(d);
  k_cg_init_r<<<grid_for(n > 0 ? n : 1, NT, 8), NT, 0, s>>>(r, g, p, d, interior_decoder(d), n, c,
                                                           accuracy, st, dpart, fpart);
}
void launch_cg_init_r(const float4 *r, const float4 *g, float4 *p, Dims4 d, OFConsts c,
                      float accuracy, CGState *st, double *dpart, float *fpart, cudaStream_t s) {
  const uint32_t n = interior_count(d);
  k_cg_init_r<<<grid_for(n > 0 ? n : 1, NT, 8), NT, 0, s>>>(r, g, p, d, interior_decoder(d), n, c,
                                                           accuracy, st, dpart, fpart);
}

void launch_add_correction(float4 *x, const float4 *e, long long n, cudaStream_t s) {
  k_add_correction<<<grid_for(n, NT), NT, 0, s>>>(x, e, n);
}

}  // namespace flof
