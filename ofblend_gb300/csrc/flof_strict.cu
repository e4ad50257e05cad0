// flof_strict.cu -- the reference's PCG arithmetic, operation for operation,
// for parity runs (context option FLOF_OPT_STRICT).
//
// GridCGOptflow4d::solve (source/plugin/optflow4d.cpp:268-329) keeps its
// vectors in float and its scalars in double:
//   dotProd   (:234-241)  d += a[i] * b[i]: float products, one serial
//                         double sum over i = 4 * cell + component;
//   addScaled (:253-258)  a[i] += b * c[i] with a double b: a double product
//                         and a double sum, rounded once to float;
//   alpha = sigma / (p . A p) and beta = sigmaNew / sigma in double.
// The fast kernels (flof_solve.cu) use float alpha and beta, fused updates
// and parallel sums.  Here every update is a separate double multiply and
// add (__dmul_rn / __dadd_rn, never contracted) rounded once to float, and
// every dot product is summed by one thread in the reference's row order.
// Border rows contribute +0 products; adding +0 leaves a double sum that
// starts at +0 unchanged, so only interior rows are visited.  The error
// metric (calcLsDiffTempl, :895-927) is summed the same way, in its t, k, j,
// i loop order.
//
// A serial sum runs at the latency of one FP64 add per term, so this mode is
// for grids of a few million cells (parity checks), not for throughput.
#include <float.h>

#include "flof_kernels.h"

namespace flof {

namespace {

constexpr int SER_NT = 512;     // one summing warp, the rest stage terms
constexpr int SER_CHUNK = 4096; // terms per shared-memory stage (16 KB)
constexpr int ST_NT = 256;

// Serial double sum of the float terms term(0), term(1), ... in that order.
// Warp 0's first thread adds one staged chunk while the other warps compute
// the next chunk's terms into the second buffer; thread 0 then hands the sum
// to fin.
template <class Term, class Fin>
__global__ void __launch_bounds__(SER_NT)
k_serial_sum(Term term, long long nterms, Fin fin) {
  __shared__ float buf[2][SER_CHUNK];
  if (fin.skip()) return;
  const int tid = threadIdx.x;
  const long long nch = (nterms + SER_CHUNK - 1) / SER_CHUNK;
  auto stage = [&](long long c, float *b, int t0, int nt) {
    const long long base = c * SER_CHUNK;
    for (int e = t0; e < SER_CHUNK; e += nt) {
      const long long g = base + e;
      b[e] = g < nterms ? term(g) : 0.f;
    }
  };
  if (nch > 0) stage(0, buf[0], tid, SER_NT);
  __syncthreads();
  double s = 0.0;
  for (long long c = 0; c < nch; ++c) {
    if (tid == 0) {
      const float *b = buf[c & 1];
      const long long rem = nterms - c * SER_CHUNK;
      const int len = rem < SER_CHUNK ? (int)rem : SER_CHUNK;
      for (int e = 0; e < len; ++e) s = __dadd_rn(s, (double)b[e]);
    } else if (tid >= 32 && c + 1 < nch) {
      stage(c + 1, buf[(c + 1) & 1], tid - 32, SER_NT - 32);
    }
    __syncthreads();
  }
  if (tid == 0) fin(s);
}

// Jacobi preconditioner entry of row (cell, c): (float)(1. / diag) of the
// block diagonal g_c g_c + diag (optflow4d.cpp:331-342, :486-488).  Double
// rounding of the double quotient to float is innocuous for p = 24,
// q = 53 >= 2p + 2 (Figueroa), so this equals the correctly rounded
// float reciprocal.
__device__ __forceinline__ float pre_of(float g, float diag) {
  return __frcp_rn(__fadd_rn(__fmul_rn(g, g), diag));
}

// Term of dotProd(a, b) for row e = 4 * (interior cell) + component.
struct DotTerm {
  const float *a, *b;
  Dims4 d;
  BoxDecoder bx;
  __device__ __forceinline__ float operator()(long long e) const {
    int i, j, k, l;
    bx.decode((uint32_t)(e >> 2), i, j, k, l);
    const idx_t id = d.index(i, j, k, l) * 4 + (idx_t)(e & 3);
    return __fmul_rn(__ldg(a + id), __ldg(b + id));
  }
};
// Term of dotProd(tmp, res) with tmp = res * precond (precondApply, :344-352).
struct ZRTerm {
  const float *r, *g;
  Dims4 d;
  BoxDecoder bx;
  float diag;
  __device__ __forceinline__ float operator()(long long e) const {
    int i, j, k, l;
    bx.decode((uint32_t)(e >> 2), i, j, k, l);
    const idx_t id = d.index(i, j, k, l) * 4 + (idx_t)(e & 3);
    const float rr = __ldg(r + id);
    const float z = __fmul_rn(rr, pre_of(__ldg(g + id), diag));
    return __fmul_rn(z, rr);
  }
};

// After the assembly: sigma = z . r and the solve's start state
// (optflow4d.cpp:278-301).  The assembly kernel has set resIni, acc and an
// early exit for a tiny initial residual.
struct FinInit {
  CGState *st;
  __device__ bool skip() const { return st->done == CG_EARLY; }
  __device__ void operator()(double s) const {
    st->sigma = s;
    if (s == 0.0 || s != s) {
      st->retResidual = 1e10f;
      st->done = CG_FAILED_SIGMA;
    } else {
      st->retResidual = 1.0f;
      st->done = CG_RUNNING;
    }
  }
};
// After q = A p: alpha = sigma / (p . q) (:306-307).
struct FinAlpha {
  CGState *st;
  __device__ bool skip() const { return st->done != CG_RUNNING; }
  __device__ void operator()(double s) const {
    st->pAp = s;
    st->alpha = st->sigma / s;
  }
};
// After the residual update: beta = sigmaNew / sigma (:316-321).
struct FinBeta {
  CGState *st;
  __device__ bool skip() const { return st->done != CG_RUNNING; }
  __device__ void operator()(double s) const {
    st->beta = s / st->sigma;
    st->sigma = s;
  }
};

// x += alpha p; r += (-alpha) q, each a double product and sum rounded to
// float (:308-309); then the signed maximum of r (:310) and the stop rule
// (:311-315).  Border rows keep r = 0, which the maximum includes.
__global__ void __launch_bounds__(ST_NT)
k_strict_update(float4 *__restrict__ x, float4 *__restrict__ r, const float4 *__restrict__ p,
                const float4 *__restrict__ q, Dims4 d, BoxDecoder bx, uint32_t nint, CGState *st,
                float *fpart, int maxIter) {
  if (st->done != CG_RUNNING) return;
  __shared__ float shf[ST_NT / 32];
  const double a = st->alpha, na = -a;
  float mx = -FLT_MAX;
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint; n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float4 pp = __ldg(p + id), qq = __ldg(q + id);
    float4 xx = x[id], rr = r[id];
    xx.x = __double2float_rn(__dadd_rn((double)xx.x, __dmul_rn(a, (double)pp.x)));
    xx.y = __double2float_rn(__dadd_rn((double)xx.y, __dmul_rn(a, (double)pp.y)));
    xx.z = __double2float_rn(__dadd_rn((double)xx.z, __dmul_rn(a, (double)pp.z)));
    xx.w = __double2float_rn(__dadd_rn((double)xx.w, __dmul_rn(a, (double)pp.w)));
    rr.x = __double2float_rn(__dadd_rn((double)rr.x, __dmul_rn(na, (double)qq.x)));
    rr.y = __double2float_rn(__dadd_rn((double)rr.y, __dmul_rn(na, (double)qq.y)));
    rr.z = __double2float_rn(__dadd_rn((double)rr.z, __dmul_rn(na, (double)qq.z)));
    rr.w = __double2float_rn(__dadd_rn((double)rr.w, __dmul_rn(na, (double)qq.w)));
    x[id] = xx;
    r[id] = rr;
    mx = fmaxf(mx, fmaxf(fmaxf(rr.x, rr.y), fmaxf(rr.z, rr.w)));
  }
  const float bm = block_max<ST_NT>(mx, shf);
  if (threadIdx.x == 0) fpart[blockIdx.x] = bm;
  if (last_block_arrives(&st->counter[2])) {
    float m = 0.0f;  // border rows hold r = 0
    for (int q2 = threadIdx.x; q2 < (int)gridDim.x; q2 += blockDim.x) m = fmaxf(m, __ldcg(fpart + q2));
    m = block_max<ST_NT>(m, shf);
    if (threadIdx.x == 0) {
      const double residual = (double)m;
      const int iter = st->iters;
      st->resMax = m;
      st->retResidual = (float)(residual / st->resIni);
      st->iters = iter + 1;
      st->counter[2] = 0;
      if (residual <= st->acc)
        st->done = CG_CONVERGED;
      else if (iter + 1 >= maxIter)
        st->done = CG_MAXITER;
    }
  }
}

// p = tmp + beta p with tmp = r * precond (:316-320): a double product and
// sum rounded to float.
__global__ void __launch_bounds__(ST_NT)
k_strict_direction(float4 *__restrict__ p, const float4 *__restrict__ r,
                   const float4 *__restrict__ g, Dims4 d, BoxDecoder bx, uint32_t nint, float diag,
                   const CGState *st) {
  if (st->done != CG_RUNNING) return;
  const double b = st->beta;
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint; n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float4 rr = __ldg(r + id), gg = __ldg(g + id);
    float4 pp = p[id];
    const float zx = __fmul_rn(rr.x, pre_of(gg.x, diag));
    const float zy = __fmul_rn(rr.y, pre_of(gg.y, diag));
    const float zz = __fmul_rn(rr.z, pre_of(gg.z, diag));
    const float zw = __fmul_rn(rr.w, pre_of(gg.w, diag));
    pp.x = __double2float_rn(__dadd_rn((double)zx, __dmul_rn(b, (double)pp.x)));
    pp.y = __double2float_rn(__dadd_rn((double)zy, __dmul_rn(b, (double)pp.y)));
    pp.z = __double2float_rn(__dadd_rn((double)zz, __dmul_rn(b, (double)pp.z)));
    pp.w = __double2float_rn(__dadd_rn((double)zw, __dmul_rn(b, (double)pp.w)));
    p[id] = pp;
  }
}

// Term of calcLsDiffTempl in its loop order; also writes the per-cell value.
struct LsTerm {
  const float *i0, *i1;
  float *out;
  Dims4 d;
  BoxDecoder bx;
  float correction;
  __device__ __forceinline__ float operator()(long long e) const {
    int i, j, k, l;
    bx.decode((uint32_t)e, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float a = __ldg(i0 + id), b = __ldg(i1 + id);
    if ((a < 0.f && b < 0.f) || (a >= 0.f && b >= 0.f)) {
      if (out) out[id] = 0.f;
      return 0.f;  // the reference adds nothing here; +0 changes no sum
    }
    float dd = __fmul_rn(fabsf(__fsub_rn(a, b)), correction);
    if (dd > 1.f) dd = 1.f;
    if (out) out[id] = dd;
    return dd;
  }
};
struct FinLs {
  Dims4 d;
  double scale;
  double *result_d;
  float *result_f;
  __device__ bool skip() const { return false; }
  __device__ void operator()(double s) const {
    double accu = __dmul_rn(s, 1000.);
    if (d.t > 1) accu = __dmul_rn(accu, 1000.);
    accu = __dmul_rn(accu, scale);
    *result_d = accu;
    *result_f = (float)accu;
  }
};

inline BoxDecoder interior_box(Dims4 d) { return make_decoder(d.x - 2, d.y - 2, d.z - 2, 1, 1, 1, 1); }
inline long long interior_cells(Dims4 d) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return 0;
  return (long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2);
}

}  // namespace

void launch_strict_init(const float4 *r, const float4 *g, Dims4 d, OFConsts c, CGState *st,
                        cudaStream_t s) {
  ZRTerm t{(const float *)r, (const float *)g, d, interior_box(d), c.diag};
  k_serial_sum<<<1, SER_NT, 0, s>>>(t, 4 * interior_cells(d), FinInit{st});
}

void launch_strict_iteration(float4 *x, float4 *r, float4 *p, float4 *q, const float4 *g, Dims4 d,
                             OFConsts c, CGState *st, double *dpart, float *fpart, int maxIter,
                             cudaStream_t s) {
  const long long nint = interior_cells(d);
  const BoxDecoder bx = interior_box(d);
  // q = A p: the fast matvec's rows are the reference's applyMat bit for bit;
  // its parallel p.q and alpha are replaced by the serial ones below
  launch_cg_matvec(p, g, q, d, c, st, dpart, s);
  k_serial_sum<<<1, SER_NT, 0, s>>>(DotTerm{(const float *)p, (const float *)q, d, bx}, 4 * nint,
                                    FinAlpha{st});
  const int nb = grid_for(nint > 0 ? nint : 1, ST_NT, 4);
  k_strict_update<<<nb, ST_NT, 0, s>>>(x, r, p, q, d, bx, (uint32_t)nint, st, fpart, maxIter);
  k_serial_sum<<<1, SER_NT, 0, s>>>(ZRTerm{(const float *)r, (const float *)g, d, bx, c.diag},
                                    4 * nint, FinBeta{st});
  k_strict_direction<<<nb, ST_NT, 0, s>>>(p, r, g, d, bx, (uint32_t)nint, c.diag, st);
}

void launch_strict_ls_diff(const float *i0, const float *i1, float *out, Dims4 d, float correction,
                           int bnd, double *result_d, float *result_f, cudaStream_t s) {
  const int ex = d.x - 2 * bnd, ey = d.y - 2 * bnd, ez = d.z - 2 * bnd, et = d.t - 2 * bnd;
  const bool empty = ex <= 0 || ey <= 0 || ez <= 0 || et <= 0;
  const long long nbox = empty ? 0 : (long long)ex * ey * ez * et;
  const BoxDecoder bx = make_decoder(empty ? 1 : ex, empty ? 1 : ey, empty ? 1 : ez, bnd, bnd, bnd,
                                     bnd);
  const double scale = 1. / (double)(ex * ey * ez * et);
  k_serial_sum<<<1, SER_NT, 0, s>>>(LsTerm{i0, i1, out, d, bx, correction}, nbox,
                                    FinLs{d, scale, result_d, result_f});
}

}  // namespace flof
