// flof_mg.cu -- multigrid-preconditioned PCG for the optical-flow system of
// one pyramid level (the learned solve mode's solver; no reference
// counterpart).
//
// The system is the reference's (opticalFlowDim, optflow4d.cpp:398-493):
// per interior cell a 4x4 block g g^T + c0 I (c0 = 8 wSmooth + wEnergy) and
// -wSmooth to each of the 8 neighbours, border rows identity.  The plain
// solver preconditions it with the diagonal (Jacobi, :331-355); its
// iteration count grows with the grid because the smoothness term is a 4D
// Laplacian.  Here a V-cycle over an aggregation hierarchy preconditions the
// same CG:
//   level 0  the system itself over the interior cells;
//   level l  one unknown (4 components) per 2^4 aggregate of level l-1,
//            Dirichlet outside;  restriction = sum over the aggregate,
//            prolongation = injection;  the coarse operator is the Galerkin
//            product P^T A P with its Laplacian part scaled by lambda per
//            level (lambda = 1/2 gives the rediscretised Laplacian):
//              block_K = sum_C G_C + lapdiag_K I,
//              A[K][K +- e_a] = -c_a,
//            kept as G (the summed g g^T + wEnergy blocks, 10 floats),
//            lapdiag and the couplings c_a to the +a neighbours;
//   smoother damped block Jacobi (the 4x4 block inverted: Sherman-Morrison
//            on level 0, Cholesky on the coarse levels), one sweep before
//            and one after the coarse correction, so the V-cycle is a fixed
//            symmetric linear operator and plain PCG applies;
//   coarsest a fixed number of damped block-Jacobi sweeps in one block.
// The damping factors and lambda are the tuned parameters (MGParams).
//
// Every kernel returns at once when the PCG state says the solve is done, so
// the host can queue iterations in chunks as the plain PCG does.  All sums
// are formed in a fixed order: results repeat bit for bit.
#include <float.h>

#include <utility>

#include "flof_kernels.h"

namespace flof {

namespace {

constexpr int MT = 256;

struct Sym4 {
  float a00, a01, a02, a03, a11, a12, a13, a22, a23, a33;
};

// Storage of a coarse cell's block: three float4, (a00 a01 a02 a03)
// (a11 a12 a13 a22) (a23 a33 lapdiag 0); the same layout holds the inverse.
__device__ __forceinline__ Sym4 sym_load(const float4 *s, idx_t i, float &lap) {
  const float4 u = __ldg(s + 3 * i), v = __ldg(s + 3 * i + 1), w = __ldg(s + 3 * i + 2);
  lap = w.z;
  return Sym4{u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w, w.x, w.y};
}
__device__ __forceinline__ void sym_store(float4 *s, idx_t i, const Sym4 &a, float lap) {
  s[3 * i] = make_float4(a.a00, a.a01, a.a02, a.a03);
  s[3 * i + 1] = make_float4(a.a11, a.a12, a.a13, a.a22);
  s[3 * i + 2] = make_float4(a.a23, a.a33, lap, 0.f);
}
__device__ __forceinline__ float4 sym_mul(const Sym4 &a, float4 x) {
  return make_float4(a.a00 * x.x + a.a01 * x.y + a.a02 * x.z + a.a03 * x.w,
                     a.a01 * x.x + a.a11 * x.y + a.a12 * x.z + a.a13 * x.w,
                     a.a02 * x.x + a.a12 * x.y + a.a22 * x.z + a.a23 * x.w,
                     a.a03 * x.x + a.a13 * x.y + a.a23 * x.z + a.a33 * x.w);
}
// Inverse of a symmetric positive definite 4x4 block by Cholesky: A = L L^T,
// A^-1 = L^-T L^-1.
__device__ __forceinline__ Sym4 sym_inv(const Sym4 &a) {
  const float l00 = sqrtf(a.a00);
  const float l10 = a.a01 / l00, l20 = a.a02 / l00, l30 = a.a03 / l00;
  const float l11 = sqrtf(a.a11 - l10 * l10);
  const float l21 = (a.a12 - l20 * l10) / l11, l31 = (a.a13 - l30 * l10) / l11;
  const float l22 = sqrtf(a.a22 - l20 * l20 - l21 * l21);
  const float l32 = (a.a23 - l30 * l20 - l31 * l21) / l22;
  const float l33 = sqrtf(a.a33 - l30 * l30 - l31 * l31 - l32 * l32);
  // M = L^-1 (lower triangular)
  const float m00 = 1.f / l00, m11 = 1.f / l11, m22 = 1.f / l22, m33 = 1.f / l33;
  const float m10 = -l10 * m00 * m11;
  const float m21 = -l21 * m11 * m22;
  const float m20 = -(l20 * m00 + l21 * m10) * m22;
  const float m32 = -l32 * m22 * m33;
  const float m31 = -(l31 * m11 + l32 * m21) * m33;
  const float m30 = -(l30 * m00 + l31 * m10 + l32 * m20) * m33;
  // (M^T M)_ij = sum_{k >= max(i,j)} m_ki m_kj
  Sym4 r;
  r.a00 = m00 * m00 + m10 * m10 + m20 * m20 + m30 * m30;
  r.a01 = m11 * m10 + m21 * m20 + m31 * m30;
  r.a02 = m22 * m20 + m32 * m30;
  r.a03 = m33 * m30;
  r.a11 = m11 * m11 + m21 * m21 + m31 * m31;
  r.a12 = m22 * m21 + m32 * m31;
  r.a13 = m33 * m31;
  r.a22 = m22 * m22 + m32 * m32;
  r.a23 = m33 * m32;
  r.a33 = m33 * m33;
  return r;
}
__device__ __forceinline__ float4 f4_add(float4 a, float4 b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 f4_sub(float4 a, float4 b) {
  return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__device__ __forceinline__ float4 f4_scale(float s, float4 a) {
  return make_float4(s * a.x, s * a.y, s * a.z, s * a.w);
}
__device__ __forceinline__ float4 f4_axpy(float s, float4 x, float4 y) {  // y + s x
  return make_float4(y.x + s * x.x, y.y + s * x.y, y.z + s * x.z, y.w + s * x.w);
}
__device__ __forceinline__ float f4_dot(float4 a, float4 b) {
  return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}

// Level-0 block (g g^T + c0 I): product and inverse (Sherman-Morrison).
__device__ __forceinline__ float4 blk0_mul(float4 g, float c0, float4 x) {
  return f4_axpy(f4_dot(g, x), g, f4_scale(c0, x));
}
__device__ __forceinline__ float4 blk0_solve(float4 g, float c0, float4 v) {
  const float s = f4_dot(g, v) / (c0 + f4_dot(g, g));
  return f4_scale(1.f / c0, f4_axpy(-s, g, v));
}

__device__ __forceinline__ bool mg_stop(const CGState *st) { return st->done != CG_RUNNING; }

// ---------------------------------------------------------------------------
// hierarchy set-up
// ---------------------------------------------------------------------------

// Level 1 from the level-0 gradient.  Aggregate K holds the interior cells
// f = 1 + 2K + delta (delta in {0,1}^4, f <= X-2).  G_K = sum (g g^T + wE I);
// lapdiag = lambda wS (edges from the aggregate's cells to cells outside
// it); c_a = lambda wS (edges from the +a face to interior cells of K+e_a).
__global__ void __launch_bounds__(MT)
k_mg_build1(const float4 *__restrict__ g, Dims4 d, Dims4 m, float4 *__restrict__ G,
            float4 *__restrict__ cpl, float4 *__restrict__ dinv, float wS, float wE, float lambda,
            const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (st->done == CG_EARLY) return;
  const int lim[4] = {d.x - 2, d.y - 2, d.z - 2, d.t - 2};  // last interior index
  const uint32_t n = (uint32_t)m.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int K[4];
    uint32_t rest = q;
    K[0] = rest % m.x; rest /= m.x;
    K[1] = rest % m.y; rest /= m.y;
    K[2] = rest % m.z; K[3] = rest / m.z;
    int two[4];  // 1: the aggregate has both children along the axis
#pragma unroll
    for (int a = 0; a < 4; ++a) two[a] = (2 + 2 * K[a] <= lim[a]) ? 1 : 0;
    Sym4 S = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    float out_edges = 0.f;
    float ca[4] = {0.f, 0.f, 0.f, 0.f};
    int cnt = 0;
    for (int dl = 0; dl <= two[3]; ++dl)
      for (int dk = 0; dk <= two[2]; ++dk)
        for (int dj = 0; dj <= two[1]; ++dj)
          for (int di = 0; di <= two[0]; ++di) {
            const int f[4] = {1 + 2 * K[0] + di, 1 + 2 * K[1] + dj, 1 + 2 * K[2] + dk,
                              1 + 2 * K[3] + dl};
            const int dlt[4] = {di, dj, dk, dl};
            const float4 gg = __ldg(g + d.index(f[0], f[1], f[2], f[3]));
            S.a00 += gg.x * gg.x; S.a01 += gg.x * gg.y; S.a02 += gg.x * gg.z; S.a03 += gg.x * gg.w;
            S.a11 += gg.y * gg.y; S.a12 += gg.y * gg.z; S.a13 += gg.y * gg.w;
            S.a22 += gg.z * gg.z; S.a23 += gg.z * gg.w; S.a33 += gg.w * gg.w;
            ++cnt;
            int inside = 0;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
              if (two[a]) inside += 1;  // the sibling along a is in the aggregate
              // on the +a face: a neighbour in K + e_a if it is interior
              const bool face = (dlt[a] == 1) || !two[a];
              if (face && f[a] + 1 <= lim[a]) ca[a] += 1.f;
            }
            out_edges += (float)(8 - inside);
          }
    const float wEn = wE * (float)cnt;
    S.a00 += wEn; S.a11 += wEn; S.a22 += wEn; S.a33 += wEn;
    const float lap = lambda * wS * out_edges;
    sym_store(G, q, S, lap);
    cpl[q] = make_float4(lambda * wS * ca[0], lambda * wS * ca[1], lambda * wS * ca[2],
                         lambda * wS * ca[3]);
    Sym4 D = S;
    D.a00 += lap; D.a11 += lap; D.a22 += lap; D.a33 += lap;
    sym_store(dinv, q, sym_inv(D), 0.f);
  }
}

// Level l from level l-1 (dims mp): aggregate K holds C = 2K + delta.
__global__ void __launch_bounds__(MT)
k_mg_build(const float4 *__restrict__ Gp, const float4 *__restrict__ cp, Dims4 mp, Dims4 m,
           float4 *__restrict__ G, float4 *__restrict__ cpl, float4 *__restrict__ dinv,
           float lambda, const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (st->done == CG_EARLY) return;
  const int ext[4] = {mp.x, mp.y, mp.z, mp.t};
  const uint32_t n = (uint32_t)m.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int K[4];
    uint32_t rest = q;
    K[0] = rest % m.x; rest /= m.x;
    K[1] = rest % m.y; rest /= m.y;
    K[2] = rest % m.z; K[3] = rest / m.z;
    int two[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) two[a] = (2 * K[a] + 1 < ext[a]) ? 1 : 0;
    Sym4 S = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    float lapsum = 0.f, internal = 0.f;
    float ca[4] = {0.f, 0.f, 0.f, 0.f};
    for (int dl = 0; dl <= two[3]; ++dl)
      for (int dk = 0; dk <= two[2]; ++dk)
        for (int dj = 0; dj <= two[1]; ++dj)
          for (int di = 0; di <= two[0]; ++di) {
            const int C[4] = {2 * K[0] + di, 2 * K[1] + dj, 2 * K[2] + dk, 2 * K[3] + dl};
            const int dlt[4] = {di, dj, dk, dl};
            const idx_t ci = mp.index(C[0], C[1], C[2], C[3]);
            float lp;
            const Sym4 c = sym_load(Gp, ci, lp);
            S.a00 += c.a00; S.a01 += c.a01; S.a02 += c.a02; S.a03 += c.a03;
            S.a11 += c.a11; S.a12 += c.a12; S.a13 += c.a13;
            S.a22 += c.a22; S.a23 += c.a23; S.a33 += c.a33;
            lapsum += lp;
            const float4 cc = __ldg(cp + ci);
            const float cv[4] = {cc.x, cc.y, cc.z, cc.w};
#pragma unroll
            for (int a = 0; a < 4; ++a) {
              if (dlt[a] == 0 && two[a]) internal += cv[a];  // edge to the sibling
              else ca[a] += cv[a];                          // edge leaving along +a
            }
          }
    const float lap = lambda * (lapsum - 2.f * internal);
    sym_store(G, q, S, lap);
    cpl[q] = make_float4(lambda * ca[0], lambda * ca[1], lambda * ca[2], lambda * ca[3]);
    Sym4 D = S;
    D.a00 += lap; D.a11 += lap; D.a22 += lap; D.a33 += lap;
    sym_store(dinv, q, sym_inv(D), 0.f);
  }
}

// ---------------------------------------------------------------------------
// level 0 (the system's own grid, interior cells)
// ---------------------------------------------------------------------------

// x = omega D^-1 b
__global__ void __launch_bounds__(MT)
k_mg0_pre(const float4 *__restrict__ b, const float4 *__restrict__ g, float4 *__restrict__ x,
          Dims4 d, BoxDecoder bx, uint32_t nint, float c0, float omega, const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint; n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    x[id] = f4_scale(omega, blk0_solve(__ldg(g + id), c0, __ldg(b + id)));
  }
}

// (A x) at one interior cell: block times x minus wS times the neighbours
// (border cells of x hold zero).
__device__ __forceinline__ float4 a0_mul(const float4 *__restrict__ x, float4 gg, idx_t id,
                                         idx_t sY, idx_t sZ, idx_t sT, float c0, float wS) {
  const float4 xc = __ldg(x + id);
  float4 nb = __ldg(x + id - sT);
  nb = f4_add(nb, __ldg(x + id - sZ));
  nb = f4_add(nb, __ldg(x + id - sY));
  nb = f4_add(nb, __ldg(x + id - 1));
  nb = f4_add(nb, __ldg(x + id + 1));
  nb = f4_add(nb, __ldg(x + id + sY));
  nb = f4_add(nb, __ldg(x + id + sZ));
  nb = f4_add(nb, __ldg(x + id + sT));
  return f4_axpy(-wS, nb, blk0_mul(gg, c0, xc));
}

// x0 + e1[parent] at interior cell (i,j,k,l) of level 0.
__device__ __forceinline__ float4 xp_at(const float4 *__restrict__ x, const float4 *__restrict__ e1,
                                        const Dims4 &d, const Dims4 &m, idx_t id, int i, int j,
                                        int k, int l) {
  return f4_add(__ldg(x + id),
                __ldg(e1 + m.index((i - 1) >> 1, (j - 1) >> 1, (k - 1) >> 1, (l - 1) >> 1)));
}

// The level-0 prolongation x += e1[parent] over the interior cells.
__global__ void __launch_bounds__(MT)
k_mg0_prolong(float4 *__restrict__ x, const float4 *__restrict__ e1, Dims4 d, BoxDecoder bx,
              uint32_t nint, Dims4 m, const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint; n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    x[id] = f4_add(x[id],
                   __ldg(e1 + m.index((i - 1) >> 1, (j - 1) >> 1, (k - 1) >> 1, (l - 1) >> 1)));
  }
}

// The last level-0 sweep, z = y + omega D^-1 (b - A y) with y the prolonged
// iterate (border cells zero), one thread per interior (x, y, z) column
// walking MG_TT consecutive t planes with y at t-1, t, t+1 in registers (the
// t neighbours cost no load); z . b for the PCG: init sets sigma (and
// beta = 0), otherwise beta = z.b / sigma and sigma = z.b.
constexpr int MG_TT = 8;
__global__ void __launch_bounds__(MT)
k_mg0_post_tw(const float4 *__restrict__ b, const float4 *__restrict__ g,
              const float4 *__restrict__ y, float4 *__restrict__ z, Dims4 d, BoxDecoder bxyz,
              uint32_t nxyz, int tchunks, float c0, float wS, float omega, CGState *st,
              double *dpart, int init) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  __shared__ double shd[MT / 32];
  __shared__ FF shff[MT / 32];
  FF dot = {0.f, 0.f};
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  const uint32_t n = nxyz * (uint32_t)tchunks;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const uint32_t cell = q % nxyz, tc = q / nxyz;
    int i, j, k, unused;
    bxyz.decode(cell, i, j, k, unused);
    const int l0 = 1 + (int)tc * MG_TT;
    const int l1 = min(l0 + MG_TT, d.t - 1);
    idx_t id = d.index(i, j, k, l0);
    // border cells of y hold zero, so the neighbour loads need no guards
    float4 ym = __ldg(y + id - sT), yc = __ldg(y + id);
    for (int l = l0; l < l1; ++l, id += sT) {
      const float4 yp = __ldg(y + id + sT);
      float4 nb = f4_add(ym, __ldg(y + id - sZ));
      nb = f4_add(nb, __ldg(y + id - sY));
      nb = f4_add(nb, __ldg(y + id - 1));
      nb = f4_add(nb, __ldg(y + id + 1));
      nb = f4_add(nb, __ldg(y + id + sY));
      nb = f4_add(nb, __ldg(y + id + sZ));
      nb = f4_add(nb, yp);
      const float4 gg = __ldg(g + id), bb = __ldg(b + id);
      const float4 res = f4_sub(bb, f4_axpy(-wS, nb, blk0_mul(gg, c0, yc)));
      const float4 zz = f4_axpy(omega, blk0_solve(gg, c0, res), yc);
      z[id] = zz;
      ff_add(dot, zz.x * bb.x);
      ff_add(dot, zz.y * bb.y);
      ff_add(dot, zz.z * bb.z);
      ff_add(dot, zz.w * bb.w);
      ym = yc;
      yc = yp;
    }
  }
  const double bd = block_sum_ff<MT>(dot, shff);
  if (threadIdx.x == 0) dpart[blockIdx.x] = bd;
  if (last_block_arrives(&st->counter[3])) {
    double s = 0.0;
    for (int q2 = threadIdx.x; q2 < (int)gridDim.x; q2 += blockDim.x) s += __ldcg(dpart + q2);
    s = block_sum<MT>(s, shd);
    if (threadIdx.x == 0) {
      st->counter[3] = 0;
      if (init) {
        st->sigma = s;
        st->beta = 0.0;
        st->betaf = 0.f;
        if (s == 0.0 || s != s) {
          st->retResidual = 1e10f;
          st->done = CG_FAILED_SIGMA;
        }
      } else {
        st->beta = s / st->sigma;
        st->betaf = (float)st->beta;
        st->sigma = s;
      }
    }
  }
}

// The level-0 residual with the restriction folded in, walking t.  A block
// is 4 warps: warp w covers the 32 interior cells x = 1 + 32 bx .. 32 + 32 bx
// of the row (y, z) = 1 + 2 (by, bz) + (w & 1, w >> 1) and walks the RR_TP
// aggregate t pairs of its chunk, with x at t-1, t and t+1 in registers (the
// t neighbours cost no load).  For each t pair, lanes 2a and 2a+1 add their
// residuals; then each of the 16 aggregates adds the 4 warps' pair sums of
// the pair's first plane and then of its second, in warp order: b1 of the 16
// aggregates, with no level-0 residual written.  The sums and their order
// are those of one cell per thread with warp (y & 1) + 2 (z & 1) + 4 (t & 1).
constexpr int RR_NT = 128, RR_TP = 4;
__global__ void __launch_bounds__(RR_NT)
k_mg0_resid_restrict(const float4 *__restrict__ b, const float4 *__restrict__ g,
                     const float4 *__restrict__ x, float4 *__restrict__ b1, Dims4 d, Dims4 m,
                     int nbx, float c0, float wS, const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  __shared__ float4 part[2][2][4][16];  // [pair parity][plane of the pair][warp][aggregate]
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int bxi = blockIdx.x % nbx, rest = blockIdx.x / nbx;
  const int by = rest % m.y, rest2 = rest / m.y;
  const int bz = rest2 % m.z, btc = rest2 / m.z;
  const int i = 1 + 32 * bxi + lane, j = 1 + 2 * by + (w & 1), k = 1 + 2 * bz + (w >> 1);
  const bool live = i <= d.x - 2 && j <= d.y - 2 && k <= d.z - 2;
  const int bt0 = btc * RR_TP, bt1 = min(bt0 + RR_TP, m.t);
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  // border cells of x hold zero, so the neighbour loads need no guards
  idx_t id = live ? d.index(i, j, k, 1 + 2 * bt0) : 0;
  float4 xm = live ? __ldg(x + id - sT) : zero4, xc = live ? __ldg(x + id) : zero4;
  for (int bt = bt0; bt < bt1; ++bt) {
    float4 r[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      r[h] = zero4;
      if (live && 1 + 2 * bt + h <= d.t - 2) {
        const float4 xp = __ldg(x + id + sT);
        float4 nb = f4_add(xm, __ldg(x + id - sZ));
        nb = f4_add(nb, __ldg(x + id - sY));
        nb = f4_add(nb, __ldg(x + id - 1));
        nb = f4_add(nb, __ldg(x + id + 1));
        nb = f4_add(nb, __ldg(x + id + sY));
        nb = f4_add(nb, __ldg(x + id + sZ));
        nb = f4_add(nb, xp);
        r[h] = f4_sub(__ldg(b + id), f4_axpy(-wS, nb, blk0_mul(__ldg(g + id), c0, xc)));
        xm = xc;
        xc = xp;
        id += sT;
      }
      r[h].x += __shfl_down_sync(0xffffffffu, r[h].x, 1);
      r[h].y += __shfl_down_sync(0xffffffffu, r[h].y, 1);
      r[h].z += __shfl_down_sync(0xffffffffu, r[h].z, 1);
      r[h].w += __shfl_down_sync(0xffffffffu, r[h].w, 1);
      if ((lane & 1) == 0) part[bt & 1][h][w][lane >> 1] = r[h];
    }
    // part[bt & 1] was last read before the barrier of pair bt - 1
    __syncthreads();
    if (threadIdx.x < 16) {
      const int K0 = 16 * bxi + threadIdx.x;
      if (K0 < m.x) {
        float4 s = part[bt & 1][0][0][threadIdx.x];
#pragma unroll
        for (int q = 1; q < 8; ++q) s = f4_add(s, part[bt & 1][q >> 2][q & 3][threadIdx.x]);
        b1[m.index(K0, by, bz, bt)] = s;
      }
    }
  }
}

// z = x + omega D^-1 (b - A x); z . b summed for the PCG (b is its residual).
// init: sigma = z.r and beta = 0; else beta = z.r / sigma, sigma = z.r.
__global__ void __launch_bounds__(MT)
k_mg0_post(const float4 *__restrict__ b, const float4 *__restrict__ g,
           const float4 *__restrict__ x, float4 *__restrict__ z, Dims4 d, BoxDecoder bx,
           uint32_t nint, float c0, float wS, float omega, CGState *st, double *dpart, int init) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  __shared__ double shd[MT / 32];
  __shared__ FF shff[MT / 32];
  FF dot = {0.f, 0.f};
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint; n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float4 gg = __ldg(g + id), bb = __ldg(b + id);
    const float4 res = f4_sub(bb, a0_mul(x, gg, id, sY, sZ, sT, c0, wS));
    const float4 zz = f4_axpy(omega, blk0_solve(gg, c0, res), __ldg(x + id));
    z[id] = zz;
    ff_add(dot, zz.x * bb.x);
    ff_add(dot, zz.y * bb.y);
    ff_add(dot, zz.z * bb.z);
    ff_add(dot, zz.w * bb.w);
  }
  const double bd = block_sum_ff<MT>(dot, shff);
  if (threadIdx.x == 0) dpart[blockIdx.x] = bd;
  if (last_block_arrives(&st->counter[3])) {
    double s = 0.0;
    for (int q2 = threadIdx.x; q2 < (int)gridDim.x; q2 += blockDim.x) s += __ldcg(dpart + q2);
    s = block_sum<MT>(s, shd);
    if (threadIdx.x == 0) {
      st->counter[3] = 0;
      if (init) {
        st->sigma = s;
        st->beta = 0.0;
        st->betaf = 0.f;
        if (s == 0.0 || s != s) {
          st->retResidual = 1e10f;
          st->done = CG_FAILED_SIGMA;
        }
      } else {
        st->beta = s / st->sigma;
        st->betaf = (float)st->beta;
        st->sigma = s;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// coarse levels (dense grids m, Dirichlet outside)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void decode_dense(uint32_t q, const Dims4 &m, int (&K)[4]) {
  uint32_t rest = q;
  K[0] = rest % m.x; rest /= m.x;
  K[1] = rest % m.y; rest /= m.y;
  K[2] = rest % m.z; K[3] = rest / m.z;
}

// (A x)_K = (G_K + lapdiag I) x_K - sum_a c_a(K) x_{K+e_a} + c_a(K-e_a) x_{K-e_a}
__device__ __forceinline__ float4 ac_mul(const float4 *__restrict__ G, const float4 *__restrict__ cpl,
                                         const float4 *__restrict__ x, const Dims4 &m,
                                         const int (&K)[4], idx_t id) {
  float lap;
  const Sym4 S = sym_load(G, id, lap);
  const float4 xc = __ldg(x + id);
  float4 y = f4_axpy(lap, xc, sym_mul(S, xc));
  const float4 c = __ldg(cpl + id);
  const idx_t str[4] = {1, m.x, m.sz(), m.st()};
  const int ext[4] = {m.x, m.y, m.z, m.t};
  const float cv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    if (K[a] + 1 < ext[a]) y = f4_axpy(-cv[a], __ldg(x + id + str[a]), y);
    if (K[a] > 0) {
      const float4 cm = __ldg(cpl + id - str[a]);
      const float cmv = a == 0 ? cm.x : a == 1 ? cm.y : a == 2 ? cm.z : cm.w;
      y = f4_axpy(-cmv, __ldg(x + id - str[a]), y);
    }
  }
  return y;
}
__device__ __forceinline__ float4 dinv_mul(const float4 *__restrict__ dinv, idx_t id, float4 v) {
  float unused;
  return sym_mul(sym_load(dinv, id, unused), v);
}

__global__ void __launch_bounds__(MT)
k_mgc_pre(const float4 *__restrict__ b, const float4 *__restrict__ dinv, float4 *__restrict__ x,
          uint32_t n, float omega, const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    x[q] = f4_scale(omega, dinv_mul(dinv, q, __ldg(b + q)));
}

__global__ void __launch_bounds__(MT)
k_mgc_resid(const float4 *__restrict__ b, const float4 *__restrict__ G,
            const float4 *__restrict__ cpl, const float4 *__restrict__ x, float4 *__restrict__ r,
            Dims4 m, const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  const uint32_t n = (uint32_t)m.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int K[4];
    decode_dense(q, m, K);
    r[q] = f4_sub(__ldg(b + q), ac_mul(G, cpl, x, m, K, q));
  }
}

__global__ void __launch_bounds__(MT)
k_mgc_restrict(const float4 *__restrict__ r, float4 *__restrict__ bn, Dims4 m, Dims4 mn,
               const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  const uint32_t n = (uint32_t)mn.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int K[4];
    decode_dense(q, mn, K);
    const int e0 = 2 * K[0] + 1 < m.x, e1 = 2 * K[1] + 1 < m.y;
    const int e2 = 2 * K[2] + 1 < m.z, e3 = 2 * K[3] + 1 < m.t;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int dl = 0; dl <= e3; ++dl)
      for (int dk = 0; dk <= e2; ++dk)
        for (int dj = 0; dj <= e1; ++dj)
          for (int di = 0; di <= e0; ++di)
            s = f4_add(s, __ldg(r + m.index(2 * K[0] + di, 2 * K[1] + dj, 2 * K[2] + dk,
                                             2 * K[3] + dl)));
    bn[q] = s;
  }
}

__global__ void __launch_bounds__(MT)
k_mgc_prolong(float4 *__restrict__ x, const float4 *__restrict__ e, Dims4 m, Dims4 mn,
              const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  const uint32_t n = (uint32_t)m.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int K[4];
    decode_dense(q, m, K);
    x[q] = f4_add(x[q], __ldg(e + mn.index(K[0] >> 1, K[1] >> 1, K[2] >> 1, K[3] >> 1)));
  }
}

// xo = x + omega D^-1 (b - A x)
__global__ void __launch_bounds__(MT)
k_mgc_post(const float4 *__restrict__ b, const float4 *__restrict__ G,
           const float4 *__restrict__ cpl, const float4 *__restrict__ dinv,
           const float4 *__restrict__ x, float4 *__restrict__ xo, Dims4 m, float omega,
           const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  const uint32_t n = (uint32_t)m.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int K[4];
    decode_dense(q, m, K);
    const float4 res = f4_sub(__ldg(b + q), ac_mul(G, cpl, x, m, K, q));
    xo[q] = f4_axpy(omega, dinv_mul(dinv, q, res), __ldg(x + q));
  }
}

// The coarsest level: `sweeps` damped block-Jacobi sweeps from zero, in one
// block of up to MG_COARSEST cells, with x in shared memory.
constexpr int MG_COARSEST = 1024;
__global__ void __launch_bounds__(MG_COARSEST)
k_mgc_coarsest(const float4 *__restrict__ b, const float4 *__restrict__ G,
               const float4 *__restrict__ cpl, const float4 *__restrict__ dinv,
               float4 *__restrict__ xout, Dims4 m, float omega, int sweeps, const CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  __shared__ float4 xs[2][MG_COARSEST];
  const int n = (int)m.cells();
  const int q = threadIdx.x;
  int K[4] = {0, 0, 0, 0};
  float lap = 0.f;
  Sym4 S = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, Di = S;
  float4 bb = make_float4(0.f, 0.f, 0.f, 0.f), c = bb;
  float cm[4] = {0.f, 0.f, 0.f, 0.f};
  const int str[4] = {1, m.x, m.x * m.y, m.x * m.y * m.z};
  const int ext[4] = {m.x, m.y, m.z, m.t};
  if (q < n) {
    decode_dense((uint32_t)q, m, K);
    S = sym_load(G, q, lap);
    float unused;
    Di = sym_load(dinv, q, unused);
    bb = __ldg(b + q);
    c = __ldg(cpl + q);
#pragma unroll
    for (int a = 0; a < 4; ++a)
      if (K[a] > 0) {
        const float4 t = __ldg(cpl + q - str[a]);
        cm[a] = a == 0 ? t.x : a == 1 ? t.y : a == 2 ? t.z : t.w;
      }
    xs[0][q] = f4_scale(omega, sym_mul(Di, bb));
  }
  __syncthreads();
  const float cv[4] = {c.x, c.y, c.z, c.w};
  int cur = 0;
  for (int s = 1; s < sweeps; ++s) {
    if (q < n) {
      const float4 xc = xs[cur][q];
      float4 y = f4_axpy(lap, xc, sym_mul(S, xc));
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        if (K[a] + 1 < ext[a]) y = f4_axpy(-cv[a], xs[cur][q + str[a]], y);
        if (K[a] > 0) y = f4_axpy(-cm[a], xs[cur][q - str[a]], y);
      }
      xs[cur ^ 1][q] = f4_axpy(omega, sym_mul(Di, f4_sub(bb, y)), xc);
    }
    cur ^= 1;
    __syncthreads();
  }
  if (q < n) xout[q] = xs[cur][q];
}

// ---------------------------------------------------------------------------
// the MG-PCG's own update and direction (the matvec is k_cg_matvec)
// ---------------------------------------------------------------------------

// x += alpha p; r -= alpha q; signed max of r and the stop rule.
__global__ void __launch_bounds__(MT)
k_mgcg_update(float4 *__restrict__ x, float4 *__restrict__ r, const float4 *__restrict__ p,
              const float4 *__restrict__ q, Dims4 d, BoxDecoder bx, uint32_t nint, CGState *st,
              float *fpart, int maxIter) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  __shared__ float shf[MT / 32];
  const float a = st->alphaf;
  float mx = -FLT_MAX;
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint; n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float4 pp = __ldg(p + id), qq = __ldg(q + id);
    x[id] = f4_axpy(a, pp, x[id]);
    const float4 rr = f4_axpy(-a, qq, r[id]);
    r[id] = rr;
    mx = fmaxf(mx, fmaxf(fmaxf(rr.x, rr.y), fmaxf(rr.z, rr.w)));
  }
  const float bm = block_max<MT>(mx, shf);
  if (threadIdx.x == 0) fpart[blockIdx.x] = bm;
  if (last_block_arrives(&st->counter[2])) {
    float m = 0.0f;  // border rows hold r = 0
    for (int q2 = threadIdx.x; q2 < (int)gridDim.x; q2 += blockDim.x) m = fmaxf(m, __ldcg(fpart + q2));
    m = block_max<MT>(m, shf);
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

// k_mgcg_update plus the V-cycle's first level-0 sweep: x0 = omega D^-1 r
// of the updated residual.  G gives the image gradient at a cell: the stored
// g, or g rebuilt from i1.
struct GradLoad {
  const float4 *__restrict__ g;
  __device__ __forceinline__ float4 operator()(idx_t id) const { return __ldg(g + id); }
};
template <class G>
__global__ void __launch_bounds__(MT)
k_mgcg_update_pre(float4 *__restrict__ x, float4 *__restrict__ r, const float4 *__restrict__ p,
                  const float4 *__restrict__ q, G grad, float4 *__restrict__ x0, Dims4 d,
                  BoxDecoder bx, uint32_t nint, float c0, float omega, CGState *st, float *fpart,
                  int maxIter) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  __shared__ float shf[MT / 32];
  const float a = st->alphaf;
  float mx = -FLT_MAX;
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint; n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float4 pp = __ldg(p + id), qq = __ldg(q + id), gg = grad(id);
    x[id] = f4_axpy(a, pp, x[id]);
    const float4 rr = f4_axpy(-a, qq, r[id]);
    r[id] = rr;
    x0[id] = f4_scale(omega, blk0_solve(gg, c0, rr));
    mx = fmaxf(mx, fmaxf(fmaxf(rr.x, rr.y), fmaxf(rr.z, rr.w)));
  }
  const float bm = block_max<MT>(mx, shf);
  if (threadIdx.x == 0) fpart[blockIdx.x] = bm;
  if (last_block_arrives(&st->counter[2])) {
    float m = 0.0f;  // border rows hold r = 0
    for (int q2 = threadIdx.x; q2 < (int)gridDim.x; q2 += blockDim.x) m = fmaxf(m, __ldcg(fpart + q2));
    m = block_max<MT>(m, shf);
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

// p = z + beta p
__global__ void __launch_bounds__(MT)
k_mgcg_direction(float4 *__restrict__ p, const float4 *__restrict__ z, Dims4 d, BoxDecoder bx,
                 uint32_t nint, const CGState *st, int init) {
  pdl_wait();
  pdl_launch_dependents();
  if (mg_stop(st)) return;
  const float b = st->betaf;
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint; n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    p[id] = init ? __ldg(z + id) : f4_axpy(b, p[id], __ldg(z + id));
  }
}

// The judge of a preconditioned solve: r = b - A x with the plain operator
// (float rows, the reference's block and neighbour terms), and the signed
// maximum of r (border rows, r = 0, included) into *rmax.
__global__ void __launch_bounds__(MT)
k_mg_judge(const float4 *__restrict__ x, const float4 *__restrict__ b,
           const float4 *__restrict__ g, float4 *__restrict__ r, Dims4 d, BoxDecoder bx,
           uint32_t nint, float c0, float wS, float *fpart, unsigned int *counter, float *rmax) {
  pdl_wait();
  pdl_launch_dependents();
  __shared__ float shf[MT / 32];
  float mx = -FLT_MAX;
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < nint; n += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float4 rr = f4_sub(__ldg(b + id), a0_mul(x, __ldg(g + id), id, sY, sZ, sT, c0, wS));
    r[id] = rr;
    mx = fmaxf(mx, fmaxf(fmaxf(rr.x, rr.y), fmaxf(rr.z, rr.w)));
  }
  const float bm = block_max<MT>(mx, shf);
  if (threadIdx.x == 0) fpart[blockIdx.x] = bm;
  if (last_block_arrives(counter)) {
    float m = 0.0f;
    for (int q2 = threadIdx.x; q2 < (int)gridDim.x; q2 += blockDim.x) m = fmaxf(m, __ldcg(fpart + q2));
    m = block_max<MT>(m, shf);
    if (threadIdx.x == 0) {
      *rmax = m;
      *counter = 0;
    }
  }
}

// Launches an MG kernel with programmatic stream serialisation: its blocks
// are scheduled while the previous kernel drains and wait in pdl_wait until
// that kernel's writes are visible.  Falls back to an ordinary launch if the
// attribute is refused.
template <typename... KArgs, typename... Args>
void mg_launch(void (*k)(KArgs...), unsigned grid, unsigned block, cudaStream_t s,
               Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, k, args...) != cudaSuccess) {
    cudaGetLastError();
    k<<<grid, block, 0, s>>>(args...);
  }
}

inline BoxDecoder interior_box(Dims4 d) { return make_decoder(d.x - 2, d.y - 2, d.z - 2, 1, 1, 1, 1); }
inline uint32_t interior_n(Dims4 d) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return 0;
  return (uint32_t)((long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2));
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

std::vector<Dims4> mg_level_dims(Dims4 d) {
  std::vector<Dims4> L;
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return L;
  Dims4 m{(d.x - 1) / 2, (d.y - 1) / 2, (d.z - 1) / 2, (d.t - 1) / 2};  // ceil((n-2)/2)
  L.push_back(m);
  while (m.cells() > MG_COARSEST && (m.x > 1 || m.y > 1 || m.z > 1 || m.t > 1)) {
    m = Dims4{(m.x + 1) / 2, (m.y + 1) / 2, (m.z + 1) / 2, (m.t + 1) / 2};
    L.push_back(m);
  }
  return L;
}

void launch_mg_build(const float4 *g, Dims4 d, const MGLevelPtrs *L, int nl, const OFConsts &c,
                     const MGParams &mp, const CGState *st, cudaStream_t s) {
  if (nl <= 0) return;
  mg_launch(k_mg_build1, grid_for(L[0].m.cells(), MT, 8), MT, s, g, d, L[0].m, L[0].G, L[0].cpl,
            L[0].dinv, c.wSmooth, c.wEnergy, mp.lambda, st);
  for (int l = 1; l < nl; ++l)
    mg_launch(k_mg_build, grid_for(L[l].m.cells(), MT, 8), MT, s, L[l - 1].G, L[l - 1].cpl,
              L[l - 1].m, L[l].m, L[l].G, L[l].cpl, L[l].dinv, mp.lambda, st);
}

void launch_mg_vcycle(const float4 *b0, const float4 *g, float4 *x0, float4 *r0, float4 *z, Dims4 d,
                      MGLevelPtrs *L, int nl, const OFConsts &c, const MGParams &mp, CGState *st,
                      double *dpart, int init, int pre_done, cudaStream_t s, int *launches) {
  const uint32_t nint = interior_n(d);
  const BoxDecoder bx = interior_box(d);
  const int nb0 = grid_for(nint > 0 ? nint : 1, MT, 8);
  const float c0 = c.diag, wS = c.wSmooth;
  int nl_ = 0;
  if (!pre_done) {
    mg_launch(k_mg0_pre, nb0, MT, s, b0, g, x0, d, bx, nint, c0, mp.omega0, st);
    ++nl_;
  }
  if (nl == 0) {
    mg_launch(k_mg0_post, nb0, MT, s, b0, g, x0, z, d, bx, nint, c0, wS, mp.omega0, st, dpart,
              init);
    if (launches) *launches += nl_;  // the caller counts one
    return;
  }
  {
    const int nbx = (d.x - 2 + 31) / 32;
    const int tchunks = (L[0].m.t + RR_TP - 1) / RR_TP;
    const long long nblk = (long long)nbx * L[0].m.y * L[0].m.z * tchunks;
    mg_launch(k_mg0_resid_restrict, (unsigned)nblk, RR_NT, s, b0, g, x0, L[0].b, d, L[0].m, nbx,
              c0, wS, st);
    ++nl_;
  }
  for (int l = 0; l + 1 < nl; ++l) {
    const uint32_t n = (uint32_t)L[l].m.cells();
    const int nb = grid_for(n, MT, 8);
    mg_launch(k_mgc_pre, nb, MT, s, L[l].b, L[l].dinv, L[l].x, n, mp.omegac, st);
    mg_launch(k_mgc_resid, nb, MT, s, L[l].b, L[l].G, L[l].cpl, L[l].x, L[l].r, L[l].m, st);
    mg_launch(k_mgc_restrict, grid_for(L[l + 1].m.cells(), MT, 8), MT, s, L[l].r, L[l + 1].b,
              L[l].m, L[l + 1].m, st);
    nl_ += 3;
  }
  const MGLevelPtrs &B = L[nl - 1];
  mg_launch(k_mgc_coarsest, 1, MG_COARSEST, s, B.b, B.G, B.cpl, B.dinv, B.x, B.m, mp.omegac,
            mp.coarse_sweeps, st);
  ++nl_;
  for (int l = nl - 2; l >= 0; --l) {
    const uint32_t n = (uint32_t)L[l].m.cells();
    const int nb = grid_for(n, MT, 8);
    mg_launch(k_mgc_prolong, nb, MT, s, L[l].x, L[l + 1].x, L[l].m, L[l + 1].m, st);
    mg_launch(k_mgc_post, nb, MT, s, L[l].b, L[l].G, L[l].cpl, L[l].dinv, L[l].x, L[l].r, L[l].m,
              mp.omegac, st);
    // the post-smoothed iterate is in r; it becomes this level's x
    std::swap(L[l].x, L[l].r);
    nl_ += 2;
  }
  {
    const BoxDecoder bxyz = make_decoder(d.x - 2, d.y - 2, d.z - 2, 1, 1, 1, 0);
    const uint32_t nxyz = (uint32_t)((long long)(d.x - 2) * (d.y - 2) * (d.z - 2));
    const int tchunks = (d.t - 2 + MG_TT - 1) / MG_TT;
    mg_launch(k_mg0_prolong, nb0, MT, s, x0, L[0].x, d, bx, nint, L[0].m, st);
    mg_launch(k_mg0_post_tw, grid_for((long long)nxyz * tchunks, MT, 8), MT, s, b0, g, x0, z, d,
              bxyz, nxyz, tchunks, c0, wS, mp.omega0, st, dpart, init);
    nl_ += 2;
  }
  if (launches) *launches += nl_ - 1;  // the caller counts one
}

void launch_mgcg_update(float4 *x, float4 *r, const float4 *p, const float4 *q, Dims4 d,
                        CGState *st, float *fpart, int maxIter, cudaStream_t s) {
  const uint32_t nint = interior_n(d);
  mg_launch(k_mgcg_update, grid_for(nint > 0 ? nint : 1, MT, 8), MT, s, x, r, p, q, d,
            interior_box(d), nint, st, fpart, maxIter);
}
void launch_mgcg_update_pre(float4 *x, float4 *r, const float4 *p, const float4 *q,
                            const float4 *g, const float *i1, float4 *x0, Dims4 d,
                            const OFConsts &c, const MGParams &mp, CGState *st, float *fpart,
                            int maxIter, cudaStream_t s) {
  const uint32_t nint = interior_n(d);
  const int nb = grid_for(nint > 0 ? nint : 1, MT, 8);
  if (i1)
    mg_launch(k_mgcg_update_pre<GradFromI1>, nb, MT, s, x, r, p, q,
              GradFromI1{i1, d.x, d.sz(), d.st(), c.dxf}, x0, d, interior_box(d), nint, c.diag,
              mp.omega0, st, fpart, maxIter);
  else
    mg_launch(k_mgcg_update_pre<GradLoad>, nb, MT, s, x, r, p, q, GradLoad{g}, x0, d,
              interior_box(d), nint, c.diag, mp.omega0, st, fpart, maxIter);
}

void launch_mg_judge(const float4 *x, const float4 *b, const float4 *g, float4 *r, Dims4 d,
                     const OFConsts &c, float *fpart, unsigned int *counter, float *rmax,
                     cudaStream_t s) {
  const uint32_t nint = interior_n(d);
  mg_launch(k_mg_judge, grid_for(nint > 0 ? nint : 1, MT, 8), MT, s, x, b, g, r, d, interior_box(d),
            nint, c.diag, c.wSmooth, fpart, counter, rmax);
}

void launch_mgcg_direction(float4 *p, const float4 *z, Dims4 d, const CGState *st, int init,
                           cudaStream_t s) {
  const uint32_t nint = interior_n(d);
  mg_launch(k_mgcg_direction, grid_for(nint > 0 ? nint : 1, MT, 8), MT, s, p, z, d, interior_box(d),
            nint, st, init);
}

// ---------------------------------------------------------------------------
// Separable extrapolation sweep (blurType 2): knCvExpolBlur4d
// (optflow4d.cpp:613-626) sets every unmarked interior cell to 1/81 of the
// sum over its 3^4 neighbourhood of the source.  That sum is formed here in
// two streaming passes, equal to the reference's 81-term sum up to rounding:
//   S2(x,y,z,t) = the 3x3 (x,y) box sum of the source, for interior x, y and
//                 every z, t;
//   out         = 1/81 of the 3x3 (z,t) box sum of S2, each thread walking
//                 t with the z sums of t-1, t, t+1 in registers.
// Every 3-term sum is (a-1 + a0) + a+1, x first, then y, z and t: the order
// of the one-pass TMA sweep (k_expol_sep_tw, flof_tma.cu), which this pair
// of kernels stands in for where TMA is unavailable.
// Marked and border cells are not written: both sweep buffers hold their
// values.
// ---------------------------------------------------------------------------
namespace {

__global__ void __launch_bounds__(MT)
k_sep_xy(const float4 *__restrict__ src, float4 *__restrict__ s2, Dims4 d, BoxDecoder bx,
         uint32_t n) {
  const idx_t sY = d.x;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    auto xsum = [&](idx_t r) {
      return f4_add(f4_add(__ldg(src + r - 1), __ldg(src + r)), __ldg(src + r + 1));
    };
    s2[id] = f4_add(f4_add(xsum(id - sY), xsum(id)), xsum(id + sY));
  }
}

constexpr int SEP_TT = 8;  // t planes per work item of the z-t pass

__global__ void __launch_bounds__(MT)
k_sep_zt(const float4 *__restrict__ s2, const float *__restrict__ mark, float4 *__restrict__ out,
         Dims4 d, BoxDecoder bx, uint32_t nxyz, int tchunks) {
  const idx_t sZ = d.sz(), sT = d.st();
  const uint32_t n = nxyz * (uint32_t)tchunks;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const uint32_t cell = q % nxyz, tc = q / nxyz;
    int i, j, k, unused;
    bx.decode(cell, i, j, k, unused);
    const int l0 = 1 + (int)tc * SEP_TT;
    const int l1 = min(l0 + SEP_TT, d.t - 1);
    idx_t id = d.index(i, j, k, l0);
    auto zsum = [&](idx_t c) {
      return f4_add(f4_add(__ldg(s2 + c - sZ), __ldg(s2 + c)), __ldg(s2 + c + sZ));
    };
    float4 zm = zsum(id - sT), zc = zsum(id);
    for (int l = l0; l < l1; ++l, id += sT) {
      const float4 zp = zsum(id + sT);
      if (__ldg(mark + id) == 0.f) {
        const float4 v = f4_add(f4_add(zm, zc), zp);
        out[id] = make_float4(mul_inv81(v.x), mul_inv81(v.y), mul_inv81(v.z), mul_inv81(v.w));
      }
      zm = zc;
      zc = zp;
    }
  }
}

}  // namespace

void launch_expol_sep(const float4 *in, float4 *out, float4 *s2, const float *mark, Dims4 d,
                      cudaStream_t s) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return;
  // S2 over interior x, y and every z, t
  const BoxDecoder bxy = make_decoder(d.x - 2, d.y - 2, d.z, 1, 1, 0, 0);
  const uint32_t nxy = (uint32_t)((long long)(d.x - 2) * (d.y - 2) * d.z * d.t);
  k_sep_xy<<<grid_for(nxy, MT, 8), MT, 0, s>>>(in, s2, d, bxy, nxy);
  // z-t sums over interior cells
  const BoxDecoder bxyz = make_decoder(d.x - 2, d.y - 2, d.z - 2, 1, 1, 1, 0);
  const uint32_t nxyz = (uint32_t)((long long)(d.x - 2) * (d.y - 2) * (d.z - 2));
  const int tchunks = (d.t - 2 + SEP_TT - 1) / SEP_TT;
  k_sep_zt<<<grid_for((long long)nxyz * tchunks, MT, 8), MT, 0, s>>>(s2, mark, out, d, bxyz, nxyz,
                                                                     tchunks);
}

}  // namespace flof
