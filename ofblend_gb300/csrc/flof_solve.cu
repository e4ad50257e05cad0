// flof_solve.cu -- optical-flow system assembly, Jacobi-PCG, Gaussian velocity
// blur and the level-set projection correction.
//
// Reference: source/plugin/optflow4d.cpp
//   opticalFlowDim        :361-553   (assembly :398-493, copy back :520-529)
//   FixedMatrixOF/applyMat :179-232  (matrix-free here: the block is g g^T +
//                                     diag I, rebuilt from the stored g)
//   GridCGOptflow4d        :268-355
//   knGaussianBlur         :132-158
//   knProjectCells et al.  :651-734
//   knCvExpolBlur4d        :613-626
#include <float.h>

#include <algorithm>

#include "flof_kernels.h"

namespace flof {

namespace {
// Launches a PCG kernel with programmatic stream serialisation, so that its
// blocks are scheduled while the previous kernel drains (the kernel starts
// with pdl_wait).  Falls back to an ordinary launch if the attribute is
// refused.
template <typename... KArgs, typename... Args>
void launch_pdl(void (*k)(KArgs...), unsigned grid, unsigned block, cudaStream_t s,
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
}  // namespace


constexpr int NT = 256;

// ---------------------------------------------------------------------------
// Assembly + PCG initialisation
// ---------------------------------------------------------------------------

int cg_blocks(Dims4 d) {
  long long n = (long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2);
  return grid_for(n > 0 ? n : 1, NT, 8);
}

static inline BoxDecoder interior_decoder(Dims4 d) {
  return make_decoder(d.x - 2 > 0 ? d.x - 2 : 1, d.y - 2 > 0 ? d.y - 2 : 1,
                      d.z - 2 > 0 ? d.z - 2 : 1, 1, 1, 1, 1);
}
static inline uint32_t interior_count(Dims4 d) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return 0;
  return (uint32_t)((long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2));
}

// Jacobi preconditioner of row (cell,d): 1/blockd[d][d] with the diagonal
// g_d*g_d + diag, rounded like the reference's (float)(1./diag).
__device__ __forceinline__ float4 precond_of(const float4 g, float diag) {
  float4 p;
  p.x = __frcp_rn(g.x * g.x + diag);
  p.y = __frcp_rn(g.y * g.y + diag);
  p.z = __frcp_rn(g.z * g.z + diag);
  p.w = __frcp_rn(g.w * g.w + diag);
  return p;
}

__global__ void __launch_bounds__(NT)
k_of_assemble_init(const float *__restrict__ i0w, const float *__restrict__ i1,
                   const float4 *__restrict__ vel, float4 *__restrict__ g,
                   float4 *__restrict__ r, float4 *__restrict__ p,
                   float4 *__restrict__ x, Dims4 d, BoxDecoder bx, uint32_t ncells,
                   OFConsts c, float accuracy, CGState *st, double *dpart,
                   float *fpart) {
  __shared__ double shd[NT / 32];
  __shared__ FF shff[NT / 32];
  __shared__ float shf[NT / 32];
  FF dot = {0.f, 0.f};
  float mx = -FLT_MAX;
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < ncells;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    const idx_t id = q;
    x[id] = zero4;  // setConst(result, 0) (optflow4d.cpp:280)
    if (!in_bounds(d, i, j, k, l, 1)) {
      // identity rows with zero rhs (optflow4d.cpp:424-433): g = r = p = 0
      g[id] = zero4;
      r[id] = zero4;
      p[id] = zero4;
      continue;
    }
    const float tderiv = (__ldg(i1 + id) - __ldg(i0w + id)) / c.mDt;
    float gr[4];
    gr[0] = (__ldg(i1 + id + 1) - __ldg(i1 + id - 1)) * c.dxf;
    gr[1] = (__ldg(i1 + id + sY) - __ldg(i1 + id - sY)) * c.dxf;
    gr[2] = (__ldg(i1 + id + sZ) - __ldg(i1 + id - sZ)) * c.dxf;
    gr[3] = (__ldg(i1 + id + sT) - __ldg(i1 + id - sT)) * c.dxf;
    float rh[4];
#pragma unroll
    for (int dd = 0; dd < 4; ++dd) rh[dd] = -gr[dd] * tderiv;
    if (vel) {
      // rhs -= wSmooth (v - v_nb) mDx mDx2Inv for m = -t,-z,-y,-x,+x,+y,+z,+t,
      // then -= wEnergy v mDx (optflow4d.cpp:450-478)
      const float4 vc = __ldg(vel + id);
      const idx_t off[8] = {-sT, -sZ, -sY, -1, 1, sY, sZ, sT};
      const float vcc[4] = {vc.x, vc.y, vc.z, vc.w};
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const float4 vn = __ldg(vel + id + off[m]);
        const float vnn[4] = {vn.x, vn.y, vn.z, vn.w};
#pragma unroll
        for (int dd = 0; dd < 4; ++dd)
          rh[dd] -= c.wSmooth * (vcc[dd] - vnn[dd]) * c.mDx * 1.0f;
      }
#pragma unroll
      for (int dd = 0; dd < 4; ++dd) rh[dd] -= c.wEnergy * vcc[dd] * c.mDx;
    }
    const float4 gg = make_float4(gr[0], gr[1], gr[2], gr[3]);
    const float4 rr = make_float4(rh[0], rh[1], rh[2], rh[3]);
    const float4 pre = precond_of(gg, c.diag);
    const float4 z = make_float4(rr.x * pre.x, rr.y * pre.y, rr.z * pre.z, rr.w * pre.w);
    g[id] = gg;
    r[id] = rr;
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
    float m = 0.0f;  // border rows hold r = 0
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
          st->retResidual = 1e10f;  // the caller's initial cgRes stays
          st->done = CG_FAILED_SIGMA;
        } else {
          st->retResidual = 1.0f;   // residual / resIni before any iteration
          st->done = CG_RUNNING;
        }
      }
    }
  }
}

void launch_of_assemble_init(const float *i0w, const float *i1,
                             const float4 *vel, float4 *g, float4 *r,
                             float4 *p, float4 *x, Dims4 d, OFConsts c,
                             float accuracy, CGState *st, double *dpart,
                             float *fpart, cudaStream_t s) {
  k_of_assemble_init<<<cg_blocks(d), NT, 0, s>>>(
      i0w, i1, vel, g, r, p, x, d, make_decoder(d.x, d.y, d.z, 0, 0, 0, 0),
      (uint32_t)d.cells(), c, accuracy, st, dpart, fpart);
}

// ---------------------------------------------------------------------------
// PCG iteration (GridCGOptflow4d::solve, optflow4d.cpp:304-326)
// ---------------------------------------------------------------------------

// q = A p over the interior rows; applyMat order: 8 neighbour terms
// (-t,-z,-y,-x,+x,+y,+z,+t) then the 4 block terms.
//
// A thread owns one interior (x,y) column cell at one z and walks MV_TT
// consecutive t planes, keeping p at t-1, t and t+1 in registers, so the -t
// and +t terms cost no extra load, and loading the next plane's operands
// while it computes the current one.  A work item is (run of MV_NT cells of
// the interior (x,y) plane, z, t chunk) with the (x,y) run fastest, so the
// blocks resident at one time cover neighbouring z at the same t chunk and
// the z-neighbour loads hit L2.  The grid is persistent (a fixed number of
// blocks per SM); p.Ap is accumulated per thread in float-float and summed
// in double by the last block to finish, in a fixed order.
constexpr int MV_NT = 128;

struct MVShape {
  FastDiv fx;        // interior x extent
  int nxy;           // interior (x,y) cells
  int runs;          // ceil(nxy / MV_NT)
  FastDiv fruns, fz;  // runs, interior z extent
  int items;         // runs * (Z-2) * tchunks
};

__device__ __forceinline__ void mv_acc(float4 &v, float o, const float4 a) {
  v.x += o * a.x;
  v.y += o * a.y;
  v.z += o * a.z;
  v.w += o * a.w;
}

// The operands of one cell other than p at t-1 and t.
struct MVLoads {
  float4 pp, gg, zm, ym, xm, xp, yp, zp;
};
template <class GT>
__device__ __forceinline__ void mv_load(MVLoads &a, const float4 *__restrict__ p,
                                        const GT *__restrict__ g, idx_t id, idx_t sY,
                                        idx_t sZ, idx_t sT) {
  a.pp = __ldg(p + id + sT);
  a.gg = ld_g(g, id);
  a.zm = __ldg(p + id - sZ);
  a.ym = __ldg(p + id - sY);
  a.xm = __ldg(p + id - 1);
  a.xp = __ldg(p + id + 1);
  a.yp = __ldg(p + id + sY);
  a.zp = __ldg(p + id + sZ);
}

// OFFD: the neighbour terms are present (applyMat skips them for a zero
// off-diagonal, optflow4d.cpp:215).  MV_TT: t planes per work item.
template <bool OFFD, int MV_TT, class GT>
__global__ void __launch_bounds__(MV_NT)
k_cg_matvec(const float4 *__restrict__ p, const GT *__restrict__ g,
            float4 *__restrict__ q, Dims4 d, MVShape sh, OFConsts c, CGState *st,
            double *dpart) {
  pdl_wait();
  pdl_launch_dependents();
  // the previous direction kernel has applied any pending x update
  if (blockIdx.x == 0 && threadIdx.x == 0) st->xpend = 0;
  if (st->done) return;
  __shared__ double shd[MV_NT / 32];
  __shared__ FF shff[MV_NT / 32];
  FF dot = {0.f, 0.f};
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  const float o = c.offd;
  for (int item = blockIdx.x; item < sh.items; item += gridDim.x) {
    const uint32_t r1 = sh.fruns.div((uint32_t)item);
    const int run = item - (int)r1 * sh.runs;
    const uint32_t tc = sh.fz.div(r1);
    const int k = 1 + (int)(r1 - tc * sh.fz.d);
    const int n = run * MV_NT + threadIdx.x;
    if (n >= sh.nxy) continue;
    const uint32_t jj = sh.fx.div((uint32_t)n);
    const int i = 1 + (n - (int)(jj * sh.fx.d)), j = 1 + (int)jj;
    const int l0 = 1 + (int)tc * MV_TT;
    const int l1 = min(l0 + MV_TT, d.t - 1);
    idx_t id = d.index(i, j, k, l0);
    float4 pm = __ldg(p + id - sT), pc = __ldg(p + id);
    MVLoads cur, nxt;
    mv_load(cur, p, g, id, sY, sZ, sT);
    for (int l = l0; l < l1; ++l, id += sT) {
      // the last plane reloads its own operands instead of reading past l1
      mv_load(nxt, p, g, l + 1 < l1 ? id + sT : id, sY, sZ, sT);
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (OFFD) {
        mv_acc(v, o, pm);
        mv_acc(v, o, cur.zm);
        mv_acc(v, o, cur.ym);
        mv_acc(v, o, cur.xm);
        mv_acc(v, o, cur.xp);
        mv_acc(v, o, cur.yp);
        mv_acc(v, o, cur.zp);
        mv_acc(v, o, cur.pp);
      }
      const float gv[4] = {cur.gg.x, cur.gg.y, cur.gg.z, cur.gg.w};
      const float pv[4] = {pc.x, pc.y, pc.z, pc.w};
      float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int dd = 0; dd < 4; ++dd) {
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          float b = gv[dd] * gv[m];
          if (dd == m) b = b + c.diag;
          vv[dd] += b * pv[m];
        }
      }
      const float4 qq = make_float4(vv[0], vv[1], vv[2], vv[3]);
      q[id] = qq;
      ff_add(dot, pc.x * qq.x);
      ff_add(dot, pc.y * qq.y);
      ff_add(dot, pc.z * qq.z);
      ff_add(dot, pc.w * qq.w);
      pm = pc;
      pc = cur.pp;
      cur = nxt;
    }
  }
  const double bd = block_sum_ff<MV_NT>(dot, shff);
  if (threadIdx.x == 0) dpart[blockIdx.x] = bd;
  if (last_block_arrives(&st->counter[1])) {
    double s = 0.0;
    for (int q2 = threadIdx.x; q2 < (int)gridDim.x; q2 += blockDim.x) s += __ldcg(dpart + q2);
    s = block_sum<MV_NT>(s, shd);
    if (threadIdx.x == 0) {
      st->pAp = s;
      st->alpha = st->sigma / s;
      st->alphaf = (float)st->alpha;
      st->counter[1] = 0;
    }
  }
}

namespace {

template <bool OFFD, int TT, class GT>
void matvec_variant(const float4 *p, const GT *g, float4 *q, Dims4 d, OFConsts c,
                    CGState *st, double *dpart, cudaStream_t s) {
  MVShape sh;
  const int ex = d.x > 2 ? d.x - 2 : 1, ey = d.y > 2 ? d.y - 2 : 1;
  const int ez = d.z > 2 ? d.z - 2 : 1;
  const int tchunks = d.t > 2 ? (d.t - 2 + TT - 1) / TT : 0;
  const bool empty = d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3;
  sh.fx = FastDiv((uint32_t)ex);
  sh.nxy = empty ? 0 : ex * ey;
  sh.runs = (ex * ey + MV_NT - 1) / MV_NT;
  sh.fruns = FastDiv((uint32_t)sh.runs);
  sh.fz = FastDiv((uint32_t)ez);
  sh.items = empty ? 0 : sh.runs * ez * tchunks;
  // resident blocks per SM of this instantiation (computed once, thread-safe)
  static const int per_sm = [] {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cg_matvec<OFFD, TT, GT>, MV_NT, 0);
    return n < 1 ? 1 : n;
  }();
  int blocks = sm_count() * per_sm;
  if (blocks > sh.items) blocks = sh.items > 0 ? sh.items : 1;
  launch_pdl(k_cg_matvec<OFFD, TT, GT>, blocks, MV_NT, s, p, g, q, d, sh, c, st, dpart);
}

template <bool OFFD, class GT>
void matvec_tt(const float4 *p, const GT *g, float4 *q, Dims4 d, OFConsts c, CGState *st,
               double *dpart, cudaStream_t s, int tt) {
  if (tt <= 4)
    matvec_variant<OFFD, 4>(p, g, q, d, c, st, dpart, s);
  else if (tt >= 16)
    matvec_variant<OFFD, 16>(p, g, q, d, c, st, dpart, s);
  else
    matvec_variant<OFFD, 8>(p, g, q, d, c, st, dpart, s);
}

template <class GT>
void matvec_any(const float4 *p, const GT *g, float4 *q, Dims4 d, OFConsts c, CGState *st,
                double *dpart, cudaStream_t s, const CGTune &tu) {
  if (c.offd != 0.f)
    matvec_tt<true>(p, g, q, d, c, st, dpart, s, tu.mv_tt);
  else
    matvec_tt<false>(p, g, q, d, c, st, dpart, s, tu.mv_tt);
}

}  // namespace

void launch_cg_matvec(const float4 *p, const float4 *g, float4 *q, Dims4 d,
                      OFConsts c, CGState *st, double *dpart, cudaStream_t s,
                      const CGTune &tu) {
  matvec_any(p, g, q, d, c, st, dpart, s, tu);
}
void launch_cg_matvec(const float4 *p, const BF4 *g, float4 *q, Dims4 d,
                      OFConsts c, CGState *st, double *dpart, cudaStream_t s,
                      const CGTune &tu) {
  matvec_any(p, g, q, d, c, st, dpart, s, tu);
}

// Where the update and direction kernels take the image gradient g for the
// Jacobi preconditioner from: the stored g (FP32 or BF16), or g rebuilt from
// the target level set i1 with the assembly's own operations (central
// differences times 1/(2 mDx), the same values bit for bit).  i1 is 4 bytes
// per cell against 16 for g; its neighbour loads hit L1 and L2.
template <class T>
struct GradStored {
  const T *__restrict__ g;
  __device__ __forceinline__ float4 operator()(idx_t id) const { return ld_g(g, id); }
};

// r -= alpha q; z = M^-1 r; sigma' = z.r; max(r).  x += alpha p is left to
// the direction kernel (st->xpend).
template <class GS>
__global__ void __launch_bounds__(NT)
k_cg_update(float4 *__restrict__ r, const float4 *__restrict__ q, GS gs, Dims4 d, BoxDecoder bx,
            uint32_t nint, OFConsts c, CGState *st, double *dpart, float *fpart, int maxIter) {
  pdl_wait();
  pdl_launch_dependents();
  if (st->done) return;
  __shared__ double shd[NT / 32];
  __shared__ FF shff[NT / 32];
  __shared__ float shf[NT / 32];
  const float a = st->alphaf;
  FF dot = {0.f, 0.f};
  float mx = -FLT_MAX;
  auto cell = [&](idx_t id, float4 qq, float4 gv, float4 rr) {
    rr.x = __fmaf_rn(-a, qq.x, rr.x);
    rr.y = __fmaf_rn(-a, qq.y, rr.y);
    rr.z = __fmaf_rn(-a, qq.z, rr.z);
    rr.w = __fmaf_rn(-a, qq.w, rr.w);
    r[id] = rr;
    const float4 pre = precond_of(gv, c.diag);
    ff_add(dot, (rr.x * pre.x) * rr.x);
    ff_add(dot, (rr.y * pre.y) * rr.y);
    ff_add(dot, (rr.z * pre.z) * rr.z);
    ff_add(dot, (rr.w * pre.w) * rr.w);
    mx = fmaxf(mx, fmaxf(fmaxf(rr.x, rr.y), fmaxf(rr.z, rr.w)));
  };
  // two cells per trip with all loads issued first (the thread's cell order,
  // and so the sum order, is that of the plain grid-stride loop)
  const uint32_t stride = gridDim.x * blockDim.x;
  uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  for (; n + stride < nint; n += 2 * stride) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t i0 = d.index(i, j, k, l);
    bx.decode(n + stride, i, j, k, l);
    const idx_t i1 = d.index(i, j, k, l);
    const float4 q0 = __ldg(q + i0), q1 = __ldg(q + i1);
    const float4 g0 = gs(i0), g1 = gs(i1);
    const float4 r0 = r[i0], r1 = r[i1];
    cell(i0, q0, g0, r0);
    cell(i1, q1, g1, r1);
  }
  if (n < nint) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t i0 = d.index(i, j, k, l);
    cell(i0, __ldg(q + i0), gs(i0), r[i0]);
  }
  const double bd = block_sum_ff<NT>(dot, shff);
  const float bm = block_max<NT>(mx, shf);
  if (threadIdx.x == 0) {
    dpart[blockIdx.x] = bd;
    fpart[blockIdx.x] = bm;
  }
  if (last_block_arrives(&st->counter[2])) {
    double s = 0.0;
    float m = 0.0f;
    for (int q2 = threadIdx.x; q2 < (int)gridDim.x; q2 += blockDim.x) {
      s += __ldcg(dpart + q2);
      m = fmaxf(m, __ldcg(fpart + q2));
    }
    s = block_sum<NT>(s, shd);
    m = block_max<NT>(m, shf);
    if (threadIdx.x == 0) {
      const double residual = (double)m;
      const int iter = st->iters;
      st->resMax = m;
      st->retResidual = (float)(residual / st->resIni);
      st->iters = iter + 1;
      st->xpend = 1;
      st->counter[2] = 0;
      if (residual <= st->acc) {
        st->done = CG_CONVERGED;
      } else {
        st->beta = s / st->sigma;
        st->betaf = (float)st->beta;
        st->sigma = s;
        if (iter + 1 >= maxIter) st->done = CG_MAXITER;
      }
    }
  }
}

// Blocks per SM for a grid-stride PCG kernel: the tuned count, capped at what
// fits at once, so that the grid is a single wave.
template <class K>
int resident_per_sm(K kernel, int want) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, NT, 0) != cudaSuccess) {
    cudaGetLastError();
    n = 1;
  }
  if (n < 1) n = 1;
  return want < n ? want : n;
}

template <class GS>
void update_launch(float4 *r, const float4 *q, GS gs, Dims4 d, OFConsts c, CGState *st,
                   double *dpart, float *fpart, int maxIter, cudaStream_t s, const CGTune &tu) {
  static const int occ = resident_per_sm(k_cg_update<GS>, 1 << 30);
  const long long n = interior_count(d);
  launch_pdl(k_cg_update<GS>, grid_for(n > 0 ? n : 1, NT, tu.per_sm < occ ? tu.per_sm : occ),
             NT, s, r, q, gs, d, interior_decoder(d), (uint32_t)n, c, st, dpart, fpart, maxIter);
}
void launch_cg_update(float4 *r, const float4 *q, const float4 *g, Dims4 d, OFConsts c,
                      CGState *st, double *dpart, float *fpart, int maxIter, cudaStream_t s,
                      const CGTune &tu, const float *i1) {
  if (i1)
    update_launch(r, q, GradFromI1{i1, d.x, d.sz(), d.st(), c.dxf}, d, c, st, dpart, fpart,
                  maxIter, s, tu);
  else
    update_launch(r, q, GradStored<float4>{g}, d, c, st, dpart, fpart, maxIter, s, tu);
}
void launch_cg_update(float4 *r, const float4 *q, const BF4 *g, Dims4 d, OFConsts c,
                      CGState *st, double *dpart, float *fpart, int maxIter, cudaStream_t s,
                      const CGTune &tu) {
  update_launch(r, q, GradStored<BF4>{g}, d, c, st, dpart, fpart, maxIter, s, tu);
}

// x += alpha p (the last update's, when pending); then, while the solve
// runs, p = z + beta p.
template <bool XP, bool PN, class GS>
__device__ __forceinline__ void direction_cells(float4 *__restrict__ x, float4 *__restrict__ p,
                                                const float4 *__restrict__ r, const GS &gs,
                                                const Dims4 &d, const BoxDecoder &bx,
                                                uint32_t nint, const OFConsts &c, float a,
                                                float b) {
  struct In {
    float4 p, x, r, g;
  };
  auto load = [&](idx_t id) {
    In v;
    v.p = p[id];
    if (XP) v.x = x[id];
    if (PN) {
      v.r = __ldg(r + id);
      v.g = gs(id);
    }
    return v;
  };
  auto cell = [&](idx_t id, const In &v) {
    float4 pp = v.p;
    if (XP) {
      float4 xx = v.x;
      xx.x = __fmaf_rn(a, pp.x, xx.x);
      xx.y = __fmaf_rn(a, pp.y, xx.y);
      xx.z = __fmaf_rn(a, pp.z, xx.z);
      xx.w = __fmaf_rn(a, pp.w, xx.w);
      x[id] = xx;
    }
    if (PN) {
      const float4 rr = v.r;
      const float4 pre = precond_of(v.g, c.diag);
      pp.x = __fmaf_rn(b, pp.x, rr.x * pre.x);
      pp.y = __fmaf_rn(b, pp.y, rr.y * pre.y);
      pp.z = __fmaf_rn(b, pp.z, rr.z * pre.z);
      pp.w = __fmaf_rn(b, pp.w, rr.w * pre.w);
      p[id] = pp;
    }
  };
  // two cells per trip with all loads issued first
  const uint32_t stride = gridDim.x * blockDim.x;
  uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
  for (; n + stride < nint; n += 2 * stride) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t i0 = d.index(i, j, k, l);
    bx.decode(n + stride, i, j, k, l);
    const idx_t i1 = d.index(i, j, k, l);
    const In v0 = load(i0), v1 = load(i1);
    cell(i0, v0);
    cell(i1, v1);
  }
  if (n < nint) {
    int i, j, k, l;
    bx.decode(n, i, j, k, l);
    const idx_t i0 = d.index(i, j, k, l);
    cell(i0, load(i0));
  }
}

template <class GS>
__global__ void __launch_bounds__(NT)
k_cg_direction(float4 *__restrict__ x, float4 *__restrict__ p, const float4 *__restrict__ r,
               GS gs, Dims4 d, BoxDecoder bx, uint32_t nint, OFConsts c, CGState *st) {
  pdl_wait();
  pdl_launch_dependents();
  // st is read-only here: the update wrote it, the next matvec clears xpend
  const bool xp = st->xpend != 0, run = st->done == 0;
  const float a = st->alphaf, b = st->betaf;
  if (xp && run)
    direction_cells<true, true>(x, p, r, gs, d, bx, nint, c, a, b);
  else if (xp)
    direction_cells<true, false>(x, p, r, gs, d, bx, nint, c, a, b);
  else if (run)
    direction_cells<false, true>(x, p, r, gs, d, bx, nint, c, a, b);
}

template <class GS>
void direction_launch(float4 *x, float4 *p, const float4 *r, GS gs, Dims4 d, OFConsts c,
                      CGState *st, cudaStream_t s, const CGTune &tu) {
  static const int occ = resident_per_sm(k_cg_direction<GS>, 1 << 30);
  const long long n = interior_count(d);
  launch_pdl(k_cg_direction<GS>, grid_for(n > 0 ? n : 1, NT, tu.per_sm < occ ? tu.per_sm : occ),
             NT, s, x, p, r, gs, d, interior_decoder(d), (uint32_t)n, c, st);
}
void launch_cg_direction(float4 *x, float4 *p, const float4 *r, const float4 *g, Dims4 d,
                         OFConsts c, CGState *st, cudaStream_t s, const CGTune &tu,
                         const float *i1) {
  if (i1)
    direction_launch(x, p, r, GradFromI1{i1, d.x, d.sz(), d.st(), c.dxf}, d, c, st, s, tu);
  else
    direction_launch(x, p, r, GradStored<float4>{g}, d, c, st, s, tu);
}
void launch_cg_direction(float4 *x, float4 *p, const float4 *r, const BF4 *g, Dims4 d,
                         OFConsts c, CGState *st, cudaStream_t s, const CGTune &tu) {
  direction_launch(x, p, r, GradStored<BF4>{g}, d, c, st, s, tu);
}

// vel = x / mDx (optflow4d.cpp:520-529); a NaN residual resets the result to
// zero first (:508-514).
__global__ void k_of_copy_back(const float4 *__restrict__ x, float4 *__restrict__ vel,
                               long long n, float mDx, const CGState *st) {
  const float res = st->retResidual;
  const bool reset = (res != res);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    float4 v = reset ? make_float4(0.f, 0.f, 0.f, 0.f) : __ldg(x + q);
    v.x = v.x / mDx;
    v.y = v.y / mDx;
    v.z = v.z / mDx;
    v.w = v.w / mDx;
    vel[q] = v;
  }
}
void launch_of_copy_back(const float4 *x, float4 *vel, long long cells,
                         float mDx, const CGState *st, cudaStream_t s) {
  k_of_copy_back<<<grid_for(cells, NT), NT, 0, s>>>(x, vel, cells, mDx, st);
}

// ---------------------------------------------------------------------------
// Gaussian blur (knGaussianBlur, optflow4d.cpp:132-158)
// ---------------------------------------------------------------------------

struct WTab {
  float w[160];  // exp weight by squared tap distance, s <= 6
};

template <int NC>
__global__ void __launch_bounds__(NT)
k_gauss_pass(const float *__restrict__ src, float *__restrict__ dst, Dims4 d,
             BoxDecoder bx, int s, WTab wt, int zero_border) {
  const uint32_t n = (uint32_t)d.cells();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    if (!in_bounds(d, i, j, k, l, 1)) {
      if (zero_border) {
        if (NC == 4) ((float4 *)dst)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        else dst[q] = 0.f;
      }
      continue;
    }
    float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
    float weight = 0.f;
    for (int vt = l - s; vt <= l + s; vt++) {
      if (vt < 0 || vt >= d.t) continue;
      for (int zk = k - s; zk <= k + s; zk++) {
        if (zk < 0 || zk >= d.z) continue;
        for (int yj = j - s; yj <= j + s; yj++) {
          if (yj < 0 || yj >= d.y) continue;
          const int base = (vt - l) * (vt - l) + (zk - k) * (zk - k) + (yj - j) * (yj - j);
          const idx_t row = d.index(0, yj, zk, vt);
          for (int xi = i - s; xi <= i + s; xi++) {
            if (xi < 0 || xi >= d.x) continue;
            const float w = wt.w[base + (xi - i) * (xi - i)];
            weight += w;
            if (NC == 4) {
              const float4 a = __ldg((const float4 *)src + row + xi);
              val.x += w * a.x;
              val.y += w * a.y;
              val.z += w * a.z;
              val.w += w * a.w;
            } else {
              val.x += w * __ldg(src + row + xi);
            }
          }
        }
      }
    }
    if (weight > 1e-6f) {
      if (NC == 4)
        ((float4 *)dst)[q] = make_float4(val.x / weight, val.y / weight, val.z / weight,
                                         val.w / weight);
      else
        dst[q] = val.x / weight;
    } else {
      if (NC == 4) ((float4 *)dst)[q] = __ldg((const float4 *)src + q);
      else dst[q] = __ldg(src + q);
    }
  }
}

void launch_gauss_pass(const float *src, float *dst, Dims4 d, int nc, int s,
                       const float *wtab, int zero_border, cudaStream_t st) {
  WTab wt;
  const int nw = 4 * s * s + 1;
  for (int q = 0; q < 160; ++q) wt.w[q] = q < nw ? wtab[q] : 0.f;
  BoxDecoder bx = make_decoder(d.x, d.y, d.z, 0, 0, 0, 0);
  const int nb = grid_for(d.cells(), NT, 8);
  if (nc == 4)
    k_gauss_pass<4><<<nb, NT, 0, st>>>(src, dst, d, bx, s, wt, zero_border);
  else
    k_gauss_pass<1><<<nb, NT, 0, st>>>(src, dst, d, bx, s, wt, zero_border);
}

// The separable blur (blurType 2).  Along one axis, the sum at coordinate c
// is sum_o w|o| src(c + o) over the in-range taps o = -S..S in increasing o,
// each added by one fused multiply-add, times 1 / (the in-range weights
// added in the same order): the 1D normalised Gaussian with clipping.  The
// four axes are applied in the order x, y, z, t by two kernels: one forms
// the y sums of x sums within each (z, t) plane, the other the t sums of z
// sums, each thread walking a run of y rows or t planes with the 2S + 1
// inner sums it needs in a register ring.  Every intermediate value is the
// single-axis pass's, rounded once to float, so the pair equals four
// single-axis passes; the 4D weight of the reference's blur is the product
// of the 1D weights and its in-bounds box the product of the 1D ranges, so
// the result equals the direct normalised stencil up to rounding.
struct W1 {
  float w[7];  // 1D weight by tap distance, S <= 6
};
template <int NC>
__device__ __forceinline__ float4 ld_nc(const float *p, idx_t i) {
  if (NC == 4) return __ldg((const float4 *)p + i);
  return make_float4(__ldg(p + i), 0.f, 0.f, 0.f);
}
template <int NC>
__device__ __forceinline__ void st_nc(float *p, idx_t i, float4 v) {
  if (NC == 4) ((float4 *)p)[i] = v;
  else p[i] = v.x;
}
__device__ __forceinline__ void fma4(float4 &v, float w, const float4 &a) {
  v.x = __fmaf_rn(w, a.x, v.x);
  v.y = __fmaf_rn(w, a.y, v.y);
  v.z = __fmaf_rn(w, a.z, v.z);
  v.w = __fmaf_rn(w, a.w, v.w);
}
__device__ __forceinline__ float4 scale4(const float4 &v, float s) {
  return make_float4(v.x * s, v.y * s, v.z * s, v.w * s);
}
// 1 / (sum of the in-range 1D weights around c on an axis of n cells)
template <int S>
__device__ __forceinline__ float sep_inv(const W1 &w, int c, int n) {
  float weight = 0.f;
#pragma unroll
  for (int o = -S; o <= S; ++o)
    if (c + o >= 0 && c + o < n) weight += w.w[o < 0 ? -o : o];
  return 1.0f / weight;
}
// the normalised 1D sum of the ring r (values at c - S .. c + S)
template <int S>
__device__ __forceinline__ float4 sep_ring(const W1 &w, const float4 (&r)[2 * S + 1], int c, int n) {
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int o = -S; o <= S; ++o)
    if (c + o >= 0 && c + o < n) fma4(v, w.w[o < 0 ? -o : o], r[o + S]);
  return scale4(v, sep_inv<S>(w, c, n));
}

constexpr int SEP_RUN = 16;  // y rows or t planes walked per thread
constexpr int SEP_ZB = 8;    // z planes per block of the z-t kernel (32 x 8 threads)
static_assert(32 * SEP_ZB == NT, "the z-t kernel's block is NT threads");

// The 2S + 1 taps of an axis sum around cell `id` with stride `step`; taps
// outside the axis (c + o out of 0..n-1) or a cell outside the walk
// (live == false) read as zero and are never used.
template <int NC, int S>
__device__ __forceinline__ void load_taps(float4 (&a)[2 * S + 1], const float *src, idx_t id,
                                          idx_t step, int c, int n, bool live) {
#pragma unroll
  for (int o = -S; o <= S; ++o)
    a[o + S] = (live && c + o >= 0 && c + o < n) ? ld_nc<NC>(src, id + o * step)
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
}
template <int S>
__device__ __forceinline__ float4 sum_taps(const W1 &w, const float4 (&a)[2 * S + 1], int c, int n,
                                           float inv) {
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int o = -S; o <= S; ++o)
    if (c + o >= 0 && c + o < n) fma4(v, w.w[o < 0 ? -o : o], a[o + S]);
  return scale4(v, inv);
}

// dst(x, y, z, t) = the y sum of the x sums, every cell.  A thread walks a
// run of y rows; the taps of the next row are loaded before the current
// row's sums are formed.
template <int NC, int S>
__global__ void __launch_bounds__(NT)
k_blur_sep_xy(const float *__restrict__ src, float *__restrict__ dst, Dims4 d, W1 w,
              uint32_t n) {
  const idx_t sY = d.x;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int x = (int)(q % (uint32_t)d.x);
    uint32_t r = q / (uint32_t)d.x;
    const int z = (int)(r % (uint32_t)d.z);
    r /= (uint32_t)d.z;
    const int t = (int)(r % (uint32_t)d.t);
    const int ya = (int)(r / (uint32_t)d.t) * SEP_RUN, yb = min(ya + SEP_RUN, d.y);
    const idx_t plane = d.index(x, 0, z, t);
    const float ix = sep_inv<S>(w, x, d.x);
    float4 ring[2 * S + 1], a[2 * S + 1];
#pragma unroll
    for (int k = 1; k <= 2 * S; ++k) {
      const int y = ya - S - 1 + k;
      const bool live = y >= 0 && y < d.y;
      load_taps<NC, S>(a, src, plane + y * sY, 1, x, d.x, live);
      ring[k] = sum_taps<S>(w, a, x, d.x, ix);
    }
    load_taps<NC, S>(a, src, plane + (ya + S) * sY, 1, x, d.x, ya + S < d.y);
    for (int y = ya; y < yb; ++y) {
      float4 cur[2 * S + 1];
#pragma unroll
      for (int k = 0; k <= 2 * S; ++k) cur[k] = a[k];
      load_taps<NC, S>(a, src, plane + (y + S + 1) * sY, 1, x, d.x, y + 1 < yb && y + S + 1 < d.y);
#pragma unroll
      for (int k = 0; k < 2 * S; ++k) ring[k] = ring[k + 1];
      ring[2 * S] = sum_taps<S>(w, cur, x, d.x, ix);
      st_nc<NC>(dst, plane + y * sY, sep_ring<S>(w, ring, y, d.y));
    }
  }
}

// dst(x, y, z, t) = the t sum of the z sums at interior cells; border_mode 1
// writes zeros on the one-cell ring, 2 leaves it alone.  A block is 32 x
// columns by SEP_ZB z planes at one y, so the z taps of a thread are mostly
// its neighbours' cells, read through L1; each thread walks a run of t
// planes, loading the next plane's taps before the current sums are formed.
template <int NC, int S>
__global__ void __launch_bounds__(NT)
k_blur_sep_zt(const float *__restrict__ src, float *__restrict__ dst, Dims4 d, W1 w,
              int border_mode, int xtiles, int ztiles, uint32_t nblocks) {
  const idx_t sZ = d.sz(), sT = d.st();
  const int tx = threadIdx.x & 31, tz = threadIdx.x >> 5;
  for (uint32_t b = blockIdx.x; b < nblocks; b += gridDim.x) {
    uint32_t r = b;
    const int xt = (int)(r % (uint32_t)xtiles);
    r /= (uint32_t)xtiles;
    const int y = (int)(r % (uint32_t)d.y);
    r /= (uint32_t)d.y;
    const int zt = (int)(r % (uint32_t)ztiles);
    const int ta = (int)(r / (uint32_t)ztiles) * SEP_RUN, tb = min(ta + SEP_RUN, d.t);
    const int x = xt * 32 + tx, z = zt * SEP_ZB + tz;
    if (x >= d.x || z >= d.z) continue;
    const idx_t col = d.index(x, y, z, 0);
    const bool ring_xyz = x < 1 || x >= d.x - 1 || y < 1 || y >= d.y - 1 || z < 1 || z >= d.z - 1;
    if (ring_xyz) {
      if (border_mode == 1)
        for (int t = ta; t < tb; ++t) st_nc<NC>(dst, col + t * sT, make_float4(0.f, 0.f, 0.f, 0.f));
      continue;
    }
    const float iz = sep_inv<S>(w, z, d.z);
    float4 ring[2 * S + 1], a[2 * S + 1];
#pragma unroll
    for (int k = 1; k <= 2 * S; ++k) {
      const int t = ta - S - 1 + k;
      load_taps<NC, S>(a, src, col + t * sT, sZ, z, d.z, t >= 0 && t < d.t);
      ring[k] = sum_taps<S>(w, a, z, d.z, iz);
    }
    load_taps<NC, S>(a, src, col + (ta + S) * sT, sZ, z, d.z, ta + S < d.t);
    for (int t = ta; t < tb; ++t) {
      float4 cur[2 * S + 1];
#pragma unroll
      for (int k = 0; k <= 2 * S; ++k) cur[k] = a[k];
      load_taps<NC, S>(a, src, col + (t + S + 1) * sT, sZ, z, d.z, t + 1 < tb && t + S + 1 < d.t);
#pragma unroll
      for (int k = 0; k < 2 * S; ++k) ring[k] = ring[k + 1];
      ring[2 * S] = sum_taps<S>(w, cur, z, d.z, iz);
      if (t < 1 || t >= d.t - 1) {
        if (border_mode == 1) st_nc<NC>(dst, col + t * sT, make_float4(0.f, 0.f, 0.f, 0.f));
        continue;
      }
      st_nc<NC>(dst, col + t * sT, sep_ring<S>(w, ring, t, d.t));
    }
  }
}

template <int NC, int S>
void launch_sep_pair(const float *src, float *dst, Dims4 d, int zt, const W1 &w, int border_mode,
                     cudaStream_t st) {
  if (!zt) {
    const uint32_t n = (uint32_t)((long long)d.x * d.z * d.t * ((d.y + SEP_RUN - 1) / SEP_RUN));
    k_blur_sep_xy<NC, S><<<grid_for(n, NT, 8), NT, 0, st>>>(src, dst, d, w, n);
  } else {
    const int xtiles = (d.x + 31) / 32, ztiles = (d.z + SEP_ZB - 1) / SEP_ZB;
    const uint32_t nb =
        (uint32_t)((long long)xtiles * d.y * ztiles * ((d.t + SEP_RUN - 1) / SEP_RUN));
    const int grid = (int)std::min<long long>(nb, (long long)sm_count() * 8);
    k_blur_sep_zt<NC, S><<<grid, 32 * SEP_ZB, 0, st>>>(src, dst, d, w, border_mode, xtiles, ztiles,
                                                       nb);
  }
}
template <int NC>
void launch_sep_pair_nc(const float *src, float *dst, Dims4 d, int zt, int s, const W1 &w,
                        int border_mode, cudaStream_t st) {
  switch (s) {
    case 1: launch_sep_pair<NC, 1>(src, dst, d, zt, w, border_mode, st); break;
    case 2: launch_sep_pair<NC, 2>(src, dst, d, zt, w, border_mode, st); break;
    case 3: launch_sep_pair<NC, 3>(src, dst, d, zt, w, border_mode, st); break;
    case 4: launch_sep_pair<NC, 4>(src, dst, d, zt, w, border_mode, st); break;
    case 5: launch_sep_pair<NC, 5>(src, dst, d, zt, w, border_mode, st); break;
    default: launch_sep_pair<NC, 6>(src, dst, d, zt, w, border_mode, st); break;
  }
}

void launch_gauss_sep_pair(const float *src, float *dst, Dims4 d, int nc, int zt, int s,
                           const float *w1d, int border_mode, cudaStream_t st) {
  W1 w;
  for (int q = 0; q < 7; ++q) w.w[q] = q <= s ? w1d[q] : 0.f;
  if (nc == 4) launch_sep_pair_nc<4>(src, dst, d, zt, s, w, border_mode, st);
  else launch_sep_pair_nc<1>(src, dst, d, zt, s, w, border_mode, st);
}

// ---------------------------------------------------------------------------
// Projection correction (optflow4d.cpp:651-734)
// ---------------------------------------------------------------------------

// The projection samples phiOrg 9 times around each cell (the centre and
// +-0.5 along each axis for the normal) and then once per search step.  The
// samples share taps: along each axis the +-0.5 bases differ from the
// centre's by at most one, so the 2^4 centre block plus one 8-tap face per
// shifted sample that moved covers all nine (48 loads instead of 144 when
// nothing is clamped).  Search steps reuse the taps while the probe stays in
// the same cell, which is every step once the normal is zero (flat, clamped
// regions).  The weights and the sum order are those of interp4_real, so the
// values are the same bit for bit.

// c[t*8 + z*4 + x*2 + y]: the interp4_sum order.
__device__ __forceinline__ float ip16(const float (&c)[16], const AxisW &ax, const AxisW &ay,
                                      const AxisW &az, const AxisW &at) {
  const float s0 = ax.w0, s1 = ax.w1, t0 = ay.w0, t1 = ay.w1;
  const float f0 = az.w0, f1 = az.w1, g0 = at.w0, g1 = at.w1;
  return (((c[0] * t0 + c[1] * t1) * s0 + (c[2] * t0 + c[3] * t1) * s1) * f0 +
          ((c[4] * t0 + c[5] * t1) * s0 + (c[6] * t0 + c[7] * t1) * s1) * f1) *
             g0 +
         (((c[8] * t0 + c[9] * t1) * s0 + (c[10] * t0 + c[11] * t1) * s1) * f0 +
          ((c[12] * t0 + c[13] * t1) * s0 + (c[14] * t0 + c[15] * t1) * s1) * f1) *
             g1;
}

__device__ __forceinline__ idx_t tap_off(int q, idx_t sY, idx_t sZ, idx_t sT) {
  return (idx_t)((q >> 1) & 1) + (idx_t)(q & 1) * sY + (idx_t)((q >> 2) & 1) * sZ +
         (idx_t)((q >> 3) & 1) * sT;
}

__device__ __forceinline__ void load_taps(const float *__restrict__ phi, idx_t i, idx_t sY,
                                          idx_t sZ, idx_t sT, float (&c)[16]) {
#pragma unroll
  for (int q = 0; q < 16; ++q) c[q] = __ldg(phi + i + tap_off(q, sY, sZ, sT));
}

// The sample at the centre position with axis D moved to `s`.
template <int D>
__device__ __forceinline__ float shifted_sample(const float *__restrict__ phi, const Dims4 &d,
                                                const float (&C)[16], idx_t ic,
                                                const AxisW (&a)[4], const AxisW &s, float p0,
                                                float p1, float p2, float p3) {
  constexpr int bit = D == 0 ? 2 : D == 1 ? 1 : D == 2 ? 4 : 8;
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  const idx_t sD = D == 0 ? 1 : D == 1 ? sY : D == 2 ? sZ : sT;
  const int delta = s.b - a[D].b;
  if (delta < -1 || delta > 1) return interp4_real(phi, d, p0, p1, p2, p3);
  float S[16];
  if (delta == 0) {
#pragma unroll
    for (int q = 0; q < 16; ++q) S[q] = C[q];
  } else if (delta > 0) {
    const idx_t f = ic + 2 * sD;
#pragma unroll
    for (int q = 0; q < 16; ++q)
      if (!(q & bit)) {
        S[q] = C[q | bit];
        S[q | bit] = __ldg(phi + f + tap_off(q, sY, sZ, sT));
      }
  } else {
    const idx_t f = ic - sD;
#pragma unroll
    for (int q = 0; q < 16; ++q)
      if (!(q & bit)) {
        S[q] = __ldg(phi + f + tap_off(q, sY, sZ, sT));
        S[q | bit] = C[q];
      }
  }
  return ip16(S, D == 0 ? s : a[0], D == 1 ? s : a[1], D == 2 ? s : a[2], D == 3 ? s : a[3]);
}

// The state of a cell whose projection search is still to run.
struct ProjState {
  float4 p;    // the advected position
  float4 nrm;  // the normalised normal
  float dd, target;
  uint32_t id, pad;
};

// The outcome of a cell's projection (optflow4d.cpp:725-732).
__device__ __forceinline__ void project_write(float4 *__restrict__ dst, float *__restrict__ marker,
                                              idx_t id, float4 nrm, float dd, float threshPhi) {
  if (fabsf(dd) > threshPhi) {
    dst[id] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  dst[id] = make_float4(nrm.x * dd, nrm.y * dd, nrm.z * dd, nrm.w * dd);
  marker[id] = 1.f;
}

// knProjectCells, first part: per box cell the advected position, the normal
// and the start of the search.  Cells with a zero normal (flat, clamped phi)
// finish here; the others are appended to `queue` (warp-aggregated, in no
// fixed order) for k_project_search.
__global__ void __launch_bounds__(128, 5)
k_project_prep(float4 *__restrict__ dst, const float4 *__restrict__ vel,
               const float *__restrict__ phiOrg, const float *__restrict__ phiTarget,
               float *__restrict__ marker, Dims4 d, BoxDecoder bx, uint32_t nbox,
               float threshPhi, int maxIter, ProjState *__restrict__ queue,
               unsigned int *__restrict__ qcount) {
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  // every lane of a warp runs the same trip count, for the warp-wide append
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t trips = (nbox + stride - 1) / stride;
  const unsigned lane = threadIdx.x & 31;
  for (uint32_t it = 0, q = blockIdx.x * blockDim.x + threadIdx.x; it < trips; ++it, q += stride) {
    bool search = false;
    ProjState S;
    if (q < nbox) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float dt = 1.0f;
    const float4 v = __ldg(vel + id);
    const float p0 = (float)(i + 0.5f) - v.x * dt;
    const float p1 = (float)(j + 0.5f) - v.y * dt;
    const float p2 = (float)(k + 0.5f) - v.z * dt;
    const float p3 = (float)(l + 0.5f) - v.w * dt;
    const AxisW a[4] = {axis_index(p0, d.x), axis_index(p1, d.y), axis_index(p2, d.z),
                        axis_index(p3, d.t)};
    const idx_t ic = d.index(a[0].b, a[1].b, a[2].b, a[3].b);
    float T[16];
    load_taps(phiOrg, ic, sY, sZ, sT, T);
    // normal at p: central differences with h = 0.5 (optflow4d.cpp:655-661)
    const float h = 0.5f;
    float4 nrm;
    nrm.x = shifted_sample<0>(phiOrg, d, T, ic, a, axis_index(p0 + h, d.x), p0 + h, p1, p2, p3) -
            shifted_sample<0>(phiOrg, d, T, ic, a, axis_index(p0 - h, d.x), p0 - h, p1, p2, p3);
    nrm.y = shifted_sample<1>(phiOrg, d, T, ic, a, axis_index(p1 + h, d.y), p0, p1 + h, p2, p3) -
            shifted_sample<1>(phiOrg, d, T, ic, a, axis_index(p1 - h, d.y), p0, p1 - h, p2, p3);
    nrm.z = shifted_sample<2>(phiOrg, d, T, ic, a, axis_index(p2 + h, d.z), p0, p1, p2 + h, p3) -
            shifted_sample<2>(phiOrg, d, T, ic, a, axis_index(p2 - h, d.z), p0, p1, p2 - h, p3);
    nrm.w = shifted_sample<3>(phiOrg, d, T, ic, a, axis_index(p3 + h, d.t), p0, p1, p2, p3 + h) -
            shifted_sample<3>(phiOrg, d, T, ic, a, axis_index(p3 - h, d.t), p0, p1, p2, p3 - h);
    // normalize (util/vector4d.h:331-345)
    {
      // |len2 - 1| < 1e-12 in double holds for a float len2 only at 1.0f:
      // the floats next to 1 are 2^-24 and 2^-23 away.  The float test keeps
      // the FP64 pipe (2 ops/clk/SM on this part) out of the kernel.
      const float len2 = nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z + nrm.w * nrm.w;
      const float eps2 = 1e-6f * 1e-6f;
      if (len2 == 1.0f) {
        // normalized enough
      } else if (len2 > eps2) {
        const float nl = __fsqrt_rn(len2);
        const float inv = __frcp_rn(nl);
        nrm.x *= inv;
        nrm.y *= inv;
        nrm.z *= inv;
        nrm.w *= inv;
      } else {
        nrm = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    // projectCell (optflow4d.cpp:675-710)
    float step = 0.25f;
    if (maxIter < 50) step = 0.5f;
    const float targetVal = __ldg(phiTarget + id);
    const float vn = ip16(T, a[0], a[1], a[2], a[3]);
    float dd = (vn - targetVal);
    if (nrm.x == 0.f && nrm.y == 0.f && nrm.z == 0.f && nrm.w == 0.f && isfinite(dd)) {
      // Zero normal (flat, clamped phi): every probe is p itself (p + 0 * dd),
      // so vn and the in-bounds test never change, the direction never flips,
      // the step never halves and the loop runs maxIter plain steps.
      if (maxIter > 0) {
        if (!in_bounds(d, trunc_i(p0), trunc_i(p1), trunc_i(p2), trunc_i(p3), 0)) {
          dd = 9999.f;
        } else if (vn < targetVal) {
          for (int s = 0; s < maxIter; ++s) dd += step;
        } else {
          for (int s = 0; s < maxIter; ++s) dd -= step;
        }
      }
      project_write(dst, marker, id, nrm, dd, threshPhi);
    } else if (maxIter <= 0) {
      project_write(dst, marker, id, nrm, dd, threshPhi);
    } else {
      search = true;
      S.p = make_float4(p0, p1, p2, p3);
      S.nrm = nrm;
      S.dd = dd;
      S.target = targetVal;
      S.id = (uint32_t)id;
      S.pad = 0;
    }
    }
    const unsigned want = __ballot_sync(0xffffffffu, search);
    if (want) {
      unsigned base = 0;
      if (lane == (unsigned)(__ffs(want) - 1)) base = atomicAdd(qcount, (unsigned)__popc(want));
      base = __shfl_sync(0xffffffffu, base, __ffs(want) - 1);
      if (search) queue[base + __popc(want & ((1u << lane) - 1u))] = S;
    }
  }
}

// knProjectCells, the search (projectCell, optflow4d.cpp:675-710) of the
// queued cells.  A lane pulls its next cell when its search ends, so the
// lanes of a warp stay busy whatever the cells' step counts (1 to maxIter).
// Warps take chunks of PROJ_CHUNK queue entries; within a chunk the lanes
// that need a cell take consecutive entries in lane order.  Every cell's
// arithmetic is the single-cell search's, so the results do not depend on
// which lane runs a cell.
constexpr int PROJ_CHUNK = 64;
__global__ void __launch_bounds__(128)
k_project_search(float4 *__restrict__ dst, const float *__restrict__ phiOrg,
                 float *__restrict__ marker, Dims4 d, float threshPhi, int maxIter,
                 const ProjState *__restrict__ queue, const unsigned int *__restrict__ qcount,
                 unsigned int *__restrict__ qhead) {
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  const unsigned lane = threadIdx.x & 31;
  const unsigned n = *qcount;
  const float dt = 1.0f;
  unsigned next = 0, end = 0;  // the warp's current chunk
  bool drained = false;        // the queue has no chunk left for this warp
  bool active = false;
  ProjState S;
  float T[16];
  idx_t ti = -1;
  float step = 0.f;
  int lastDir = 0, s = 0;
  for (;;) {
    unsigned need = __ballot_sync(0xffffffffu, !active);
    while (need && !drained) {
      if (next >= end) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(qhead, (unsigned)PROJ_CHUNK);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) {
          drained = true;
          break;
        }
        next = base;
        end = min(base + (unsigned)PROJ_CHUNK, n);
      }
      const unsigned k = next + __popc(need & ((1u << lane) - 1u));
      if (!active && k < end) {
        S = queue[k];
        active = true;
        ti = -1;
        step = maxIter < 50 ? 0.5f : 0.25f;
        lastDir = 0;
        s = 0;
      }
      next = min(next + (unsigned)__popc(need), end);
      need = __ballot_sync(0xffffffffu, !active);
    }
    if (!__any_sync(0xffffffffu, active)) break;
    if (active) {
    // one step of the search
    bool done = false;
    const float n0 = S.p.x + (S.nrm.x * S.dd) * dt;
    const float n1 = S.p.y + (S.nrm.y * S.dd) * dt;
    const float n2 = S.p.z + (S.nrm.z * S.dd) * dt;
    const float n3 = S.p.w + (S.nrm.w * S.dd) * dt;
    if (!in_bounds(d, trunc_i(n0), trunc_i(n1), trunc_i(n2), trunc_i(n3), 0)) {
      S.dd = 9999.f;
      done = true;
    } else {
      const AxisW b0 = axis_index(n0, d.x), b1 = axis_index(n1, d.y);
      const AxisW b2 = axis_index(n2, d.z), b3 = axis_index(n3, d.t);
      const idx_t ni = d.index(b0.b, b1.b, b2.b, b3.b);
      if (ni != ti) {
        load_taps(phiOrg, ni, sY, sZ, sT, T);
        ti = ni;
      }
      const float vn = ip16(T, b0, b1, b2, b3);
      if (vn < S.target) {
        if (lastDir < 0) step *= 0.5f;
        S.dd += step;
        lastDir = 1;
      } else {
        if (lastDir > 0) step *= 0.5f;
        S.dd -= step;
        lastDir = -1;
      }
      // (double)step < 0.1 equals step < 0.1f for every float: 0.1f is the
      // smallest float above 0.1.
      if (step < 0.1f) done = true;
    }
    if (++s >= maxIter) done = true;
    if (done) {
      project_write(dst, marker, S.id, S.nrm, S.dd, threshPhi);
      active = false;
    }
    }
  }
}

__global__ void k_zero_counters(unsigned int *c) {
  c[0] = 0;
  c[1] = 0;
}

// Queue entries: the whole box, or at least PROJ_QMIN cells and a quarter of
// the box, whichever is less; a larger box runs in t slabs of that many
// cells.
constexpr long long PROJ_QMIN = 16ll << 20;
long long project_queue_cells(Dims4 d) {
  if (d.x < 5 || d.y < 5 || d.z < 5 || d.t < 5) return 1;
  const long long vol = (long long)(d.x - 4) * (d.y - 4) * (d.z - 4);
  const long long nbox = vol * (d.t - 4);
  long long cap = nbox / 4 > PROJ_QMIN ? nbox / 4 : PROJ_QMIN;
  if (cap < vol) cap = vol;  // at least one t plane
  return cap < nbox ? cap : nbox;
}

size_t project_queue_bytes(Dims4 d) { return sizeof(ProjState) * (size_t)project_queue_cells(d); }

void launch_project_cells(float4 *dst, const float4 *vel, const float *phiOrg,
                          const float *phiTarget, float *marker, Dims4 d,
                          float threshPhi, int maxIter, void *queue, unsigned int *counters,
                          cudaStream_t s) {
  if (d.x < 5 || d.y < 5 || d.z < 5 || d.t < 5) return;
  const long long vol = (long long)(d.x - 4) * (d.y - 4) * (d.z - 4);
  const int tslab = (int)(project_queue_cells(d) / vol);  // t planes per slab
  // every block of the search resident at once: warps leave when the queue
  // is drained
  static const int per_sm = [] {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_project_search, 128, 0);
    return n < 1 ? 1 : n;
  }();
  for (int t0 = 0; t0 < d.t - 4; t0 += tslab) {
    const int nt = min(tslab, d.t - 4 - t0);
    const BoxDecoder bx = make_decoder(d.x - 4, d.y - 4, d.z - 4, 2, 2, 2, 2 + t0);
    const long long nbox = vol * nt;
    if (t0 > 0) k_zero_counters<<<1, 1, 0, s>>>(counters);
    k_project_prep<<<grid_for(nbox, 128, 16), 128, 0, s>>>(dst, vel, phiOrg, phiTarget, marker,
                                                           d, bx, (uint32_t)nbox, threshPhi,
                                                           maxIter, (ProjState *)queue, counters);
    k_project_search<<<sm_count() * per_sm, 128, 0, s>>>(dst, phiOrg, marker, d, threshPhi,
                                                         maxIter, (const ProjState *)queue,
                                                         counters, counters + 1);
  }
}

// knCvExpolBlur4d (optflow4d.cpp:613-626) fused with the preceding copy:
// unmarked interior cells get avg of the 3^4 neighbourhood, scaled by the
// double constant 1/81 and rounded back to float; others copy through.
__global__ void __launch_bounds__(NT)
k_expol_sweep(const float4 *__restrict__ in, float4 *__restrict__ out,
              const float *__restrict__ mark, Dims4 d, BoxDecoder bx) {
  const uint32_t n = (uint32_t)d.cells();
  const idx_t sY = d.x, sZ = d.sz(), sT = d.st();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    if (!in_bounds(d, i, j, k, l, 1) || __ldg(mark + q) != 0.f) {
      out[q] = __ldg(in + q);
      continue;
    }
    float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int vt = -1; vt <= 1; ++vt)
      for (int zk = -1; zk <= 1; ++zk)
        for (int yj = -1; yj <= 1; ++yj) {
          const idx_t row = (idx_t)q + vt * sT + zk * sZ + yj * sY;
#pragma unroll
          for (int xi = -1; xi <= 1; ++xi) {
            const float4 a = __ldg(in + row + xi);
            val.x += a.x;
            val.y += a.y;
            val.z += a.z;
            val.w += a.w;
          }
        }
    out[q] = make_float4(mul_inv81(val.x), mul_inv81(val.y), mul_inv81(val.z), mul_inv81(val.w));
  }
}

void launch_expol_sweep(const float4 *in, float4 *out, const float *mark,
                        Dims4 d, cudaStream_t s) {
  BoxDecoder bx = make_decoder(d.x, d.y, d.z, 0, 0, 0, 0);
  k_expol_sweep<<<grid_for(d.cells(), NT, 8), NT, 0, s>>>(in, out, mark, d, bx);
}

}  // namespace flof
