// flof_host.cu -- context, device grid pool, the FlOF multiscale driver and
// the C ABI declared in include/flof_gb300.h.
//
// The driver restates the control flow of the reference
// (source/plugin/optflow4d.cpp): opticalFlowMultiscaleTemplate :936-1173,
// opticalFlowDim :361-553, corrVelsOfTempl :737-802, gaussianBlurGeneric
// :160-174, advectCflHelper4d :1309-1321, loadAdvectTimeSlice_OptRun
// :1951-2105.  All data stays in device memory; the host only decides the
// data-dependent control (CG convergence, multistep stop rule, CFL substeps,
// extrapolation sweep count), reading those scalars back on the context
// stream.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <chrono>
#include <map>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "flof_internal.h"

using namespace flof;
using namespace fh;

namespace {

// ---------------------------------------------------------------------------
// Building blocks of the driver
// ---------------------------------------------------------------------------

// interpolGridTempl (optflow4d.cpp:40-57): factor = Real(src)/target per
// axis, offset = factor * 0.5.
void interpol_grid(flof_ctx *c, float *target, Dims4 td, const float *source, Dims4 sd,
                   int nc) {
  const int sa[4] = {sd.x, sd.y, sd.z, sd.t}, ta[4] = {td.x, td.y, td.z, td.t};
  float fac[4], off[4];
  for (int q = 0; q < 4; ++q) {
    fac[q] = (float)sa[q] / (float)ta[q];
    off[q] = (float)((double)fac[q] * 0.5);
  }
  KLP(c, KC_RESAMPLE, td.x, (td.cells() + sd.cells()) * nc * 4,
      launch_resample(target, td, source, sd, nc, make_float4(fac[0], fac[1], fac[2], fac[3]),
                        make_float4(off[0], off[1], off[2], off[3]), c->stream));
}

// max |v| of a Vec4 grid (getMaxValue, grid4d.cpp:274-277), synchronising.
float vec_max_norm(flof_ctx *c, const float4 *v, Dims4 d) {
  KLP(c, KC_REDUCE, d.x, d.cells() * 16,
      launch_reduce_minmax((const float *)v, d.cells(), 4, 0, c->fpart, c->counter + 4,
                             c->fres + 0, c->stream));
  const float m2 = read_f(c, c->fres + 0);
  return sqrtf(m2);
}

// advectCflTemplate<Grid4d<int>,...> (optflow4d.cpp:2170-2180) ->
// advectCflHelper4d (:1309-1321) with the solver dt = 1 and velFactor = 1
// (a multiplication by 1 is exact, so the velocity copy is skipped).
void advect_cfl(flof_ctx *c, Dims4 d, float cfl, const float4 *vel, float *grid, int nc) {
  if (!c->cfl_sync) {
    KLP(c, KC_REDUCE, d.x, d.cells() * 16,
        launch_reduce_minmax((const float *)vel, d.cells(), 4, 0, c->fpart, c->counter + 4,
                             c->fres + 0, c->stream));
    DBuf tmp(c, (size_t)d.cells() * nc * sizeof(float));
    KLP(c, KC_ADVECT, d.x, d.cells() * (16 + 8 * nc),
        launch_advect_cfl1(vel, grid, tmp.f(), d, nc, c->fres + 0, cfl, c->cfl_flag, c->stream));
    CK(cudaMemcpyAsync(grid, tmp.p, (size_t)d.cells() * nc * sizeof(float),
                       cudaMemcpyDeviceToDevice, c->stream));
    return;
  }
  const float orgDt = 1.0f;
  const float maxVel = vec_max_norm(c, vel, d) * orgDt;
  const int steps = trunc_f(maxVel / cfl) + 1;
  if (steps < 1 || steps > (1 << 16))
    fail(FLOF_E_NAN, "CFL substep count out of range (non-finite or huge velocities)");
  const float mdt = orgDt / (float)steps;
  DBuf tmp(c, (size_t)d.cells() * nc * sizeof(float));
  float *a = grid, *b = tmp.f();
  for (int s = 0; s < steps; ++s) {
    KLP(c, KC_ADVECT, d.x, d.cells() * (16 + 8 * nc),
        launch_advect(vel, a, b, d, nc, mdt * 1.0f, c->stream));
    float *sw = a;
    a = b;
    b = sw;
  }
  if (a != grid)
    CK(cudaMemcpyAsync(grid, a, (size_t)d.cells() * nc * sizeof(float),
                       cudaMemcpyDeviceToDevice, c->stream));
}

// calcLsDiffTempl (optflow4d.cpp:895-927), synchronising.
float ls_diff(flof_ctx *c, const float *i0, const float *i1, float *out, Dims4 d, float corr,
              int bnd) {
  if (c->strict)
    KLP(c, KC_LSDIFF, d.x, d.cells() * 8,
        launch_strict_ls_diff(i0, i1, out, d, corr, bnd, c->dres + 0, c->fres + 1, c->stream));
  else
    KLP(c, KC_LSDIFF, d.x, d.cells() * 8,
        launch_ls_diff(i0, i1, out, d, corr, bnd, c->dpart, c->counter + 5, c->dres + 0,
                         c->fres + 1, c->stream));
  return read_f(c, c->fres + 1);
}

// In-bounds weight sums of knGaussianBlur by clipping pattern: per axis the
// number of taps cut below 0 and above size-1; summed in the reference's tap
// order (t, z, y, x), skipping the cut taps.
const float *wsum_table(flof_ctx *c, float sigma, int s, const float *wtab) {
  uint32_t bits;
  memcpy(&bits, &sigma, sizeof(bits));
  auto key = std::make_pair(bits, s);
  auto it = c->wsum_cache.find(key);
  if (it != c->wsum_cache.end()) return it->second;
  const int P = s + 1, P1 = P * P;
  std::vector<float> h((size_t)P1 * P1 * P1 * P1);
  for (int ct = 0; ct < P1; ++ct)
    for (int cz = 0; cz < P1; ++cz)
      for (int cy = 0; cy < P1; ++cy)
        for (int cx = 0; cx < P1; ++cx) {
          const int lo_t = -s + ct / P, hi_t = s - ct % P;
          const int lo_z = -s + cz / P, hi_z = s - cz % P;
          const int lo_y = -s + cy / P, hi_y = s - cy % P;
          const int lo_x = -s + cx / P, hi_x = s - cx % P;
          float w = 0.f;
          for (int vt = lo_t; vt <= hi_t; ++vt)
            for (int zk = lo_z; zk <= hi_z; ++zk)
              for (int yj = lo_y; yj <= hi_y; ++yj)
                for (int xi = lo_x; xi <= hi_x; ++xi) w += wtab[vt * vt + zk * zk + yj * yj + xi * xi];
          h[((size_t)(ct * P1 + cz) * P1 + cy) * P1 + cx] = w;
        }
  float *dptr = nullptr;
  CK(cudaMalloc(&dptr, h.size() * sizeof(float)));
  // On the context's stream and waited for: a plain cudaMemcpy from pageable
  // memory runs on the legacy stream and may return before the data lands,
  // and the context's non-blocking stream is not ordered after it.
  CK(cudaMemcpyAsync(dptr, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->wsum_cache[key] = dptr;
  return dptr;
}

// gaussianBlurGeneric(a, sigma, iter = 1) (optflow4d.cpp:160-174).
void gauss_blur(flof_ctx *c, float *a, Dims4 d, int nc, float sigma, int blurType) {
  int s = trunc_d(1. * (double)sigma + 0.5);
  if (s == 0) s = 1;
  if (s > 6 || s < 0) fail(FLOF_E_ARG, "Gaussian blur radius above 6 cells is not supported");
  const size_t nb = (size_t)d.cells() * nc * sizeof(float);
  if (blurType != FLOF_BLUR_GAUSS_SEPARABLE) {
    float wtab[160];
    for (int q = 0; q <= 4 * s * s; ++q)
      wtab[q] = (float)exp((double)(-(float)q) / (2. * (double)sigma * (double)sigma));
    DBuf tmp(c, nb);
    // pass 1: a -> fresh tmp (zero ring); pass 2: tmp -> a (ring keeps the
    // original values): the state after the reference's two swaps.
    if (gauss_slab_supported(s, d)) {
      const float *ws = wsum_table(c, sigma, s, wtab);
      for (int pass = 0; pass < 2; ++pass) {
        const float *src = pass == 0 ? a : tmp.f();
        float *dst = pass == 0 ? tmp.f() : a;
        const int zb = pass == 0 ? 1 : 0;
        bool tma = false;
        if (nc == 4 && c->slab_tma)
          KLP(c, KC_BLUR, d.x, d.cells() * nc * 8,
              tma = launch_gauss_tma((const float4 *)src, (float4 *)dst, d, s, wtab, ws, zb,
                                     c->dev_err, c->stream));
        if (!tma)
          KLP(c, KC_BLUR, d.x, d.cells() * nc * 8,
              launch_gauss_slab(src, dst, d, nc, s, wtab, ws, zb, c->stream));
      }
    } else {
      KLP(c, KC_BLUR, d.x, d.cells() * nc * 8,
          launch_gauss_pass(a, tmp.f(), d, nc, s, wtab, 1, c->stream));
      KLP(c, KC_BLUR, d.x, d.cells() * nc * 8,
          launch_gauss_pass(tmp.f(), a, d, nc, s, wtab, 0, c->stream));
    }
  } else {
    float w1[8];
    for (int q = 0; q <= s; ++q)
      w1[q] = (float)exp((double)(-(float)(q * q)) / (2. * (double)sigma * (double)sigma));
    // the reference's two passes: a -> t2 (zero ring), t2 -> a (ring kept)
    DBuf t1(c, nb), t2(c, nb);
    KLP(c, KC_BLUR, d.x, d.cells() * nc * 8,
        launch_gauss_sep_pair(a, t1.f(), d, nc, 0, s, w1, 0, c->stream));
    KLP(c, KC_BLUR, d.x, d.cells() * nc * 8,
        launch_gauss_sep_pair(t1.f(), t2.f(), d, nc, 1, s, w1, 1, c->stream));
    KLP(c, KC_BLUR, d.x, d.cells() * nc * 8,
        launch_gauss_sep_pair(t2.f(), t1.f(), d, nc, 0, s, w1, 0, c->stream));
    KLP(c, KC_BLUR, d.x, d.cells() * nc * 8,
        launch_gauss_sep_pair(t1.f(), a, d, nc, 1, s, w1, 2, c->stream));
  }
}

struct OFArgs {
  float wSmooth, wEnergy, postVelBlur, cgAccuracy, resetBndWidth;
  int blurType, cgMaxIter;
  int precision = FLOF_PRECISION_FP32;
  int solver = FLOF_SOLVER_PCG;
};

// opticalFlowDim<Grid4d<Real>,Grid4d<Vec4>,4> (optflow4d.cpp:361-553).
// velIn (nullable) is the input velocity used in the rhs; the result goes
// to velOut (may alias velIn).
// PCG launch shapes for grid size d: the defaults, or (FLOF_OPT_AUTOTUNE)
// the fastest of a few candidates timed once per size on scratch buffers.
// The candidates give the same per-cell arithmetic; the grouping of the dot
// product partial sums, and so the last bits of alpha and beta, differ.
CGTune cg_tune(flof_ctx *c, Dims4 d, const OFConsts &k) {
  CGTune best;
  if (!c->autotune || d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return best;
  const std::array<int, 4> key = {d.x, d.y, d.z, d.t};
  flof_ctx *owner = c->tune_owner ? c->tune_owner : c;
  std::lock_guard<std::mutex> lock(owner->tune_mu);
  auto it = owner->tunes.find(key);
  if (it != owner->tunes.end()) return it->second;
  const size_t vb = vec_bytes(d);
  DBuf p(c, vb), g(c, vb), q(c, vb), x(c, vb), r(c, vb), stb(c, sizeof(CGState));
  CK(cudaMemsetAsync(p.p, 0, vb, c->stream));
  CK(cudaMemsetAsync(g.p, 0, vb, c->stream));
  CK(cudaMemsetAsync(x.p, 0, vb, c->stream));
  CK(cudaMemsetAsync(r.p, 0, vb, c->stream));
  // a private PCG state that never converges (acc < 0) and never divides by 0
  CGState init;
  memset(&init, 0, sizeof(init));
  init.sigma = 1.0;
  init.acc = -1.0;
  init.resIni = 1.0;
  CK(cudaMemcpyAsync(stb.p, &init, sizeof(init), cudaMemcpyHostToDevice, c->stream));
  CGState *st = (CGState *)stb.p;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto time_it = [&](auto &&launch) {
    launch();  // warm-up
    CK(cudaEventRecord(e0, c->stream));
    for (int rep = 0; rep < 3; ++rep) launch();
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    return ms;
  };
  float bt = 1e30f;
  for (int tt : {4, 8, 16}) {
    CGTune cand = best;
    cand.mv_tt = tt;
    const float ms = time_it([&] {
      launch_cg_matvec(p.v(), g.v(), q.v(), d, k, st, c->dpart, c->stream, cand);
    });
    if (ms < bt) {
      bt = ms;
      best.mv_tt = tt;
    }
  }
  bt = 1e30f;
  const int pick_tt = best.mv_tt;
  for (int ps : {4, 8, 16}) {
    CGTune cand = best;
    cand.per_sm = ps;
    const float ms = time_it([&] {
      launch_cg_update(r.v(), q.v(), g.v(), d, k, st, c->dpart, c->fpart, 1 << 30, c->stream,
                       cand);
      launch_cg_direction(x.v(), p.v(), r.v(), g.v(), d, k, st, c->stream, cand);
    });
    if (ms < bt) {
      bt = ms;
      best.per_sm = ps;
    }
  }
  best.mv_tt = pick_tt;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  owner->tunes[key] = best;
  return best;
}

// PCG iterations (GridCGOptflow4d::solve, optflow4d.cpp:304-326) from the
// state the initialisation left.  Iterations are launched in chunks without
// waiting; every kernel returns at once when the state says done.  After each
// chunk the host reads the state (into c->st_h) and sizes the next chunk from
// the observed reduction rate.
void pcg_update(flof_ctx *c, Dims4 d, const OFConsts &k, const CGTune &tu, float4 *r,
                const float4 *q, const float4 *g, const float *i1, int maxIter) {
  launch_cg_update(r, q, g, d, k, c->st, c->dpart, c->fpart, maxIter, c->stream, tu, i1);
}
void pcg_update(flof_ctx *c, Dims4 d, const OFConsts &k, const CGTune &tu, float4 *r,
                const float4 *q, const BF4 *g, const float *, int maxIter) {
  launch_cg_update(r, q, g, d, k, c->st, c->dpart, c->fpart, maxIter, c->stream, tu);
}
void pcg_direction(flof_ctx *c, Dims4 d, const OFConsts &k, const CGTune &tu, float4 *x,
                   float4 *p, const float4 *r, const float4 *g, const float *i1) {
  launch_cg_direction(x, p, r, g, d, k, c->st, c->stream, tu, i1);
}
void pcg_direction(flof_ctx *c, Dims4 d, const OFConsts &k, const CGTune &tu, float4 *x,
                   float4 *p, const float4 *r, const BF4 *g, const float *) {
  launch_cg_direction(x, p, r, g, d, k, c->st, c->stream, tu);
}

// i1: the FP32 solve's target level set; the update and direction kernels
// rebuild the preconditioner's gradient from it (null: they read g).
template <class GT>
void pcg_loop(flof_ctx *c, Dims4 d, const OFConsts &k, const CGTune &tu, float4 *x, float4 *r,
              float4 *p, float4 *q, const GT *g, int maxIter, const float *i1 = nullptr) {
  const double gb = sizeof(GT) == 8 ? 8.0 : 16.0;  // bytes of g per cell
  const double gpc = i1 ? 4.0 : gb;                 // bytes of g or i1 per cell in update/direction
  int it = 0;
  int chunk = 4;
  for (;;) {
    const int n = (maxIter - it) < chunk ? (maxIter - it) : chunk;
    for (int s = 0; s < n; ++s) {
      KLP(c, KC_MATVEC, d.x, nint(d) * (32 + gb),
          launch_cg_matvec(p, g, q, d, k, c->st, c->dpart, c->stream, tu));
      KLP(c, KC_UPDATE, d.x, nint(d) * (48 + gpc),
          pcg_update(c, d, k, tu, r, q, g, i1, maxIter));
      KLP(c, KC_DIRECTION, d.x, nint(d) * (80 + gpc), pcg_direction(c, d, k, tu, x, p, r, g, i1));
    }
    it += n;
    CK(cudaMemcpyAsync(c->st_h, c->st, sizeof(CGState), cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    if (c->st_h->done != CG_RUNNING) break;
    if (it >= maxIter) break;
    const double ratio = (double)c->st_h->resMax / c->st_h->resIni;
    const double target = c->st_h->acc / c->st_h->resIni;
    if (ratio > 0 && ratio < 1 && target > 0) {
      const double rate = log(ratio) / it;
      const double est = rate < 0 ? (log(target) - log(ratio)) / rate : 64;
      const int e = (int)(est * 1.1) + 2;
      chunk = e < 2 ? 2 : (e > 64 ? 64 : e);
    } else {
      chunk = chunk * 2 > 64 ? 64 : chunk * 2;
    }
  }
}

// The PCG with the reference's arithmetic (FLOF_OPT_STRICT): the same
// chunked launches and host checks as pcg_loop, one strict iteration per
// step.
void pcg_loop_strict(flof_ctx *c, Dims4 d, const OFConsts &k, float4 *x, float4 *r, float4 *p,
                     float4 *q, const float4 *g, int maxIter) {
  KL(c, launch_strict_init(r, g, d, k, c->st, c->stream));
  int it = 0;
  for (;;) {
    CK(cudaMemcpyAsync(c->st_h, c->st, sizeof(CGState), cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    if (c->st_h->done != CG_RUNNING || it >= maxIter) break;
    const int n = (maxIter - it) < 16 ? (maxIter - it) : 16;
    for (int s = 0; s < n; ++s)
      KLP(c, KC_MATVEC, d.x, nint(d) * 160,
          launch_strict_iteration(x, r, p, q, g, d, k, c->st, c->dpart, c->fpart, maxIter,
                                  c->stream));
    it += n;
  }
}

// Multigrid-preconditioned PCG (solver FLOF_SOLVER_MG, flof_mg.cu) from the
// state the assembly left (x = 0, r = b, resIni = signed max of b, acc =
// cgAccuracy * resIni): the stop rule is the reference's, on the same
// residual.  The plain operator then judges the result: r = b - A x is
// formed anew (FP64 row sums) and, when its signed max is above the same
// threshold, or the preconditioned solve did not converge within its
// iteration cap, the plain Jacobi-PCG continues from x to that threshold.
// Returns the status; *iters counts both solvers' iterations.
int mg_pcg(flof_ctx *c, Dims4 d, const OFConsts &k, const CGTune &tu, const OFArgs &a, float4 *x,
           float4 *r, float4 *p, float4 *q, const float4 *g, const float *i1, int *iters,
           float *res) {
  const size_t vb = vec_bytes(d);
  const std::vector<Dims4> dims = mg_level_dims(d);
  const int nl = (int)dims.size();
  std::vector<DBuf> bufs;
  std::vector<MGLevelPtrs> L(nl);
  for (int l = 0; l < nl; ++l) {
    const size_t n = (size_t)dims[l].cells();
    auto take = [&](size_t nf4) {
      bufs.emplace_back(c, nf4 * sizeof(float4));
      return bufs.back().v();
    };
    L[l].m = dims[l];
    L[l].G = take(3 * n);
    L[l].dinv = take(3 * n);
    L[l].cpl = take(n);
    L[l].b = take(n);
    L[l].x = take(n);
    L[l].r = take(n);
  }
  DBuf x0(c, vb), r0(c, vb), z(c, vb), b(c, vb);
  CK(cudaMemcpyAsync(b.p, r, vb, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemsetAsync(x0.p, 0, vb, c->stream));  // its border stays zero
  MGParams mp = c->mg;
  const double nb = (double)nint(d);
  KLP(c, KC_MG, d.x, nb * 16, launch_mg_build(g, d, L.data(), nl, k, mp, c->st, c->stream));
  int vl = nl > 1 ? nl - 1 : 0;  // the build's launches beyond the one counted
  KLP(c, KC_MG, d.x, nb * 96,
      launch_mg_vcycle(r, g, x0.v(), r0.v(), z.v(), d, L.data(), nl, k, mp, c->st, c->dpart, 1, 0,
                       c->stream, &vl));
  KLP(c, KC_DIRECTION, d.x, nb * 32, launch_mgcg_direction(p, z.v(), d, c->st, 1, c->stream));
  const int cap = a.cgMaxIter < mp.max_iter ? a.cgMaxIter : mp.max_iter;
  int it = 0, chunk = 2;
  for (;;) {
    const int n = (cap - it) < chunk ? (cap - it) : chunk;
    for (int s = 0; s < n; ++s) {
      KLP(c, KC_MATVEC, d.x, nb * 48, launch_cg_matvec(p, g, q, d, k, c->st, c->dpart, c->stream, tu));
      KLP(c, KC_UPDATE, d.x, nb * (i1 ? 116 : 128),
          launch_mgcg_update_pre(x, r, p, q, g, i1, x0.v(), d, k, mp, c->st, c->fpart, cap,
                                 c->stream));
      KLP(c, KC_MG, d.x, nb * 128,
          launch_mg_vcycle(r, g, x0.v(), r0.v(), z.v(), d, L.data(), nl, k, mp, c->st, c->dpart, 0,
                           1, c->stream, &vl));
      KLP(c, KC_DIRECTION, d.x, nb * 48, launch_mgcg_direction(p, z.v(), d, c->st, 0, c->stream));
    }
    it += n;
    CK(cudaMemcpyAsync(c->st_h, c->st, sizeof(CGState), cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    if (c->st_h->done != CG_RUNNING || it >= cap) break;
    chunk = chunk * 2 > 16 ? 16 : chunk * 2;
  }
  c->launches += vl;
  int status = c->st_h->done;
  if (status == CG_RUNNING) status = CG_MAXITER;
  int total = c->st_h->iters;
  float ret = c->st_h->retResidual;
  if (status == CG_CONVERGED || status == CG_MAXITER) {
    // the plain operator judges the result
    const double bmax = c->st_h->resIni;
    const double goal = (double)a.cgAccuracy * bmax;
    KLP(c, KC_MG, d.x, nb * 64,
        launch_mg_judge(x, b.v(), g, r, d, k, c->fpart, c->counter + 7, c->fres + 8, c->stream));
    CK(cudaMemcpyAsync(c->fres_h + 10, c->fres + 8, sizeof(float), cudaMemcpyDeviceToHost,
                       c->stream));
    sync(c);
    const double rmax = (double)c->fres_h[10];
    ret = (float)(rmax / bmax);
    if (rmax > goal) {
      // the plain Jacobi-PCG finishes from x, to the same absolute threshold
      const float acc_rel = (float)(goal / rmax);
      KLP(c, KC_ASSEMBLE, d.x, nb * 40,
          launch_cg_init_r(r, g, p, d, k, acc_rel, c->st, c->dpart, c->fpart, c->stream));
      pcg_loop(c, d, k, tu, x, r, p, q, g, a.cgMaxIter, i1);
      status = c->st_h->done;
      if (status == CG_RUNNING) status = CG_MAXITER;
      if (status == CG_EARLY) status = CG_CONVERGED;
      total += c->st_h->iters;
      ret = (float)((double)c->st_h->resMax / bmax);
      c->mg_fallbacks++;
    } else {
      status = CG_CONVERGED;
    }
  }
  if (iters) *iters = total;
  if (res) *res = ret;
  return status;
}

// Mixed-precision solve with iterative refinement.  The PCG runs on the
// matrix of the BF16-stored gradient, first to sqrt(cgAccuracy) (restarting
// from the assembly's r = b with that matrix's preconditioner).  Then, up to
// MAX_REFINE times: r = b - A x of the FP32 matrix with FP64 row sums; stop
// when the reference's criterion holds for this true residual (signed max
// <= cgAccuracy x the signed max of b); else solve the BF16 system for the
// correction just far enough to meet it (at least 10x, at most 1000x) and
// add it in FP64.  Each refinement restarts the Krylov space, so the
// accuracy is split between the solves instead of demanded of each.  The true
// relative residual ||b - A x|| / ||b|| (FP64) goes to the solve record.
void mixed_solve(flof_ctx *c, Dims4 d, const OFConsts &k, const CGTune &tu, const OFArgs &a,
                 const float4 *g, float4 *x, float4 *r, float4 *p, float4 *q, int *itersOut,
                 float *resOut) {
  constexpr int MAX_REFINE = 4;
  const size_t vb = vec_bytes(d);
  DBuf g16(c, (size_t)d.cells() * sizeof(BF4)), b(c, vb), e(c, vb);
  CK(cudaMemcpyAsync(b.p, r, vb, cudaMemcpyDeviceToDevice, c->stream));
  KLP(c, KC_ELEMWISE, d.x, d.cells() * 24,
      launch_to_bf4(g, (BF4 *)g16.p, d.cells(), c->stream));
  const BF4 *gh = (const BF4 *)g16.p;
  const float first_acc = a.cgAccuracy < 1e-2f ? sqrtf(a.cgAccuracy) : a.cgAccuracy;
  KLP(c, KC_ASSEMBLE, d.x, nint(d) * 40,
      launch_cg_init_r(r, gh, p, d, k, first_acc, c->st, c->dpart, c->fpart, c->stream));
  pcg_loop(c, d, k, tu, x, r, p, q, gh, a.cgMaxIter);
  int status = c->st_h->done;
  if (status == CG_RUNNING) status = CG_MAXITER;
  int iters = c->st_h->iters;
  const float res = c->st_h->retResidual;
  const double bmax = c->st_h->resIni;  // signed max of b
  double true_rel = -1.0;
  auto true_residual = [&]() {
    CK(cudaMemsetAsync(c->dres + 8, 0, 2 * sizeof(double), c->stream));
    KLP(c, KC_UPDATE, d.x, nint(d) * 64,
        launch_residual64(x, b.v(), g, r, d, k, c->dpart, c->counter + 7, c->dres + 8,
                          c->fres + 8, c->stream));
    CK(cudaMemcpyAsync(c->dres_h + 8, c->dres + 8, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaMemcpyAsync(c->fres_h + 10, c->fres + 8, sizeof(float), cudaMemcpyDeviceToHost,
                       c->stream));
    sync(c);
    true_rel = c->dres_h[9] > 0 ? sqrt(c->dres_h[8] / c->dres_h[9]) : 0.0;
    return (double)c->fres_h[10];
  };
  if (status == CG_CONVERGED || status == CG_MAXITER) {
    for (int ref = 0; ref < MAX_REFINE; ++ref) {
      const double rmax = true_residual();
      const double goal = (double)a.cgAccuracy * bmax;
      if (!(rmax > goal)) break;
      double inner = 0.5 * goal / rmax;  // the reduction still needed, with margin
      inner = inner > 0.1 ? 0.1 : (inner < 1e-3 ? 1e-3 : inner);
      CK(cudaMemsetAsync(e.p, 0, vb, c->stream));
      KLP(c, KC_ASSEMBLE, d.x, nint(d) * 40,
          launch_cg_init_r(r, gh, p, d, k, (float)inner, c->st, c->dpart, c->fpart, c->stream));
      pcg_loop(c, d, k, tu, e.v(), r, p, q, gh, a.cgMaxIter);
      iters += c->st_h->iters;
      KLP(c, KC_ELEMWISE, d.x, d.cells() * 48,
          launch_add_correction(x, e.v(), d.cells(), c->stream));
    }
    true_residual();
  }
  record_solve(c, d.x, iters, res, status, (float)true_rel);
  if (itersOut) *itersOut = iters;
  if (resOut) *resOut = res;
}

void optical_flow_dim(flof_ctx *c, Dims4 d, float4 *velOut, const float4 *velIn,
                      const float *i0w, const float *i1, const OFArgs &a, int *itersOut,
                      float *resOut) {
  const size_t vb = vec_bytes(d);
  DBuf g(c, vb), r(c, vb), p(c, vb), q(c, vb), x(c, vb);
  OFConsts k;
  k.mDx = (float)(1. / d.x);
  k.mDt = 1.0f;
  k.dxf = (float)(1. / (2. * (double)k.mDx));
  k.wSmooth = a.wSmooth;
  k.wEnergy = a.wEnergy;
  k.offd = -a.wSmooth * 1.0f;
  float diag = 0.f;
  diag += (float)(2 * 4) * a.wSmooth * 1.0f;
  diag += a.wEnergy;
  k.diag = diag;

  const CGTune tu = cg_tune(c, d, k);
  KLP(c, KC_ASSEMBLE, d.x, nint(d) * 8 + d.cells() * 64,
      launch_of_assemble_init(i0w, i1, velIn, g.v(), r.v(), p.v(), x.v(), d, k,
                                a.cgAccuracy, c->st, c->dpart, c->fpart, c->stream));
  if (a.solver == FLOF_SOLVER_MG && a.precision != FLOF_PRECISION_MIXED && !c->strict) {
    int iters = 0;
    float res = 0.f;
    const int status = mg_pcg(c, d, k, tu, a, x.v(), r.v(), p.v(), q.v(), g.v(), i1, &iters, &res);
    record_solve(c, d.x, iters, res, status);
    if (itersOut) *itersOut = iters;
    if (resOut) *resOut = res;
  } else if (a.precision != FLOF_PRECISION_MIXED) {
    if (c->strict)
      pcg_loop_strict(c, d, k, x.v(), r.v(), p.v(), q.v(), g.v(), a.cgMaxIter);
    else
      pcg_loop(c, d, k, tu, x.v(), r.v(), p.v(), q.v(), g.v(), a.cgMaxIter, i1);
    int status = c->st_h->done;
    if (status == CG_RUNNING) status = CG_MAXITER;  // cgMaxIter == 0
    const int iters = c->st_h->iters;
    const float res = c->st_h->retResidual;
    record_solve(c, d.x, iters, res, status);
    if (itersOut) *itersOut = iters;
    if (resOut) *resOut = res;
  } else {
    mixed_solve(c, d, k, tu, a, g.v(), x.v(), r.v(), p.v(), q.v(), itersOut, resOut);
  }

  KLP(c, KC_COPYBACK, d.x, d.cells() * 32,
      launch_of_copy_back(x.v(), velOut, d.cells(), k.mDx, c->st, c->stream));
  if (a.postVelBlur > 0.f) {
    if (a.blurType != 1 && a.blurType != FLOF_BLUR_GAUSS_SEPARABLE)
      fail(FLOF_E_ARG, "blurType must be 1 (Gaussian) or 2 (separable Gaussian)");
    gauss_blur(c, (float *)velOut, d, 4, (float)(0.5 * a.postVelBlur), a.blurType);
  }
  if (a.resetBndWidth > 0.f) {
    const int rb = trunc_f(a.resetBndWidth * (float)d.x) + 1;
    KLP(c, KC_BORDER, d.x, 0, launch_reset_outside(velOut, d, rb, c->stream));
  }
}

// corrVelsOfTempl (optflow4d.cpp:737-802).  dst receives the correction of
// the last round; vel is corrected in place.
void corr_vels_of(flof_ctx *c, Dims4 d, float4 *dst, float4 *vel, const float *phiOrg,
                  const float *phiTarget, float threshPhi, float postVelBlur,
                  float resetBndWidth, int maxIter, int blurType) {
  const float blurThreshold = 0.98f;
  const int doCvExtrapol = trunc_f(vec_max_norm(c, vel, d) + 4);
  if (doCvExtrapol > (1 << 16)) {
    check_device_errors(c);  // a kernel that gave up is the likelier cause
    fail(FLOF_E_NAN, "extrapolation sweep count out of range (non-finite or huge velocities)");
  }
  if (!(postVelBlur < 1e30f) && postVelBlur == postVelBlur)
    fail(FLOF_E_ARG, "postVelBlur must be finite");
  DBuf marker(c, real_bytes(d)), tmp(c, vec_bytes(d));
  DBuf mask(c, expol_mask_words(d) * sizeof(uint16_t));
  // the projection's queue of cells that need a search, and its two counters
  DBuf pqueue(c, project_queue_bytes(d)), pcount(c, 2 * sizeof(unsigned int));
  DBuf s2;  // the separable sweep's (x,y) box sums (blurType 2)
  int singleStep = 0;
  if (postVelBlur < blurThreshold) singleStep = 1;
  float4 *A = dst;
  while ((postVelBlur >= blurThreshold) || singleStep) {
    A = dst;
    float4 *B = tmp.v();
    CK(cudaMemsetAsync(dst, 0, vec_bytes(d), c->stream));
    CK(cudaMemsetAsync(marker.p, 0, real_bytes(d), c->stream));
    CK(cudaMemsetAsync(pcount.p, 0, 2 * sizeof(unsigned int), c->stream));
    KLP(c, KC_PROJECT, d.x, d.cells() * 44,
        launch_project_cells(dst, vel, phiOrg, phiTarget, marker.f(), d, threshPhi, maxIter,
                             pqueue.p, (unsigned int *)pcount.p, c->stream));
    if (doCvExtrapol > 0) {
      // The sweeps only rewrite unmarked interior cells; both buffers carry
      // the projected values everywhere else (the reference's tmp copy).
      CK(cudaMemcpyAsync(B, A, vec_bytes(d), cudaMemcpyDeviceToDevice, c->stream));
      if (c->slab_tma)  // the plain-load sweeps read the marker
        KLP(c, KC_EXPOL_MASK, d.x, d.cells() * 4,
            launch_expol_mask(marker.f(), (uint16_t *)mask.p, d, c->stream));
    }
    const uint16_t *keep = (const uint16_t *)mask.p;
    for (int s = 0; s < doCvExtrapol; ++s) {
      bool tma = false;
      if (blurType == FLOF_BLUR_GAUSS_SEPARABLE) {
        if (c->slab_tma)
          KLP(c, KC_EXPOL, d.x, d.cells() * 32,
              tma = launch_expol_sep_tw(A, B, keep, d, c->dev_err, c->stream));
        if (!tma) {
          if (!s2.p) s2 = DBuf(c, vec_bytes(d));
          KLP(c, KC_EXPOL, d.x, d.cells() * 68,
              launch_expol_sep(A, B, s2.v(), marker.f(), d, c->stream));
        }
      } else {
        if (c->slab_tma)
          KLP(c, KC_EXPOL, d.x, d.cells() * 32,
              tma = launch_expol_tw(A, B, keep, d, c->dev_err, c->stream));
        if (!tma)
          KLP(c, KC_EXPOL, d.x, d.cells() * 36,
              launch_expol_slab(A, B, marker.f(), d, c->stream));
      }
      std::swap(A, B);
    }
    if (postVelBlur > 1e-6f) gauss_blur(c, (float *)A, d, 4, (float)(0.5 * postVelBlur), blurType);
    const int resetBnd = trunc_f(resetBndWidth * (float)d.x) + 1;
    if (resetBndWidth > 0.f)
      KLP(c, KC_BORDER, d.x, 0,
          launch_set_bound((float *)A, d, 4, make_float4(0.f, 0.f, 0.f, 0.f), resetBnd,
                             c->stream));
    KLP(c, KC_ELEMWISE, d.x, d.cells() * 48,
        launch_add_scaled((float *)vel, (const float *)A, d.cells(), 4,
                            make_float4(-1.f, -1.f, -1.f, -1.f), c->stream));
    postVelBlur = (float)((double)postVelBlur * 0.5);
    if (singleStep > 0) singleStep--;
    if (A != dst) {
      // keep the round's correction in dst (the reference swaps pointers)
      CK(cudaMemcpyAsync(dst, A, vec_bytes(d), cudaMemcpyDeviceToDevice, c->stream));
      A = dst;
    }
  }
}

struct MSArgs {
  float wSmooth, wEnergy, postVelBlur, cgAccuracy, cfl, resetBndWidth;
  int blurType, multiStep, projSizeThresh, minGridSize, doFinalProject, cgMaxIter;
  int precision = FLOF_PRECISION_FP32;
  int warmStart = 0;
  int solver = FLOF_SOLVER_PCG;
};

// opticalFlowMultiscaleTemplate (optflow4d.cpp:936-1173).
float multiscale(flof_ctx *c, Dims4 d, float4 *vel, const float *i0, const float *i1,
                 const MSArgs &p, int level) {
  const long long n4 = d.cells() * 4;
  const int resetBnd = p.resetBndWidth > 0 ? trunc_f(p.resetBndWidth * (float)d.x) + 1 : 0;
  const float projMaxDist = 4.f;
  const int projMaxIter = 40;
  const float lsDiffFac = (float)(0.1 / 20.);
  OFArgs oa;
  oa.wSmooth = p.wSmooth;
  oa.wEnergy = p.wEnergy;
  oa.cgAccuracy = p.cgAccuracy;
  oa.resetBndWidth = p.resetBndWidth;
  oa.blurType = p.blurType;
  oa.cgMaxIter = p.cgMaxIter;
  oa.precision = p.precision;
  oa.solver = p.solver;

  DBuf i0warped(c, real_bytes(d));
  CK(cudaMemcpyAsync(i0warped.p, i0, real_bytes(d), cudaMemcpyDeviceToDevice, c->stream));

  if (d.x > p.minGridSize) {
    Dims4 sd{d.x / 2, d.y / 2, d.z / 2, d.t / 2};
    DBuf velSm(c, vec_bytes(sd)), i0Sm(c, real_bytes(sd)), i1Sm(c, real_bytes(sd));
    interpol_grid(c, i0Sm.f(), sd, i0, d, 1);
    interpol_grid(c, i1Sm.f(), sd, i1, d, 1);
    interpol_grid(c, velSm.f(), sd, (const float *)vel, d, 4);
    KL(c, launch_mult_const(velSm.f(), sd.cells(), 4, make_float4(0.5f, 0.5f, 0.5f, 0.5f),
                            c->stream));
    multiscale(c, sd, velSm.v(), i0Sm.f(), i1Sm.f(), p, level + 1);
    interpol_grid(c, (float *)vel, d, velSm.f(), sd, 4);
    KL(c, launch_mult_const((float *)vel, d.cells(), 4, make_float4(2.f, 2.f, 2.f, 2.f),
                            c->stream));
  }

  if (p.warmStart && !(d.x > p.minGridSize) && c->model) {
    // learned warm start: the coarsest level starts from the network's
    // prediction if that lowers the level's error metric, else as usual
    const int R = model_res(c->model);
    if (d.x == R && d.y == R && d.z == R && d.t == R) {
      DBuf pred(c, vec_bytes(d)), tmp(c, real_bytes(d));
      model_predict_raw(c->model, i0, i1, pred.v());
      float err[2];
      const float4 *cand[2] = {vel, pred.v()};
      for (int q = 0; q < 2; ++q) {
        CK(cudaMemcpyAsync(tmp.p, i0, real_bytes(d), cudaMemcpyDeviceToDevice, c->stream));
        advect_cfl(c, d, p.cfl, cand[q], tmp.f(), 1);
        KLP(c, KC_BORDER, d.x, 0, launch_set_bound_neumann(tmp.f(), d, 1, 0, c->stream));
        err[q] = ls_diff(c, tmp.f(), i1, nullptr, d, lsDiffFac, resetBnd);
      }
      const bool use = err[1] < err[0];
      if (use) CK(cudaMemcpyAsync(vel, pred.p, vec_bytes(d), cudaMemcpyDeviceToDevice, c->stream));
      if (c->stats) {
        c->stats->warm_start = use ? 1 : 0;
        c->stats->warm_start_err[0] = err[0];
        c->stats->warm_start_err[1] = err[1];
      }
    }
  }

  advect_cfl(c, d, p.cfl, vel, i0warped.f(), 1);
  KLP(c, KC_BORDER, d.x, 0, launch_set_bound_neumann(i0warped.f(), d, 1, 0, c->stream));
  float errCurr = ls_diff(c, i0warped.f(), i1, nullptr, d, lsDiffFac, resetBnd);

  bool doProject = false;
  int multiStep = p.multiStep;
  int doFinalProject = p.doFinalProject;
  if (d.x > p.projSizeThresh) {
    doProject = true;
    multiStep = 1;
    if (doFinalProject) doFinalProject = 0;
  }
  if (multiStep >= 10) fail(FLOF_E_ARG, "Too many of substeps!");

  if (multiStep > 1) {
    std::vector<DBuf> vs(multiStep), vs2(multiStep);
    for (int of = 0; of < multiStep; ++of) vs2[of] = DBuf(c, vec_bytes(d));
    DBuf tmpVel(c, vec_bytes(d)), i0warp2(c, real_bytes(d));
    float velBlur = p.postVelBlur;
    float errLast = errCurr;
    int ofStepsCurr = multiStep;
    for (int of = 0; of < ofStepsCurr; ++of) {
      vs[of] = DBuf(c, vec_bytes(d));
      oa.postVelBlur = velBlur;
      // a fresh zero grid: its rhs terms in vel vanish, so velIn = null
      optical_flow_dim(c, d, vs[of].v(), nullptr, i0warped.f(), i1, oa, nullptr, nullptr);
      velBlur = (float)((double)velBlur * (3. / 4.));
      if (velBlur < 2.f) velBlur = 2.f;
      for (int k = of; k >= 0; --k)
        CK(cudaMemcpyAsync(vs2[k].p, vs[k].p, vec_bytes(d), cudaMemcpyDeviceToDevice,
                           c->stream));
      for (int k = of - 1; k >= 0; --k)
        for (int l = 0; l < k; ++l) advect_cfl(c, d, p.cfl, vs2[k].v(), vs2[l].f(), 4);
      CK(cudaMemcpyAsync(tmpVel.p, vel, vec_bytes(d), cudaMemcpyDeviceToDevice, c->stream));
      for (int k = of; k >= 0; --k)
        KLP(c, KC_ELEMWISE, d.x, n4 * 12, launch_add(tmpVel.f(), vs2[k].f(), n4, c->stream));
      CK(cudaMemcpyAsync(i0warp2.p, i0, real_bytes(d), cudaMemcpyDeviceToDevice, c->stream));
      advect_cfl(c, d, p.cfl, tmpVel.v(), i0warp2.f(), 1);
      KLP(c, KC_BORDER, d.x, 0, launch_set_bound_neumann(i0warp2.f(), d, 1, 0, c->stream));
      const float errC = ls_diff(c, i0warp2.f(), i1, nullptr, d, lsDiffFac, resetBnd);
      CK(cudaMemcpyAsync(i0warped.p, i0warp2.p, real_bytes(d), cudaMemcpyDeviceToDevice,
                         c->stream));
      if (of > 0 && (double)(errC / errLast) > 0.95) {
        CK(cudaMemsetAsync(vs[of].p, 0, vec_bytes(d), c->stream));
        ofStepsCurr = of + 1;
      }
      errLast = errC;
    }
    for (int of = ofStepsCurr - 1; of >= 0; --of)
      for (int l = 0; l < of; ++l) advect_cfl(c, d, p.cfl, vs[of].v(), vs[l].f(), 4);
    for (int of = 0; of < ofStepsCurr; ++of)
      KLP(c, KC_ELEMWISE, d.x, n4 * 12, launch_add((float *)vel, vs[of].f(), n4, c->stream));
  } else {
    DBuf velCurr(c, vec_bytes(d));
    if (!doProject) {
      oa.postVelBlur = p.postVelBlur;
      optical_flow_dim(c, d, velCurr.v(), nullptr, i0warped.f(), i1, oa, nullptr, nullptr);
      KL(c, launch_add((float *)vel, velCurr.f(), n4, c->stream));
    } else {
      DBuf velTmp2(c, vec_bytes(d));
      CK(cudaMemsetAsync(velTmp2.p, 0, vec_bytes(d), c->stream));
      corr_vels_of(c, d, velCurr.v(), velTmp2.v(), i0warped.f(), i1, projMaxDist,
                   p.postVelBlur, p.resetBndWidth, projMaxIter, p.blurType);
      KL(c, launch_add((float *)vel, velTmp2.f(), n4, c->stream));
      KL(c, launch_mult_const(velCurr.f(), d.cells(), 4, make_float4(-1.f, -1.f, -1.f, -1.f),
                              c->stream));
      KL(c, launch_add((float *)vel, velCurr.f(), n4, c->stream));
    }
  }

  if (level == 0 && doFinalProject) {
    DBuf velCurr(c, vec_bytes(d));
    const float finalProjBlur = 4.f;
    corr_vels_of(c, d, velCurr.v(), vel, i0, i1, projMaxDist, finalProjBlur, p.resetBndWidth,
                 projMaxIter, p.blurType);
  }

  if (level == 0) {
    CK(cudaMemcpyAsync(i0warped.p, i0, real_bytes(d), cudaMemcpyDeviceToDevice, c->stream));
    advect_cfl(c, d, p.cfl, vel, i0warped.f(), 1);
    KLP(c, KC_BORDER, d.x, 0, launch_set_bound_neumann(i0warped.f(), d, 1, 0, c->stream));
    errCurr = ls_diff(c, i0warped.f(), i1, nullptr, d, lsDiffFac, resetBnd);
  }
  return errCurr;
}

}  // namespace

namespace flof {
void set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }
}  // namespace flof

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

FLOF_API const char *flof_version(void) { return "flof-gb300 0.1 (sm_103a)"; }
FLOF_API const char *flof_last_error(void) { return g_last_error.c_str(); }
FLOF_API const char *flof_status_string(int s) {
  switch (s) {
    case FLOF_OK: return "ok";
    case FLOF_E_ARG: return "invalid argument";
    case FLOF_E_CUDA: return "CUDA error";
    case FLOF_E_OOM: return "out of device memory";
    case FLOF_E_NAN: return "non-finite value";
    case FLOF_E_STALL: return "solve stalled";
    case FLOF_E_TIMEOUT: return "device wait timed out";
    case FLOF_E_STATE: return "call out of order";
    case FLOF_E_NOTFOUND: return "not found";
    default: return "unknown status";
  }
}

FLOF_API void flof_of_params_default(flof_of_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->wSmooth = 0.f;
  p->wEnergy = 0.f;
  p->level = 0;
  p->postVelBlur = 0.f;
  p->cgAccuracy = 1e-04f;
  p->blurType = 1;
  p->cfl = 999.f;
  p->orderTime = 1;
  p->orderSpace = 1;
  p->resetBndWidth = -1.f;
  p->multiStep = 1;
  p->projSizeThresh = 9999;
  p->minGridSize = 10;
  p->doFinalProject = 0;
  p->cgMaxIter = 1000;
}

FLOF_API void flof_of_params_flof(flof_of_params *p) {
  flof_of_params_default(p);
  if (!p) return;
  p->wSmooth = 0.001f;
  p->wEnergy = 0.0001f;
  p->cgAccuracy = 0.01f;
  p->postVelBlur = 4.f;
  p->cfl = 999.f;
  p->multiStep = 3;
  p->minGridSize = 20;
  p->doFinalProject = 1;
  p->resetBndWidth = 0.1f;
}

FLOF_API int flof_ctx_create(int device, flof_ctx **out) {
  return guarded([&] {
    need(out != nullptr, "out is NULL");
    *out = nullptr;
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    need(device >= 0 && device < n, "no such CUDA device");
    CK(cudaSetDevice(device));
    flof_ctx *c = new flof_ctx();
    c->device = device;
    try {
      CK(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
      c->stream = c->own_stream;
      const int maxBlocks = 65536;
      CK(cudaMalloc(&c->st, sizeof(CGState)));
      CK(cudaMemset(c->st, 0, sizeof(CGState)));
      CK(cudaMallocHost(&c->st_h, sizeof(CGState)));
      CK(cudaMalloc(&c->dpart, sizeof(double) * maxBlocks));
      CK(cudaMalloc(&c->fpart, sizeof(float) * maxBlocks));
      CK(cudaMalloc(&c->cfl_flag, sizeof(int)));
      CK(cudaMemset(c->cfl_flag, 0, sizeof(int)));
      CK(cudaMalloc(&c->dev_err, sizeof(int)));
      CK(cudaMemset(c->dev_err, 0, sizeof(int)));
      CK(cudaMalloc(&c->counter, sizeof(unsigned int) * 8));
      CK(cudaMemset(c->counter, 0, sizeof(unsigned int) * 8));
      CK(cudaMalloc(&c->fres, sizeof(float) * 16));
      CK(cudaMalloc(&c->dres, sizeof(double) * 16));
      CK(cudaMallocHost(&c->fres_h, sizeof(float) * 16));
      CK(cudaMallocHost(&c->dres_h, sizeof(double) * 16));
      CK(cudaDeviceSynchronize());
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
  });
}

FLOF_API int flof_ctx_destroy(flof_ctx *c) {
  if (!c) return FLOF_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  for (auto &kv : c->lats) {
    if (kv.second.vt) c->pool.put(kv.second.vt);
    if (kv.second.defo) grid_unpin(const_cast<flof_grid *>(kv.second.defo));
  }
  c->lats.clear();
  for (flof_model *m : c->models) model_orphan(m);
  c->models.clear();
  c->model = nullptr;
  // grids still alive: free their storage now and orphan the handles
  for (flof_grid *g : c->grids) {
    if (g->owned && g->d) cudaFree(g->d);
    g->d = nullptr;
    g->ctx = nullptr;
  }
  c->grids.clear();
  c->pool.release_all();
  cudaFree(c->st);
  cudaFreeHost(c->st_h);
  cudaFree(c->dpart);
  cudaFree(c->fpart);
  cudaFree(c->counter);
  cudaFree(c->cfl_flag);
  cudaFree(c->dev_err);
  cudaFree(c->fres);
  cudaFree(c->dres);
  cudaFreeHost(c->fres_h);
  cudaFreeHost(c->dres_h);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  for (auto &kv : c->wsum_cache) cudaFree(kv.second);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->copy_order) cudaEventDestroy(c->copy_order);
  for (flof_ctx *w : c->workers) flof_ctx_destroy(w);
  delete c;
  // teardown reports nothing; leave no error behind for the next call
  cudaGetLastError();
  return FLOF_OK;
}

FLOF_API int flof_ctx_synchronize(flof_ctx *c) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    CK(cudaStreamSynchronize(c->stream));
    if (c->copy_stream) CK(cudaStreamSynchronize(c->copy_stream));
  });
}

FLOF_API int flof_ctx_set_stream(flof_ctx *c, void *stream) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    CK(cudaStreamSynchronize(c->stream));
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  });
}

FLOF_API void *flof_ctx_stream(flof_ctx *c) { return c ? (void *)c->stream : nullptr; }

FLOF_API long long flof_ctx_kernel_launches(flof_ctx *c) { return c ? c->launches : 0; }

FLOF_API int flof_ctx_profile(flof_ctx *c, int enable) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    CK(cudaStreamSynchronize(c->stream));
    c->recs.clear();
    c->ev_used = 0;
    c->profiling = enable ? 1 : 0;
  });
}

FLOF_API int flof_ctx_profile_count(flof_ctx *c, int *n) {
  return guarded([&] {
    need(c != nullptr && n != nullptr, "NULL argument");
    CK(cudaStreamSynchronize(c->stream));
    *n = (int)c->recs.size();
  });
}

FLOF_API int flof_ctx_profile_record(flof_ctx *c, int i, int *cls, int *size_x, double *bytes,
                                     float *ms) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need(i >= 0 && i < (int)c->recs.size(), "record index out of range");
    const ProfRec &r = c->recs[i];
    if (cls) *cls = r.cls;
    if (size_x) *size_x = r.size_x;
    if (bytes) *bytes = r.bytes;
    if (ms) {
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, r.e0, r.e1));
      *ms = t;
    }
  });
}

FLOF_API const char *flof_kernel_class_name(int cls) {
  if (cls < 0 || cls >= KC_COUNT) return "unknown";
  return kc_names[cls];
}

FLOF_API int flof_ctx_set_option(flof_ctx *c, int option, int value) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    if (option == FLOF_OPT_CFL_SYNC) {
      need(value == 0 || value == 1, "FLOF_OPT_CFL_SYNC takes 0 or 1");
      c->cfl_force_sync = value;
    } else if (option == FLOF_OPT_STRICT) {
      need(value == 0 || value == 1, "FLOF_OPT_STRICT takes 0 or 1");
      c->strict = value;
      for (flof_ctx *w : c->workers) w->strict = value;
    } else if (option == FLOF_OPT_SLAB_TMA) {
      need(value == 0 || value == 1, "FLOF_OPT_SLAB_TMA takes 0 or 1");
      c->slab_tma = value;
      for (flof_ctx *w : c->workers) w->slab_tma = value;
    } else if (option == FLOF_OPT_AUTOTUNE) {
      need(value == 0 || value == 1, "FLOF_OPT_AUTOTUNE takes 0 or 1");
      c->autotune = value;
      for (flof_ctx *w : c->workers) w->autotune = value;
    } else {
      fail(FLOF_E_ARG, "unknown context option");
    }
  });
}

FLOF_API int flof_ctx_set_mg_params(flof_ctx *c, float omega0, float omegac, float lambda,
                                    int coarse_sweeps, int max_iter) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need(omega0 > 0.f && omega0 <= 1.f && omegac > 0.f && omegac <= 1.f,
         "the damping factors must be in (0, 1]");
    need(lambda > 0.f && lambda <= 1.f, "lambda must be in (0, 1]");
    need(coarse_sweeps >= 1 && coarse_sweeps <= 256, "coarse_sweeps must be in 1..256");
    need(max_iter >= 0, "max_iter must be >= 0");
    c->mg.max_iter = max_iter;
    c->mg.omega0 = omega0;
    c->mg.omegac = omegac;
    c->mg.lambda = lambda;
    c->mg.coarse_sweeps = coarse_sweeps;
    for (flof_ctx *w : c->workers) w->mg = c->mg;
  });
}

FLOF_API long long flof_ctx_mg_fallbacks(flof_ctx *c) { return c ? c->mg_fallbacks : 0; }

FLOF_API int flof_ctx_trim(flof_ctx *c) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    CK(cudaStreamSynchronize(c->stream));
    c->pool.trim();
    for (flof_ctx *w : c->workers) {
      CK(cudaStreamSynchronize(w->stream));
      w->pool.trim();
    }
  });
}

// ---- grids -------------------------------------------------------------------

FLOF_API int flof_grid_create(flof_ctx *c, const int dims[4], int elem, flof_grid **out) {
  return guarded([&] {
    need(c != nullptr && dims != nullptr && out != nullptr, "NULL argument");
    need(elem == FLOF_REAL || elem == FLOF_VEC4, "elem must be FLOF_REAL or FLOF_VEC4");
    for (int q = 0; q < 4; ++q) need(dims[q] >= 1, "grid extents must be positive");
    const long long cells = (long long)dims[0] * dims[1] * dims[2] * dims[3];
    need(cells < (1ll << 31), "grid too large (cells must stay below 2^31)");
    set_ctx_device(c);
    flof_grid *g = new flof_grid();
    g->ctx = c;
    memcpy(g->dims, dims, sizeof(g->dims));
    g->elem = elem;
    size_t bytes = g->bytes();
    cudaError_t e = cudaMalloc(&g->d, bytes ? bytes : 16);
    if (e != cudaSuccess) {
      cudaGetLastError();
      delete g;
      fail(FLOF_E_OOM, "device allocation of a grid failed");
    }
    g->owned = true;
    c->grids.insert(g);
    cudaError_t e2 = cudaMemsetAsync(g->d, 0, bytes, c->stream);
    if (e2 != cudaSuccess) {
      cudaFree(g->d);
      delete g;
      cuda_check(e2, "cudaMemsetAsync");
    }
    *out = g;
  });
}

FLOF_API int flof_grid_wrap(flof_ctx *c, const int dims[4], int elem, void *ptr,
                            flof_grid **out) {
  return guarded([&] {
    need(c != nullptr && dims != nullptr && out != nullptr, "NULL argument");
    need(elem == FLOF_REAL || elem == FLOF_VEC4, "elem must be FLOF_REAL or FLOF_VEC4");
    for (int q = 0; q < 4; ++q) need(dims[q] >= 1, "grid extents must be positive");
    need(ptr != nullptr, "device pointer is NULL");
    need(((uintptr_t)ptr & 15) == 0, "device pointer must be 16-byte aligned");
    const long long cells = (long long)dims[0] * dims[1] * dims[2] * dims[3];
    need(cells < (1ll << 31), "grid too large (cells must stay below 2^31)");
    flof_grid *g = new flof_grid();
    g->ctx = c;
    memcpy(g->dims, dims, sizeof(g->dims));
    g->elem = elem;
    g->d = ptr;
    g->owned = false;
    c->grids.insert(g);
    *out = g;
  });
}

FLOF_API int flof_grid_destroy(flof_grid *g) {
  if (!g) return FLOF_OK;
  if (g->pins > 0) {
    g->destroy_pending = true;
    return FLOF_OK;
  }
  grid_free(g);
  return FLOF_OK;
}

FLOF_API int flof_grid_dims(const flof_grid *g, int dims[4], int *elem) {
  return guarded([&] {
    need(g != nullptr, "grid is NULL");
    if (dims) memcpy(dims, g->dims, sizeof(g->dims));
    if (elem) *elem = g->elem;
  });
}

FLOF_API void *flof_grid_data(flof_grid *g) { return g ? g->d : nullptr; }

namespace {
// The context stream waits (on the device) for the grid's last asynchronous
// transfer.
void after_grid_copy(const flof_grid *g) {
  if (g->copy_ev) CK(cudaStreamWaitEvent(g->ctx->stream, g->copy_ev, 0));
}

// Queues a host transfer of the whole grid on the context's copy stream,
// after everything already queued on the context stream.
void grid_copy_async(flof_grid *g, void *dst, const void *src, cudaMemcpyKind kind) {
  flof_ctx *c = g->ctx;
  if (!c->copy_stream) {
    CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->copy_order, cudaEventDisableTiming));
  }
  if (!g->copy_ev) CK(cudaEventCreateWithFlags(&g->copy_ev, cudaEventDisableTiming));
  CK(cudaEventRecord(c->copy_order, c->stream));
  CK(cudaStreamWaitEvent(c->copy_stream, c->copy_order, 0));
  CK(cudaMemcpyAsync(dst, src, g->bytes(), kind, c->copy_stream));
  CK(cudaEventRecord(g->copy_ev, c->copy_stream));
}
}  // namespace

FLOF_API int flof_grid_upload(flof_grid *g, const void *host) {
  return guarded([&] {
    need_grid(g, "grid");
    need(host != nullptr, "host buffer is NULL");
    set_ctx_device(g->ctx);
    after_grid_copy(g);
    CK(cudaMemcpyAsync(g->d, host, g->bytes(), cudaMemcpyHostToDevice, g->ctx->stream));
    CK(cudaStreamSynchronize(g->ctx->stream));
  });
}

FLOF_API int flof_grid_download(const flof_grid *g, void *host) {
  return guarded([&] {
    need_grid(g, "grid");
    need(host != nullptr, "host buffer is NULL");
    set_ctx_device(g->ctx);
    after_grid_copy(g);
    CK(cudaMemcpyAsync(host, g->d, g->bytes(), cudaMemcpyDeviceToHost, g->ctx->stream));
    CK(cudaStreamSynchronize(g->ctx->stream));
  });
}

FLOF_API int flof_grid_upload_async(flof_grid *g, const void *host) {
  return guarded([&] {
    need_grid(g, "grid");
    need(host != nullptr, "host buffer is NULL");
    set_ctx_device(g->ctx);
    grid_copy_async(g, g->d, host, cudaMemcpyHostToDevice);
  });
}

FLOF_API int flof_grid_download_async(flof_grid *g, void *host) {
  return guarded([&] {
    need_grid(g, "grid");
    need(host != nullptr, "host buffer is NULL");
    set_ctx_device(g->ctx);
    grid_copy_async(g, host, g->d, cudaMemcpyDeviceToHost);
  });
}

FLOF_API int flof_grid_copy_wait(flof_grid *g) {
  return guarded([&] {
    need_grid(g, "grid");
    set_ctx_device(g->ctx);
    after_grid_copy(g);
  });
}

FLOF_API int flof_ctx_copies_sync(flof_ctx *c) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    set_ctx_device(c);
    if (c->copy_stream) CK(cudaStreamSynchronize(c->copy_stream));
  });
}

FLOF_API int flof_grid_copyFrom(flof_grid *dst, const flof_grid *src) {
  return guarded([&] {
    need_grid(dst, "dst");
    need_grid(src, "src");
    same_size(dst, src, "copyFrom");
    need(dst->elem == src->elem, "copyFrom: element types differ");
    CK(cudaMemcpyAsync(dst->d, src->d, dst->bytes(), cudaMemcpyDeviceToDevice,
                       dst->ctx->stream));
  });
}

FLOF_API int flof_grid_add(flof_grid *a, const flof_grid *b) {
  return guarded([&] {
    need_grid(a, "a");
    need_grid(b, "b");
    same_size(a, b, "add");
    need(a->elem == b->elem, "add: element types differ");
    KL(a->ctx, launch_add(a->f(), b->f(), a->cells() * a->nc(), a->ctx->stream));
  });
}

FLOF_API int flof_grid_sub(flof_grid *a, const flof_grid *b) {
  return guarded([&] {
    need_grid(a, "a");
    need_grid(b, "b");
    same_size(a, b, "sub");
    need(a->elem == b->elem, "sub: element types differ");
    KL(a->ctx, launch_sub(a->f(), b->f(), a->cells() * a->nc(), a->ctx->stream));
  });
}

FLOF_API int flof_grid_setConst(flof_grid *a, const float v[4]) {
  return guarded([&] {
    need_grid(a, "grid");
    need(v != nullptr, "value is NULL");
    KL(a->ctx, launch_set_const(a->f(), a->cells(), a->nc(), f4(v, a->nc()), a->ctx->stream));
  });
}

FLOF_API int flof_grid_addConst(flof_grid *a, const float v[4]) {
  return guarded([&] {
    need_grid(a, "grid");
    need(v != nullptr, "value is NULL");
    KL(a->ctx, launch_add_const(a->f(), a->cells(), a->nc(), f4(v, a->nc()), a->ctx->stream));
  });
}

FLOF_API int flof_grid_multConst(flof_grid *a, const float v[4]) {
  return guarded([&] {
    need_grid(a, "grid");
    need(v != nullptr, "value is NULL");
    KL(a->ctx, launch_mult_const(a->f(), a->cells(), a->nc(), f4(v, a->nc()), a->ctx->stream));
  });
}

FLOF_API int flof_grid_addScaled(flof_grid *a, const flof_grid *b, const float factor[4]) {
  return guarded([&] {
    need_grid(a, "a");
    need_grid(b, "b");
    same_size(a, b, "addScaled");
    need(a->elem == b->elem, "addScaled: element types differ");
    need(factor != nullptr, "factor is NULL");
    KL(a->ctx, launch_add_scaled(a->f(), b->f(), a->cells(), a->nc(), f4(factor, a->nc()),
                                 a->ctx->stream));
  });
}

FLOF_API int flof_grid_clear(flof_grid *a) {
  return guarded([&] {
    need_grid(a, "grid");
    CK(cudaMemsetAsync(a->d, 0, a->bytes(), a->ctx->stream));
  });
}

static int grid_reduce(flof_grid *a, int which, float *out) {
  return guarded([&] {
    need_grid(a, "grid");
    need(out != nullptr, "out is NULL");
    flof_ctx *c = a->ctx;
    if (a->nc() == 4) {
      KL(c, launch_reduce_minmax(a->f(), a->cells(), 4, which == 1 ? 1 : 0, c->fpart,
                                 c->counter + 6, c->fres + 2, c->stream));
      *out = sqrtf(read_f(c, c->fres + 2));
      return;
    }
    if (which == 2) {
      KL(c, launch_reduce_minmax(a->f(), a->cells(), 1, 1, c->fpart, c->counter + 6,
                                 c->fres + 2, c->stream));
      const float amin = read_f(c, c->fres + 2);
      KL(c, launch_reduce_minmax(a->f(), a->cells(), 1, 0, c->fpart, c->counter + 6,
                                 c->fres + 3, c->stream));
      const float amax = read_f(c, c->fres + 3);
      const float x = fabsf(amin), y = fabsf(amax);
      *out = x > y ? x : y;
      return;
    }
    KL(c, launch_reduce_minmax(a->f(), a->cells(), 1, which, c->fpart, c->counter + 6,
                               c->fres + 2, c->stream));
    *out = read_f(c, c->fres + 2);
  });
}

FLOF_API int flof_grid_getMax(flof_grid *a, float *out) { return grid_reduce(a, 0, out); }
FLOF_API int flof_grid_getMin(flof_grid *a, float *out) { return grid_reduce(a, 1, out); }
FLOF_API int flof_grid_getMaxAbs(flof_grid *a, float *out) { return grid_reduce(a, 2, out); }

FLOF_API int flof_grid_setBound(flof_grid *a, const float v[4], int w) {
  return guarded([&] {
    need_grid(a, "grid");
    need(v != nullptr, "value is NULL");
    KL(a->ctx, launch_set_bound(a->f(), a->D(), a->nc(), f4(v, a->nc()), w, a->ctx->stream));
  });
}

FLOF_API int flof_grid_setBoundNeumann(flof_grid *a, int w) {
  return guarded([&] {
    need_grid(a, "grid");
    for (int q = 0; q < 4; ++q)
      need(a->dims[q] > 2 * (w + 1), "setBoundNeumann: boundary wider than the grid");
    KL(a->ctx, launch_set_bound_neumann(a->f(), a->D(), a->nc(), w, a->ctx->stream));
  });
}

// ---- plugins --------------------------------------------------------------------

FLOF_API int flof_opticalFlowMultiscale4d(flof_ctx *c, flof_grid *vel, const flof_grid *i0,
                                          const flof_grid *i1, const flof_of_params *params,
                                          float *err, flof_solve_stats *stats) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(vel, "vel");
    need_grid(i0, "i0");
    need_grid(i1, "i1");
    need_elem(vel, FLOF_VEC4, "vel");
    need_elem(i0, FLOF_REAL, "i0");
    need_elem(i1, FLOF_REAL, "i1");
    same_size(vel, i0, "opticalFlowMultiscale4d");
    same_size(vel, i1, "opticalFlowMultiscale4d");
    need_4d(vel, "vel");
    flof_of_params def;
    flof_of_params_default(&def);
    const flof_of_params &pp = params ? *params : def;
    need(pp.blurType == 1 || pp.blurType == 2, "blurType must be 1 or 2");
    need(pp.cgMaxIter >= 0, "cgMaxIter must be >= 0");
    need(pp.cfl > 0.f, "cfl must be positive");
    need(pp.precision == FLOF_PRECISION_FP32 || pp.precision == FLOF_PRECISION_MIXED,
         "precision must be FLOF_PRECISION_FP32 or FLOF_PRECISION_MIXED");
    need(pp.solver == FLOF_SOLVER_PCG || pp.solver == FLOF_SOLVER_MG,
         "solver must be FLOF_SOLVER_PCG or FLOF_SOLVER_MG");
    set_ctx_device(c);
    const auto t0 = std::chrono::steady_clock::now();
    flof_solve_stats local;
    memset(&local, 0, sizeof(local));
    local.warm_start = -1;
    c->stats = &local;
    const int syncs0 = c->syncs;
    MSArgs m;
    m.wSmooth = pp.wSmooth;
    m.wEnergy = pp.wEnergy;
    m.postVelBlur = pp.postVelBlur;
    m.cgAccuracy = pp.cgAccuracy;
    m.cfl = pp.cfl;
    m.resetBndWidth = pp.resetBndWidth;
    m.blurType = pp.blurType;
    m.multiStep = pp.multiStep;
    m.projSizeThresh = pp.projSizeThresh;
    m.minGridSize = pp.minGridSize;
    m.doFinalProject = pp.doFinalProject;
    m.cgMaxIter = pp.cgMaxIter;
    m.precision = pp.precision;
    m.warmStart = pp.warmStart;
    m.solver = pp.solver;
    float e;
    try {
      // speculative pass: CFL substep counts checked on the device
      DBuf vel_in(c, vel->bytes());
      CK(cudaMemcpyAsync(vel_in.p, vel->d, vel->bytes(), cudaMemcpyDeviceToDevice, c->stream));
      CK(cudaMemsetAsync(c->cfl_flag, 0, sizeof(int), c->stream));
      c->cfl_sync = c->cfl_force_sync;
      e = multiscale(c, vel->D(), vel->v(), i0->f(), i1->f(), m, pp.level);
      int flag = 0;
      CK(cudaMemcpyAsync(c->fres_h + 8, c->cfl_flag, sizeof(int), cudaMemcpyDeviceToHost,
                         c->stream));
      CK(cudaStreamSynchronize(c->stream));
      memcpy(&flag, c->fres_h + 8, sizeof(int));
      if (flag) {
        // some advection needed more than one CFL substep: redo the call
        // with host-side substep counts
        memset(&local, 0, sizeof(local));
        local.warm_start = -1;
        CK(cudaMemcpyAsync(vel->d, vel_in.p, vel->bytes(), cudaMemcpyDeviceToDevice, c->stream));
        c->cfl_sync = 1;
        e = multiscale(c, vel->D(), vel->v(), i0->f(), i1->f(), m, pp.level);
        c->cfl_sync = 0;
        CK(cudaStreamSynchronize(c->stream));
      }
    } catch (...) {
      c->stats = nullptr;
      c->cfl_sync = 0;
      throw;
    }
    c->stats = nullptr;
    check_device_errors(c);
    local.err_final = e;
    local.syncs = c->syncs - syncs0;
    local.seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (err) *err = e;
    if (stats) *stats = local;
  });
}

FLOF_API int flof_opticalFlow4d(flof_ctx *c, flof_grid *vel, const flof_grid *i0,
                                const flof_grid *i1, float wSmooth, float wEnergy,
                                float postVelBlur, float cgAccuracy, int blurType,
                                float resetBndWidth, int cgMaxIter, int *iterations,
                                float *residual) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(vel, "vel");
    need_grid(i0, "i0");
    need_grid(i1, "i1");
    need_elem(vel, FLOF_VEC4, "vel");
    need_elem(i0, FLOF_REAL, "i0");
    need_elem(i1, FLOF_REAL, "i1");
    same_size(vel, i0, "opticalFlow4d");
    same_size(vel, i1, "opticalFlow4d");
    need_4d(vel, "vel");
    need(blurType == 1 || blurType == 2, "blurType must be 1 or 2");
    set_ctx_device(c);
    OFArgs a;
    a.wSmooth = wSmooth;
    a.wEnergy = wEnergy;
    a.postVelBlur = postVelBlur;
    a.cgAccuracy = cgAccuracy;
    a.resetBndWidth = resetBndWidth;
    a.blurType = blurType;
    a.cgMaxIter = cgMaxIter;
    // the input vel enters the rhs; the result replaces it
    DBuf vin(c, vel->bytes());
    CK(cudaMemcpyAsync(vin.p, vel->d, vel->bytes(), cudaMemcpyDeviceToDevice, c->stream));
    optical_flow_dim(c, vel->D(), vel->v(), vin.v(), i0->f(), i1->f(), a, iterations, residual);
    check_device_errors(c);
  });
}

FLOF_API int flof_corrVelsOf4d(flof_ctx *c, flof_grid *dst, flof_grid *vel,
                               const flof_grid *phiOrg, const flof_grid *phiCurr,
                               const flof_grid *phiTarget, float threshPhi, float threshNorm,
                               float postVelBlur, float resetBndWidth, int maxIter) {
  (void)phiCurr;
  (void)threshNorm;
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(dst, "dst");
    need_grid(vel, "vel");
    need_grid(phiOrg, "phiOrg");
    need_grid(phiTarget, "phiTarget");
    need_elem(dst, FLOF_VEC4, "dst");
    need_elem(vel, FLOF_VEC4, "vel");
    need_elem(phiOrg, FLOF_REAL, "phiOrg");
    need_elem(phiTarget, FLOF_REAL, "phiTarget");
    same_size(dst, vel, "corrVelsOf4d");
    same_size(vel, phiOrg, "corrVelsOf4d");
    same_size(vel, phiTarget, "corrVelsOf4d");
    need_4d(vel, "vel");
    set_ctx_device(c);
    corr_vels_of(c, vel->D(), dst->v(), vel->v(), phiOrg->f(), phiTarget->f(), threshPhi,
                 postVelBlur, resetBndWidth, maxIter, 1);
    check_device_errors(c);
  });
}

FLOF_API int flof_gaussianBlur4d(flof_ctx *c, flof_grid *a, float sigma, int blurType) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(a, "grid");
    need_4d(a, "grid");
    need(blurType == 1 || blurType == 2, "blurType must be 1 or 2");
    set_ctx_device(c);
    gauss_blur(c, a->f(), a->D(), a->nc(), sigma, blurType);
    check_device_errors(c);
  });
}

FLOF_API int flof_advect4d(flof_ctx *c, const flof_grid *vel, flof_grid *grid, float dtFac) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(vel, "vel");
    need_grid(grid, "grid");
    need_elem(vel, FLOF_VEC4, "vel");
    same_size(vel, grid, "advect4d");
    need_4d(vel, "vel");
    set_ctx_device(c);
    const float dt = 1.0f * dtFac;
    DBuf fwd(c, grid->bytes());
    KLP(c, KC_ADVECT, grid->dims[0], grid->cells() * (16 + 8 * grid->nc()),
        launch_advect(vel->v(), grid->f(), fwd.f(), grid->D(), grid->nc(), dt, c->stream));
    CK(cudaMemcpyAsync(grid->d, fwd.p, grid->bytes(), cudaMemcpyDeviceToDevice, c->stream));
  });
}

FLOF_API int flof_calcLsDiff4d(flof_ctx *c, const flof_grid *i0, const flof_grid *i1,
                               flof_grid *out, float correction, int bnd, float *result) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(i0, "i0");
    need_grid(i1, "i1");
    need_elem(i0, FLOF_REAL, "i0");
    need_elem(i1, FLOF_REAL, "i1");
    same_size(i0, i1, "calcLsDiff4d");
    if (out) {
      need_elem(out, FLOF_REAL, "out");
      same_size(i0, out, "calcLsDiff4d");
    }
    // a bnd that leaves no cells gives the reference's 0 * (1 / count)
    need(bnd >= 0 && bnd <= (1 << 20), "calcLsDiff4d: bnd must be in [0, 2^20]");
    set_ctx_device(c);
    const float r = ls_diff(c, i0->f(), i1->f(), out ? out->f() : nullptr, i0->D(), correction,
                            bnd);
    if (result) *result = r;
  });
}

static int interpolate_common(flof_ctx *c, flof_grid *target, const flof_grid *source,
                              const float *offset, const float *scale, const float *size,
                              int elem) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(target, "target");
    need_grid(source, "source");
    need_elem(target, elem, "target");
    need_elem(source, elem, "source");
    need_4d(source, "source");
    set_ctx_device(c);
    const float zero[4] = {0, 0, 0, 0}, one[4] = {1, 1, 1, 1}, neg[4] = {-1, -1, -1, -1};
    const float *o = offset ? offset : zero, *s = scale ? scale : one, *z = size ? size : neg;
    float s1[4], s2[4], fac[4], off[4];
    for (int q = 0; q < 4; ++q) {
      s1[q] = (float)source->dims[q];
      s2[q] = (float)target->dims[q];
      off[q] = o[q];
    }
    grid_factor4d(s1, s2, z, s, fac, off);
    KL(c, launch_resample(target->f(), target->D(), source->f(), source->D(), target->nc(),
                          make_float4(fac[0], fac[1], fac[2], fac[3]),
                          make_float4(off[0], off[1], off[2], off[3]), c->stream));
  });
}

FLOF_API int flof_interpolateGrid4d(flof_ctx *c, flof_grid *target, const flof_grid *source,
                                    const float offset[4], const float scale[4],
                                    const float size[4]) {
  return interpolate_common(c, target, source, offset, scale, size, FLOF_REAL);
}

FLOF_API int flof_interpolateGrid4dVec(flof_ctx *c, flof_grid *target, const flof_grid *source,
                                       const float offset[4], const float scale[4],
                                       const float size[4]) {
  return interpolate_common(c, target, source, offset, scale, size, FLOF_VEC4);
}

FLOF_API int flof_deform4d(flof_ctx *c, flof_grid *out, const flof_grid *i0,
                           const flof_grid *i1, const flof_grid *vel, const flof_grid *velInv,
                           float alpha, float alphaInv, int twoway) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(out, "out");
    need_grid(i0, "i0");
    need_grid(vel, "vel");
    need_elem(out, FLOF_REAL, "out");
    need_elem(i0, FLOF_REAL, "i0");
    need_elem(vel, FLOF_VEC4, "vel");
    same_size(out, i0, "deform4d");
    same_size(out, vel, "deform4d");
    need_4d(out, "out");
    need(twoway >= 0 && twoway <= 2, "twoway must be 0, 1 or 2");
    set_ctx_device(c);
    const Dims4 d = out->D();
    if (twoway == 1) {
      need_grid(i1, "i1");
      need_grid(velInv, "velInv");
      need_elem(i1, FLOF_REAL, "i1");
      need_elem(velInv, FLOF_VEC4, "velInv");
      same_size(out, i1, "deform4d");
      same_size(out, velInv, "deform4d");
      need(out->d != i0->d && out->d != i1->d, "deform4d: out must not alias the inputs");
      KLP(c, KC_DEFORM, d.x, d.cells() * 44,
          launch_deform_twoway(vel->v(), velInv->v(), i0->f(), i1->f(), out->f(), d, alpha,
                                 alphaInv, c->stream));
      return;
    }
    need(out->d != i0->d, "deform4d: out must not alias i0");
    KLP(c, KC_ADVECT, d.x, d.cells() * 24,
        launch_advect(vel->v(), i0->f(), out->f(), d, 1, 1.0f * alpha, c->stream));
    if (twoway == 2) {
      need_grid(i1, "i1");
      same_size(out, i1, "deform4d");
      KL(c, launch_mult_const(out->f(), d.cells(), 1, make_float4(alphaInv, 0, 0, 0), c->stream));
      KL(c, launch_add_scaled(out->f(), i1->f(), d.cells(), 1, make_float4(alpha, 0, 0, 0),
                              c->stream));
    }
  });
}

// ---- mode-3 slice application ---------------------------------------------------------

FLOF_API int flof_loadAdvectTimeSlice_OptInit(flof_ctx *c, int id, const flof_grid *defo,
                                              int useDefoVols, int doAligned,
                                              float partialLoadFac) {
  (void)doAligned;
  (void)partialLoadFac;
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(defo, "defo");
    need_elem(defo, FLOF_VEC4, "defo");
    need(!useDefoVols, "deformation volumes (useDefoVols) are not supported");
    // the trilinear slice sample reads a 2x2x2 neighbourhood
    need(defo->dims[0] >= 2 && defo->dims[1] >= 2 && defo->dims[2] >= 2 && defo->dims[3] >= 1,
         "Invalid src size of the deformation (x, y, z extents must be at least 2)");
    set_ctx_device(c);
    LatsData &L = c->lats[id];
    if (L.vt) c->pool.put(L.vt);
    if (L.defo) grid_unpin(const_cast<flof_grid *>(L.defo));
    const_cast<flof_grid *>(defo)->pins++;
    L.defo = defo;
    L.vt = c->pool.get((size_t)defo->dims[0] * defo->dims[1] * defo->dims[2] * sizeof(float4));
    L.lastT = -1;
  });
}

// OptInit with the deformation named by a .uni file (the reference's call):
// the whole file is loaded into a device grid that the context owns and
// frees at Finish.
FLOF_API int flof_loadAdvectTimeSlice_OptInitFile(flof_ctx *c, int id, const char *fname,
                                                  int useDefoVols, int doAligned,
                                                  float partialLoadFac) {
  flof_grid *g = nullptr;
  const int st = guarded([&] {
    need(c != nullptr && fname != nullptr, "NULL argument");
    need(!useDefoVols, "deformation volumes (useDefoVols) are not supported");
    const UniInfo u = uni_info(fname);
    need(u.is4d && u.bytesPerElement == 16,
         std::string(fname) + " is not a 4D Vec4 (M4T2) deformation file");
    const int dims[4] = {u.dims[0], u.dims[1], u.dims[2], u.dims[3]};
    if (flof_grid_create(c, dims, FLOF_VEC4, &g) != FLOF_OK) fail(FLOF_E_OOM, g_last_error);
    uni_load(g, fname);
  });
  if (st != FLOF_OK) {
    if (g) flof_grid_destroy(g);
    return st;
  }
  const int st2 = flof_loadAdvectTimeSlice_OptInit(c, id, g, useDefoVols, doAligned,
                                                   partialLoadFac);
  // OptInit pinned g; the destroy is deferred until Finish unpins it
  flof_grid_destroy(g);
  return st2;
}

FLOF_API int flof_loadAdvectTimeSlice_Finish(flof_ctx *c, int id) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    auto it = c->lats.find(id);
    if (it == c->lats.end()) return;
    CK(cudaStreamSynchronize(c->stream));
    if (it->second.vt) c->pool.put(it->second.vt);
    if (it->second.defo) grid_unpin(const_cast<flof_grid *>(it->second.defo));
    c->lats.erase(it);
  });
}

namespace {

struct SliceSetup {
  float sf[4], off2[4];
  int t, tp1;
  float tw;
};

// The size/offset arithmetic of loadAdvectTimeSlice_OptRun
// (optflow4d.cpp:1961-1985).
SliceSetup slice_setup(const flof_grid *defo, const flof_grid *phi, float time,
                       float loadTimeScale, const float *defoOffset, const float *defoScale,
                       const float *overrideSize) {
  SliceSetup S;
  const float dim4[4] = {(float)defo->dims[0], (float)defo->dims[1], (float)defo->dims[2],
                         (float)defo->dims[3]};
  int ds[4] = {phi->dims[0], phi->dims[1], phi->dims[2], phi->dims[3]};
  if (overrideSize && overrideSize[0] > 0.f)
    for (int q = 0; q < 4; ++q) ds[q] = trunc_f(overrideSize[q]);
  float defoSize[4], neg1[4] = {-1, -1, -1, -1}, one[4] = {1, 1, 1, 1};
  for (int q = 0; q < 4; ++q) {
    defoSize[q] = (float)ds[q];
    S.off2[q] = defoOffset ? defoOffset[q] : 0.f;
  }
  grid_factor4d(dim4, defoSize, neg1, defoScale ? defoScale : one, S.sf, S.off2);
  const float srcTime = (float)((double)(time * S.sf[3] * loadTimeScale + S.off2[3]) - 0.5);
  int t = trunc_f(srcTime);
  int tp1 = t + 1;
  S.tw = srcTime - (float)t;
  const int dimT = defo->dims[3];
  if (t > dimT - 1) t = dimT - 1;
  if (tp1 > dimT - 1) tp1 = dimT - 1;
  need(t >= 0 && tp1 >= 0, "loadAdvectTimeSlice: time maps before the first deformation slice");
  S.t = t;
  S.tp1 = tp1;
  return S;
}

void blend_vt(flof_ctx *c, LatsData &L, const SliceSetup &S, int zeroVel) {
  const flof_grid *defo = L.defo;
  const long long slice = (long long)defo->dims[0] * defo->dims[1] * defo->dims[2];
  const float4 *base = defo->v();
  if (zeroVel) {
    CK(cudaMemsetAsync(L.vt, 0, slice * sizeof(float4), c->stream));
  } else {
    KLP(c, KC_BLEND, defo->dims[0], slice * 48,
        launch_blend_slices(base + (long long)S.t * slice, base + (long long)S.tp1 * slice,
                              (float4 *)L.vt, slice, 1.0f - S.tw, S.tw, c->stream));
  }
  L.lastT = S.t;
}

// Both directions' blends of a two-way frame (equal deformation sizes) in
// one launch.
void blend_vt2(flof_ctx *c, LatsData &L0, const SliceSetup &S0, LatsData &L1,
               const SliceSetup &S1) {
  const flof_grid *d0 = L0.defo, *d1 = L1.defo;
  const long long slice = (long long)d0->dims[0] * d0->dims[1] * d0->dims[2];
  KLP(c, KC_BLEND, d0->dims[0], 2 * slice * 48,
      launch_blend_slices2(d0->v() + (long long)S0.t * slice, d0->v() + (long long)S0.tp1 * slice,
                           (float4 *)L0.vt, 1.0f - S0.tw, S0.tw,
                           d1->v() + (long long)S1.t * slice, d1->v() + (long long)S1.tp1 * slice,
                           (float4 *)L1.vt, 1.0f - S1.tw, S1.tw, slice, c->stream));
  L0.lastT = S0.t;
  L1.lastT = S1.t;
}

LatsData &lats_of(flof_ctx *c, int id) {
  auto it = c->lats.find(id);
  if (it == c->lats.end() || !it->second.defo)
    fail(FLOF_E_STATE, "Load-advect data id " + std::to_string(id) + " not initialized!");
  need(it->second.defo->ctx != nullptr,
       "the deformation grid of load-advect id " + std::to_string(id) +
           " belongs to a destroyed context");
  return it->second;
}

}  // namespace

FLOF_API int flof_loadAdvectTimeSlice_OptRun(
    flof_ctx *c, int id, flof_grid *dst, const flof_grid *phi, float time, float blendAlpha,
    float loadTimeScale, const float defoOffset[4], const float defoScale[4],
    const float defoFactor[4], const float overrideSize[4], float overrideTimeOff, int zeroVel,
    float thirdAlpha, int bordSkip, float fourthAlpha, float defoAniFac) {
  (void)thirdAlpha;
  (void)fourthAlpha;
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(dst, "dst");
    need_grid(phi, "phi");
    need_elem(dst, FLOF_REAL, "dst");
    need_elem(phi, FLOF_REAL, "phi");
    need(dst->dims[3] == 1, "dst must be a 3D grid (t extent 1)");
    need_4d(phi, "phi");
    set_ctx_device(c);
    LatsData &L = lats_of(c, id);
    const SliceSetup S =
        slice_setup(L.defo, phi, time, loadTimeScale, defoOffset, defoScale, overrideSize);
    blend_vt(c, L, S, zeroVel);
    const float one[4] = {1, 1, 1, 1};
    const float *dfac = defoFactor ? defoFactor : one;
    const float4 df = make_float4(dfac[0] * defoAniFac, dfac[1] * defoAniFac,
                                  dfac[2] * defoAniFac, dfac[3] * defoAniFac);
    KLP(c, KC_LOOKUP, dst->dims[0], dst->cells() * 8,
        launch_lookup_slice(dst->f(), dst->dims[0], dst->dims[1], dst->dims[2], phi->f(),
                              phi->D(), time + overrideTimeOff, blendAlpha,
                              (const float4 *)L.vt, L.defo->dims[0], L.defo->dims[1],
                              L.defo->dims[2], make_float4(S.sf[0], S.sf[1], S.sf[2], 0.f),
                              make_float4(S.off2[0], S.off2[1], S.off2[2], 0.f), df, bordSkip,
                              c->stream));
  });
}

// loadAdvectTimeSlice (optflow4d.cpp:1671-1760), the non-optimised twin of
// OptRun: the deformation comes from `defo` (device Vec4 grid) or, when defo
// is NULL, from slices t and t+1 of the .uni file fname; the lookup covers
// the bnd = 1 box of dst (bordSkip and thirdAlpha are not supported by the
// reference either).
FLOF_API int flof_loadAdvectTimeSlice(flof_ctx *c, const flof_grid *defo, const char *fname,
                                      flof_grid *dst, const flof_grid *phi, float time,
                                      float blendAlpha, float loadTimeScale,
                                      const float defoOffset[4], const float defoScale[4],
                                      const float defoFactor[4], const float overrideSize[4],
                                      float overrideTimeOff, int zeroVel, float defoAniFac) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need(defo != nullptr || fname != nullptr, "either defo or fname is required");
    need_grid(dst, "dst");
    need_grid(phi, "phi");
    need_elem(dst, FLOF_REAL, "dst");
    need_elem(phi, FLOF_REAL, "phi");
    need(dst->dims[3] == 1, "dst must be a 3D grid (t extent 1)");
    need_4d(phi, "phi");
    set_ctx_device(c);
    // a stand-in grid with the deformation's extents (file mode) for the
    // size arithmetic
    flof_grid shape;
    if (defo) {
      need_grid(defo, "defo");
      need_elem(defo, FLOF_VEC4, "defo");
      shape = *defo;
    } else {
      const UniInfo u = uni_info(fname);
      need(u.is4d && u.bytesPerElement == 16,
           std::string(fname) + " is not a 4D Vec4 (M4T2) deformation file");
      memcpy(shape.dims, u.dims, sizeof(shape.dims));
      shape.elem = FLOF_VEC4;
      shape.ctx = c;
    }
    need(shape.dims[0] >= 2 && shape.dims[1] >= 2 && shape.dims[2] >= 2,
         "Invalid src size of the deformation");
    const SliceSetup S =
        slice_setup(&shape, phi, time, loadTimeScale, defoOffset, defoScale, overrideSize);
    const long long slice = (long long)shape.dims[0] * shape.dims[1] * shape.dims[2];
    DBuf vt(c, slice * sizeof(float4));
    const float4 *v1, *v2;
    DBuf s1, s2;
    if (defo) {
      v1 = defo->v() + (long long)S.t * slice;
      v2 = defo->v() + (long long)S.tp1 * slice;
    } else {
      // readGrid4dUni(fname, NULL, t, &v1) and (.., tp1, &v2)
      s1 = DBuf(c, slice * sizeof(float4));
      s2 = DBuf(c, slice * sizeof(float4));
      flof_grid g1 = shape, g2 = shape;
      g1.dims[3] = g2.dims[3] = 1;
      g1.d = s1.p;
      g2.d = s2.p;
      g1.owned = g2.owned = false;
      uni_read_slice(&g1, fname, S.t);
      uni_read_slice(&g2, fname, S.tp1);
      v1 = s1.v();
      v2 = s2.v();
    }
    if (zeroVel) {
      CK(cudaMemsetAsync(vt.p, 0, slice * sizeof(float4), c->stream));
    } else {
      KLP(c, KC_BLEND, shape.dims[0], slice * 48,
          launch_blend_slices(v1, v2, vt.v(), slice, 1.0f - S.tw, S.tw, c->stream));
    }
    const float one[4] = {1, 1, 1, 1};
    const float *dfac = defoFactor ? defoFactor : one;
    const float4 df = make_float4(dfac[0] * defoAniFac, dfac[1] * defoAniFac,
                                  dfac[2] * defoAniFac, dfac[3] * defoAniFac);
    KLP(c, KC_LOOKUP, dst->dims[0], dst->cells() * 8,
        launch_lookup_slice(dst->f(), dst->dims[0], dst->dims[1], dst->dims[2], phi->f(),
                            phi->D(), time + overrideTimeOff, blendAlpha, vt.v(),
                            shape.dims[0], shape.dims[1], shape.dims[2],
                            make_float4(S.sf[0], S.sf[1], S.sf[2], 0.f),
                            make_float4(S.off2[0], S.off2[1], S.off2[2], 0.f), df, 0, c->stream,
                            1));
    CK(cudaStreamSynchronize(c->stream));
  });
}

FLOF_API int flof_loadAdvectTimeSlice_OptRunTwoway(
    flof_ctx *c, int id0, int id1, flof_grid *dst, const flof_grid *phi0,
    const flof_grid *phi1, float time, float blendAlpha, float alphaInv, float loadTimeScale,
    const float defoOffset[4], const float defoScale[4], const float defoFactor[4],
    const float overrideSize[4], float overrideTimeOff, int bordSkip, float defoAniFac) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need_grid(dst, "dst");
    need_grid(phi0, "phi0");
    need_grid(phi1, "phi1");
    need_elem(dst, FLOF_REAL, "dst");
    need(dst->dims[3] == 1, "dst must be a 3D grid (t extent 1)");
    same_size(phi0, phi1, "OptRunTwoway");
    need_4d(phi0, "phi0");
    set_ctx_device(c);
    LatsData &L0 = lats_of(c, id0);
    LatsData &L1 = lats_of(c, id1);
    need(L0.defo->dims[0] == L1.defo->dims[0] && L0.defo->dims[1] == L1.defo->dims[1] &&
             L0.defo->dims[2] == L1.defo->dims[2] && L0.defo->dims[3] == L1.defo->dims[3],
         "OptRunTwoway: both deformations must have the same size");
    const SliceSetup S0 =
        slice_setup(L0.defo, phi0, time, loadTimeScale, defoOffset, defoScale, overrideSize);
    const SliceSetup S1 =
        slice_setup(L1.defo, phi1, time, loadTimeScale, defoOffset, defoScale, overrideSize);
    if (&L0 != &L1) {
      blend_vt2(c, L0, S0, L1, S1);
    } else {  // one data set for both directions: the second blend wins, as in sequence
      blend_vt(c, L0, S0, 0);
      blend_vt(c, L1, S1, 0);
    }
    const float one[4] = {1, 1, 1, 1};
    const float *dfac = defoFactor ? defoFactor : one;
    const float4 df = make_float4(dfac[0] * defoAniFac, dfac[1] * defoAniFac,
                                  dfac[2] * defoAniFac, dfac[3] * defoAniFac);
    KLP(c, KC_LOOKUP, dst->dims[0], dst->cells() * 12,
        launch_lookup_slice_twoway(
              dst->f(), dst->dims[0], dst->dims[1], dst->dims[2], phi0->f(), phi1->f(),
              phi0->D(), time + overrideTimeOff, blendAlpha, alphaInv, (const float4 *)L0.vt,
              (const float4 *)L1.vt, L0.defo->dims[0], L0.defo->dims[1], L0.defo->dims[2],
              make_float4(S0.sf[0], S0.sf[1], S0.sf[2], 0.f),
              make_float4(S0.off2[0], S0.off2[1], S0.off2[2], 0.f), df, bordSkip, c->stream));
  });
}

}  // extern "C"
