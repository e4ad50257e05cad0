/*
 * flof_oracle.c -- CPU restatement of the FlOF hot path of thunil/ofblend.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle for the
 * GB300 library in ofblend_gb300/.  Only tests/, __graft_entry__.smoke() and
 * the cpu_baseline / reference legs of bench.py may load it, and only as the
 * oracle the GPU results are compared with or as the timed CPU baseline.  The
 * product never calls it.
 *
 * What it is: a from-scratch C restatement of the reference's algorithm,
 * following the reference's operation order so that per-cell results can be
 * compared bit for bit.  Every function cites the reference file:line it
 * restates (paths relative to the reference project root).  It is compiled
 * twice: with REAL = float (the reference's default "fp1" build) and with
 * REAL = double (the reference's "fp2" build, -DDOUBLEPRECISION), always with
 * -ffp-contract=off so that no multiply-add is fused (the reference's x86
 * build emits no FMA; on aarch64 GCC would contract by default).
 *
 * Parity status:
 *   - Grid4d arithmetic (setConst/addConst/multConst/copyFrom/add/addScaled,
 *     getMaxAbs) is pinned against the closed-form constants of the
 *     reference test tools/tests/test_0032_grid4dop.py:54-115.
 *   - interpolateGrid4d / interpolateGrid4dVec is checked against the
 *     properties exercised by tools/tests/test_0042_interpol4d.py:95-140
 *     (the test's golden grids are not shipped with the reference).
 *   - Everything else (assembly, PCG, blur, projection, multiscale driver,
 *     slice lookup): parity unpinned.  The reference's kernels need code
 *     generated by its own source preprocessor (the files under
 *     source/preprocessor), so
 *     they cannot be compiled from their source files alone, and the
 *     reference's tests never run the optical-flow solve
 *     (tools/tests/ofCheckerboardTest.py:59 sets doRunOf = 0).
 *
 * Layout conventions (source/grid4d.h:92-97): a 4D grid of size (X,Y,Z,T) is
 * stored x-fastest, idx = i + X*j + X*Y*k + X*Y*Z*t.  Vec4 grids store four
 * REAL per cell, interleaved (x,y,z,t).
 *
 * Loop conventions (source/kernel.cpp:38-46, preprocessor/codegen_kernel.cpp
 * :124-131): a KERNEL(fourd, bnd=b) visits every cell with b <= c < size-b in
 * all four dimensions.  Kernels that write a fresh output grid leave the
 * unvisited ring at zero (the Grid4d constructor zero-fills, grid4d.cpp:82).
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef ORC_DOUBLE
typedef double REAL;
#define R_SQRT sqrt
#define R_FABS fabs
#define R_BIG DBL_MAX
#define VEC_EPS 1e-10 /* source/util/vectorbase.h:57 */
#define ORC_SYM(name) orc64_##name
#else
typedef float REAL;
#define R_SQRT sqrtf
#define R_FABS fabsf
#define R_BIG FLT_MAX
#define VEC_EPS 1e-6f /* source/util/vectorbase.h:53 */
#define ORC_SYM(name) orc32_##name
#endif

#define EXPORT __attribute__((visibility("default")))

typedef long long idx_t;

typedef struct {
  int x, y, z, t;
} dims4;

typedef struct {
  REAL v[4];
} vec4;

static inline dims4 mkdims(const int *d) {
  dims4 r = {d[0], d[1], d[2], d[3]};
  return r;
}
static inline idx_t ncell(dims4 d) { return (idx_t)d.x * d.y * d.z * d.t; }
static inline idx_t index4(dims4 d, int i, int j, int k, int t) {
  return (idx_t)i + (idx_t)d.x * j + (idx_t)d.x * d.y * k +
         (idx_t)d.x * d.y * d.z * t;
}
/* Grid4dBase::isInBounds(Vec4i, bnd), source/grid4d.h:319-326 */
static inline int in_bounds(dims4 d, int i, int j, int k, int t, int b) {
  return i >= b && j >= b && i < d.x - b && j < d.y - b && k >= b &&
         k < d.z - b && t >= b && t < d.t - b;
}

/* float -> int truncation as the GPU's cvt.rzi performs it.  The reference
 * casts with (int), which is undefined for NaN / out-of-range values; for all
 * in-range values the two agree. */
static inline int trunc_int(REAL p) {
  if (p != p) return 0;
  if (p >= (REAL)2147483647.0) return INT_MAX;
  if (p <= (REAL)-2147483648.0) return INT_MIN;
  return (int)p;
}

static inline int trunc_int_d(double p) {
  if (p != p) return 0;
  if (p >= 2147483647.0) return INT_MAX;
  if (p <= -2147483648.0) return INT_MIN;
  return (int)p;
}

static void *xcalloc(idx_t n, size_t sz) {
  void *p = calloc((size_t)n, sz);
  if (!p) abort();
  return p;
}

/* ------------------------------------------------------------------------ */
/* Interpolation                                                              */
/* ------------------------------------------------------------------------ */

typedef struct {
  idx_t idx;
  REAL s0, s1, t0, t1, f0, f1, g0, g1;
} iw4;

/* BUILD_INDEX_4D, source/util/vector4d.h:422-470.  Cell-centred sampling at
 * pos-0.5, truncating index, clamp to border with one-sided weights.  The
 * `1. - s1` expressions are evaluated in double and rounded to REAL, as the
 * reference does. */
static inline iw4 build_index4(dims4 sz, const REAL *pos) {
  iw4 w;
  REAL px = pos[0] - 0.5f, py = pos[1] - 0.5f, pz = pos[2] - 0.5f,
       pt = pos[3] - 0.5f;
  int xi = trunc_int(px), yi = trunc_int(py), zi = trunc_int(pz),
      ti = trunc_int(pt);
  w.s1 = px - (REAL)xi;
  w.s0 = (REAL)(1. - w.s1);
  w.t1 = py - (REAL)yi;
  w.t0 = (REAL)(1. - w.t1);
  w.f1 = pz - (REAL)zi;
  w.f0 = (REAL)(1. - w.f1);
  w.g1 = pt - (REAL)ti;
  w.g0 = (REAL)(1. - w.g1);
  if (px < 0.) { xi = 0; w.s0 = 1.0; w.s1 = 0.0; }
  if (py < 0.) { yi = 0; w.t0 = 1.0; w.t1 = 0.0; }
  if (pz < 0.) { zi = 0; w.f0 = 1.0; w.f1 = 0.0; }
  if (pt < 0.) { ti = 0; w.g0 = 1.0; w.g1 = 0.0; }
  if (xi >= sz.x - 1) { xi = sz.x - 2; w.s0 = 0.0; w.s1 = 1.0; }
  if (yi >= sz.y - 1) { yi = sz.y - 2; w.t0 = 0.0; w.t1 = 1.0; }
  if (zi >= sz.z - 1) { zi = sz.z - 2; w.f0 = 0.0; w.f1 = 1.0; }
  if (ti >= sz.t - 1) { ti = sz.t - 2; w.g0 = 0.0; w.g1 = 1.0; }
  w.idx = index4(sz, xi, yi, zi, ti);
  return w;
}

/* interpol4d<T>, source/util/vector4d.h:484-513: sum order y, x, z, t.
 * `data` holds nc REAL per cell; component c is sampled. */
static inline REAL interp4c(const REAL *data, int nc, int c, dims4 sz,
                            const iw4 *w) {
  const idx_t sX = nc, sY = (idx_t)sz.x * nc, sZ = (idx_t)sz.x * sz.y * nc,
              sT = (idx_t)sz.x * sz.y * sz.z * nc;
  const REAL *d = data + w->idx * nc + c;
  const REAL t0 = w->t0, t1 = w->t1, s0 = w->s0, s1 = w->s1, f0 = w->f0,
             f1 = w->f1, g0 = w->g0, g1 = w->g1;
  return (((d[0] * t0 + d[sY] * t1) * s0 + (d[sX] * t0 + d[sX + sY] * t1) * s1) *
              f0 +
          ((d[sZ] * t0 + d[sY + sZ] * t1) * s0 +
           (d[sX + sZ] * t0 + d[sX + sY + sZ] * t1) * s1) *
              f1) *
             g0 +
         (((d[sT] * t0 + d[sT + sY] * t1) * s0 +
           (d[sT + sX] * t0 + d[sT + sX + sY] * t1) * s1) *
              f0 +
          ((d[sT + sZ] * t0 + d[sT + sY + sZ] * t1) * s0 +
           (d[sT + sX + sZ] * t0 + d[sT + sX + sY + sZ] * t1) * s1) *
              f1) *
             g1;
}

static inline REAL interp4_real(const REAL *data, dims4 sz, const REAL *pos) {
  iw4 w = build_index4(sz, pos);
  return interp4c(data, 1, 0, sz, &w);
}
static inline vec4 interp4_vec(const REAL *data, dims4 sz, const REAL *pos) {
  iw4 w = build_index4(sz, pos);
  vec4 r;
  for (int c = 0; c < 4; ++c) r.v[c] = interp4c(data, 4, c, sz, &w);
  return r;
}

/* BUILD_INDEX + interpol<T>, source/util/interpol.h:57-116 (3D trilinear;
 * z is clamped only when size.z > 1).  `data` is a Vec4 field of size
 * (sx,sy,sz) with z stride Zs (in cells). */
static inline vec4 interp3_vec4(const REAL *data, const int *size, idx_t Zs,
                                const REAL *pos) {
  REAL px = pos[0] - 0.5f, py = pos[1] - 0.5f, pz = pos[2] - 0.5f;
  int xi = trunc_int(px), yi = trunc_int(py), zi = trunc_int(pz);
  REAL s1 = px - (REAL)xi, s0 = (REAL)(1. - s1);
  REAL t1 = py - (REAL)yi, t0 = (REAL)(1. - t1);
  REAL f1 = pz - (REAL)zi, f0 = (REAL)(1. - f1);
  if (px < 0.) { xi = 0; s0 = 1.0; s1 = 0.0; }
  if (py < 0.) { yi = 0; t0 = 1.0; t1 = 0.0; }
  if (pz < 0.) { zi = 0; f0 = 1.0; f1 = 0.0; }
  if (xi >= size[0] - 1) { xi = size[0] - 2; s0 = 0.0; s1 = 1.0; }
  if (yi >= size[1] - 1) { yi = size[1] - 2; t0 = 0.0; t1 = 1.0; }
  if (size[2] > 1) {
    if (zi >= size[2] - 1) { zi = size[2] - 2; f0 = 0.0; f1 = 1.0; }
  }
  const idx_t X = 4, Y = (idx_t)size[0] * 4, Z = Zs * 4;
  const idx_t idx = ((idx_t)xi + (idx_t)size[0] * yi + Zs * zi) * 4;
  vec4 r;
  for (int c = 0; c < 4; ++c) {
    const REAL *d = data + idx + c;
    r.v[c] = ((d[0] * t0 + d[Y] * t1) * s0 + (d[X] * t0 + d[X + Y] * t1) * s1) *
                 f0 +
             ((d[Z] * t0 + d[Y + Z] * t1) * s0 +
              (d[X + Z] * t0 + d[X + Y + Z] * t1) * s1) *
                 f1;
  }
  return r;
}

EXPORT REAL ORC_SYM(interp4)(const int *dims, const REAL *data, int nc, int c,
                             const REAL *pos) {
  dims4 d = mkdims(dims);
  iw4 w = build_index4(d, pos);
  return interp4c(data, nc, c, d, &w);
}

/* ------------------------------------------------------------------------ */
/* Grid4d operations, source/grid4d.cpp:198-412, grid4d.h:334-394            */
/* ------------------------------------------------------------------------ */

/* nc = REAL per cell (1 Real, 4 Vec4). Elementwise ops act per REAL. */
EXPORT void ORC_SYM(setConst)(const int *dims, REAL *a, int nc, const REAL *v) {
  idx_t n = ncell(mkdims(dims));
  for (idx_t i = 0; i < n; ++i)
    for (int c = 0; c < nc; ++c) a[i * nc + c] = v[c];
}
EXPORT void ORC_SYM(addConst)(const int *dims, REAL *a, int nc, const REAL *v) {
  idx_t n = ncell(mkdims(dims));
  for (idx_t i = 0; i < n; ++i)
    for (int c = 0; c < nc; ++c) a[i * nc + c] += v[c];
}
EXPORT void ORC_SYM(multConst)(const int *dims, REAL *a, int nc, const REAL *v) {
  idx_t n = ncell(mkdims(dims));
  for (idx_t i = 0; i < n; ++i)
    for (int c = 0; c < nc; ++c) a[i * nc + c] *= v[c];
}
EXPORT void ORC_SYM(add)(const int *dims, REAL *a, int nc, const REAL *b) {
  idx_t n = ncell(mkdims(dims)) * nc;
  for (idx_t i = 0; i < n; ++i) a[i] += b[i];
}
EXPORT void ORC_SYM(sub)(const int *dims, REAL *a, int nc, const REAL *b) {
  idx_t n = ncell(mkdims(dims)) * nc;
  for (idx_t i = 0; i < n; ++i) a[i] -= b[i];
}
/* Grid4dScaledAdd: me += factor * other (grid4d.h:367-371) */
EXPORT void ORC_SYM(addScaled)(const int *dims, REAL *a, int nc, const REAL *b,
                               const REAL *f) {
  idx_t n = ncell(mkdims(dims));
  for (idx_t i = 0; i < n; ++i)
    for (int c = 0; c < nc; ++c) a[i * nc + c] += f[c] * b[i * nc + c];
}

/* kn4dMaxVec / getMax for Vec4: sqrt(max |v|^2) (grid4d.cpp:165-172, :274-285) */
static REAL vec4_maxnorm(dims4 d, const REAL *a) {
  idx_t n = ncell(d);
  REAL m = -R_BIG;
  for (idx_t i = 0; i < n; ++i) {
    const REAL *v = a + i * 4;
    const REAL s = v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3];
    if (s > m) m = s;
  }
  return R_SQRT(m);
}
/* kn4dMinVec / getMin for Vec4: sqrt(min |v|^2) */
static REAL vec4_minnorm(dims4 d, const REAL *a) {
  idx_t n = ncell(d);
  REAL m = R_BIG;
  for (idx_t i = 0; i < n; ++i) {
    const REAL *v = a + i * 4;
    const REAL s = v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3];
    if (s < m) m = s;
  }
  return R_SQRT(m);
}
static REAL real_max(dims4 d, const REAL *a) {
  idx_t n = ncell(d);
  REAL m = -R_BIG;
  for (idx_t i = 0; i < n; ++i)
    if (a[i] > m) m = a[i];
  return m;
}
static REAL real_min(dims4 d, const REAL *a) {
  idx_t n = ncell(d);
  REAL m = R_BIG;
  for (idx_t i = 0; i < n; ++i)
    if (a[i] < m) m = a[i];
  return m;
}
/* which: 0 max, 1 min, 2 maxabs (grid4d.cpp:263-285) */
EXPORT REAL ORC_SYM(reduce)(const int *dims, const REAL *a, int nc, int which) {
  dims4 d = mkdims(dims);
  if (nc == 4) {
    if (which == 1) return vec4_minnorm(d, a);
    return vec4_maxnorm(d, a);
  }
  if (which == 0) return real_max(d, a);
  if (which == 1) return real_min(d, a);
  {
    REAL amin = real_min(d, a), amax = real_max(d, a);
    REAL x = R_FABS(amin), y = R_FABS(amax);
    return x > y ? x : y; /* std::max(fabs(amin), fabs(amax)) */
  }
}

/* knSetBnd4d: sets cells with c <= w or c >= size-1-w (grid4d.cpp:355-368) */
EXPORT void ORC_SYM(setBound)(const int *dims, REAL *a, int nc, const REAL *v,
                              int w) {
  dims4 d = mkdims(dims);
  for (int t = 0; t < d.t; ++t)
    for (int k = 0; k < d.z; ++k)
      for (int j = 0; j < d.y; ++j)
        for (int i = 0; i < d.x; ++i) {
          int b = (i <= w || i >= d.x - 1 - w || j <= w || j >= d.y - 1 - w ||
                   k <= w || k >= d.z - 1 - w || t <= w || t >= d.t - 1 - w);
          if (b) {
            idx_t id = index4(d, i, j, k, t);
            for (int c = 0; c < nc; ++c) a[id * nc + c] = v[c];
          }
        }
}

/* knSetBnd4dNeumann (grid4d.cpp:370-407).  Source cells are never inside the
 * written ring, so the in-place update is order independent. */
EXPORT void ORC_SYM(setBoundNeumann)(const int *dims, REAL *a, int nc, int w) {
  dims4 d = mkdims(dims);
  for (int t = 0; t < d.t; ++t)
    for (int k = 0; k < d.z; ++k)
      for (int j = 0; j < d.y; ++j)
        for (int i = 0; i < d.x; ++i) {
          int set = 0, si = i, sj = j, sk = k, st = t;
          if (i <= w) { si = w + 1; set = 1; }
          if (i >= d.x - 1 - w) { si = d.x - 1 - w - 1; set = 1; }
          if (j <= w) { sj = w + 1; set = 1; }
          if (j >= d.y - 1 - w) { sj = d.y - 1 - w - 1; set = 1; }
          if (k <= w) { sk = w + 1; set = 1; }
          if (k >= d.z - 1 - w) { sk = d.z - 1 - w - 1; set = 1; }
          if (t <= w) { st = w + 1; set = 1; }
          if (t >= d.t - 1 - w) { st = d.t - 1 - w - 1; set = 1; }
          if (set) {
            idx_t dst = index4(d, i, j, k, t), src = index4(d, si, sj, sk, st);
            for (int c = 0; c < nc; ++c) a[dst * nc + c] = a[src * nc + c];
          }
        }
}

/* ------------------------------------------------------------------------ */
/* Resampling                                                                 */
/* ------------------------------------------------------------------------ */

/* knInterpol4d / KnInterpolateGrid4dTempl (grid4d.cpp:531-538,
 * grid4d.h:463-471): target(ijkt) = source.getInterpolated(ijkt*fac + off),
 * over all target cells. */
EXPORT void ORC_SYM(resample4d)(const int *tdims, REAL *target, const int *sdims,
                                const REAL *source, int nc, const REAL *fac,
                                const REAL *off) {
  dims4 td = mkdims(tdims), sd = mkdims(sdims);
#pragma omp parallel for schedule(static)
  for (int t = 0; t < td.t; ++t)
    for (int k = 0; k < td.z; ++k)
      for (int j = 0; j < td.y; ++j)
        for (int i = 0; i < td.x; ++i) {
          REAL pos[4];
          pos[0] = (REAL)i * fac[0] + off[0];
          pos[1] = (REAL)j * fac[1] + off[1];
          pos[2] = (REAL)k * fac[2] + off[2];
          pos[3] = (REAL)t * fac[3] + off[3];
          iw4 w = build_index4(sd, pos);
          idx_t o = index4(td, i, j, k, t) * nc;
          for (int c = 0; c < nc; ++c)
            target[o + c] = interp4c(source, nc, c, sd, &w);
        }
}

/* gridFactor4d (grid4d.cpp:559-569): srcFac = (s1/s2)/scale,
 * off = -off*srcFac + srcFac*0.5, with optional size override of s2. */
EXPORT void ORC_SYM(gridFactor4d)(const REAL *s1, const REAL *s2in,
                                  const REAL *optSize, const REAL *scale,
                                  REAL *srcFac, REAL *retOff) {
  REAL s2[4];
  for (int c = 0; c < 4; ++c) s2[c] = optSize[c] > 0. ? optSize[c] : s2in[c];
  for (int c = 0; c < 4; ++c) {
    REAL f = s1[c] / s2[c]; /* calcGridSizeFactor4d(Vec4,Vec4), grid4d.h:279 */
    srcFac[c] = f / scale[c];
  }
  for (int c = 0; c < 4; ++c) {
    REAL neg = -retOff[c];
    retOff[c] = neg * srcFac[c] + (REAL)((double)srcFac[c] * 0.5);
  }
}

/* interpolateGrid4d / interpolateGrid4dVec (grid4d.cpp:540-557) */
EXPORT void ORC_SYM(interpolateGrid4d)(const int *tdims, REAL *target,
                                       const int *sdims, const REAL *source,
                                       int nc, const REAL *offset,
                                       const REAL *scale, const REAL *size) {
  REAL s1[4], s2[4], fac[4], off[4];
  for (int c = 0; c < 4; ++c) {
    s1[c] = (REAL)sdims[c];
    s2[c] = (REAL)tdims[c];
    off[c] = offset[c];
  }
  ORC_SYM(gridFactor4d)(s1, s2, size, scale, fac, off);
  ORC_SYM(resample4d)(tdims, target, sdims, source, nc, fac, off);
}

/* interpolGridTempl (optflow4d.cpp:40-57): factor = src/target sizes as
 * Real(s1)/s2, offset = factor*0.5. */
static void interpol_grid(dims4 td, REAL *target, dims4 sd, const REAL *source,
                          int nc) {
  REAL fac[4], off[4];
  int sa[4] = {sd.x, sd.y, sd.z, sd.t}, ta[4] = {td.x, td.y, td.z, td.t};
  for (int c = 0; c < 4; ++c) {
    fac[c] = (REAL)sa[c] / (REAL)ta[c];
    off[c] = (REAL)((double)fac[c] * 0.5);
  }
  ORC_SYM(resample4d)(ta, target, sa, source, nc, fac, off);
}
EXPORT void ORC_SYM(interpolGrid)(const int *tdims, REAL *target,
                                  const int *sdims, const REAL *source, int nc) {
  interpol_grid(mkdims(tdims), target, mkdims(sdims), source, nc);
}

/* ------------------------------------------------------------------------ */
/* Semi-Lagrangian advection                                                  */
/* ------------------------------------------------------------------------ */

/* semiLagrange4d (optflow4d.cpp:1275-1281) over bnd=1 cells into a fresh
 * zeroed grid, then swap (advectSemiLagrange4d, :1283-1290). */
static void semi_lagrange4d(dims4 d, const REAL *vel, REAL *grid, int nc,
                            REAL dt) {
  idx_t n = ncell(d);
  REAL *fwd = (REAL *)xcalloc(n * nc, sizeof(REAL));
#pragma omp parallel for schedule(static)
  for (int t = 1; t < d.t - 1; ++t)
    for (int k = 1; k < d.z - 1; ++k)
      for (int j = 1; j < d.y - 1; ++j)
        for (int i = 1; i < d.x - 1; ++i) {
          idx_t id = index4(d, i, j, k, t);
          const REAL *v = vel + id * 4;
          REAL pos[4];
          pos[0] = (REAL)(i + 0.5f) - v[0] * dt;
          pos[1] = (REAL)(j + 0.5f) - v[1] * dt;
          pos[2] = (REAL)(k + 0.5f) - v[2] * dt;
          pos[3] = (REAL)(t + 0.5f) - v[3] * dt;
          iw4 w = build_index4(d, pos);
          for (int c = 0; c < nc; ++c) fwd[id * nc + c] = interp4c(grid, nc, c, d, &w);
        }
  memcpy(grid, fwd, (size_t)(n * nc) * sizeof(REAL));
  free(fwd);
}

/* advect4d(vel, grid, dtFac) with the solver dt = 1 (optflow4d.cpp:1292-1306) */
EXPORT void ORC_SYM(advect4d)(const int *dims, const REAL *vel, REAL *grid,
                              int nc, REAL dtFac) {
  REAL dt = (REAL)1.0 * dtFac;
  semi_lagrange4d(mkdims(dims), vel, grid, nc, dt);
}

/* advectCflTemplate<Grid4d<int>,...> -> advectCflHelper4d
 * (optflow4d.cpp:2170-2180, :1309-1321), solver dt = 1, velFactor = 1. */
static void advect_cfl(dims4 d, REAL cfl, const REAL *vel, REAL *grid, int nc) {
  idx_t n = ncell(d);
  REAL *velTmp = (REAL *)xcalloc(n * 4, sizeof(REAL));
  memcpy(velTmp, vel, (size_t)n * 4 * sizeof(REAL));
  /* velTmp.multConst(Vec4(1)) is exact */
  REAL orgDt = 1.0;
  REAL maxVel = vec4_maxnorm(d, velTmp) * orgDt;
  int steps = trunc_int(maxVel / cfl) + 1;
  REAL mdt = orgDt / (REAL)steps;
  for (int s = 0; s < steps; ++s) semi_lagrange4d(d, velTmp, grid, nc, mdt * (REAL)1.);
  free(velTmp);
}
EXPORT void ORC_SYM(advectCfl4d)(const int *dims, REAL cfl, const REAL *vel,
                                 REAL *grid, int nc) {
  advect_cfl(mkdims(dims), cfl, vel, grid, nc);
}

/* ------------------------------------------------------------------------ */
/* Error metric                                                               */
/* ------------------------------------------------------------------------ */

/* calcLsDiffTempl (optflow4d.cpp:895-927) */
EXPORT REAL ORC_SYM(calcLsDiff4d)(const int *dims, const REAL *i0,
                                  const REAL *i1, REAL *out, REAL correction,
                                  int bnd) {
  dims4 d = mkdims(dims);
  double accu = 0.;
  for (int t = bnd; t < d.t - bnd; ++t)
    for (int k = bnd; k < d.z - bnd; ++k)
      for (int j = bnd; j < d.y - bnd; ++j)
        for (int i = bnd; i < d.x - bnd; ++i) {
          idx_t id = index4(d, i, j, k, t);
          REAL a = i0[id], b = i1[id];
          if ((a < 0. && b < 0.) || (a >= 0. && b >= 0.)) {
            if (out) out[id] = 0.;
          } else {
            REAL dd = R_FABS(a - b) * correction;
            if (dd > 1.) dd = 1.;
            accu += dd;
            if (out) out[id] = dd;
          }
        }
  int sx = d.x - 2 * bnd, sy = d.y - 2 * bnd, sz = d.z - 2 * bnd,
      st = d.t - 2 * bnd;
  accu *= 1000.;
  if (d.t > 1) accu *= 1000.;
  accu *= 1. / (double)(sx * sy * sz * st);
  return (REAL)accu;
}

/* ------------------------------------------------------------------------ */
/* Gaussian blur                                                              */
/* ------------------------------------------------------------------------ */

/* gaussianWeight (optflow4d.cpp:127-130): exp evaluated in double */
static REAL gauss_weight(REAL sigma, REAL dSqr) {
  return (REAL)exp((double)(-dSqr) / (2. * (double)sigma * (double)sigma));
}

/* knGaussianBlur (optflow4d.cpp:132-158), bnd=1, Vec4 or Real grid */
static void gaussian_pass(dims4 d, const REAL *a, REAL *tmp, int nc, REAL sigma,
                          int s) {
  REAL *wtab = (REAL *)xcalloc(4 * s * s + 1, sizeof(REAL));
  for (int q = 0; q <= 4 * s * s; ++q) wtab[q] = gauss_weight(sigma, (REAL)q);
#pragma omp parallel for schedule(static)
  for (int t = 1; t < d.t - 1; ++t)
    for (int k = 1; k < d.z - 1; ++k)
      for (int j = 1; j < d.y - 1; ++j)
        for (int i = 1; i < d.x - 1; ++i) {
          REAL val[4] = {0, 0, 0, 0};
          REAL weight = 0.;
          for (int vt = t - s; vt <= t + s; vt++)
            for (int zk = k - s; zk <= k + s; zk++)
              for (int yj = j - s; yj <= j + s; yj++)
                for (int xi = i - s; xi <= i + s; xi++) {
                  if (!in_bounds(d, xi, yj, zk, vt, 0)) continue;
                  int dq = (xi - i) * (xi - i) + (yj - j) * (yj - j) +
                           (zk - k) * (zk - k) + (vt - t) * (vt - t);
                  REAL wcurr = wtab[dq];
                  weight += wcurr;
                  const REAL *src = a + index4(d, xi, yj, zk, vt) * nc;
                  for (int c = 0; c < nc; ++c) val[c] += wcurr * src[c];
                }
          idx_t o = index4(d, i, j, k, t) * nc;
          if (weight > VEC_EPS) {
            for (int c = 0; c < nc; ++c) tmp[o + c] = val[c] / weight;
          } else {
            for (int c = 0; c < nc; ++c) tmp[o + c] = a[o + c];
          }
        }
  free(wtab);
}

/* gaussianBlurGeneric (optflow4d.cpp:160-174): 2*iter passes, each
 * followed by a pointer swap; the fresh tmp grid starts at zero.  After the
 * even number of swaps the result is back in the caller's buffer. */
static void gaussian_blur(dims4 d, REAL *a, int nc, REAL sigma, int iter) {
  idx_t n = ncell(d);
  REAL *tmp = (REAL *)xcalloc(n * nc, sizeof(REAL));
  int s = trunc_int_d(1. * (double)sigma + 0.5);
  if (s == 0) s = 1;
  REAL *A = a, *B = tmp;
  for (int it = 0; it < 2 * iter; ++it) {
    gaussian_pass(d, A, B, nc, sigma, s);
    REAL *sw = A;
    A = B;
    B = sw;
  }
  free(A == a ? B : A);
}
EXPORT void ORC_SYM(gaussianBlur4d)(const int *dims, REAL *a, int nc,
                                    REAL sigma, int iter) {
  gaussian_blur(mkdims(dims), a, nc, sigma, iter);
}

/* ------------------------------------------------------------------------ */
/* Optical flow system and Jacobi-PCG                                          */
/* ------------------------------------------------------------------------ */

typedef struct {
  int iterations;
  REAL residual;   /* ret_residual: max(r)/max(r0) */
  int converged;   /* return value of solve() */
  double sigma0;   /* first z.r */
  REAL resIni;
} orc_cg_info;

/* Neighbour order m = 0..7: -t, -z, -y, -x, +x, +y, +z, +t
 * (optflow4d.cpp:389-392). */
static const int NBX[8] = {0, 0, 0, -1, +1, 0, 0, 0};
static const int NBY[8] = {0, 0, -1, 0, 0, +1, 0, 0};
static const int NBZ[8] = {0, -1, 0, 0, 0, 0, +1, 0};
static const int NBT[8] = {-1, 0, 0, 0, 0, 0, 0, +1};

typedef struct {
  idx_t n;          /* 4 * cells */
  idx_t off[8];     /* row offsets of the 8 neighbours */
  REAL *offd;       /* n */
  REAL *blockd;     /* 4n */
} ofmat;

/* The element-wise loops of the PCG (applyMat, addScaled, precondApply,
 * getMaxNorm) run their rows on OpenMP threads: each row is computed alone,
 * and the signed maximum does not depend on the order, so the results are
 * the serial loops' bit for bit.  dotProd stays one serial double sum, the
 * reference's order. */

/* applyMat (optflow4d.cpp:211-232) */
static void apply_mat(const ofmat *A, const REAL *x, REAL *res) {
#pragma omp parallel for schedule(static)
  for (idx_t i = 0; i < A->n; ++i) {
    REAL v = 0;
    const REAL od = A->offd[i];
    if (od != 0.) {
      for (int m = 0; m < 8; ++m) v += od * x[i + A->off[m]];
    }
    const idx_t bi = (i / 4) * 4;
    for (int m = 0; m < 4; ++m) v += A->blockd[i * 4 + m] * x[bi + m];
    res[i] = v;
  }
}
/* dotProd (:234-241): double accumulator over REAL products */
static double dot_prod(const REAL *a, const REAL *b, idx_t n) {
  double d = 0.;
  for (idx_t i = 0; i < n; ++i) d += a[i] * b[i];
  return d;
}
/* getMaxNorm (:243-250): signed maximum.  Every thread starts from a[0]
 * and keeps the same ">" rule, so NaN entries are skipped (and a NaN a[0]
 * sticks) exactly as in the serial loop. */
static REAL max_norm(const REAL *a, idx_t n) {
  REAL m = a[0];
#pragma omp parallel
  {
    REAL mt = a[0];
#pragma omp for schedule(static) nowait
    for (idx_t i = 1; i < n; ++i)
      if (a[i] > mt) mt = a[i];
#pragma omp critical
    {
      if (mt > m) m = mt;
    }
  }
  return m;
}
/* addScaled (:253-258): a += (double)b * c, stored as REAL */
static void add_scaled(REAL *a, double b, const REAL *c, idx_t n) {
#pragma omp parallel for schedule(static)
  for (idx_t i = 0; i < n; ++i) a[i] += b * c[i];
}

/* GridCGOptflow4d::solve + precondInit/Apply (:268-355). x0 may be given
 * (NULL = the reference's x0 = 0). */
static int cg_solve(const ofmat *A, const REAL *rhs, REAL *result,
                    orc_cg_info *info, REAL accuracy, int maxIter) {
  const idx_t n = A->n;
  REAL *srch = (REAL *)xcalloc(n, sizeof(REAL));
  REAL *tmp = (REAL *)xcalloc(n, sizeof(REAL));
  REAL *res = (REAL *)xcalloc(n, sizeof(REAL));
  REAL *pre = (REAL *)xcalloc(n, sizeof(REAL));
  int ok = 0;
  info->iterations = 0;
  info->converged = 0;
  for (idx_t i = 0; i < n; ++i) result[i] = 0.;
  memcpy(res, rhs, (size_t)n * sizeof(REAL));
  double residual = max_norm(res, n);
  info->resIni = (REAL)residual;
  if (residual < VEC_EPS) {
    info->residual = 0;
    info->iterations = 0;
    info->converged = 1;
    ok = 1;
    goto done;
  }
  {
    const double acc = accuracy * residual;
    const double resIni = residual;
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < n; ++i) {
      REAL diag = A->blockd[i * 4 + (i - (i / 4) * 4)];
      pre[i] = (REAL)(1. / diag);
    }
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < n; ++i) tmp[i] = res[i] * pre[i];
    double sigma = dot_prod(tmp, res, n);
    info->sigma0 = sigma;
    if (sigma == 0 || sigma != sigma) {
      info->iterations = 0;
      ok = 0;
      goto done;
    }
    memcpy(srch, tmp, (size_t)n * sizeof(REAL));
    for (int iter = 0; iter < maxIter; ++iter) {
      apply_mat(A, srch, tmp);
      double alpha1 = dot_prod(srch, tmp, n);
      double alpha = sigma / alpha1;
      add_scaled(result, alpha, srch, n);
      add_scaled(res, -alpha, tmp, n);
      residual = max_norm(res, n);
      info->residual = (REAL)(residual / resIni);
      if (residual <= acc) {
        info->iterations = iter + 1;
        info->converged = 1;
        ok = 1;
        goto done;
      }
#pragma omp parallel for schedule(static)
      for (idx_t i = 0; i < n; ++i) tmp[i] = res[i] * pre[i];
      double sigmaNew = dot_prod(tmp, res, n);
      double beta = sigmaNew / sigma;
      add_scaled(tmp, beta, srch, n);
      memcpy(srch, tmp, (size_t)n * sizeof(REAL));
      sigma = sigmaNew;
      info->iterations = iter + 1;
    }
    info->residual = (REAL)(residual / resIni);
    ok = 0;
  }
done:
  free(srch);
  free(tmp);
  free(res);
  free(pre);
  return ok;
}

typedef struct {
  REAL wSmooth, wEnergy, postVelBlur, cgAccuracy, resetBndWidth;
  int blurType, cgMaxIter;
} orc_of_params;

/* System assembly of opticalFlowDim<...,4> (optflow4d.cpp:361-493).  Fills
 * the matrix and rhs from vel (usually zero), i0, i1. */
static void of_assemble(dims4 d, const REAL *vel, const REAL *i0,
                        const REAL *i1, REAL wSmooth, REAL wEnergy, ofmat *A,
                        REAL *rhs) {
  const REAL mDt = 1.0;
  const REAL mDx = (REAL)(1. / d.x);
  const REAL mDx2Inv = 1.;
  const int dim[4] = {d.x, d.y, d.z, d.t};
  const idx_t nc = ncell(d);
  A->n = nc * 4;
  A->offd = (REAL *)xcalloc(A->n, sizeof(REAL));
  A->blockd = (REAL *)xcalloc(A->n * 4, sizeof(REAL));
  for (idx_t q = 0; q < A->n; ++q) rhs[q] = 0.;
  /* neighbour offsets from cell (1,1,1,1) (:406-419) */
  {
    idx_t id = index4(d, 1, 1, 1, 1) * 4;
    for (int m = 0; m < 8; ++m) {
      int ti = 1 + NBX[m], tj = 1 + NBY[m], tk = 1 + NBZ[m], tt = 1 + NBT[m];
      A->off[m] = 0;
      if (in_bounds(d, ti, tj, tk, tt, 0))
        A->off[m] = index4(d, ti, tj, tk, tt) * 4 - id;
    }
  }
  const REAL dxf = (REAL)(1. / (2. * (double)mDx));
  /* rows are independent: OpenMP over t as the reference's kernels */
#pragma omp parallel for schedule(static)
  for (int t = 0; t < d.t; ++t)
    for (int k = 0; k < d.z; ++k)
      for (int j = 0; j < d.y; ++j)
        for (int i = 0; i < d.x; ++i) {
          idx_t cell = index4(d, i, j, k, t);
          if (!in_bounds(d, i, j, k, t, 1)) {
            for (int dd = 0; dd < 4; ++dd) {
              idx_t v = cell * 4 + dd;
              A->blockd[v * 4 + dd] = 1.;
            }
            continue;
          }
          REAL tderiv = (i1[cell] - i0[cell]) / mDt;
          REAL grad[4];
          grad[0] = (i1[index4(d, i + 1, j, k, t)] - i1[index4(d, i - 1, j, k, t)]) * dxf;
          grad[1] = (i1[index4(d, i, j + 1, k, t)] - i1[index4(d, i, j - 1, k, t)]) * dxf;
          grad[2] = (i1[index4(d, i, j, k + 1, t)] - i1[index4(d, i, j, k - 1, t)]) * dxf;
          grad[3] = (i1[index4(d, i, j, k, t + 1)] - i1[index4(d, i, j, k, t - 1)]) * dxf;
          for (int dd = 0; dd < 4; ++dd) {
            idx_t v = cell * 4 + dd;
            rhs[v] = -grad[dd] * tderiv;
            for (int m = 0; m < 8; ++m) {
              int ti = i + NBX[m], tj = j + NBY[m], tk = k + NBZ[m], tt = t + NBT[m];
              ti = ti < 0 ? 0 : (ti > dim[0] - 1 ? dim[0] - 1 : ti);
              tj = tj < 0 ? 0 : (tj > dim[1] - 1 ? dim[1] - 1 : tj);
              tk = tk < 0 ? 0 : (tk > dim[2] - 1 ? dim[2] - 1 : tk);
              tt = tt < 0 ? 0 : (tt > dim[3] - 1 ? dim[3] - 1 : tt);
              rhs[v] -= wSmooth * (vel[cell * 4 + dd] - vel[index4(d, ti, tj, tk, tt) * 4 + dd]) *
                        mDx * mDx2Inv;
            }
            A->offd[v] = -wSmooth * mDx2Inv;
            REAL diag = 0.;
            diag += (REAL)(2 * 4) * wSmooth * mDx2Inv;
            diag += wEnergy;
            for (int m = 0; m < 4; ++m) {
              if (dd == m)
                A->blockd[v * 4 + m] = grad[dd] * grad[m] + diag;
              else
                A->blockd[v * 4 + m] = grad[dd] * grad[m];
            }
            rhs[v] -= wEnergy * vel[cell * 4 + dd] * mDx;
          }
        }
}

/* Stage helper for parity tests: the per-cell gradient g (= the rank-one
 * part of the block), the rhs and the block matrix. */
EXPORT void ORC_SYM(ofAssemble)(const int *dims, const REAL *vel, const REAL *i0,
                                const REAL *i1, REAL wSmooth, REAL wEnergy,
                                REAL *rhs_out, REAL *blockd_out, REAL *offd_out) {
  dims4 d = mkdims(dims);
  ofmat A;
  of_assemble(d, vel, i0, i1, wSmooth, wEnergy, &A, rhs_out);
  if (blockd_out) memcpy(blockd_out, A.blockd, (size_t)A.n * 4 * sizeof(REAL));
  if (offd_out) memcpy(offd_out, A.offd, (size_t)A.n * sizeof(REAL));
  free(A.offd);
  free(A.blockd);
}

/* Statistics of the last driver call, for tests and the bench. */
#define ORC_MAX_SOLVES 256
static int g_nsolves = 0;
static int g_solve_iters[ORC_MAX_SOLVES];
static int g_solve_size[ORC_MAX_SOLVES];
static REAL g_solve_res[ORC_MAX_SOLVES];
EXPORT void ORC_SYM(statsReset)(void) { g_nsolves = 0; }
EXPORT int ORC_SYM(statsGet)(int *iters, int *sizes, REAL *res, int cap) {
  int n = g_nsolves < cap ? g_nsolves : cap;
  for (int q = 0; q < n; ++q) {
    iters[q] = g_solve_iters[q];
    sizes[q] = g_solve_size[q];
    res[q] = g_solve_res[q];
  }
  return g_nsolves;
}

/* opticalFlowDim<Grid4d<Real>,Grid4d<Vec4>,4> (optflow4d.cpp:361-553) */
static void optical_flow_dim(dims4 d, REAL *vel, const REAL *i0, const REAL *i1,
                             const orc_of_params *p, orc_cg_info *info_out) {
  const idx_t nc = ncell(d), n = nc * 4;
  const REAL mDx = (REAL)(1. / d.x);
  REAL *rhs = (REAL *)xcalloc(n, sizeof(REAL));
  REAL *result = (REAL *)xcalloc(n, sizeof(REAL));
  ofmat A;
  of_assemble(d, vel, i0, i1, p->wSmooth, p->wEnergy, &A, rhs);
  orc_cg_info info;
  memset(&info, 0, sizeof(info));
  info.residual = (REAL)1e10;
  info.iterations = -1;
  cg_solve(&A, rhs, result, &info, p->cgAccuracy, p->cgMaxIter);
  REAL cgRes = info.residual;
  if (cgRes != cgRes) {
    for (idx_t q = 0; q < n; ++q) result[q] = 0.;
  }
  if (g_nsolves < ORC_MAX_SOLVES) {
    g_solve_iters[g_nsolves] = info.iterations;
    g_solve_size[g_nsolves] = d.x;
    g_solve_res[g_nsolves] = info.residual;
  }
  g_nsolves++;
  if (info_out) *info_out = info;
  for (idx_t q = 0; q < n; ++q) vel[q] = result[q] / mDx;
  if (p->postVelBlur > 0.) {
    REAL sigma = (REAL)(0.5 * p->postVelBlur);
    gaussian_blur(d, vel, 4, sigma, 1);
  }
  if (p->resetBndWidth > 0.) {
    int resetBnd = trunc_int(p->resetBndWidth * (REAL)d.x) + 1;
    for (int t = 0; t < d.t; ++t)
      for (int k = 0; k < d.z; ++k)
        for (int j = 0; j < d.y; ++j)
          for (int i = 0; i < d.x; ++i) {
            if (in_bounds(d, i, j, k, t, resetBnd)) continue;
            idx_t id = index4(d, i, j, k, t) * 4;
            vel[id] = vel[id + 1] = vel[id + 2] = vel[id + 3] = 0.;
          }
  }
  free(rhs);
  free(result);
  free(A.offd);
  free(A.blockd);
}

EXPORT void ORC_SYM(opticalFlow4d)(const int *dims, REAL *vel, const REAL *i0,
                                   const REAL *i1, REAL wSmooth, REAL wEnergy,
                                   REAL postVelBlur, REAL cgAccuracy,
                                   REAL resetBndWidth, int cgMaxIter,
                                   int *iters, REAL *residual) {
  orc_of_params p;
  p.wSmooth = wSmooth;
  p.wEnergy = wEnergy;
  p.postVelBlur = postVelBlur;
  p.cgAccuracy = cgAccuracy;
  p.resetBndWidth = resetBndWidth;
  p.blurType = 1;
  p.cgMaxIter = cgMaxIter;
  orc_cg_info info;
  optical_flow_dim(mkdims(dims), vel, i0, i1, &p, &info);
  if (iters) *iters = info.iterations;
  if (residual) *residual = info.residual;
}

/* Stand-alone PCG on an assembled system, for stage-wise tests. */
EXPORT int ORC_SYM(cgSolve)(const int *dims, const REAL *vel, const REAL *i0,
                            const REAL *i1, REAL wSmooth, REAL wEnergy,
                            REAL accuracy, int maxIter, REAL *result,
                            int *iters, REAL *residual) {
  dims4 d = mkdims(dims);
  idx_t n = ncell(d) * 4;
  REAL *rhs = (REAL *)xcalloc(n, sizeof(REAL));
  ofmat A;
  of_assemble(d, vel, i0, i1, wSmooth, wEnergy, &A, rhs);
  orc_cg_info info;
  memset(&info, 0, sizeof(info));
  info.residual = (REAL)1e10;
  int ok = cg_solve(&A, rhs, result, &info, accuracy, maxIter);
  if (iters) *iters = info.iterations;
  if (residual) *residual = info.residual;
  free(rhs);
  free(A.offd);
  free(A.blockd);
  return ok;
}

/* ------------------------------------------------------------------------ */
/* Level-set projection correction                                            */
/* ------------------------------------------------------------------------ */

/* knCvExpolBlur4d (optflow4d.cpp:613-626), bnd=1; the sum is scaled by the
 * double constant 1/81 and rounded back to REAL. */
static void expol_sweep(dims4 d, const REAL *a, REAL *tmp, const REAL *mark) {
#pragma omp parallel for schedule(static)
  for (int t = 1; t < d.t - 1; ++t)
    for (int k = 1; k < d.z - 1; ++k)
      for (int j = 1; j < d.y - 1; ++j)
        for (int i = 1; i < d.x - 1; ++i) {
          idx_t id = index4(d, i, j, k, t);
          if (mark[id] != 0.) continue;
          REAL val[4] = {0, 0, 0, 0};
          for (int vt = t - 1; vt <= t + 1; vt++)
            for (int zk = k - 1; zk <= k + 1; zk++)
              for (int yj = j - 1; yj <= j + 1; yj++)
                for (int xi = i - 1; xi <= i + 1; xi++) {
                  const REAL *s = a + index4(d, xi, yj, zk, vt) * 4;
                  for (int c = 0; c < 4; ++c) val[c] += s[c];
                }
          for (int c = 0; c < 4; ++c)
            tmp[id * 4 + c] = (REAL)((double)val[c] * (1. / 81.0));
        }
}
/* The sweep loop of corrVelsOfTempl (optflow4d.cpp:766-781):
 * tmp.copyFrom(dst); knCvExpolBlur4d(dst, tmp, marker); dst.swap(tmp). */
static void expol_sweeps(dims4 d, REAL *dst, REAL *tmp, const REAL *mark,
                         int sweeps) {
  idx_t n = ncell(d) * 4;
  REAL *A = dst, *B = tmp;
  for (int s = 0; s < sweeps; ++s) {
    memcpy(B, A, (size_t)n * sizeof(REAL));
    expol_sweep(d, A, B, mark);
    REAL *sw = A;
    A = B;
    B = sw;
  }
  if (A != dst) memcpy(dst, A, (size_t)n * sizeof(REAL));
}
EXPORT void ORC_SYM(expolSweeps)(const int *dims, REAL *dst, const REAL *mark,
                                 int sweeps) {
  dims4 d = mkdims(dims);
  REAL *tmp = (REAL *)xcalloc(ncell(d) * 4, sizeof(REAL));
  expol_sweeps(d, dst, tmp, mark, sweeps);
  free(tmp);
}

/* getNormalInterpTempl (optflow4d.cpp:651-673) + normalize
 * (util/vector4d.h:331-345) */
static vec4 normal_interp(dims4 d, const REAL *phi, const REAL *pos) {
  const REAL h = 0.5;
  vec4 n;
  for (int c = 0; c < 4; ++c) {
    REAL pa[4] = {pos[0], pos[1], pos[2], pos[3]};
    REAL pb[4] = {pos[0], pos[1], pos[2], pos[3]};
    pa[c] = pos[c] + h;
    pb[c] = pos[c] - h;
    n.v[c] = interp4_real(phi, d, pa) - interp4_real(phi, d, pb);
  }
  REAL l = n.v[0] * n.v[0] + n.v[1] * n.v[1] + n.v[2] * n.v[2] + n.v[3] * n.v[3];
  const REAL eps2 = VEC_EPS * VEC_EPS;
  if (fabs((double)l - 1.) < (double)eps2) {
    /* normalized enough */
  } else if (l > eps2) {
    REAL nrm = R_SQRT(l);
    REAL inv = (REAL)(1. / (double)nrm);
    for (int c = 0; c < 4; ++c) n.v[c] *= inv;
  } else {
    n.v[0] = n.v[1] = n.v[2] = n.v[3] = 0.;
  }
  return n;
}

/* projectCell (optflow4d.cpp:675-710), solver dt = 1 */
static REAL project_cell(dims4 d, vec4 nrm, const REAL *phiOrg,
                         const REAL *phiTarget, const REAL *pos, int ci, int cj,
                         int ck, int ct, int maxIter) {
  const REAL dt = 1.0;
  REAL step = 0.25;
  if (maxIter < 50) step = 0.5;
  int lastDir = 0;
  REAL targetVal = phiTarget[index4(d, ci, cj, ck, ct)];
  REAL vn = interp4_real(phiOrg, d, pos);
  REAL dd = (vn - targetVal);
  for (int s = 0; s < maxIter; ++s) {
    REAL pn[4];
    for (int c = 0; c < 4; ++c) pn[c] = pos[c] + (nrm.v[c] * dd) * dt;
    /* isInBounds(Vec4) truncates to int (grid4d.h:73-76) */
    if (!in_bounds(d, trunc_int(pn[0]), trunc_int(pn[1]), trunc_int(pn[2]),
                   trunc_int(pn[3]), 0)) {
      s = maxIter;
      dd = 9999.;
      continue;
    }
    vn = interp4_real(phiOrg, d, pn);
    if (vn < targetVal) {
      if (lastDir < 0) step *= 0.5;
      dd += step;
      lastDir = 1;
    } else {
      if (lastDir > 0) step *= 0.5;
      dd -= step;
      lastDir = -1;
    }
    if (step < 1e-01) s = maxIter + 1;
  }
  return dd;
}

/* knProjectCells (optflow4d.cpp:713-734), bnd=2 */
static void project_cells(dims4 d, REAL *dst, const REAL *vel,
                          const REAL *phiOrg, const REAL *phiTarget,
                          REAL *marker, REAL threshPhi, int maxIter) {
  const REAL dt = 1.0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 2; t < d.t - 2; ++t)
    for (int k = 2; k < d.z - 2; ++k)
      for (int j = 2; j < d.y - 2; ++j)
        for (int i = 2; i < d.x - 2; ++i) {
          idx_t id = index4(d, i, j, k, t);
          const REAL *v = vel + id * 4;
          REAL pos[4];
          pos[0] = (REAL)(i + 0.5f) - v[0] * dt;
          pos[1] = (REAL)(j + 0.5f) - v[1] * dt;
          pos[2] = (REAL)(k + 0.5f) - v[2] * dt;
          pos[3] = (REAL)(t + 0.5f) - v[3] * dt;
          vec4 n = normal_interp(d, phiOrg, pos);
          REAL dd = project_cell(d, n, phiOrg, phiTarget, pos, i, j, k, t, maxIter);
          if (R_FABS(dd) > threshPhi) {
            dst[id * 4 + 0] = dst[id * 4 + 1] = dst[id * 4 + 2] = dst[id * 4 + 3] = 0.;
            continue;
          }
          for (int c = 0; c < 4; ++c) dst[id * 4 + c] = n.v[c] * dd;
          marker[id] = 1.;
        }
}
EXPORT void ORC_SYM(projectCells)(const int *dims, REAL *dst, const REAL *vel,
                                  const REAL *phiOrg, const REAL *phiTarget,
                                  REAL *marker, REAL threshPhi, int maxIter) {
  project_cells(mkdims(dims), dst, vel, phiOrg, phiTarget, marker, threshPhi,
                maxIter);
}

/* corrVelsOfTempl (optflow4d.cpp:737-802) */
static void corr_vels_of(dims4 d, REAL *dst, REAL *vel, const REAL *phiOrg,
                         const REAL *phiTarget, REAL threshPhi,
                         REAL postVelBlur, REAL resetBndWidth, int maxIter,
                         int *expolOut) {
  const idx_t nc = ncell(d), n = nc * 4;
  const REAL blurThreshold = 0.98;
  int doCvExtrapol = trunc_int(vec4_maxnorm(d, vel) + 4);
  if (expolOut) *expolOut = doCvExtrapol;
  REAL *marker = (REAL *)xcalloc(nc, sizeof(REAL));
  REAL *tmp = (REAL *)xcalloc(n, sizeof(REAL));
  int singleStep = 0;
  if (postVelBlur < blurThreshold) singleStep = 1;
  while ((postVelBlur >= blurThreshold) || singleStep) {
    for (idx_t q = 0; q < n; ++q) dst[q] = 0.;
    for (idx_t q = 0; q < nc; ++q) marker[q] = 0;
    project_cells(d, dst, vel, phiOrg, phiTarget, marker, threshPhi, maxIter);
    expol_sweeps(d, dst, tmp, marker, doCvExtrapol);
    if (postVelBlur > VEC_EPS) gaussian_blur(d, dst, 4, (REAL)(0.5 * postVelBlur), 1);
    const int resetBnd = trunc_int(resetBndWidth * (REAL)d.x) + 1;
    if (resetBndWidth > 0.) {
      const REAL z4[4] = {0, 0, 0, 0};
      int dd[4] = {d.x, d.y, d.z, d.t};
      ORC_SYM(setBound)(dd, dst, 4, z4, resetBnd);
    }
    /* vel.addScaled(dst, Vec4(-1.)) */
    for (idx_t q = 0; q < n; ++q) vel[q] += (REAL)-1. * dst[q];
    postVelBlur *= 0.5;
    if (singleStep > 0) singleStep--;
  }
  free(marker);
  free(tmp);
}
EXPORT void ORC_SYM(corrVelsOf4d)(const int *dims, REAL *dst, REAL *vel,
                                  const REAL *phiOrg, const REAL *phiTarget,
                                  REAL threshPhi, REAL postVelBlur,
                                  REAL resetBndWidth, int maxIter,
                                  int *expolOut) {
  corr_vels_of(mkdims(dims), dst, vel, phiOrg, phiTarget, threshPhi,
               postVelBlur, resetBndWidth, maxIter, expolOut);
}

/* ------------------------------------------------------------------------ */
/* Multiscale driver                                                          */
/* ------------------------------------------------------------------------ */

typedef struct {
  REAL wSmooth, wEnergy;
  int level;
  REAL postVelBlur, cgAccuracy;
  int blurType;
  REAL cfl;
  int orderTime, orderSpace;
  REAL resetBndWidth;
  int multiStep, projSizeThresh, minGridSize, doFinalProject;
  int cgMaxIter;
} orc_ms_params;

static void vadd(REAL *a, const REAL *b, idx_t n) {
#pragma omp parallel for schedule(static)
  for (idx_t q = 0; q < n; ++q) a[q] += b[q];
}

/* opticalFlowMultiscaleTemplate (optflow4d.cpp:936-1173) */
static REAL of_multiscale(dims4 d, REAL *vel, const REAL *i0, const REAL *i1,
                          orc_ms_params p, int level) {
  const idx_t nc = ncell(d), n4 = nc * 4;
  const int resetBnd =
      p.resetBndWidth > 0 ? trunc_int(p.resetBndWidth * (REAL)d.x) + 1 : 0;
  const REAL projMaxDist = 4.;
  const REAL projMaxIter = 40.;
  const REAL lsDiffFac = (REAL)(0.1 / 20.);
  int dd4[4] = {d.x, d.y, d.z, d.t};
  orc_of_params op;
  op.wSmooth = p.wSmooth;
  op.wEnergy = p.wEnergy;
  op.cgAccuracy = p.cgAccuracy;
  op.resetBndWidth = p.resetBndWidth;
  op.blurType = p.blurType;
  op.cgMaxIter = p.cgMaxIter;

  REAL *i0warped = (REAL *)xcalloc(nc, sizeof(REAL));
  memcpy(i0warped, i0, (size_t)nc * sizeof(REAL));
  REAL errPreOf = ORC_SYM(calcLsDiff4d)(dd4, i0, i1, NULL, lsDiffFac, resetBnd);

  if (d.x > p.minGridSize) {
    dims4 sd = {d.x / 2, d.y / 2, d.z / 2, d.t / 2};
    idx_t snc = ncell(sd);
    REAL *velSm = (REAL *)xcalloc(snc * 4, sizeof(REAL));
    REAL *i0Sm = (REAL *)xcalloc(snc, sizeof(REAL));
    REAL *i1Sm = (REAL *)xcalloc(snc, sizeof(REAL));
    interpol_grid(sd, i0Sm, d, i0, 1);
    interpol_grid(sd, i1Sm, d, i1, 1);
    interpol_grid(sd, velSm, d, vel, 4);
    for (idx_t q = 0; q < snc * 4; ++q) velSm[q] *= (REAL)0.5;
    of_multiscale(sd, velSm, i0Sm, i1Sm, p, level + 1);
    interpol_grid(d, vel, sd, velSm, 4);
    for (idx_t q = 0; q < n4; ++q) vel[q] *= (REAL)2.;
    free(velSm);
    free(i0Sm);
    free(i1Sm);
  }

  advect_cfl(d, p.cfl, vel, i0warped, 1);
  ORC_SYM(setBoundNeumann)(dd4, i0warped, 1, 0);
  REAL errCurr = ORC_SYM(calcLsDiff4d)(dd4, i0warped, i1, NULL, lsDiffFac, resetBnd);

  int doProject = 0;
  int multiStep = p.multiStep;
  int doFinalProject = p.doFinalProject;
  if (d.x > p.projSizeThresh) {
    doProject = 1;
    multiStep = 1;
    if (doFinalProject) doFinalProject = 0;
  }

  if (multiStep > 1) {
    REAL *vs[10];
    REAL *vs2[10];
    for (int of = 0; of < multiStep; ++of) {
      vs[of] = NULL;
      vs2[of] = (REAL *)xcalloc(n4, sizeof(REAL));
    }
    REAL *tmpVel = (REAL *)xcalloc(n4, sizeof(REAL));
    memcpy(tmpVel, vel, (size_t)n4 * sizeof(REAL));
    REAL *i0warp2 = (REAL *)xcalloc(nc, sizeof(REAL));
    REAL velBlur = p.postVelBlur;
    REAL errLast = errCurr;
    int ofStepsCurr = multiStep;
    for (int of = 0; of < ofStepsCurr; ++of) {
      vs[of] = (REAL *)xcalloc(n4, sizeof(REAL));
      op.postVelBlur = velBlur;
      optical_flow_dim(d, vs[of], i0warped, i1, &op, NULL);
      velBlur *= (REAL)(3. / 4.);
      if (velBlur < 2.) velBlur = 2.;
      for (int k = of; k >= 0; --k) memcpy(vs2[k], vs[k], (size_t)n4 * sizeof(REAL));
      for (int k = of - 1; k >= 0; --k)
        for (int l = 0; l < k; ++l) advect_cfl(d, p.cfl, vs2[k], vs2[l], 4);
      memcpy(tmpVel, vel, (size_t)n4 * sizeof(REAL));
      for (int k = of; k >= 0; --k) vadd(tmpVel, vs2[k], n4);
      memcpy(i0warp2, i0, (size_t)nc * sizeof(REAL));
      advect_cfl(d, p.cfl, tmpVel, i0warp2, 1);
      ORC_SYM(setBoundNeumann)(dd4, i0warp2, 1, 0);
      REAL errC = ORC_SYM(calcLsDiff4d)(dd4, i0warp2, i1, NULL, lsDiffFac, resetBnd);
      memcpy(i0warped, i0warp2, (size_t)nc * sizeof(REAL));
      if (of > 0 && (errC / errLast) > 0.95) {
        for (idx_t q = 0; q < n4; ++q) vs[of][q] = 0.;
        ofStepsCurr = of + 1;
      }
      errLast = errC;
    }
    for (int of = ofStepsCurr - 1; of >= 0; --of)
      for (int l = 0; l < of; ++l) advect_cfl(d, p.cfl, vs[of], vs[l], 4);
    for (int of = 0; of < ofStepsCurr; ++of) {
      vadd(vel, vs[of], n4);
      free(vs[of]);
    }
    for (int of = 0; of < multiStep; ++of) free(vs2[of]);
    free(tmpVel);
    free(i0warp2);
  } else {
    REAL *velCurr = (REAL *)xcalloc(n4, sizeof(REAL));
    if (!doProject) {
      op.postVelBlur = p.postVelBlur;
      optical_flow_dim(d, velCurr, i0warped, i1, &op, NULL);
      vadd(vel, velCurr, n4);
    } else {
      REAL *velTmp2 = (REAL *)xcalloc(n4, sizeof(REAL));
      corr_vels_of(d, velCurr, velTmp2, i0warped, i1, projMaxDist,
                   p.postVelBlur, p.resetBndWidth, (int)projMaxIter, NULL);
      vadd(vel, velTmp2, n4);
      for (idx_t q = 0; q < n4; ++q) velCurr[q] *= (REAL)-1.;
      vadd(vel, velCurr, n4);
      free(velTmp2);
    }
    free(velCurr);
  }

  if (level == 0 && doFinalProject) {
    REAL *velCurr = (REAL *)xcalloc(n4, sizeof(REAL));
    REAL finalProjBlur = 4.;
    corr_vels_of(d, velCurr, vel, i0, i1, projMaxDist, finalProjBlur,
                 p.resetBndWidth, (int)projMaxIter, NULL);
    free(velCurr);
  }

  if (level == 0) {
    memcpy(i0warped, i0, (size_t)nc * sizeof(REAL));
    advect_cfl(d, p.cfl, vel, i0warped, 1);
    ORC_SYM(setBoundNeumann)(dd4, i0warped, 1, 0);
    REAL errFinal = ORC_SYM(calcLsDiff4d)(dd4, i0warped, i1, NULL, lsDiffFac, resetBnd);
    errCurr = errFinal;
  }
  (void)errPreOf;
  free(i0warped);
  return errCurr;
}

/* opticalFlowMultiscale4d (optflow4d.cpp:2182-2195).  params layout:
 * f[0] wSmooth, f[1] wEnergy, f[2] postVelBlur, f[3] cgAccuracy, f[4] cfl,
 * f[5] resetBndWidth; k[0] level, k[1] blurType, k[2] orderTime,
 * k[3] orderSpace, k[4] multiStep, k[5] projSizeThresh, k[6] minGridSize,
 * k[7] doFinalProject, k[8] cgMaxIter. */
EXPORT REAL ORC_SYM(opticalFlowMultiscale4d)(const int *dims, REAL *vel,
                                             const REAL *i0, const REAL *i1,
                                             const REAL *f, const int *k) {
  orc_ms_params p;
  p.wSmooth = f[0];
  p.wEnergy = f[1];
  p.postVelBlur = f[2];
  p.cgAccuracy = f[3];
  p.cfl = f[4];
  p.resetBndWidth = f[5];
  p.level = k[0];
  p.blurType = k[1];
  p.orderTime = k[2];
  p.orderSpace = k[3];
  p.multiStep = k[4];
  p.projSizeThresh = k[5];
  p.minGridSize = k[6];
  p.doFinalProject = k[7];
  p.cgMaxIter = k[8];
  return of_multiscale(mkdims(dims), vel, i0, i1, p, p.level);
}

/* ------------------------------------------------------------------------ */
/* Applying a deformation                                                     */
/* ------------------------------------------------------------------------ */

/* deform4d of scenes/flof.py:591-615 (modes 2): one-way advect at alpha,
 * two-way (twoway=1) blends with the inverse advect at 1-alpha. */
EXPORT void ORC_SYM(deform4d)(const int *dims, const REAL *vel,
                              const REAL *velInv, const REAL *i0,
                              const REAL *i1, REAL *out, REAL alpha,
                              REAL alphaInv, int twoway) {
  dims4 d = mkdims(dims);
  idx_t nc = ncell(d);
  memcpy(out, i0, (size_t)nc * sizeof(REAL));
  ORC_SYM(advect4d)(dims, vel, out, 1, alpha);
  if (twoway == 1) {
    REAL *i1adv = (REAL *)xcalloc(nc, sizeof(REAL));
    memcpy(i1adv, i1, (size_t)nc * sizeof(REAL));
    ORC_SYM(advect4d)(dims, velInv, i1adv, 1, alphaInv);
    for (idx_t q = 0; q < nc; ++q) out[q] *= alphaInv;
    for (idx_t q = 0; q < nc; ++q) out[q] += alpha * i1adv[q];
    free(i1adv);
  } else if (twoway == 2) {
    for (idx_t q = 0; q < nc; ++q) out[q] *= alphaInv;
    for (idx_t q = 0; q < nc; ++q) out[q] += alpha * i1[q];
  }
}

/* knSemiLagrangeLookupSlice4d_WithVel (optflow4d.cpp:1648-1665), a
 * KERNEL(bnd=10) over the 3D dst grid plus the bordSkip test.  v1 is the
 * time-blended Vec4 defo slice of size vdims[0..2]. */
static void lookup_slice(const int *dstDims, REAL *dst, dims4 pd,
                         const REAL *phi, REAL time, REAL dt, const REAL *v1,
                         const int *vdims, const REAL *sf3, const REAL *off3,
                         const REAL *defoFactor, int bordSkip) {
  const int X = dstDims[0], Y = dstDims[1], Z = dstDims[2];
  const idx_t vZ = (idx_t)vdims[0] * vdims[1];
#pragma omp parallel for schedule(static)
  for (int k = 10; k < Z - 10; ++k)
    for (int j = 10; j < Y - 10; ++j)
      for (int i = 10; i < X - 10; ++i) {
        if (!(i >= bordSkip && j >= bordSkip && i < X - bordSkip &&
              j < Y - bordSkip && k >= bordSkip && k < Z - bordSkip))
          continue;
        REAL pos3[3];
        pos3[0] = (REAL)i * sf3[0] + off3[0];
        pos3[1] = (REAL)j * sf3[1] + off3[1];
        pos3[2] = (REAL)k * sf3[2] + off3[2];
        vec4 v = interp3_vec4(v1, vdims, vZ, pos3);
        for (int c = 0; c < 4; ++c) v.v[c] *= defoFactor[c];
        REAL pos4[4];
        pos4[0] = (REAL)(i + 0.5f) - v.v[0] * dt;
        pos4[1] = (REAL)(j + 0.5f) - v.v[1] * dt;
        pos4[2] = (REAL)(k + 0.5f) - v.v[2] * dt;
        pos4[3] = (REAL)(time + 0.5f) - v.v[3] * dt;
        dst[(idx_t)i + (idx_t)X * j + (idx_t)X * Y * k] = interp4_real(phi, pd, pos4);
      }
}

/* One loadAdvectTimeSlice_OptRun call (optflow4d.cpp:1951-2105) without
 * defo volumes: the defo (defoDims, Vec4) is held in memory instead of being
 * streamed from a .uni file slice by slice.  dst is 3D (dstDims[0..2]) and is
 * only written inside the bnd=10 / bordSkip region. */
EXPORT void ORC_SYM(optRunFrame)(const int *defoDims, const REAL *defo,
                                 const int *dstDims, REAL *dst,
                                 const int *phiDims, const REAL *phi, REAL time,
                                 REAL blendAlpha, REAL loadTimeScale,
                                 const REAL *defoOffset, const REAL *defoScale,
                                 const REAL *defoFactor, const REAL *overrideSize,
                                 REAL overrideTimeOff, int bordSkip,
                                 REAL defoAniFac) {
  const int dimT = defoDims[3];
  REAL dim4[4] = {(REAL)defoDims[0], (REAL)defoDims[1], (REAL)defoDims[2],
                  (REAL)defoDims[3]};
  int defoSizeI[4] = {phiDims[0], phiDims[1], phiDims[2], phiDims[3]};
  if (overrideSize[0] > 0.) {
    for (int c = 0; c < 4; ++c) defoSizeI[c] = trunc_int(overrideSize[c]);
  }
  REAL defoSize[4], sf[4], off2[4], neg1[4] = {-1, -1, -1, -1};
  for (int c = 0; c < 4; ++c) {
    defoSize[c] = (REAL)defoSizeI[c];
    off2[c] = defoOffset[c];
  }
  ORC_SYM(gridFactor4d)(dim4, defoSize, neg1, defoScale, sf, off2);
  REAL srcTime = (REAL)((double)(time * sf[3] * loadTimeScale + off2[3]) - 0.5);
  int t = trunc_int(srcTime);
  int tp1 = t + 1;
  REAL tw = srcTime - (REAL)t;
  if (t > dimT - 1) t = dimT - 1;
  if (tp1 > dimT - 1) tp1 = dimT - 1;
  const idx_t slice = (idx_t)defoDims[0] * defoDims[1] * defoDims[2];
  REAL *vt = (REAL *)xcalloc(slice * 4, sizeof(REAL));
  const REAL *v1 = defo + (idx_t)t * slice * 4;
  const REAL *v2 = defo + (idx_t)tp1 * slice * 4;
  const REAL f1 = (REAL)(1. - tw), f2 = tw;
  for (idx_t q = 0; q < slice * 4; ++q) {
    vt[q] = 0.;
    vt[q] += f1 * v1[q];
    vt[q] += f2 * v2[q];
  }
  REAL df[4];
  for (int c = 0; c < 4; ++c) df[c] = defoFactor[c] * defoAniFac;
  REAL sf3[3] = {sf[0], sf[1], sf[2]}, off3[3] = {off2[0], off2[1], off2[2]};
  lookup_slice(dstDims, dst, mkdims(phiDims), phi, time + overrideTimeOff,
               blendAlpha, vt, defoDims, sf3, off3, df, bordSkip);
  free(vt);
}

/* ------------------------------------------------------------------------ */
/* Input conditioning (scenes/flof.py postProcessPhiData :491-531)          */
/* ------------------------------------------------------------------------ */

/* repeatFrame4d (optflow4d.cpp:1254-1266): serial and in place like the
 * reference.  The reference does not range-check t; slices outside [0, T)
 * are skipped here. */
EXPORT void ORC_SYM(repeatFrame4d)(const int *dims, REAL *phi, REAL srct,
                                   REAL range, int bnd) {
  const dims4 d = mkdims(dims);
  const int t0 = trunc_int_d((double)(srct - range) + 0.5);
  const int t1 = trunc_int(srct);
  for (int t = t0; t <= t1; t++) {
    if (t < 0 || t >= d.t) continue;
    for (int k = bnd; k < d.z - bnd; ++k)
      for (int j = bnd; j < d.y - bnd; j++)
        for (int i = bnd; i < d.x - bnd; i++) {
          const REAL pos[4] = {(REAL)i + (REAL)0.5, (REAL)j + (REAL)0.5,
                               (REAL)k + (REAL)0.5, srct + (REAL)0.5};
          phi[index4(d, i, j, k, t)] = interp4_real(phi, d, pos);
        }
  }
}

/* extrap4dLsSimple (optflow4d.cpp:1332-1406) with its Grid4d<int> marks;
 * knExtrap4dLsSimple (:1328-1350) and knSetRemaining4d (:1352-1357) run
 * serially over the bnd = 1 box (both are race-free as parallel kernels: a
 * sweep reads only cells marked d and writes only cells marked 0). */
EXPORT void ORC_SYM(extrap4dLsSimple)(const int *dims, REAL *phi, int distance,
                                      int inside) {
  const dims4 d = mkdims(dims);
  const idx_t n = ncell(d);
  int *tmp = (int *)xcalloc(n, sizeof(int));
  /* nbs4d (optflow4d.cpp:1323-1326): -x,+x,-y,+y,-z,+z,-t,+t */
  const idx_t off[8] = {-1, 1, -(idx_t)d.x, (idx_t)d.x, -(idx_t)d.x * d.y,
                        (idx_t)d.x * d.y, -(idx_t)d.x * d.y * d.z,
                        (idx_t)d.x * d.y * d.z};
  REAL direction = 1.;
  if (inside) direction = -1.;
  for (int t = 1; t < d.t - 1; ++t)
    for (int k = 1; k < d.z - 1; ++k)
      for (int j = 1; j < d.y - 1; ++j)
        for (int i = 1; i < d.x - 1; ++i) {
          const idx_t q = index4(d, i, j, k, t);
          if (!inside ? (phi[q] < 0.) : (phi[q] > 0.)) tmp[q] = 1;
        }
  for (int t = 1; t < d.t - 1; ++t)
    for (int k = 1; k < d.z - 1; ++k)
      for (int j = 1; j < d.y - 1; ++j)
        for (int i = 1; i < d.x - 1; ++i) {
          const idx_t q = index4(d, i, j, k, t);
          if (tmp[q]) continue;
          for (int m = 0; m < 8; ++m)
            if (tmp[q + off[m]] == 1) {
              tmp[q] = 2;
              break;
            }
        }
  for (int dd = 2; dd < 1 + distance; ++dd)
    for (int t = 1; t < d.t - 1; ++t)
      for (int k = 1; k < d.z - 1; ++k)
        for (int j = 1; j < d.y - 1; ++j)
          for (int i = 1; i < d.x - 1; ++i) {
            const idx_t q = index4(d, i, j, k, t);
            if (tmp[q] != 0) continue;
            int nbs = 0;
            REAL avg = 0.;
            for (int m = 0; m < 8; ++m)
              if (tmp[q + off[m]] == dd) {
                avg += phi[q + off[m]];
                nbs++;
              }
            if (nbs > 0) {
              tmp[q] = dd + 1;
              phi[q] = avg / (REAL)nbs + direction;
            }
          }
  for (int t = 1; t < d.t - 1; ++t)
    for (int k = 1; k < d.z - 1; ++k)
      for (int j = 1; j < d.y - 1; ++j)
        for (int i = 1; i < d.x - 1; ++i) {
          const idx_t q = index4(d, i, j, k, t);
          if (tmp[q] == 0) phi[q] = (REAL)(direction * (REAL)(distance + 2));
        }
  free(tmp);
}

/* ------------------------------------------------------------------------ */
/* 3D Grid<Real> methods of the mode-3 output stage                          */
/* ------------------------------------------------------------------------ */

/* LevelsetGrid::join (levelset.cpp:114-118): a = std::min(a, b). */
EXPORT void ORC_SYM(join)(idx_t n, REAL *a, const REAL *b) {
  for (idx_t q = 0; q < n; ++q) a[q] = (b[q] < a[q]) ? b[q] : a[q];
}

/* Grid<T>::setBound (grid.cpp:462-473) of a 3D grid (dims3 = X, Y, Z). */
EXPORT void ORC_SYM(setBound3)(const int *dims3, REAL *a, int nc, const REAL *v,
                               int w) {
  const int X = dims3[0], Y = dims3[1], Z = dims3[2];
  const int is3d = Z > 1;
  for (int k = 0; k < Z; ++k)
    for (int j = 0; j < Y; ++j)
      for (int i = 0; i < X; ++i) {
        const int b = (i <= w || i >= X - 1 - w || j <= w || j >= Y - 1 - w ||
                       (is3d && (k <= w || k >= Z - 1 - w)));
        if (!b) continue;
        const idx_t q = (idx_t)i + (idx_t)X * j + (idx_t)X * Y * k;
        for (int c = 0; c < nc; ++c) a[q * nc + c] = v[c];
      }
}

/* Grid<T>::setBoundNeumann (grid.cpp:475-511) of a 3D grid. */
EXPORT void ORC_SYM(setBoundNeumann3)(const int *dims3, REAL *a, int nc, int w) {
  const int X = dims3[0], Y = dims3[1], Z = dims3[2];
  const int is3d = Z > 1;
  for (int k = 0; k < Z; ++k)
    for (int j = 0; j < Y; ++j)
      for (int i = 0; i < X; ++i) {
        int set = 0, si = i, sj = j, sk = k;
        if (i <= w) { si = w + 1; set = 1; }
        if (i >= X - 1 - w) { si = X - 1 - w - 1; set = 1; }
        if (j <= w) { sj = w + 1; set = 1; }
        if (j >= Y - 1 - w) { sj = Y - 1 - w - 1; set = 1; }
        if (is3d) {
          if (k <= w) { sk = w + 1; set = 1; }
          if (k >= Z - 1 - w) { sk = Z - 1 - w - 1; set = 1; }
        }
        if (!set) continue;
        const idx_t q = (idx_t)i + (idx_t)X * j + (idx_t)X * Y * k;
        const idx_t s = (idx_t)si + (idx_t)X * sj + (idx_t)X * Y * sk;
        for (int c = 0; c < nc; ++c) a[q * nc + c] = a[s * nc + c];
      }
}

/* simpleBlurSpecial / knSimpleBlurSpecial (test.cpp:94-131) of a 3D grid:
 * `iter` passes into a fresh zeroed grid with a swap after each. */
EXPORT void ORC_SYM(simpleBlurSpecial)(const int *dims3, REAL *a, int iter,
                                       REAL thresh, int bord) {
  const int X = dims3[0], Y = dims3[1], Z = dims3[2];
  const int is3d = Z > 1;
  const idx_t n = (idx_t)X * Y * Z, sY = X, sZ = (idx_t)X * Y;
  REAL *tmp = (REAL *)xcalloc(n, sizeof(REAL));
  REAL *cur = a, *nxt = tmp;
  for (int it = 0; it < iter; ++it) {
    for (int k = is3d ? 1 : 0; k < (is3d ? Z - 1 : 1); ++k)
      for (int j = 1; j < Y - 1; ++j)
        for (int i = 1; i < X - 1; ++i) {
          const idx_t q = (idx_t)i + sY * j + sZ * k;
          int inb = i >= bord && j >= bord && i < X - bord && j < Y - bord;
          inb = inb && (is3d ? (k >= bord && k < Z - bord) : (k == 0));
          if (!inb || cur[q] < thresh) {
            nxt[q] = cur[q];
            continue;
          }
          nxt[q] = cur[q + 1] + cur[q - 1] + cur[q + sY] + cur[q - sY];
          if (is3d) {
            nxt[q] += cur[q + sZ] + cur[q - sZ];
            nxt[q] = (REAL)((double)nxt[q] * (1. / 6.));
          } else {
            nxt[q] = (REAL)((double)nxt[q] * (1. / 4.));
          }
        }
    REAL *sw = cur;
    cur = nxt;
    nxt = sw;
  }
  if (cur != a) memcpy(a, cur, (size_t)n * sizeof(REAL));
  free(tmp);
}

/* ------------------------------------------------------------------------ */
/* Hi-res 4D assembly (scenes/flof.py :707-723)                              */
/* ------------------------------------------------------------------------ */

/* interpol<Real> (interpol.h:57-95) on a 3D Real grid. */
static inline REAL interp3_real(const REAL *data, const int *size, idx_t Zs,
                                const REAL *pos) {
  REAL px = pos[0] - 0.5f, py = pos[1] - 0.5f, pz = pos[2] - 0.5f;
  int xi = trunc_int(px), yi = trunc_int(py), zi = trunc_int(pz);
  REAL s1 = px - (REAL)xi, s0 = (REAL)(1. - s1);
  REAL t1 = py - (REAL)yi, t0 = (REAL)(1. - t1);
  REAL f1 = pz - (REAL)zi, f0 = (REAL)(1. - f1);
  if (px < 0.) { xi = 0; s0 = 1.0; s1 = 0.0; }
  if (py < 0.) { yi = 0; t0 = 1.0; t1 = 0.0; }
  if (pz < 0.) { zi = 0; f0 = 1.0; f1 = 0.0; }
  if (xi >= size[0] - 1) { xi = size[0] - 2; s0 = 0.0; s1 = 1.0; }
  if (yi >= size[1] - 1) { yi = size[1] - 2; t0 = 0.0; t1 = 1.0; }
  if (size[2] > 1) {
    if (zi >= size[2] - 1) { zi = size[2] - 2; f0 = 0.0; f1 = 1.0; }
  }
  const idx_t X = 1, Y = size[0], Z = Zs;
  const idx_t i = (idx_t)xi + (idx_t)size[0] * yi + Zs * zi;
  return ((data[i] * t0 + data[i + Y] * t1) * s0 +
          (data[i + X] * t0 + data[i + X + Y] * t1) * s1) *
             f0 +
         ((data[i + Z] * t0 + data[i + Y + Z] * t1) * s0 +
          (data[i + X + Z] * t0 + data[i + X + Y + Z] * t1) * s1) *
             f1;
}

/* loadPlaceGrid4d (optflow4d.cpp:1460-1594) with the 3D slice files held in
 * memory: slices + q * sdims3[0]*sdims3[1]*sdims3[2] is file index
 * fileIdxStart + q (q < nfiles).  knLoadPlaceGridIpol (:1443-1450) and
 * knLoadPlaceGridRescale (:1452-1458) run serially over the bnd = 1 box. */
EXPORT void ORC_SYM(loadPlaceGrid4d)(
    const int *dims, REAL *phi, const int *sdims3, const REAL *slices, int nfiles,
    const REAL *offset, const REAL *scale, int fileIdxStart, int fileIdxEnd,
    int debugSkipLoad, REAL spread, const REAL *overrideSize, REAL overrideTimeOff,
    int overrideGoodRegion, REAL loadTimeScale, int rescaleSdfValues,
    REAL sdfIsoOff, REAL repeatStartFrame) {
  const dims4 d = mkdims(dims);
  const idx_t n3 = (idx_t)sdims3[0] * sdims3[1] * sdims3[2];
  const idx_t Zs = sdims3[2] > 1 ? (idx_t)sdims3[0] * sdims3[1] : 0;
  REAL v1[4] = {(REAL)sdims3[0], (REAL)sdims3[1], (REAL)sdims3[2], 1};
  REAL defoSize[4] = {(REAL)d.x, (REAL)d.y, (REAL)d.z, (REAL)d.t};
  if (overrideSize[0] > 0.)
    for (int c = 0; c < 4; ++c) defoSize[c] = overrideSize[c];
  REAL sf[4], off2[4], neg1[4] = {-1, -1, -1, -1};
  for (int c = 0; c < 4; ++c) off2[c] = offset[c];
  ORC_SYM(gridFactor4d)(v1, defoSize, neg1, scale, sf, off2);
  REAL valueScale = 1.;
  if (rescaleSdfValues) valueScale = (REAL)(1. / sf[0]);
  REAL *w = (REAL *)xcalloc(d.t, sizeof(REAL));
  const idx_t sT = (idx_t)d.x * d.y * d.z;
  if (overrideGoodRegion <= 0) {
    memset(phi, 0, sizeof(REAL) * (size_t)(sT * d.t));
  } else if (overrideGoodRegion < d.t) {
    memset(phi + sT * overrideGoodRegion, 0,
           sizeof(REAL) * (size_t)(sT * (d.t - overrideGoodRegion)));
  }
  if (fileIdxStart < 0) fileIdxStart = 0;
  if (fileIdxEnd < 0) fileIdxEnd = trunc_int(defoSize[3]);
  int repeatOff = 0;
  if (repeatStartFrame > 0)
    repeatOff = trunc_int_d((double)((REAL)(fileIdxEnd - fileIdxStart) * repeatStartFrame) + 1.0);
  REAL *tmp = (REAL *)xcalloc(n3, sizeof(REAL));
  const int endId = fileIdxEnd < debugSkipLoad ? fileIdxEnd : debugSkipLoad;
  for (int fileid = fileIdxStart - repeatOff; fileid < endId; ++fileid) {
    const int fileidClamp = fileid > fileIdxStart ? fileid : fileIdxStart;
    int didLoad = 0;
    const REAL duration =
        (REAL)(1. * (double)(defoSize[3] * scale[3] / loadTimeScale) /
               (double)(REAL)(fileIdxEnd - fileIdxStart));
    const REAL dstt = offset[3] + overrideTimeOff + duration * (REAL)(fileid - fileIdxStart);
    const int s0 = trunc_int(dstt - spread * duration) + 0;
    const int s1 = trunc_int(dstt + spread * duration) + 2;
    for (int slice = s0; slice < s1; ++slice) {
      if (slice < overrideGoodRegion || slice >= d.t) continue;
      const REAL q = R_FABS((REAL)slice - dstt) / (duration * spread);
      const REAL wc = (REAL)(1. - (double)q);
      if (wc < VEC_EPS) continue;
      w[slice] += wc;
      if (!didLoad) {
        const int qi = fileidClamp - fileIdxStart;
        if (qi < 0 || qi >= nfiles) abort(); /* the caller supplies every file */
        memcpy(tmp, slices + (idx_t)qi * n3, sizeof(REAL) * (size_t)n3);
        if (rescaleSdfValues && sdfIsoOff != 0.) {
          const int X = sdims3[0], Y = sdims3[1], Z = sdims3[2];
          for (int k = Z > 1 ? 1 : 0; k < (Z > 1 ? Z - 1 : 1); ++k)
            for (int j = 1; j < Y - 1; ++j)
              for (int i = 1; i < X - 1; ++i)
                tmp[(idx_t)i + (idx_t)X * j + (idx_t)X * Y * k] += sdfIsoOff;
          const REAL one = 1.;
          ORC_SYM(setBound3)(sdims3, tmp, 1, &one, 1);
        }
        didLoad = 1;
      }
      for (int k = 1; k < d.z - 1; ++k)
        for (int j = 1; j < d.y - 1; ++j)
          for (int i = 1; i < d.x - 1; ++i) {
            REAL p[3];
            p[0] = (REAL)i * sf[0] + off2[0];
            p[1] = (REAL)j * sf[1] + off2[1];
            p[2] = (REAL)k * sf[2] + off2[2];
            phi[index4(d, i, j, k, slice)] += wc * interp3_real(tmp, sdims3, Zs, p);
          }
    }
  }
  for (int s = 0; s < d.t; ++s) {
    if (w[s] < 1e-03) {
      w[s] = 0.;
    } else {
      w[s] = (REAL)(1. / w[s]);
      w[s] *= valueScale;
    }
  }
  for (int t = 1; t < d.t - 1; ++t) {
    if (w[t] <= 0.) continue;
    for (int k = 1; k < d.z - 1; ++k)
      for (int j = 1; j < d.y - 1; ++j)
        for (int i = 1; i < d.x - 1; ++i) phi[index4(d, i, j, k, t)] *= w[t];
  }
  free(tmp);
  free(w);
}

/* loadAdvectTimeSlice (optflow4d.cpp:1671-1760), the non-optimised twin of
 * loadAdvectTimeSlice_OptRun: the deformation slices t and t+1 (defo, held
 * in memory) are blended, interpolated to the 3D dst size over its bnd = 1
 * box (loadAdvReInterpol), and knSemiLagrangeLookupSlice4d (:1622-1629)
 * looks phi up over the same box.  With a t extent of 1 the reference's
 * fourd kernel runs its 3D branch at t = 0 (codegen_kernel.cpp:243-263). */
EXPORT void ORC_SYM(loadAdvectTimeSlice)(
    const int *defoDims, const REAL *defo, const int *dstDims, REAL *dst,
    const int *phiDims, const REAL *phi, REAL time, REAL blendAlpha,
    REAL loadTimeScale, const REAL *defoOffset, const REAL *defoScale,
    const REAL *defoFactor, const REAL *overrideSize, REAL overrideTimeOff,
    int zeroVel, REAL defoAniFac) {
  const int dimT = defoDims[3];
  REAL dim4[4] = {(REAL)defoDims[0], (REAL)defoDims[1], (REAL)defoDims[2],
                  (REAL)defoDims[3]};
  int defoSizeI[4] = {phiDims[0], phiDims[1], phiDims[2], phiDims[3]};
  if (overrideSize[0] > 0.)
    for (int c = 0; c < 4; ++c) defoSizeI[c] = trunc_int(overrideSize[c]);
  REAL defoSize[4], sf[4], off2[4], neg1[4] = {-1, -1, -1, -1};
  for (int c = 0; c < 4; ++c) {
    defoSize[c] = (REAL)defoSizeI[c];
    off2[c] = defoOffset[c];
  }
  ORC_SYM(gridFactor4d)(dim4, defoSize, neg1, defoScale, sf, off2);
  REAL srcTime = (REAL)((double)(time * sf[3] * loadTimeScale + off2[3]) - 0.5);
  int t = trunc_int(srcTime);
  int tp1 = t + 1;
  REAL tw = srcTime - (REAL)t;
  if (t > dimT - 1) t = dimT - 1;
  if (tp1 > dimT - 1) tp1 = dimT - 1;
  const idx_t slice = (idx_t)defoDims[0] * defoDims[1] * defoDims[2];
  REAL *v1 = (REAL *)xcalloc(slice * 4, sizeof(REAL));
  const REAL *a = defo + (idx_t)t * slice * 4;
  const REAL *b = defo + (idx_t)tp1 * slice * 4;
  const REAL f1 = (REAL)(1. - tw), f2 = tw;
  /* v1.multConst(1-tw); v2.multConst(tw); v1.add(v2) */
  for (idx_t q = 0; q < slice * 4; ++q) v1[q] = a[q] * f1 + b[q] * f2;
  if (zeroVel)
    for (idx_t q = 0; q < slice * 4; ++q) v1[q] = 0.;
  const int X = dstDims[0], Y = dstDims[1], Z = dstDims[2];
  const idx_t vZ = (idx_t)defoDims[0] * defoDims[1];
  REAL df[4];
  for (int c = 0; c < 4; ++c) df[c] = defoFactor[c] * defoAniFac;
  const dims4 pd = mkdims(phiDims);
  const REAL T0 = time + overrideTimeOff;
  for (int k = 1; k < Z - 1; ++k)
    for (int j = 1; j < Y - 1; ++j)
      for (int i = 1; i < X - 1; ++i) {
        REAL pos3[3];
        pos3[0] = (REAL)i * sf[0] + off2[0];
        pos3[1] = (REAL)j * sf[1] + off2[1];
        pos3[2] = (REAL)k * sf[2] + off2[2];
        vec4 v = interp3_vec4(v1, defoDims, vZ, pos3);
        for (int c = 0; c < 4; ++c) v.v[c] *= df[c];
        REAL pos4[4];
        pos4[0] = (REAL)(i + 0.5f) - v.v[0] * blendAlpha;
        pos4[1] = (REAL)(j + 0.5f) - v.v[1] * blendAlpha;
        pos4[2] = (REAL)(k + 0.5f) - v.v[2] * blendAlpha;
        pos4[3] = (REAL)(T0 + 0.5f) - v.v[3] * blendAlpha;
        dst[(idx_t)i + (idx_t)X * j + (idx_t)X * Y * k] = interp4_real(phi, pd, pos4);
      }
  free(v1);
}
