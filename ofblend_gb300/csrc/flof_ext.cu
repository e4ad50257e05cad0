// flof_ext.cu -- C ABI of the steps either side of the solve: input
// conditioning of the 4D level sets (repeatFrame4d, extrap4dLsSimple), the
// 3D Grid<Real> methods of the output stage (join, setBound,
// setBoundNeumann, simpleBlurSpecial) and the partial-load helpers of the
// hi-res 4D assembly (shiftForwGrid4d, the device part of loadPlaceGrid4d).
#include "flof_internal.h"

using namespace flof;
using namespace fh;

namespace {

void need_3d(const flof_grid *g, const char *name) {
  need(g->dims[3] == 1, std::string(name) + " must be a 3D grid (t extent 1)");
}

}  // namespace

// repeatFrame4d (source/plugin/optflow4d.cpp:1254-1266).  The reference loops
// t from int(srct - range + 0.5) to int(srct) without a range check; slices
// outside [0, T) are skipped here.
FLOF_API int flof_repeatFrame4d(flof_grid *phi, float srct, float range, int bnd) {
  return guarded([&] {
    need_grid(phi, "phi");
    need_elem(phi, FLOF_REAL, "phi");
    need(bnd >= 0, "bnd must not be negative");
    need(srct == srct && range == range, "srct and range must be numbers");
    const Dims4 d = phi->D();
    need(d.x >= 2 && d.y >= 2 && d.z >= 2 && d.t >= 2, "phi: every extent must be at least 2");
    int t0 = trunc_d((double)(srct - range) + 0.5);
    int t1 = trunc_f(srct);
    if (t0 < 0) t0 = 0;
    if (t1 > d.t - 1) t1 = d.t - 1;
    if (t1 < t0) return;
    flof_ctx *c = phi->ctx;
    set_ctx_device(c);
    DBuf slice(c, (size_t)d.x * d.y * d.z * sizeof(float));
    KLP(c, KC_ELEMWISE, d.x, (double)d.x * d.y * d.z * 4 * (2 + (t1 - t0 + 1)),
        launch_repeat_frame(phi->f(), d, srct, t0, t1, bnd, slice.f(), c->stream));
  });
}

// extrap4dLsSimple (source/plugin/optflow4d.cpp:1332-1406): mark the cells
// below zero (inside: above zero), the first layer around them, then
// `distance - 1` sweeps that give each newly reached cell the mean of its
// reached neighbours plus one step (+1 outside, -1 inside), and finally the
// cells never reached get direction * (distance + 2).
FLOF_API int flof_extrap4dLsSimple(flof_grid *phi, int distance, int inside) {
  return guarded([&] {
    need_grid(phi, "phi");
    need_elem(phi, FLOF_REAL, "phi");
    const Dims4 d = phi->D();
    need(d.x >= 3 && d.y >= 3 && d.z >= 3 && d.t >= 3,
         "extrap4dLsSimple: every extent must be at least 3");
    need(distance >= 0 && distance < (1 << 20), "distance out of range");
    flof_ctx *c = phi->ctx;
    set_ctx_device(c);
    const float direction = inside ? -1.f : 1.f;
    DBuf tmp(c, (size_t)d.cells() * sizeof(int));
    const double cells = (double)d.cells();
    KLP(c, KC_ELEMWISE, d.x, cells * 8,
        launch_extrap_mark(phi->f(), (int *)tmp.p, d, inside ? 1 : 0, c->stream));
    KLP(c, KC_ELEMWISE, d.x, cells * 4, launch_extrap_layer((int *)tmp.p, d, c->stream));
    for (int dd = 2; dd < 1 + distance; ++dd)
      KLP(c, KC_ELEMWISE, d.x, cells * 8,
          launch_extrap_step(phi->f(), (int *)tmp.p, d, dd, direction, c->stream));
    KLP(c, KC_ELEMWISE, d.x, cells * 8,
        launch_extrap_remaining(phi->f(), (const int *)tmp.p, d,
                                direction * (float)(distance + 2), c->stream));
  });
}

// LevelsetGrid::join (source/levelset.cpp:114-118): a = min(a, b).
FLOF_API int flof_grid_join(flof_grid *a, const flof_grid *b) {
  return guarded([&] {
    need_grid(a, "a");
    need_grid(b, "b");
    need_elem(a, FLOF_REAL, "a");
    need_elem(b, FLOF_REAL, "b");
    same_size(a, b, "join");
    KLP(a->ctx, KC_ELEMWISE, a->dims[0], (double)a->cells() * 12,
        launch_join(a->f(), b->f(), a->cells(), a->ctx->stream));
  });
}

// Grid<T>::setBound / setBoundNeumann of a 3D grid (source/grid.cpp:462-511):
// the k planes count only when the grid is 3D (Z > 1).
FLOF_API int flof_grid3_setBound(flof_grid *a, const float v[4], int w) {
  return guarded([&] {
    need_grid(a, "grid");
    need_3d(a, "grid");
    need(v != nullptr, "value is NULL");
    KLP(a->ctx, KC_BORDER, a->dims[0], 0,
        launch_set_bound3(a->f(), a->dims[0], a->dims[1], a->dims[2], a->nc(), f4(v, a->nc()), w,
                          a->ctx->stream));
  });
}

FLOF_API int flof_grid3_setBoundNeumann(flof_grid *a, int w) {
  return guarded([&] {
    need_grid(a, "grid");
    need_3d(a, "grid");
    need(a->dims[0] > 2 * (w + 1) && a->dims[1] > 2 * (w + 1) &&
             (a->dims[2] == 1 || a->dims[2] > 2 * (w + 1)),
         "setBoundNeumann: boundary wider than the grid");
    KLP(a->ctx, KC_BORDER, a->dims[0], 0,
        launch_set_bound_neumann3(a->f(), a->dims[0], a->dims[1], a->dims[2], a->nc(), w,
                                  a->ctx->stream));
  });
}

// simpleBlurSpecial (source/test.cpp:116-131): `iter` passes through a fresh
// zeroed scratch grid with a swap after each, so after an odd number of
// passes the ring outside the bnd = 1 box is zero and after an even number
// it holds the grid's own ring again.
FLOF_API int flof_simpleBlurSpecial(flof_grid *a, int iter, float thresh, int bord) {
  return guarded([&] {
    need_grid(a, "grid");
    need_3d(a, "grid");
    need_elem(a, FLOF_REAL, "grid");
    const int X = a->dims[0], Y = a->dims[1], Z = a->dims[2];
    need(X >= 3 && Y >= 3 && (Z == 1 || Z >= 3),
         "simpleBlurSpecial: extents must be at least 3 (z may be 1 for a 2D grid)");
    if (iter <= 0) return;
    flof_ctx *c = a->ctx;
    set_ctx_device(c);
    const size_t bytes = a->bytes();
    DBuf tmp(c, bytes);
    CK(cudaMemsetAsync(tmp.p, 0, bytes, c->stream));
    float *cur = a->f(), *nxt = tmp.f();
    for (int it = 0; it < iter; ++it) {
      KLP(c, KC_ELEMWISE, X, (double)a->cells() * 8,
          launch_simple_blur_special(cur, nxt, X, Y, Z, thresh, bord, c->stream));
      float *sw = cur;
      cur = nxt;
      nxt = sw;
    }
    if (cur != a->f())
      CK(cudaMemcpyAsync(a->f(), cur, bytes, cudaMemcpyDeviceToDevice, c->stream));
  });
}

// shiftForwGrid4d (source/plugin/optflow4d.cpp:1596-1616): moves the t slices
// [shift, T) forward to [0, good), shift = T - good, in blocks of `shift`
// slices so that no copy overlaps itself.
FLOF_API int flof_shiftForwGrid4d(flof_grid *phi, int overrideGoodRegion) {
  return guarded([&] {
    need_grid(phi, "phi");
    const int T = phi->dims[3];
    const int good = overrideGoodRegion;
    if (good <= 0) return;
    // the reference's loop does not end for good >= T (shift <= 0)
    need(good < T, "shiftForwGrid4d: overrideGoodRegion must be below the t extent");
    const int shift = T - good;
    const size_t slice = (size_t)phi->dims[0] * phi->dims[1] * phi->dims[2] * phi->nc() * 4;
    char *base = (char *)phi->d;
    for (int s = 0; s < good; s += shift) {
      const int len = (s + shift >= good) ? good - s : shift;
      CK(cudaMemcpyAsync(base + (size_t)s * slice, base + (size_t)(s + shift) * slice,
                         (size_t)len * slice, cudaMemcpyDeviceToDevice, phi->ctx->stream));
    }
  });
}
