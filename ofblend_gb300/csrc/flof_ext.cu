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

// snprintf(pattern, idx) for a file-name pattern with at most one integer
// conversion (%d, %i, with flags and width) and %% escapes; anything else in
// a conversion is rejected rather than handed to printf.
std::string file_name(const char *pattern, int idx) {
  std::string out;
  int convs = 0;
  for (const char *p = pattern; *p; ++p) {
    if (*p != '%') {
      out += *p;
      continue;
    }
    if (p[1] == '%') {
      out += '%';
      ++p;
      continue;
    }
    const char *q = p + 1;
    std::string spec = "%";
    while (*q == '0' || *q == '-' || *q == '+' || *q == ' ') spec += *q++;
    while (*q >= '0' && *q <= '9') spec += *q++;
    need(*q == 'd' || *q == 'i', std::string("file name pattern '") + pattern +
                                     "': only one integer conversion (%d) is supported");
    need(++convs == 1, std::string("file name pattern '") + pattern +
                           "' has more than one conversion");
    spec += 'd';
    char buf[64];
    snprintf(buf, sizeof(buf), spec.c_str(), idx);
    out += buf;
    p = q;
  }
  return out;
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

// loadPlaceGrid4d (source/plugin/optflow4d.cpp:1460-1594): builds the hi-res
// 4D level set from a sequence of 3D slice files.  File fileid goes to the
// t slices around dstt = offset.t + overrideTimeOff + duration * (fileid -
// fileIdxStart) with hat weights; each placed slice is the trilinear
// resample of the file to phi's x, y, z extent (bnd = 1 box), and the
// accumulated weights are divided out at the end.  The slices come from the
// files fname % fileid (.uni MNT2) or, when fname is NULL, from the device
// grids slices[fileid - fileIdxStart].
FLOF_API int flof_loadPlaceGrid4d(flof_grid *phi, const char *fname,
                                  const flof_grid *const *slices, int nslices,
                                  const float offset[4], const float scale[4], int fileIdxStart,
                                  int fileIdxEnd, int debugSkipLoad, float spread,
                                  const float overrideSize[4], float overrideTimeOff,
                                  int overrideGoodRegion, float loadTimeScale,
                                  int rescaleSdfValues, float sdfIsoOff, float repeatStartFrame) {
  return guarded([&] {
    need_grid(phi, "phi");
    need_elem(phi, FLOF_REAL, "phi");
    need(fname != nullptr || (slices != nullptr && nslices > 0),
         "either fname or a list of slice grids is required");
    need(offset != nullptr && scale != nullptr, "offset and scale are required");
    const Dims4 d = phi->D();
    need(d.x >= 3 && d.y >= 3 && d.z >= 3 && d.t >= 3,
         "loadPlaceGrid4d: every extent of phi must be at least 3");
    flof_ctx *c = phi->ctx;
    set_ctx_device(c);
    int sd[3];
    if (fname) {
      // the reference probes the size with the raw fileIdxStart
      const std::string first = file_name(fname, fileIdxStart);
      const UniInfo u = uni_info(first.c_str());
      need(!u.is4d && u.bytesPerElement == 4,
           first + " is not a 3D Real (MNT2) file");
      sd[0] = u.dims[0];
      sd[1] = u.dims[1];
      sd[2] = u.dims[2];
    } else {
      for (int q = 0; q < nslices; ++q) {
        need_grid(slices[q], "slice");
        need_elem(slices[q], FLOF_REAL, "slice");
        need_3d(slices[q], "slice");
        need(q == 0 || (slices[q]->dims[0] == slices[0]->dims[0] &&
                        slices[q]->dims[1] == slices[0]->dims[1] &&
                        slices[q]->dims[2] == slices[0]->dims[2]),
             "all slices must have the same size");
      }
      for (int q = 0; q < 3; ++q) sd[q] = slices[0]->dims[q];
    }
    need(sd[0] >= 2 && sd[1] >= 2 && sd[2] >= 1, "Invalid src size of the slices");
    const float v1[4] = {(float)sd[0], (float)sd[1], (float)sd[2], 1.f};
    float defoSize[4] = {(float)d.x, (float)d.y, (float)d.z, (float)d.t};
    if (overrideSize && overrideSize[0] > 0.f)
      for (int q = 0; q < 4; ++q) defoSize[q] = overrideSize[q];
    float sf[4], off2[4];
    const float neg1[4] = {-1, -1, -1, -1};
    for (int q = 0; q < 4; ++q) off2[q] = offset[q];
    grid_factor4d(v1, defoSize, neg1, scale, sf, off2);
    const float sf3[3] = {sf[0], sf[1], sf[2]}, off3[3] = {off2[0], off2[1], off2[2]};
    float valueScale = 1.f;
    if (rescaleSdfValues) valueScale = (float)(1. / (double)sf[0]);
    std::vector<float> w(d.t, 0.f);
    const size_t sliceBytes = (size_t)d.x * d.y * d.z * sizeof(float);
    if (overrideGoodRegion <= 0) {
      CK(cudaMemsetAsync(phi->d, 0, phi->bytes(), c->stream));
    } else if (overrideGoodRegion < d.t) {
      CK(cudaMemsetAsync((char *)phi->d + sliceBytes * overrideGoodRegion, 0,
                         sliceBytes * (d.t - overrideGoodRegion), c->stream));
    }
    if (fileIdxStart < 0) fileIdxStart = 0;
    if (fileIdxEnd < 0) fileIdxEnd = trunc_f(defoSize[3]);
    int repeatOff = 0;
    if (repeatStartFrame > 0.f)
      repeatOff = trunc_d((double)((float)(fileIdxEnd - fileIdxStart) * repeatStartFrame) + 1.0);
    const size_t n3 = (size_t)sd[0] * sd[1] * sd[2];
    DBuf tmp(c, n3 * sizeof(float));
    flof_grid tg;
    tg.ctx = c;
    tg.dims[0] = sd[0];
    tg.dims[1] = sd[1];
    tg.dims[2] = sd[2];
    tg.dims[3] = 1;
    tg.elem = FLOF_REAL;
    tg.d = tmp.p;
    tg.owned = false;
    const int endId = fileIdxEnd < debugSkipLoad ? fileIdxEnd : debugSkipLoad;
    for (int fileid = fileIdxStart - repeatOff; fileid < endId; ++fileid) {
      const int fileidClamp = fileid > fileIdxStart ? fileid : fileIdxStart;
      bool didLoad = false;
      const float duration = (float)(1. * (double)(defoSize[3] * scale[3] / loadTimeScale) /
                                     (double)(float)(fileIdxEnd - fileIdxStart));
      const float dstt = offset[3] + overrideTimeOff + duration * (float)(fileid - fileIdxStart);
      const int s0 = trunc_f(dstt - spread * duration) + 0;
      const int s1 = trunc_f(dstt + spread * duration) + 2;
      for (int slice = s0; slice < s1; ++slice) {
        if (slice < overrideGoodRegion || slice >= d.t) continue;
        const float q = fabsf((float)slice - dstt) / (duration * spread);
        const float wc = (float)(1. - (double)q);
        if (wc < 1e-6f) continue;
        w[slice] += wc;
        if (!didLoad) {
          if (fname) {
            const std::string nm = file_name(fname, fileidClamp);
            uni_load(&tg, nm.c_str());
          } else {
            const int qi = fileidClamp - fileIdxStart;
            need(qi >= 0 && qi < nslices,
                 "loadPlaceGrid4d: no slice grid for file index " + std::to_string(fileidClamp));
            CK(cudaMemcpyAsync(tmp.p, slices[qi]->d, n3 * sizeof(float),
                               cudaMemcpyDeviceToDevice, c->stream));
          }
          if (rescaleSdfValues && sdfIsoOff != 0.f) {
            KLP(c, KC_ELEMWISE, sd[0], (double)n3 * 8,
                launch_add_inner3(tmp.f(), sd[0], sd[1], sd[2], sdfIsoOff, c->stream));
            KLP(c, KC_BORDER, sd[0], 0,
                launch_set_bound3(tmp.f(), sd[0], sd[1], sd[2], 1,
                                  make_float4(1.f, 1.f, 1.f, 1.f), 1, c->stream));
          }
          didLoad = true;
        }
        KLP(c, KC_RESAMPLE, d.x, (double)d.x * d.y * d.z * 8,
            launch_place_slice(phi->f(), d, slice, tmp.f(), sd, sf3, off3, wc, c->stream));
      }
    }
    for (int t = 0; t < d.t; ++t) {
      if (w[t] < 1e-03f) {
        w[t] = 0.f;
      } else {
        w[t] = (float)(1. / (double)w[t]);
        w[t] *= valueScale;
      }
    }
    DBuf wd(c, (size_t)d.t * sizeof(float));
    CK(cudaMemcpyAsync(wd.p, w.data(), (size_t)d.t * sizeof(float), cudaMemcpyHostToDevice,
                       c->stream));
    KLP(c, KC_ELEMWISE, d.x, (double)d.cells() * 8,
        launch_rescale_slices(phi->f(), d, wd.f(), c->stream));
    CK(cudaStreamSynchronize(c->stream));
  });
}
