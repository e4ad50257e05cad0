/*
 * c_client.c -- a plain C99 caller of the C ABI (include/flof_gb300.h), the
 * way a reference-side plugin would bind it: opaque handles, host buffers,
 * status codes.  `c_client 0` expects no usable device and checks that the
 * library reports that cleanly; `c_client 1` runs a small multiscale solve
 * on two drops moving along x and checks the result.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "flof_gb300.h"

static float sphere_sdf(int x, int y, int z, float cx, float cy, float cz, float r) {
  const float dx = (float)x + 0.5f - cx, dy = (float)y + 0.5f - cy, dz = (float)z + 0.5f - cz;
  float d = sqrtf(dx * dx + dy * dy + dz * dz) - r;
  if (d < -4.f) d = -4.f;
  if (d > 4.f) d = 4.f;
  return d * -0.005f; /* lsFactor = -0.1 / 20 */
}

int main(int argc, char **argv) {
  const int want_gpu = argc > 1 && atoi(argv[1]) != 0;
  flof_ctx *ctx = NULL;
  int st = flof_ctx_create(0, &ctx);
  if (!want_gpu) {
    if (st == FLOF_OK) {
      printf("context created without a device\n");
      flof_ctx_destroy(ctx);
      return 2;
    }
    printf("no device: status %d (%s): %s\n", st, flof_status_string(st), flof_last_error());
    return 0;
  }
  if (st != FLOF_OK) {
    printf("flof_ctx_create: %s\n", flof_last_error());
    return 1;
  }
  const int X = 24, Y = 24, Z = 24, T = 16;
  const int dims[4] = {X, Y, Z, T};
  const size_t n = (size_t)X * Y * Z * T;
  float *i0 = malloc(n * sizeof(float)), *i1 = malloc(n * sizeof(float));
  float *v = malloc(n * 4 * sizeof(float));
  if (!i0 || !i1 || !v) return 1;
  for (int t = 0; t < T; ++t)
    for (int z = 0; z < Z; ++z)
      for (int y = 0; y < Y; ++y)
        for (int x = 0; x < X; ++x) {
          const size_t id = (size_t)x + (size_t)X * (y + (size_t)Y * (z + (size_t)Z * t));
          i0[id] = sphere_sdf(x, y, z, 9.f + 0.25f * t, 12.f, 12.f, 5.f);
          i1[id] = sphere_sdf(x, y, z, 11.f + 0.25f * t, 12.f, 12.f, 5.f);
        }
  flof_grid *g0 = NULL, *g1 = NULL, *gv = NULL;
  if (flof_grid_create(ctx, dims, FLOF_REAL, &g0) || flof_grid_create(ctx, dims, FLOF_REAL, &g1) ||
      flof_grid_create(ctx, dims, FLOF_VEC4, &gv) || flof_grid_upload(g0, i0) ||
      flof_grid_upload(g1, i1)) {
    printf("grids: %s\n", flof_last_error());
    return 1;
  }
  flof_of_params p;
  flof_of_params_flof(&p); /* scenes/flof.py's mode-1 parameters */
  float err = -1.f;
  flof_solve_stats stats;
  st = flof_opticalFlowMultiscale4d(ctx, gv, g0, g1, &p, &err, &stats);
  if (st != FLOF_OK) {
    printf("flof_opticalFlowMultiscale4d: %s\n", flof_last_error());
    return 1;
  }
  if (flof_grid_download(gv, v)) {
    printf("download: %s\n", flof_last_error());
    return 1;
  }
  /* the drops move +x: the mean x velocity inside the drop band is positive */
  double vx = 0.0, vmax = 0.0;
  long cnt = 0;
  for (size_t q = 0; q < n; ++q) {
    for (int c = 0; c < 4; ++c) {
      const float a = v[4 * q + c];
      if (!isfinite(a)) {
        printf("non-finite velocity\n");
        return 1;
      }
      if (fabsf(a) > vmax) vmax = fabsf(a);
    }
    if (fabsf(i0[q]) < 0.02f * 0.999f) {
      vx += v[4 * q];
      ++cnt;
    }
  }
  printf("err %.6f solves %d iterations %d max|v| %.4f mean vx in band %.4f\n", err,
         stats.nsolves, stats.cg_total_iterations, vmax, cnt ? vx / cnt : 0.0);
  flof_grid_destroy(g0);
  flof_grid_destroy(g1);
  flof_grid_destroy(gv);
  flof_ctx_destroy(ctx);
  free(i0);
  free(i1);
  free(v);
  return (stats.nsolves > 0 && vmax > 0.0 && cnt > 0 && vx > 0.0) ? 0 : 3;
}
