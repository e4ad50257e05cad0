// flof_internal.h -- host-side internals shared by the translation units
// that implement the C ABI: the context and grid objects behind the opaque
// handles of include/flof_gb300.h, the device buffer pool, launch tracing
// and the error plumbing (status code + thread-local message; no exception
// crosses the C ABI).
#pragma once

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <array>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/flof_gb300.h"
#include "flof_kernels.h"

using flof::CGState;
using flof::Dims4;

namespace fh {

inline thread_local std::string g_last_error;

struct FlofError {
  int code;
  std::string msg;
};

[[noreturn]] inline void fail(int code, const std::string &msg) { throw FlofError{code, msg}; }

inline void cuda_check(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return;
  const int code = (e == cudaErrorMemoryAllocation) ? FLOF_E_OOM : FLOF_E_CUDA;
  fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call) cuda_check((call), #call)

struct Pool {
  std::unordered_map<size_t, std::vector<void *>> free_list;
  std::unordered_map<void *, size_t> owned;
  size_t bytes = 0;

  void *get(size_t n) {
    if (n == 0) n = 16;
    n = (n + 255) & ~size_t(255);
    auto it = free_list.find(n);
    if (it != free_list.end() && !it->second.empty()) {
      void *p = it->second.back();
      it->second.pop_back();
      return p;
    }
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      cudaGetLastError();
      trim();
      e = cudaMalloc(&p, n);
      if (e != cudaSuccess) {
        cudaGetLastError();
        fail(FLOF_E_OOM, "device allocation of " + std::to_string(n) + " bytes failed");
      }
    }
    owned[p] = n;
    bytes += n;
    return p;
  }
  void put(void *p) {
    if (!p) return;
    auto it = owned.find(p);
    if (it == owned.end()) return;
    free_list[it->second].push_back(p);
  }
  void trim() {
    for (auto &kv : free_list) {
      for (void *p : kv.second) {
        cudaFree(p);
        owned.erase(p);
        bytes -= kv.first;
      }
      kv.second.clear();
    }
  }
  void release_all() {
    for (auto &kv : owned) cudaFree(kv.first);
    owned.clear();
    free_list.clear();
    bytes = 0;
  }
};

enum KClass {
  KC_OTHER = 0, KC_ASSEMBLE, KC_MATVEC, KC_UPDATE, KC_DIRECTION, KC_COPYBACK, KC_BLUR,
  KC_PROJECT, KC_EXPOL, KC_ADVECT, KC_RESAMPLE, KC_LSDIFF, KC_REDUCE, KC_ELEMWISE, KC_BORDER,
  KC_LOOKUP, KC_DEFORM, KC_BLEND, KC_EXPOL_MASK, KC_MG, KC_COUNT
};
inline const char *kc_names[KC_COUNT] = {
    "other", "of_assemble_init", "cg_matvec", "cg_update", "cg_direction", "of_copy_back",
    "gauss_blur", "project_cells", "expol_sweep", "advect", "resample", "ls_diff", "reduce",
    "elementwise", "border", "lookup_slice", "deform_twoway", "blend_slices", "expol_mask",
    "mg_vcycle"};

struct ProfRec {
  int cls;
  int size_x;
  double bytes;
  cudaEvent_t e0, e1;
};

struct LatsData {
  const flof_grid *defo = nullptr;
  void *vt = nullptr;  // blended t-slice (Vec4, X*Y*Z of the defo)
  int lastT = -1;
};

}  // namespace fh

struct flof_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // asynchronous host transfers (flof_grid_*_async): their own stream, ordered
  // after the work queued on `stream` when each copy is issued
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_order = nullptr;
  fh::Pool pool;
  CGState *st = nullptr;    // device
  CGState *st_h = nullptr;  // pinned host mirror
  double *dpart = nullptr;
  float *fpart = nullptr;
  unsigned int *counter = nullptr;  // 8 zeroed counters
  float *fres = nullptr;            // 16 device scalars
  double *dres = nullptr;
  float *fres_h = nullptr;          // pinned
  double *dres_h = nullptr;
  long long launches = 0;
  int syncs = 0;
  std::map<int, fh::LatsData> lats;
  flof_solve_stats *stats = nullptr;
  // 0: CFL substep counts are checked on the device (one substep assumed,
  // exceptions flagged in cfl_flag); 1: the host reads max |v| each time.
  int cfl_sync = 0;
  int *cfl_flag = nullptr;
  int *dev_err = nullptr;  // device error word written by bounded waits
  int cfl_force_sync = 0;
  int profiling = 0;
  std::map<std::pair<uint32_t, int>, float *> wsum_cache;  // (sigma bits, radius)
  // autotuned PCG launch shapes per grid size (FLOF_OPT_AUTOTUNE); worker
  // contexts share their parent's table (tune_owner)
  int autotune = 0;
  // FLOF_OPT_STRICT: the reference's PCG and error-metric arithmetic
  int strict = 0;
  // FLOF_OPT_SLAB_TMA: 1 the TMA slab kernels for the Vec4 blur and the
  // extrapolation sweeps, 0 their plain-load counterparts
  int slab_tma = 1;
  // parameters of the multigrid preconditioner (FLOF_SOLVER_MG) and the
  // number of its solves the plain PCG had to finish
  flof::MGParams mg;
  long long mg_fallbacks = 0;
  std::map<std::array<int, 4>, flof::CGTune> tunes;
  std::mutex tune_mu;
  flof_ctx *tune_owner = nullptr;
  // worker contexts of the batched solve (created on demand)
  std::vector<flof_ctx *> workers;
  // live grids of this context: destroying the context frees their storage
  // and leaves the handles orphaned (ctx == nullptr) until they are destroyed
  std::unordered_set<flof_grid *> grids;
  // learned warm start used by the multiscale driver (flof_ctx_set_model)
  flof_model *model = nullptr;
  std::unordered_set<flof_model *> models;
  std::vector<fh::ProfRec> recs;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
};

struct flof_grid {
  flof_ctx *ctx = nullptr;
  int dims[4] = {0, 0, 0, 0};
  int elem = FLOF_REAL;
  void *d = nullptr;
  bool owned = false;
  // OptInit pins the deformation grid it reads from; destroying a pinned
  // grid is deferred until the last Finish releases it.
  int pins = 0;
  bool destroy_pending = false;
  // completion of the grid's last asynchronous host transfer (null: none yet)
  cudaEvent_t copy_ev = nullptr;
  Dims4 D() const { return Dims4{dims[0], dims[1], dims[2], dims[3]}; }
  int nc() const { return elem == FLOF_VEC4 ? 4 : 1; }
  long long cells() const { return (long long)dims[0] * dims[1] * dims[2] * dims[3]; }
  size_t bytes() const { return (size_t)cells() * nc() * sizeof(float); }
  float *f() const { return (float *)d; }
  float4 *v() const { return (float4 *)d; }
};

namespace fh {

// Frees a grid's storage (owned grids) and its handle.  A grid whose context
// is gone has no storage left (the context freed it) and only the handle goes.
inline void grid_free(flof_grid *g) {
  if (g->copy_ev) cudaEventSynchronize(g->copy_ev);  // no transfer outlives the storage
  if (g->ctx) {
    if (g->owned && g->d) {
      cudaSetDevice(g->ctx->device);
      cudaStreamSynchronize(g->ctx->stream);
      cudaFree(g->d);
    }
    g->ctx->grids.erase(g);
  }
  if (g->copy_ev) cudaEventDestroy(g->copy_ev);
  delete g;
}

inline void grid_unpin(flof_grid *g) {
  if (!g) return;
  if (g->pins > 0) g->pins--;
  if (g->pins == 0 && g->destroy_pending) grid_free(g);
}


// RAII device buffer from the context pool.
struct DBuf {
  flof_ctx *c = nullptr;
  void *p = nullptr;
  DBuf() {}
  DBuf(flof_ctx *ctx, size_t n) : c(ctx), p(ctx->pool.get(n)) {}
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : c(o.c), p(o.p) { o.p = nullptr; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) {
      release();
      c = o.c;
      p = o.p;
      o.p = nullptr;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void release() {
    if (p && c) c->pool.put(p);
    p = nullptr;
  }
  float *f() const { return (float *)p; }
  float4 *v() const { return (float4 *)p; }
};

inline size_t real_bytes(Dims4 d) { return (size_t)d.cells() * sizeof(float); }
inline size_t vec_bytes(Dims4 d) { return (size_t)d.cells() * sizeof(float4); }

// Kernel launch with optional event tracing: when the context profiles,
// every launch is bracketed by two CUDA events on the context stream and
// recorded with its kernel class, the X extent of its grid and its
// algorithmic bytes (compulsory reads + writes).
#define KLP(ctx, cls, sx, nbytes, call)                                   \
  do {                                                                     \
    flof_ctx *_c = (ctx);                                                  \
    cudaEvent_t _e0 = nullptr, _e1 = nullptr;                              \
    if (_c->profiling) {                                                   \
      _e0 = prof_event(_c);                                                \
      _e1 = prof_event(_c);                                                \
      CK(cudaEventRecord(_e0, _c->stream));                                \
    }                                                                      \
    call;                                                                  \
    ++_c->launches;                                                        \
    if (_c->profiling) {                                                   \
      CK(cudaEventRecord(_e1, _c->stream));                                \
      _c->recs.push_back(ProfRec{(cls), (sx), (double)(nbytes), _e0, _e1}); \
    }                                                                      \
  } while (0)
#define KL(ctx, call) KLP(ctx, KC_OTHER, 0, 0, call)

inline long long nint(Dims4 d) {
  if (d.x < 3 || d.y < 3 || d.z < 3 || d.t < 3) return 0;
  return (long long)(d.x - 2) * (d.y - 2) * (d.z - 2) * (d.t - 2);
}

inline cudaEvent_t prof_event(flof_ctx *c) {
  if (c->ev_used == c->ev_pool.size()) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    c->ev_pool.push_back(e);
  }
  return c->ev_pool[c->ev_used++];
}

inline void sync(flof_ctx *c) {
  CK(cudaStreamSynchronize(c->stream));
  c->syncs++;
}

inline float read_f(flof_ctx *c, const float *dev) {
  CK(cudaMemcpyAsync(c->fres_h, dev, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  return c->fres_h[0];
}

inline int trunc_f(float v) {
  if (v != v) return 0;
  if (v >= 2147483647.f) return 2147483647;
  if (v <= -2147483648.f) return (-2147483647 - 1);
  return (int)v;
}
inline int trunc_d(double v) {
  if (v != v) return 0;
  if (v >= 2147483647.0) return 2147483647;
  if (v <= -2147483648.0) return (-2147483647 - 1);
  return (int)v;
}

// Reads and clears the device error word (after the stream has drained).
inline void check_device_errors(flof_ctx *c) {
  CK(cudaMemcpyAsync(c->fres_h + 9, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  int e = 0;
  memcpy(&e, c->fres_h + 9, sizeof(int));
  if (e) {
    CK(cudaMemsetAsync(c->dev_err, 0, sizeof(int), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    fail(FLOF_E_TIMEOUT, std::string("a bounded wait on ") +
                             (e == flof::FLOF_DEV_ERR_TC_TIMEOUT ? "tensor-core MMAs" : "a TMA copy") +
                             " gave up (device error " + std::to_string(e) + ")");
  }
}

inline void record_solve(flof_ctx *c, int sx, int iters, float res, int status,
                         float true_res = -1.f) {
  flof_solve_stats *s = c->stats;
  if (!s) return;
  if (s->nsolves < FLOF_MAX_SOLVE_STATS) {
    s->size_x[s->nsolves] = sx;
    s->iterations[s->nsolves] = iters;
    s->residual[s->nsolves] = res;
    s->status[s->nsolves] = status;
    s->true_residual[s->nsolves] = true_res;
  }
  s->nsolves++;
  s->cg_total_iterations += iters > 0 ? iters : 0;
}


// ---------------------------------------------------------------------------
// C ABI helpers
// ---------------------------------------------------------------------------

// Host-only work (file headers): no CUDA error to collect.
template <class F>
inline int guarded_host(F &&f) {
  try {
    f();
    return FLOF_OK;
  } catch (const FlofError &e) {
    g_last_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return FLOF_E_OOM;
  } catch (...) {
    g_last_error = "unknown error";
    return FLOF_E_CUDA;
  }
}

template <class F>
inline int guarded(F &&f) {
  // an error left by an earlier call that had no way to report it (a
  // teardown path) must not be charged to this one
  cudaGetLastError();
  try {
    f();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) fail(FLOF_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return FLOF_OK;
  } catch (const FlofError &e) {
    g_last_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return FLOF_E_OOM;
  } catch (...) {
    g_last_error = "unknown error";
    return FLOF_E_CUDA;
  }
}

inline void need(bool cond, const std::string &msg) {
  if (!cond) fail(FLOF_E_ARG, msg);
}
inline void need_grid(const flof_grid *g, const char *name) {
  need(g != nullptr, std::string(name) + " is NULL");
  need(g->ctx != nullptr, std::string(name) + " belongs to a destroyed context");
  need(g->d != nullptr || g->cells() == 0, std::string(name) + " has no storage");
}
inline void same_size(const flof_grid *a, const flof_grid *b, const char *what) {
  need(a->dims[0] == b->dims[0] && a->dims[1] == b->dims[1] && a->dims[2] == b->dims[2] &&
           a->dims[3] == b->dims[3],
       std::string(what) + ": different grid resolutions");
}
inline void need_elem(const flof_grid *g, int elem, const char *name) {
  need(g->elem == elem, std::string(name) + (elem == FLOF_VEC4 ? " must be a Vec4 grid"
                                                               : " must be a Real grid"));
}
inline void need_4d(const flof_grid *g, const char *name) {
  for (int q = 0; q < 4; ++q)
    need(g->dims[q] >= 2, std::string(name) + ": every extent must be at least 2");
}
inline void set_ctx_device(flof_ctx *c) { CK(cudaSetDevice(c->device)); }

inline float4 f4(const float *v, int nc) {
  if (!v) return make_float4(0.f, 0.f, 0.f, 0.f);
  if (nc == 1) return make_float4(v[0], v[0], v[0], v[0]);
  return make_float4(v[0], v[1], v[2], v[3]);
}

// gridFactor4d (grid4d.cpp:559-569)
inline void grid_factor4d(const float s1[4], const float s2in[4], const float optSize[4],
                   const float scale[4], float srcFac[4], float retOff[4]) {
  float s2[4];
  for (int q = 0; q < 4; ++q) s2[q] = optSize[q] > 0.f ? optSize[q] : s2in[q];
  for (int q = 0; q < 4; ++q) srcFac[q] = (s1[q] / s2[q]) / scale[q];
  for (int q = 0; q < 4; ++q) {
    const float neg = -retOff[q];
    retOff[q] = neg * srcFac[q] + (float)((double)srcFac[q] * 0.5);
  }
}

}  // namespace fh

// ---- learned warm start (flof_model.cu) -----------------------------------------
namespace fh {
void model_predict_raw(flof_model *m, const float *i0, const float *i1, float4 *vel);
int model_res(const flof_model *m);
// frees a model's device memory when its context goes (the handle stays)
void model_orphan(flof_model *m);
}  // namespace fh

// ---- .uni files (flof_uni.cu) ----------------------------------------------------
namespace fh {
struct UniInfo {
  int dims[4];  // x, y, z and the t extent (1 for a 3D file)
  bool is4d;
  int gridType, elementType, bytesPerElement;
};
UniInfo uni_info(const char *name);
void uni_load(flof_grid *g, const char *name);
void uni_save(const flof_grid *g, const char *name, bool is4d, int gridType);
void uni_read_slice(flof_grid *g, const char *name, int t);
}  // namespace fh
