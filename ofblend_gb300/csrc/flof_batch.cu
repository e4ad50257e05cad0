// flof_batch.cu -- many independent deformation solves of uneven grid sizes
// on one GPU.  A solve at 24^3 x 16 cells launches kernels of a few
// microseconds, far too small to fill 152 SMs, and spends much of its time
// in host round trips (CG convergence checks, multistep decisions).  The
// batch runs the solves concurrently: each worker context owns a CUDA stream,
// a buffer pool and the PCG state, and one host thread drives it through the
// same multiscale driver as the single call, so kernels of different solves
// overlap on the GPU and one solve's host round trip hides behind another's
// kernels.  Solves are handed out largest first from a shared counter, and
// a budget of cells in flight keeps large solves, which fill the GPU alone,
// from running side by side.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <mutex>
#include <thread>

#include "flof_internal.h"

using namespace flof;
using namespace fh;

namespace {

flof_ctx *worker(flof_ctx *c, size_t q) {
  while (c->workers.size() <= q) {
    flof_ctx *w = nullptr;
    if (flof_ctx_create(c->device, &w) != FLOF_OK) fail(FLOF_E_CUDA, g_last_error);
    w->cfl_force_sync = c->cfl_force_sync;
    w->autotune = c->autotune;
    w->strict = c->strict;
    w->slab_tma = c->slab_tma;
    w->mg = c->mg;
    w->tune_owner = c;
    c->workers.push_back(w);
  }
  return c->workers[q];
}

// Cells of the solves in flight at once.  A solve of a few million cells
// keeps the PCG kernels near the HBM roofline on its own (on GB300: 3.5M-cell
// solves gain nothing from a second stream, 1M-cell solves 1.4x from several,
// 0.2M-cell solves 2.8x from sixteen), so a larger solve runs alone and
// smaller ones share the budget.
constexpr long long kCellsInFlight = 4ll << 20;

// Worker count when the caller leaves it open: enough streams that the
// smallest solves fill the budget, at most 16 and at most one per solve.
int auto_workers(const std::vector<long long> &cells) {
  long long small = cells.empty() ? 1 : cells[0];
  for (long long n : cells) small = n < small ? n : small;
  long long w = kCellsInFlight / (small > 0 ? small : 1);
  if (w < 1) w = 1;
  if (w > 16) w = 16;
  if (w > (long long)cells.size()) w = (long long)cells.size();
  return (int)w;
}

// Shares of the cells budget: a solve waits until its share fits; a solve
// larger than the budget takes all of it.
struct CellBudget {
  std::mutex mu;
  std::condition_variable cv;
  long long used = 0;
  long long acquire(long long n) {
    if (n > kCellsInFlight) n = kCellsInFlight;
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return used + n <= kCellsInFlight; });
    used += n;
    return n;
  }
  void release(long long n) {
    {
      std::lock_guard<std::mutex> lk(mu);
      used -= n;
    }
    cv.notify_all();
  }
};

}  // namespace

FLOF_API int flof_opticalFlowMultiscale4d_batch(flof_ctx *c, int n, flof_grid *const *vels,
                                                const flof_grid *const *i0s,
                                                const flof_grid *const *i1s,
                                                const flof_of_params *params, float *errs,
                                                int workers) {
  return guarded([&] {
    need(c != nullptr, "ctx is NULL");
    need(n >= 0, "n must not be negative");
    if (n == 0) return;
    need(vels != nullptr && i0s != nullptr && i1s != nullptr, "NULL grid list");
    std::vector<long long> cells(n);
    for (int q = 0; q < n; ++q) {
      need_grid(vels[q], "vel");
      need_grid(i0s[q], "i0");
      need_grid(i1s[q], "i1");
      need_elem(vels[q], FLOF_VEC4, "vel");
      need_elem(i0s[q], FLOF_REAL, "i0");
      need_elem(i1s[q], FLOF_REAL, "i1");
      same_size(vels[q], i0s[q], "opticalFlowMultiscale4d_batch");
      same_size(vels[q], i1s[q], "opticalFlowMultiscale4d_batch");
      need_4d(vels[q], "vel");
      cells[q] = vels[q]->cells();
    }
    set_ctx_device(c);
    if (params && params->warmStart && c->model) {
      // The attached model keeps its activations in one set of buffers on
      // its context's stream, so warm-started solves run in turn on this
      // context: the single call's results, one after another.
      for (int q = 0; q < n; ++q) {
        float e = 0.f;
        const int st = flof_opticalFlowMultiscale4d(c, vels[q], i0s[q], i1s[q], params, &e,
                                                    nullptr);
        if (st != FLOF_OK) fail(st, "solve " + std::to_string(q) + ": " + g_last_error);
        if (errs) errs[q] = e;
      }
      return;
    }
    int nw = workers > 0 ? workers : auto_workers(cells);
    if (nw > n) nw = n;
    // largest first
    std::vector<int> order(n);
    for (int q = 0; q < n; ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return cells[a] > cells[b]; });
    // the inputs may still be in flight on the caller's stream
    cudaEvent_t ready;
    CK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    CK(cudaEventRecord(ready, c->stream));
    std::vector<flof_ctx *> ws(nw);
    for (int q = 0; q < nw; ++q) {
      ws[q] = worker(c, q);
      CK(cudaStreamWaitEvent(ws[q]->stream, ready, 0));
    }
    CK(cudaEventDestroy(ready));

    std::atomic<int> next(0);
    CellBudget budget;
    std::mutex mu;
    int first_status = FLOF_OK;
    std::string first_msg;
    auto run = [&](flof_ctx *w) {
      cudaSetDevice(w->device);
      for (;;) {
        const int k = next.fetch_add(1);
        if (k >= n) break;
        const int q = order[k];
        float e = 0.f;
        const long long share = budget.acquire(cells[q]);
        const int st = flof_opticalFlowMultiscale4d(w, vels[q], i0s[q], i1s[q], params, &e,
                                                    nullptr);
        budget.release(share);
        if (st != FLOF_OK) {
          std::lock_guard<std::mutex> lk(mu);
          if (first_status == FLOF_OK) {
            first_status = st;
            first_msg = "solve " + std::to_string(q) + ": " + g_last_error;
          }
          next.store(n);  // stop handing out work
          break;
        }
        if (errs) errs[q] = e;
      }
    };
    std::vector<std::thread> threads;
    threads.reserve(nw > 0 ? nw - 1 : 0);
    for (int q = 1; q < nw; ++q) threads.emplace_back(run, ws[q]);
    run(ws[0]);
    for (auto &t : threads) t.join();
    for (flof_ctx *w : ws) CK(cudaStreamSynchronize(w->stream));
    if (first_status != FLOF_OK) fail(first_status, first_msg);
  });
}
