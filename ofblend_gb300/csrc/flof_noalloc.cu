// flof_noalloc.cu -- calcLsDiff4d for callers that cannot allocate device
// memory.
//
// Some callers of this library cannot call cudaMalloc at the point where they
// need the level-set error metric.  Examples are host applications that
// reserve all device memory at start-up and forbid allocations afterwards,
// and loops that must not pay for an allocation, which may synchronise the
// whole device.  flof_calcLsDiff4d needs a context, and a context owns a
// device pool.  flof_calcLsDiff4d_noalloc takes the caller's device buffers
// and keeps its only scratch, the per-block partial sums of the reduction,
// in a file-scope device array instead.
//
// The array is part of the library image: every GPU that loads the library
// holds it (8 KiB) until the process exits.  All calls share it and it keeps
// the contents of the last call.  Calls that overlap on the GPU (on two
// streams, or from two threads) therefore race on it; serialise them.
#include <mutex>
#include <string>

#include "../../include/flof_gb300.h"
#include "flof_kernels.h"

namespace flof {

namespace {

constexpr int NA_THREADS = 256;
// Block partials, then the arrival counter (as a double slot).
constexpr int NA_MAX_BLOCKS = 1024;
constexpr int NA_SLOTS = NA_MAX_BLOCKS + 1;
constexpr int NA_MAX_DEVICES = 64;

static __device__ __align__(256) double g_lsdiff_scratch[NA_SLOTS];

// Device address of g_lsdiff_scratch per device, looked up once.
double *g_scratch_ptr[NA_MAX_DEVICES] = {nullptr};
std::mutex g_scratch_mu;

// The same arithmetic as k_ls_diff (calcLsDiffTempl, optflow4d.cpp:895-927),
// with the block partials and the arrival counter in `scratch`.
__global__ void __launch_bounds__(NA_THREADS)
k_ls_diff_noalloc(const float *__restrict__ i0, const float *__restrict__ i1, float *out, Dims4 d,
                  BoxDecoder bx, uint32_t nbox, float correction, double scale, double *scratch,
                  float *result) {
  __shared__ double sh[NA_THREADS / 32];
  double acc = 0.0;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nbox; q += gridDim.x * blockDim.x) {
    int i, j, k, l;
    bx.decode(q, i, j, k, l);
    const idx_t id = d.index(i, j, k, l);
    const float a = __ldg(i0 + id), b = __ldg(i1 + id);
    if ((a < 0.f && b < 0.f) || (a >= 0.f && b >= 0.f)) {
      if (out) out[id] = 0.f;
    } else {
      float dd = fabsf(a - b) * correction;
      if (dd > 1.f) dd = 1.f;
      acc += (double)dd;
      if (out) out[id] = dd;
    }
  }
  const double b = block_sum<NA_THREADS>(acc, sh);
  if (threadIdx.x == 0) scratch[blockIdx.x] = b;
  unsigned int *counter = (unsigned int *)(scratch + NA_MAX_BLOCKS);
  if (last_block_arrives(counter)) {
    double m = 0.0;
    for (int q2 = threadIdx.x; q2 < (int)gridDim.x; q2 += blockDim.x) m += __ldcg(scratch + q2);
    m = block_sum<NA_THREADS>(m, sh);
    if (threadIdx.x == 0) {
      double accu = m * 1000.;
      if (d.t > 1) accu *= 1000.;
      accu *= scale;
      *result = (float)accu;
      *counter = 0;
    }
  }
}

}  // namespace

}  // namespace flof

using namespace flof;

static int na_fail(int code, const char *msg) {
  set_last_error(msg);
  return code;
}

extern "C" FLOF_API int flof_calcLsDiff4d_noalloc(const float *i0, const float *i1, float *out,
                                                  const int dims[4], float correction, int bnd,
                                                  float *result, void *stream) {
  if (!i0 || !i1 || !result || !dims) return na_fail(FLOF_E_ARG, "i0, i1, result and dims are required");
  for (int q = 0; q < 4; ++q)
    if (dims[q] < 1) return na_fail(FLOF_E_ARG, "grid extents must be positive");
  const long long cells = (long long)dims[0] * dims[1] * dims[2] * dims[3];
  if (cells >= (1ll << 31))
    return na_fail(FLOF_E_ARG, "grid too large for calcLsDiff4d_noalloc: at most 2^31-1 cells");
  if (bnd < 0 || bnd > (1 << 20))
    return na_fail(FLOF_E_ARG, "calcLsDiff4d_noalloc: bnd must be in [0, 2^20]");
  const int ex = dims[0] - 2 * bnd, ey = dims[1] - 2 * bnd, ez = dims[2] - 2 * bnd,
            et = dims[3] - 2 * bnd;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES)
    return na_fail(FLOF_E_CUDA, "calcLsDiff4d_noalloc: no usable current device");
  cudaStream_t s = (cudaStream_t)stream;
  // The array's device address belongs to the context current now.  Outside
  // stream capture it is looked up on every call, so that a device reset or
  // another context on the same device gets its own address; while the
  // stream is being captured the address of the last eager call is used.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
    cudaGetLastError();
    return na_fail(FLOF_E_CUDA, "calcLsDiff4d_noalloc: cannot query the stream");
  }
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (cap == cudaStreamCaptureStatusNone || !g_scratch_ptr[dev]) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_lsdiff_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return na_fail(FLOF_E_CUDA, "calcLsDiff4d_noalloc: scratch address lookup failed");
      }
      g_scratch_ptr[dev] = (double *)p;
    }
    scratch = g_scratch_ptr[dev];
  }
  // the arrival counter must start at zero; the partials are overwritten
  if (cudaMemsetAsync(scratch + NA_MAX_BLOCKS, 0, sizeof(double), s) != cudaSuccess)
    return na_fail(FLOF_E_CUDA, "calcLsDiff4d_noalloc: clearing the arrival counter failed");
  const Dims4 d{dims[0], dims[1], dims[2], dims[3]};
  // Grid4d's is3D() and is4D() are constant true (grid4d.h:82-83): every
  // axis loses 2 bnd cells.  A bnd that leaves none gives the reference's
  // 0 * (1 / count), which one block computes.
  const bool empty = ex <= 0 || ey <= 0 || ez <= 0 || et <= 0;
  const long long nbox = empty ? 0 : (long long)ex * ey * ez * et;
  const BoxDecoder bx = make_decoder(empty ? 1 : ex, empty ? 1 : ey, empty ? 1 : ez, bnd, bnd,
                                     bnd, bnd);
  long long nb = (nbox + NA_THREADS - 1) / NA_THREADS;
  if (nb > NA_MAX_BLOCKS) nb = NA_MAX_BLOCKS;
  if (nb < 1) nb = 1;
  const double scale = 1. / (double)(ex * ey * ez * et);
  // an error the caller left pending is not ours to report or to clear
  const cudaError_t before = cudaPeekAtLastError();
  k_ls_diff_noalloc<<<(int)nb, NA_THREADS, 0, s>>>(i0, i1, out, d, bx, (uint32_t)nbox, correction,
                                                   scale, scratch, result);
  const cudaError_t after = cudaPeekAtLastError();
  if (after != cudaSuccess && after != before) {
    cudaGetLastError();
    const std::string msg =
        std::string("calcLsDiff4d_noalloc: kernel launch failed: ") + cudaGetErrorString(after);
    return na_fail(FLOF_E_CUDA, msg.c_str());
  }
  return FLOF_OK;
}
