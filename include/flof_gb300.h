/*
 * flof_gb300.h -- C ABI of the GB300 implementation of the FlOF hot path
 * (thunil/ofblend, source/plugin/optflow4d.cpp and the Grid4d type of
 * source/grid4d.{h,cpp}).
 *
 * Every entry point is a plain C function over opaque handles, plain
 * pointers and sizes; none throws.  Each returns an flof_status and, on
 * failure, leaves a message retrievable with flof_last_error() (thread
 * local).  The reference raises a C++ exception through errMsg()
 * (source/general.h:96-99) which its Python wrapper turns into a Python
 * error; a binding maps a non-zero status to its own error type.
 *
 * Data layout is the reference's (source/grid4d.h:92-97): a 4D grid of size
 * (X,Y,Z,T) is stored x-fastest, idx = i + X*j + X*Y*k + X*Y*Z*t.  Real
 * grids hold one float per cell, Vec4 grids four (x,y,z,t interleaved).  A
 * 3D Grid<Real> (the mode-3 output slice) is a grid with T == 1.
 *
 * Grids live in device memory (HBM) and are owned by a context, as the
 * reference's grids are owned by a FluidSolver pool
 * (source/fluidsolver.cpp:87-124).  Host buffers enter and leave through
 * flof_grid_upload / flof_grid_download.  All work of one context runs in
 * order on the context's CUDA stream; calls that return scalars (errors,
 * maxima) synchronise on that stream.  A context is used by one thread at a
 * time, like the reference's plugins, which run with the Python GIL held.
 */
#ifndef FLOF_GB300_H
#define FLOF_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FLOF_API __attribute__((visibility("default")))

typedef enum {
  FLOF_OK = 0,
  FLOF_E_ARG = 1,      /* invalid argument, size or type mismatch         */
  FLOF_E_CUDA = 2,     /* CUDA runtime error                               */
  FLOF_E_OOM = 3,      /* device allocation failed                         */
  FLOF_E_NAN = 4,      /* non-finite values where finite ones are required */
  FLOF_E_STALL = 5,    /* iterative solve stopped without converging       */
  FLOF_E_TIMEOUT = 6,  /* a bounded device wait gave up                    */
  FLOF_E_STATE = 7,    /* call out of order (e.g. OptRun before OptInit)   */
  FLOF_E_NOTFOUND = 8  /* unknown handle or id                             */
} flof_status;

/* Element types, numbered as Grid4dBase::Grid4dType (source/grid4d.h:29-35). */
typedef enum { FLOF_REAL = 1, FLOF_VEC4 = 8 } flof_elem;

/* Gaussian blur variants for postVelBlur (optflow4d.cpp:531-541).
 * 1 = the reference's direct 4D stencil (knGaussianBlur, :132-158), bitwise
 *     equal to the reference;
 * 2 = separable stencils: the blur as a 4x1D stencil with the same in-bounds
 *     normalisation, and the projection's extrapolation sweep
 *     (knCvExpolBlur4d, :613-626) with its 3^4 box sum formed as 3x3 (x,y)
 *     sums added over z and t; equal to 1 up to float rounding, the blur
 *     about five times and the sweep about a quarter cheaper. */
enum { FLOF_BLUR_GAUSS = 1, FLOF_BLUR_GAUSS_SEPARABLE = 2 };

typedef struct flof_ctx flof_ctx;
typedef struct flof_grid flof_grid;
typedef struct flof_model flof_model;

/* Keyword arguments of opticalFlowMultiscale4d
 * (optflow4d.cpp:2182-2189), same names and meaning, plus cgMaxIter, which
 * the reference hard-codes to 1000 (:502). */
typedef struct flof_of_params {
  float wSmooth;
  float wEnergy;
  int level;
  float postVelBlur;
  float cgAccuracy;
  int blurType;
  float cfl;
  int orderTime;
  int orderSpace;
  float resetBndWidth;
  int multiStep;
  int projSizeThresh;
  int minGridSize;
  int doFinalProject;
  int cgMaxIter;
  /* FLOF_PRECISION_FP32 (default): the reference's float solve.
   * FLOF_PRECISION_MIXED: PCG on the BF16-stored image gradient, FP64
   * residuals of the FP32 system and iterative refinement (no reference
   * counterpart). */
  int precision;
  /* 1: start the coarsest level from the learned warm start attached with
   * flof_ctx_set_model (dropped when it does not lower that level's error
   * metric); 0 (default): the reference's zero start. */
  int warmStart;
  /* FLOF_SOLVER_PCG (default): the reference's Jacobi-preconditioned CG.
   * FLOF_SOLVER_MG: the same CG preconditioned by a multigrid V-cycle with
   * the same stop rule on the same residual; the plain operator re-forms the
   * final residual and the plain Jacobi-PCG finishes the solve when it is
   * above the threshold (no reference counterpart). */
  int solver;
  int reserved[4];
} flof_of_params;
enum { FLOF_PRECISION_FP32 = 0, FLOF_PRECISION_MIXED = 1 };
enum { FLOF_SOLVER_PCG = 0, FLOF_SOLVER_MG = 1 };

#define FLOF_MAX_SOLVE_STATS 64
/* Per-call record of the linear solves (the reference logs the same facts
 * with debMsg, optflow4d.cpp:496-517). */
typedef struct flof_solve_stats {
  int nsolves;
  int size_x[FLOF_MAX_SOLVE_STATS];     /* X extent of the level            */
  int iterations[FLOF_MAX_SOLVE_STATS]; /* PCG iterations                   */
  float residual[FLOF_MAX_SOLVE_STATS]; /* max(r)/max(r0) at exit           */
  int status[FLOF_MAX_SOLVE_STATS];     /* 1 converged, 2 sigma==0/NaN,
                                           3 tiny initial residual,
                                           4 iteration limit                */
  int cg_total_iterations;
  int syncs;                            /* host synchronisations            */
  float err_final;                      /* returned error metric            */
  double seconds;                       /* wall time of the call            */
  /* ||b - A x||_2 / ||b||_2 of the FP32 system in FP64 (mixed precision;
   * -1 when not computed) */
  float true_residual[FLOF_MAX_SOLVE_STATS];
  /* learned warm start: 1 used, 0 dropped by the error check, -1 not tried */
  int warm_start;
  float warm_start_err[2];              /* coarse error: zero start, prediction */
} flof_solve_stats;

/* ---- library / context -------------------------------------------------- */
FLOF_API const char *flof_version(void);
FLOF_API const char *flof_last_error(void);
FLOF_API const char *flof_status_string(int status);
/* Fills the reference's defaults of opticalFlowMultiscale4d
 * (optflow4d.cpp:2182-2189), cgMaxIter = 1000, blurType = 1. */
FLOF_API void flof_of_params_default(flof_of_params *p);
/* Fills the parameters scenes/flof.py:913-915 passes in mode 1. */
FLOF_API void flof_of_params_flof(flof_of_params *p);

FLOF_API int flof_ctx_create(int device, flof_ctx **out);
FLOF_API int flof_ctx_destroy(flof_ctx *ctx);
FLOF_API int flof_ctx_synchronize(flof_ctx *ctx);
/* Use an external CUDA stream (cudaStream_t passed as void*); NULL restores
 * the context's own stream. */
FLOF_API int flof_ctx_set_stream(flof_ctx *ctx, void *stream);
FLOF_API void *flof_ctx_stream(flof_ctx *ctx);
/* Number of kernels this context has launched so far. */
FLOF_API long long flof_ctx_kernel_launches(flof_ctx *ctx);
/* Kernel tracing.  flof_ctx_profile(ctx, 1) clears the record list and
 * brackets every later kernel launch with CUDA events on the context stream;
 * each record holds the kernel class, the X extent of the launch's grid, its
 * algorithmic bytes (compulsory reads + writes) and its device time.  The
 * reference times whole plugin calls instead (pbPreparePlugin /
 * pbFinalizePlugin, source/pwrapper/pclass.cpp:27-45). */
FLOF_API int flof_ctx_profile(flof_ctx *ctx, int enable);
FLOF_API int flof_ctx_profile_count(flof_ctx *ctx, int *n);
FLOF_API int flof_ctx_profile_record(flof_ctx *ctx, int i, int *cls,
                                     int *size_x, double *bytes, float *ms);
FLOF_API const char *flof_kernel_class_name(int cls);
/* Context options (flof_ctx_set_option).
 * FLOF_OPT_CFL_SYNC: 0 (default) the CFL substep count of advectCflHelper4d
 *   (optflow4d.cpp:1309-1321) is checked on the device and a call that needs
 *   more than one substep is redone; 1 the host reads max |v| before every
 *   CFL-guarded advection.
 * FLOF_OPT_AUTOTUNE: 1 times a few launch shapes of the PCG kernels once per
 *   grid size and keeps the fastest; 0 (default) uses fixed shapes.  Shapes
 *   group the dot-product partial sums differently, so tuned and untuned runs
 *   agree to rounding, not bit for bit.
 * FLOF_OPT_STRICT: 1 runs the FP32 PCG with the reference's arithmetic
 *   operation for operation (GridCGOptflow4d::solve, optflow4d.cpp:268-329:
 *   double alpha and beta, addScaled's double multiply and add rounded once
 *   to float, dotProd's serial double sum in row order) and sums the error
 *   metric serially in calcLsDiffTempl's loop order (:895-927), so that
 *   whole solves equal the reference's bit for bit.  One thread forms each
 *   sum: for parity checks on grids of a few million cells, not for speed.
 *   0 (default): the parallel kernels.
 * FLOF_OPT_SLAB_TMA: 1 (default) the Vec4 Gaussian blur and the extrapolation
 *   sweeps of corrVelsOf4d use the TMA slab kernels; 0 their plain-load
 *   counterparts, which take the same sums in the same order (equal results;
 *   for checking one against the other). */
enum { FLOF_OPT_CFL_SYNC = 2, FLOF_OPT_AUTOTUNE = 3, FLOF_OPT_STRICT = 4, FLOF_OPT_SLAB_TMA = 5 };
FLOF_API int flof_ctx_set_option(flof_ctx *ctx, int option, int value);
/* Parameters of the multigrid V-cycle of FLOF_SOLVER_MG (no reference
 * counterpart): damping of the block-Jacobi sweeps on the system's own grid
 * (omega0) and on the coarse levels (omegac), in (0, 1]; the scale of each
 * coarse level's Laplacian against its Galerkin product (lambda, in
 * (0, 1]; 1/2 rediscretises it); sweeps on the coarsest level (1..256);
 * preconditioned iterations before the plain Jacobi-PCG takes over (>= 0).
 * Defaults 0.95, 1.0, 0.9, 8, 200 (fitted on solver-generated systems). */
FLOF_API int flof_ctx_set_mg_params(flof_ctx *ctx, float omega0, float omegac, float lambda,
                                    int coarse_sweeps, int max_iter);
/* Solves of FLOF_SOLVER_MG so far whose result the plain Jacobi-PCG had to
 * finish (residual above the threshold, or no convergence within the
 * preconditioned solve's iteration cap). */
FLOF_API long long flof_ctx_mg_fallbacks(flof_ctx *ctx);
/* Release cached device buffers of the context's pool (and its workers'). */
FLOF_API int flof_ctx_trim(flof_ctx *ctx);

/* ---- grids: Grid4d<Real>, Grid4d<Vec4> (source/grid4d.h:117-265) -------- */
/* New zero-filled device grid (the Grid4d constructor clears, grid4d.cpp:82). */
FLOF_API int flof_grid_create(flof_ctx *ctx, const int dims[4], int elem,
                              flof_grid **out);
/* Non-owning view of caller device memory (x-fastest, 16-byte aligned). */
FLOF_API int flof_grid_wrap(flof_ctx *ctx, const int dims[4], int elem,
                            void *device_ptr, flof_grid **out);
FLOF_API int flof_grid_destroy(flof_grid *g);
FLOF_API int flof_grid_dims(const flof_grid *g, int dims[4], int *elem);
FLOF_API void *flof_grid_data(flof_grid *g);
/* Host <-> device copies of the whole grid (bytes = cells * 4 * ncomp). */
FLOF_API int flof_grid_upload(flof_grid *g, const void *host);
FLOF_API int flof_grid_download(const flof_grid *g, void *host);
/* Asynchronous copies on the context's copy stream, so that transfers
 * overlap the kernels of the context stream (no counterpart in the
 * reference).  Each copy starts after the work queued on the context stream
 * when it is issued.  After an upload, call flof_grid_copy_wait before work
 * that reads the grid; after a download, call it before work that writes the
 * grid.  flof_grid_copy_wait makes the context stream wait on the device for
 * the grid's last asynchronous copy; the host does not block.
 * flof_ctx_copies_sync waits on the host for all of them, and so does
 * flof_ctx_synchronize.  Host buffers must stay valid until then; pinned
 * buffers give the overlap, pageable ones are staged synchronously. */
FLOF_API int flof_grid_upload_async(flof_grid *g, const void *host);
FLOF_API int flof_grid_download_async(flof_grid *g, void *host);
FLOF_API int flof_grid_copy_wait(flof_grid *g);
FLOF_API int flof_ctx_copies_sync(flof_ctx *ctx);

/* Grid4d methods (grid4d.cpp:198-412).  Constants are float[4]; Real grids
 * use element 0. */
FLOF_API int flof_grid_copyFrom(flof_grid *dst, const flof_grid *src);
FLOF_API int flof_grid_add(flof_grid *a, const flof_grid *b);
FLOF_API int flof_grid_sub(flof_grid *a, const flof_grid *b);
FLOF_API int flof_grid_setConst(flof_grid *a, const float v[4]);
FLOF_API int flof_grid_addConst(flof_grid *a, const float v[4]);
FLOF_API int flof_grid_multConst(flof_grid *a, const float v[4]);
FLOF_API int flof_grid_addScaled(flof_grid *a, const flof_grid *b,
                                 const float factor[4]);
FLOF_API int flof_grid_clear(flof_grid *a);
/* getMax / getMin / getMaxAbs (grid4d.cpp:263-285); Vec4 grids reduce the
 * vector norm. */
FLOF_API int flof_grid_getMax(flof_grid *a, float *out);
FLOF_API int flof_grid_getMin(flof_grid *a, float *out);
FLOF_API int flof_grid_getMaxAbs(flof_grid *a, float *out);
/* setBound: cells with c <= w or c >= size-1-w (knSetBnd4d, :355-368). */
FLOF_API int flof_grid_setBound(flof_grid *a, const float v[4], int w);
/* setBoundNeumann (knSetBnd4dNeumann, :370-407). */
FLOF_API int flof_grid_setBoundNeumann(flof_grid *a, int w);

/* ---- plugins --------------------------------------------------------------- */

/* opticalFlowMultiscale4d (optflow4d.cpp:2182-2195 ->
 * opticalFlowMultiscaleTemplate :936-1173).  vel is in/out (flof passes a
 * zero grid); i0, i1 are Real grids of the same size.  err (nullable)
 * receives the returned error metric; stats (nullable) the solve record.
 * rhsT of the reference is a debug output and is not offered. */
FLOF_API int flof_opticalFlowMultiscale4d(flof_ctx *ctx, flof_grid *vel,
                                          const flof_grid *i0,
                                          const flof_grid *i1,
                                          const flof_of_params *params,
                                          float *err, flof_solve_stats *stats);

/* Batched opticalFlowMultiscale4d: n independent solves with the same
 * parameters and any grid sizes (vels[q], i0s[q], i1s[q] of one size per q).
 * They run concurrently on `workers` worker streams of the context, each
 * driven by its own host thread; workers <= 0 picks the count from the
 * smallest size.  At most 4M cells of solves are in flight at once, so a
 * larger solve runs alone.  With params->warmStart and a model attached to
 * ctx, the solves run one after another on ctx itself (the model's buffers
 * serve one prediction at a time).  Every solve gives the same result as the
 * single call on the same grids.  errs (nullable) receives n error metrics. */
FLOF_API int flof_opticalFlowMultiscale4d_batch(flof_ctx *ctx, int n,
                                                flof_grid *const *vels,
                                                const flof_grid *const *i0s,
                                                const flof_grid *const *i1s,
                                                const flof_of_params *params,
                                                float *errs, int workers);

/* opticalFlow4d (optflow4d.cpp:2110-2119 -> opticalFlowDim :361-553): one
 * level, one solve.  iterations / residual (nullable) report the PCG. */
FLOF_API int flof_opticalFlow4d(flof_ctx *ctx, flof_grid *vel,
                                const flof_grid *i0, const flof_grid *i1,
                                float wSmooth, float wEnergy, float postVelBlur,
                                float cgAccuracy, int blurType,
                                float resetBndWidth, int cgMaxIter,
                                int *iterations, float *residual);

/* corrVelsOf4d (optflow4d.cpp:2121-2130 -> corrVelsOfTempl :737-802).
 * phiCurr is unused by the reference and may be NULL. */
FLOF_API int flof_corrVelsOf4d(flof_ctx *ctx, flof_grid *dst, flof_grid *vel,
                               const flof_grid *phiOrg,
                               const flof_grid *phiCurr,
                               const flof_grid *phiTarget, float threshPhi,
                               float threshNorm, float postVelBlur,
                               float resetBndWidth, int maxIter);

/* gaussianBlurGeneric(a, sigma, iter=1) (optflow4d.cpp:160-174), the
 * reference's internal velocity blur, exposed for stage-wise checks.
 * blurType as in flof_of_params (1 direct stencil, 2 separable). */
FLOF_API int flof_gaussianBlur4d(flof_ctx *ctx, flof_grid *a, float sigma,
                                 int blurType);

/* advect4d (optflow4d.cpp:1292-1306): semi-Lagrangian advection of a Real
 * or Vec4 grid by vel with dt = solver dt (1) * dtFac. */
FLOF_API int flof_advect4d(flof_ctx *ctx, const flof_grid *vel,
                           flof_grid *grid, float dtFac);

/* calcLsDiff4d (optflow4d.cpp:2132-2137 -> calcLsDiffTempl :895-927).
 * Every axis loses 2 bnd cells, T and Z included: Grid4d's is3D() and
 * is4D() are constant true (grid4d.h:82-83).  A bnd that leaves no cells
 * gives the reference's 0 * (1 / count): -0 for a negative count, NaN for
 * a zero one.  bnd must be in [0, 2^20]. */
FLOF_API int flof_calcLsDiff4d(flof_ctx *ctx, const flof_grid *i0,
                               const flof_grid *i1, flof_grid *out,
                               float correction, int bnd, float *result);

/* interpolateGrid4d / interpolateGrid4dVec (grid4d.cpp:540-557).  offset,
 * scale and size are float[4] (defaults 0, 1, -1). */
FLOF_API int flof_interpolateGrid4d(flof_ctx *ctx, flof_grid *target,
                                    const flof_grid *source,
                                    const float offset[4], const float scale[4],
                                    const float size[4]);
FLOF_API int flof_interpolateGrid4dVec(flof_ctx *ctx, flof_grid *target,
                                       const flof_grid *source,
                                       const float offset[4],
                                       const float scale[4],
                                       const float size[4]);

/* Mode-2 apply of scenes/flof.py deform4d (:591-615) into `out`:
 * twoway 0: out = advect4d(vel, i0, alpha)
 * twoway 1: out = advect(vel,i0,alpha)*(1-alpha) + alpha*advect(velInv,i1,1-alpha)
 * twoway 2: out = advect(vel,i0,alpha)*(1-alpha) + alpha*i1  (naive blend)
 * alphaInv is the float (1 - alpha) the scene computes in double. */
FLOF_API int flof_deform4d(flof_ctx *ctx, flof_grid *out, const flof_grid *i0,
                           const flof_grid *i1, const flof_grid *vel,
                           const flof_grid *velInv, float alpha,
                           float alphaInv, int twoway);

/* calcLsDiff4d without any device allocation.  This entry point has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory where they need the error metric: applications that reserve
 * all device memory at start-up and forbid allocations afterwards, and loops
 * that cannot afford one (an allocation may synchronise the device).  It
 * computes the same value as flof_calcLsDiff4d (calcLsDiffTempl,
 * optflow4d.cpp:895-927) from the caller's device buffers on the caller's
 * stream (void* cudaStream_t, NULL for the legacy default stream) and writes
 * it to the device float `result`; `out` (device, nullable) receives the
 * per-cell values.  A bnd that leaves no cells gives the reference's
 * 0 * (1 / count) (-0 or NaN), as flof_calcLsDiff4d does.
 * Grids up to 2^31-1 cells; larger ones are rejected with FLOF_E_ARG.
 * Its scratch is a fixed 8 KiB device array in the library (1024 block
 * partials plus a counter), held by every GPU that loads the library until
 * exit and shared by all calls: calls that overlap on the GPU race on it.
 * Every call looks the array's address up for the current context, except
 * while its stream is being captured, when the address found by the last
 * call on that device is used. */
FLOF_API int flof_calcLsDiff4d_noalloc(const float *i0, const float *i1,
                                       float *out, const int dims[4],
                                       float correction, int bnd,
                                       float *result, void *stream);

/* loadAdvectTimeSlice_OptInit (optflow4d.cpp:1871-1913).  The reference
 * names a .uni file that OptRun streams t-slices from; here the whole
 * deformation `defo` (Vec4 grid) is already resident in device memory and
 * the context pins it until Finish (a flof_grid_destroy in between is
 * deferred until then).  Defo volumes
 * (useDefoVols, the three-data-set mode) are not supported: FLOF_E_ARG. */
FLOF_API int flof_loadAdvectTimeSlice_OptInit(flof_ctx *ctx, int id,
                                              const flof_grid *defo,
                                              int useDefoVols, int doAligned,
                                              float partialLoadFac);
/* loadAdvectTimeSlice_OptRun (optflow4d.cpp:1951-2105) for one output frame:
 * blends defo t-slices t and t+1, then knSemiLagrangeLookupSlice4d_WithVel
 * (:1648-1665) writes dst (a T == 1 grid) inside the bnd=10 / bordSkip box.
 * Vector arguments are float[4]. */
FLOF_API int flof_loadAdvectTimeSlice_OptRun(
    flof_ctx *ctx, int id, flof_grid *dst, const flof_grid *phi, float time,
    float blendAlpha, float loadTimeScale, const float defoOffset[4],
    const float defoScale[4], const float defoFactor[4],
    const float overrideSize[4], float overrideTimeOff, int zeroVel,
    float thirdAlpha, int bordSkip, float fourthAlpha, float defoAniFac);
/* Two-way frame in one pass: dst = OptRun(id0, phi0, alpha) * (1-alpha) +
 * alpha * OptRun(id1, phi1, 1-alpha), the blend of scenes/flof.py:750-755.
 * Cells outside the lookup box keep their previous contents (the scene
 * overwrites that ring with setBound afterwards, flof.py:830-832). */
FLOF_API int flof_loadAdvectTimeSlice_OptRunTwoway(
    flof_ctx *ctx, int id0, int id1, flof_grid *dst, const flof_grid *phi0,
    const flof_grid *phi1, float time, float blendAlpha, float alphaInv,
    float loadTimeScale, const float defoOffset[4], const float defoScale[4],
    const float defoFactor[4], const float overrideSize[4],
    float overrideTimeOff, int bordSkip, float defoAniFac);
/* loadAdvectTimeSlice_Finish (optflow4d.cpp:1930-1950). */
FLOF_API int flof_loadAdvectTimeSlice_Finish(flof_ctx *ctx, int id);

/* ---- .uni grid files (source/fileio.cpp:834-1000) ------------------------
 * gzip streams: a 4-byte tag ("MNT2" 3D, "M4T2" 4D), the 288-byte UniHeader,
 * for 4D an int32 t extent, then float32 cells x fastest.  zlib is loaded at
 * run time (libz.so.1). */

/* Header of a file: dims = x, y, z, t (t = 1 for a 3D file). */
FLOF_API int flof_uni_info(const char *fname, int dims[4], int *is4d,
                           int *gridType, int *bytesPerElement);
/* Grid4d::load / Grid<T>::load: the file's extents and element size must
 * match the grid (a 3D file needs t extent 1). */
FLOF_API int flof_grid_load(flof_grid *grid, const char *fname);
/* Grid4d::save (is4d != 0, M4T2) / Grid<Real>::save (is4d == 0, MNT2). */
FLOF_API int flof_grid_save(const flof_grid *grid, const char *fname,
                            int is4d);
/* readGrid4dUni(name, NULL, t, slice) (fileio.cpp:912-990): t slice of a 4D
 * file into a grid with the file's x, y, z extents and t extent 1. */
FLOF_API int flof_uni_read_slice(flof_grid *slice, const char *fname, int t);

/* ---- learned warm start ------------------------------------------------
 * A 4D convolutional encoder-decoder (3 levels, 16/32/64 channels, BF16
 * weights, FP32 accumulation) mapping the coarsest-level inputs (i0, i1) of
 * the multiscale solve on a res^4 grid to that level's deformation.  It has
 * no counterpart in the reference.  Training and inference run on the GPU;
 * the plain PCG refines every level afterwards. */
FLOF_API int flof_model_create(flof_ctx *ctx, int res, flof_model **out);
FLOF_API int flof_model_destroy(flof_model *model);
FLOF_API int flof_model_num_params(const flof_model *model, long long *n);
/* He-normal weights from a seeded RNG, zero biases, fresh Adam state. */
FLOF_API int flof_model_init(flof_model *model, unsigned long long seed);
/* FP32 master parameters, layer by layer (weights [tap][cin][cout], bias). */
FLOF_API int flof_model_get_params(const flof_model *model, float *host);
FLOF_API int flof_model_set_params(flof_model *model, const float *host);
/* vel (Vec4 res^4) = network(i0, i1) (Real res^4 grids). */
FLOF_API int flof_model_predict(flof_model *model, const flof_grid *i0,
                                const flof_grid *i1, flof_grid *vel);
/* Mean squared error against target and its gradient (grad nullable, host,
 * num_params floats) for one sample. */
FLOF_API int flof_model_loss_grad(flof_model *model, const flof_grid *i0,
                                  const flof_grid *i1, const flof_grid *target,
                                  double *loss, float *grad);
/* One Adam step on the mean loss of n samples. */
FLOF_API int flof_model_train_step(flof_model *model, int n,
                                   const flof_grid *const *i0s,
                                   const flof_grid *const *i1s,
                                   const flof_grid *const *targets, float lr,
                                   double *loss);
/* The model used when flof_of_params.warmStart is 1 (NULL detaches). */
FLOF_API int flof_ctx_set_model(flof_ctx *ctx, flof_model *model);

/* ---- input conditioning (scenes/flof.py postProcessPhiData :491-531) ---- */

/* repeatFrame4d (optflow4d.cpp:1254-1266): slices int(srct-range+0.5) ..
 * int(srct) of the bnd box get phi interpolated at time srct.  Slices
 * outside [0, T) are skipped (the reference does not check). */
FLOF_API int flof_repeatFrame4d(flof_grid *phi, float srct, float range,
                                int bnd);
/* extrap4dLsSimple (optflow4d.cpp:1332-1406) of a Real grid, every extent
 * at least 3; inside != 0 marches into the positive region. */
FLOF_API int flof_extrap4dLsSimple(flof_grid *phi, int distance, int inside);

/* ---- 3D Grid<Real> methods of the mode-3 output stage -------------------- */
/* A 3D grid is a flof_grid with t extent 1; it is 2D when its z extent is
 * 1, as for the reference's Grid<T>::is3D(). */

/* LevelsetGrid::join (levelset.cpp:114-118): a = min(a, b), any Real grid. */
FLOF_API int flof_grid_join(flof_grid *a, const flof_grid *b);
/* Grid<T>::setBound / setBoundNeumann (grid.cpp:462-511) of a 3D grid. */
FLOF_API int flof_grid3_setBound(flof_grid *a, const float value[4], int w);
FLOF_API int flof_grid3_setBoundNeumann(flof_grid *a, int w);
/* simpleBlurSpecial(a, iter, thresh, bord) (test.cpp:94-131) of a 3D Real
 * grid: the writeResults smoothing and time-SDF merge of scenes/flof.py
 * (:818-828) and scenes/ofHelpers.py (:108-113). */
FLOF_API int flof_simpleBlurSpecial(flof_grid *a, int iter, float thresh,
                                    int bord);

/* ---- hi-res 4D assembly with partial loads (flof.py:707-723) ------------ */

/* shiftForwGrid4d (optflow4d.cpp:1596-1616): t slices [T-good, T) move to
 * [0, good).  good must be below T (the reference loops forever for
 * good >= T). */
FLOF_API int flof_shiftForwGrid4d(flof_grid *phi, int overrideGoodRegion);
/* loadPlaceGrid4d (optflow4d.cpp:1460-1594): places the 3D slice files
 * fname % fileid (a printf pattern with one integer conversion; .uni MNT2)
 * into the Real 4D grid phi.  With fname NULL the slices are the device
 * grids slices[fileid - fileIdxStart], q < nslices.  Vector arguments are
 * float[4]; overrideSize may be NULL. */
FLOF_API int flof_loadPlaceGrid4d(flof_grid *phi, const char *fname,
                                  const flof_grid *const *slices, int nslices,
                                  const float offset[4], const float scale[4],
                                  int fileIdxStart, int fileIdxEnd,
                                  int debugSkipLoad, float spread,
                                  const float overrideSize[4],
                                  float overrideTimeOff, int overrideGoodRegion,
                                  float loadTimeScale, int rescaleSdfValues,
                                  float sdfIsoOff, float repeatStartFrame);

/* ---- mode 3 from files ---------------------------------------------------- */

/* loadAdvectTimeSlice_OptInit with the reference's file argument: the M4T2
 * Vec4 deformation file is loaded whole into device memory owned by the
 * context until Finish. */
FLOF_API int flof_loadAdvectTimeSlice_OptInitFile(flof_ctx *ctx, int id,
                                                  const char *fname,
                                                  int useDefoVols,
                                                  int doAligned,
                                                  float partialLoadFac);
/* loadAdvectTimeSlice (optflow4d.cpp:1671-1760), the non-optimised twin of
 * OptRun: blends deformation slices t and t+1 of `defo` (device Vec4 grid)
 * or, when defo is NULL, of the file fname, and looks phi up over the
 * bnd = 1 box of dst (no bordSkip, as in the reference). */
FLOF_API int flof_loadAdvectTimeSlice(flof_ctx *ctx, const flof_grid *defo,
                                      const char *fname, flof_grid *dst,
                                      const flof_grid *phi, float time,
                                      float blendAlpha, float loadTimeScale,
                                      const float defoOffset[4],
                                      const float defoScale[4],
                                      const float defoFactor[4],
                                      const float overrideSize[4],
                                      float overrideTimeOff, int zeroVel,
                                      float defoAniFac);

#ifdef __cplusplus
}
#endif

#endif /* FLOF_GB300_H */
