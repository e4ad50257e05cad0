// flof_kernels.h -- host-side launchers of the FlOF CUDA kernels.  Every
// launcher enqueues work on the given stream and returns immediately; errors
// surface through cudaGetLastError() / the next synchronisation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "flof_common.cuh"

namespace flof {

// Sets the thread-local message returned by flof_last_error().
void set_last_error(const char *msg);

// Number of SMs of the current device (cached), used to size grids.
int sm_count();
// Blocks for a grid-stride launch over n items with `nt` threads per block.
int grid_for(long long n, int nt, int per_sm = 8);

// ---- elementwise (n = number of floats) -----------------------------------
void launch_set_const(float *a, long long ncell, int nc, float4 v, cudaStream_t s);
void launch_add_const(float *a, long long ncell, int nc, float4 v, cudaStream_t s);
void launch_mult_const(float *a, long long ncell, int nc, float4 v, cudaStream_t s);
void launch_add(float *a, const float *b, long long n, cudaStream_t s);
void launch_sub(float *a, const float *b, long long n, cudaStream_t s);
// a += factor * b, per component
void launch_add_scaled(float *a, const float *b, long long ncell, int nc, float4 f,
                       cudaStream_t s);

// ---- borders -----------------------------------------------------------------
void launch_set_bound(float *a, Dims4 d, int nc, float4 v, int w, cudaStream_t s);
void launch_set_bound_neumann(float *a, Dims4 d, int nc, int w, cudaStream_t s);
// zero every cell outside isInBounds(resetBnd)
void launch_reset_outside(float4 *a, Dims4 d, int resetBnd, cudaStream_t s);

// ---- reductions (result written to device memory) ---------------------------
// which: 0 max, 1 min.  For nc == 4 the value is max/min |v|^2 (no sqrt).
// `partials` holds grid_for(...) floats, `counter` one zeroed uint.
void launch_reduce_minmax(const float *a, long long ncell, int nc, int which,
                          float *partials, unsigned int *counter, float *result,
                          cudaStream_t s);
// calcLsDiffTempl sum over the bnd box (double), scaled as the reference
// does; result as double and as float.
void launch_ls_diff(const float *i0, const float *i1, float *out, Dims4 d,
                    float correction, int bnd, double *partials,
                    unsigned int *counter, double *result_d, float *result_f,
                    cudaStream_t s);
int ls_diff_blocks(Dims4 d, int bnd);

// ---- resampling / advection ---------------------------------------------------
void launch_resample(float *target, Dims4 td, const float *source, Dims4 sd,
                     int nc, float4 fac, float4 off, cudaStream_t s);
// dst (fresh) = src sampled at ijkt+0.5 - vel*dt over bnd=1 cells; the
// border ring of dst is written with zeros.
void launch_advect(const float4 *vel, const float *src, float *dst, Dims4 d,
                   int nc, float dt, cudaStream_t s);
// One substep of the CFL-guarded advection with the substep count checked
// on the device: maxn2 is the device max |v|^2; *flag is set when
// int(maxVel/cfl)+1 != 1.
void launch_advect_cfl1(const float4 *vel, const float *src, float *dst, Dims4 d, int nc,
                        const float *maxn2, float cfl, int *flag, cudaStream_t s);
// Two-way blend of deform4d (scenes/flof.py:603-610) in one pass:
// out = (advect(vel,i0,a) * (1-a)) + a * advect(velInv,i1,1-a).
void launch_deform_twoway(const float4 *vel, const float4 *velInv,
                          const float *i0, const float *i1, float *out, Dims4 d,
                          float alpha, float alphaInv, cudaStream_t s);

// ---- mode-3 slice lookup -------------------------------------------------------
// vt = (0 + f1*v1) + f2*v2 over one defo t-slice of `cells` cells
void launch_blend_slices(const float4 *v1, const float4 *v2, float4 *vt,
                         long long cells, float f1, float f2, cudaStream_t s);
// the same for two sets (both directions of a two-way frame) in one launch
void launch_blend_slices2(const float4 *v1a, const float4 *v2a, float4 *vta, float fa1, float fa2,
                          const float4 *v1b, const float4 *v2b, float4 *vtb, float fb1, float fb2,
                          long long cells, cudaStream_t s);
// minBnd: the KERNEL bnd of the lookup, 10 for knSemiLagrangeLookupSlice4d_
// WithVel (OptRun), 1 for knSemiLagrangeLookupSlice4d (loadAdvectTimeSlice).
void launch_lookup_slice(float *dst, int dx, int dy, int dz, const float *phi,
                         Dims4 pd, float time, float dt, const float4 *vt,
                         int vx, int vy, int vz, float4 sf3, float4 off3,
                         float4 defoFactor, int bordSkip, cudaStream_t s, int minBnd = 10);
// Both directions of a two-way frame plus the blend of scenes/flof.py
// :750-755, in one pass.
void launch_lookup_slice_twoway(float *dst, int dx, int dy, int dz,
                                const float *phi0, const float *phi1, Dims4 pd,
                                float time, float alpha, float alphaInv,
                                const float4 *vt0, const float4 *vt1, int vx,
                                int vy, int vz, float4 sf3, float4 off3,
                                float4 defoFactor, int bordSkip, cudaStream_t s);

// ---- optical flow system and PCG ---------------------------------------------------
struct CGState {
  double sigma;     // z . r of the current iterate
  double alpha;     // sigma / (p . A p)
  double beta;      // sigmaNew / sigma
  double acc;       // accuracy * max(r0)
  double resIni;    // max(r0)
  double pAp;
  float alphaf;     // (float)alpha and (float)beta, the values the kernels use
  float betaf;
  float resMax;     // max(r) after the last update
  float retResidual;  // resMax / resIni
  int done;         // 0 running; see CG_* below
  int iters;
  int xpend;        // 1: x += alpha p of the last update is still to be applied
  unsigned int counter[4];
};
enum { CG_RUNNING = 0, CG_CONVERGED = 1, CG_FAILED_SIGMA = 2, CG_EARLY = 3,
       CG_MAXITER = 4 };

struct OFConsts {
  float dxf;        // 1 / (2 mDx)
  float mDx;
  float mDt;
  float wSmooth;
  float wEnergy;
  float offd;       // -wSmooth * mDx2Inv
  float diag;       // 8 wSmooth mDx2Inv + wEnergy
};

int cg_blocks(Dims4 d);
// Launch shapes of the PCG kernels, chosen per grid size by the autotuner
// (defaults otherwise): t planes per matvec work item (4, 8 or 16) and
// resident blocks per SM of the update / direction kernels.
struct CGTune {
  int mv_tt = 8;
  int per_sm = 8;
};
// Assembly + PCG initialisation over all cells.  vel may be null (zero).
// Writes g, r = rhs, p = z on the interior, zeros on the border ring, and
// x = 0 everywhere.
void launch_of_assemble_init(const float *i0w, const float *i1,
                             const float4 *vel, float4 *g, float4 *r,
                             float4 *p, float4 *x, Dims4 d, OFConsts c,
                             float accuracy, CGState *st, double *dpart,
                             float *fpart, cudaStream_t s);
void launch_cg_matvec(const float4 *p, const float4 *g, float4 *q, Dims4 d,
                      OFConsts c, CGState *st, double *dpart, cudaStream_t s,
                      const CGTune &tu = CGTune());
// The update (r -= alpha q, z.r, max r) takes the iteration number from
// st->iters and leaves x += alpha p to the direction kernel, which reads p
// anyway (st->xpend); the direction kernel applies it even after the update
// has ended the solve.  The x values are those of the textbook order bit for
// bit.
// With i1 (the level's target level set, from which the assembly built g)
// the two kernels rebuild g from it instead of reading g.
void launch_cg_update(float4 *r, const float4 *q, const float4 *g, Dims4 d, OFConsts c,
                      CGState *st, double *dpart, float *fpart, int maxIter, cudaStream_t s,
                      const CGTune &tu = CGTune(), const float *i1 = nullptr);
void launch_cg_direction(float4 *x, float4 *p, const float4 *r, const float4 *g, Dims4 d,
                         OFConsts c, CGState *st, cudaStream_t s,
                         const CGTune &tu = CGTune(), const float *i1 = nullptr);
// The same three kernels with the image gradient stored in BF16 (mixed
// precision: the matrix g g^T + diag I is built from the rounded gradient).
void launch_cg_matvec(const float4 *p, const BF4 *g, float4 *q, Dims4 d,
                      OFConsts c, CGState *st, double *dpart, cudaStream_t s,
                      const CGTune &tu = CGTune());
void launch_cg_update(float4 *r, const float4 *q, const BF4 *g, Dims4 d, OFConsts c,
                      CGState *st, double *dpart, float *fpart, int maxIter, cudaStream_t s,
                      const CGTune &tu = CGTune());
void launch_cg_direction(float4 *x, float4 *p, const float4 *r, const BF4 *g, Dims4 d,
                         OFConsts c, CGState *st, cudaStream_t s,
                         const CGTune &tu = CGTune());
// ---- strict arithmetic (flof_strict.cu, FLOF_OPT_STRICT) ----------------------
// The reference's PCG arithmetic operation for operation: double alpha and
// beta, double multiply-and-add updates rounded once to float, and dot
// products summed serially in the reference's row order by one thread.
// launch_strict_init follows launch_of_assemble_init (it replaces the
// parallel z.r with the serial one); one launch_strict_iteration is one PCG
// iteration (matvec, p.q, x and r updates with the stop rule, z.r, new p).
void launch_strict_init(const float4 *r, const float4 *g, Dims4 d, OFConsts c, CGState *st,
                        cudaStream_t s);
void launch_strict_iteration(float4 *x, float4 *r, float4 *p, float4 *q, const float4 *g, Dims4 d,
                             OFConsts c, CGState *st, double *dpart, float *fpart, int maxIter,
                             cudaStream_t s);
// calcLsDiffTempl with the serial double sum in the reference's loop order.
void launch_strict_ls_diff(const float *i0, const float *i1, float *out, Dims4 d, float correction,
                           int bnd, double *result_d, float *result_f, cudaStream_t s);
// ---- multigrid-preconditioned PCG (flof_mg.cu) --------------------------------
// Parameters of the V-cycle: damping of the block-Jacobi sweeps on level 0
// and on the coarse levels, the scale of each coarse level's Laplacian
// against its Galerkin product (1/2: rediscretised), and the sweeps on the
// coarsest level.  The defaults are the fit of ofblend_gb300/mgfit.py on six
// seeded 32^4 drop pairs at cgAccuracy 1e-4 (290 -> 213 iterations against
// 0.8 / 0.8 / 0.5 / 24).
struct MGParams {
  float omega0 = 0.95f;
  float omegac = 1.0f;
  float lambda = 0.9f;
  int coarse_sweeps = 8;
  int max_iter = 200;  // preconditioned iterations before the plain PCG takes over
};
// One coarse level: dense dims m; G (3 float4 per cell: the summed
// g g^T + wEnergy block and lapdiag), couplings to the +a neighbours, the
// block inverse (3 float4 per cell), and the V-cycle's rhs, iterate and
// scratch vectors (x and r are swapped by the V-cycle).
struct MGLevelPtrs {
  Dims4 m;
  float4 *G, *cpl, *dinv, *b, *x, *r;
};
// Dims of the coarse levels of a system on grid d (interior cells
// aggregated 2^4 at a time until at most 1024 cells remain); empty for a
// grid without interior cells.
std::vector<Dims4> mg_level_dims(Dims4 d);
// Builds the coarse operators from the level-0 gradient g.
void launch_mg_build(const float4 *g, Dims4 d, const MGLevelPtrs *L, int nl, const OFConsts &c,
                     const MGParams &mp, const CGState *st, cudaStream_t s);
// z = V-cycle(b0) on level 0 (x0, r0: level-0 scratch, x0's border zero),
// plus z.b0 into the PCG state: init 1 sets sigma (and beta = 0), init 0
// sets beta = z.b0 / sigma and sigma.  Counts its launches into *launches.
// pre_done: x0 already holds the first level-0 sweep (launch_mgcg_update_pre).
void launch_mg_vcycle(const float4 *b0, const float4 *g, float4 *x0, float4 *r0, float4 *z, Dims4 d,
                      MGLevelPtrs *L, int nl, const OFConsts &c, const MGParams &mp, CGState *st,
                      double *dpart, int init, int pre_done, cudaStream_t s, int *launches);
// x += alpha p, r -= alpha q, signed max of r and the stop rule.
void launch_mgcg_update(float4 *x, float4 *r, const float4 *p, const float4 *q, Dims4 d,
                        CGState *st, float *fpart, int maxIter, cudaStream_t s);
// The same plus the V-cycle's first level-0 sweep x0 = omega0 D^-1 r; with
// i1 (the level's target level set, from which the assembly built g) the
// block solve rebuilds g from it instead of reading g.
void launch_mgcg_update_pre(float4 *x, float4 *r, const float4 *p, const float4 *q,
                            const float4 *g, const float *i1, float4 *x0, Dims4 d,
                            const OFConsts &c, const MGParams &mp, CGState *st, float *fpart,
                            int maxIter, cudaStream_t s);
// The plain operator's residual r = b - A x of a preconditioned solve (float
// rows) and its signed maximum into the device float *rmax.
void launch_mg_judge(const float4 *x, const float4 *b, const float4 *g, float4 *r, Dims4 d,
                     const OFConsts &c, float *fpart, unsigned int *counter, float *rmax,
                     cudaStream_t s);
// p = z + beta p (init: p = z).
void launch_mgcg_direction(float4 *p, const float4 *z, Dims4 d, const CGState *st, int init,
                           cudaStream_t s);

// ---- mixed precision (flof_mixed.cu) ------------------------------------------
// g16 = bf16(g) over n cells
void launch_to_bf4(const float4 *g, BF4 *g16, long long n, cudaStream_t s);
// r = b - A x over the interior with A built from the FP32 gradient g and the
// row sums accumulated in FP64; res[0] = ||r||^2, res[1] = ||b||^2 (FP64),
// fres[0] = signed max of r (0 included: border rows).  res/fres must be
// zeroed (reset by the kernel's last block for the next call).
void launch_residual64(const float4 *x, const float4 *b, const float4 *g, float4 *r, Dims4 d,
                       OFConsts c, double *dpart, unsigned int *counter, double *res,
                       float *fres, cudaStream_t s);
// PCG start from a given residual r (x0 = 0, the caller zeroes x): p = z =
// M^-1 r on the interior, sigma = z.r, resIni = signed max of r; the state
// logic of the assembly's initialisation.
void launch_cg_init_r(const float4 *r, const BF4 *g, float4 *p, Dims4 d, OFConsts c,
                      float accuracy, CGState *st, double *dpart, float *fpart, cudaStream_t s);
void launch_cg_init_r(const float4 *r, const float4 *g, float4 *p, Dims4 d, OFConsts c,
                      float accuracy, CGState *st, double *dpart, float *fpart, cudaStream_t s);
// x = float((double)x + (double)e) over n cells
void launch_add_correction(float4 *x, const float4 *e, long long n, cudaStream_t s);
// vel = x / mDx over all cells (x border entries are zero)
void launch_of_copy_back(const float4 *x, float4 *vel, long long cells,
                         float mDx, const CGState *st, cudaStream_t s);

// ---- Gaussian blur (gaussianBlurGeneric, strict 4D stencil) -----------------
// One pass of knGaussianBlur over bnd=1 cells; when zero_border, the border
// ring of dst is written with zeros.  wtab holds exp weights by squared
// distance (host-computed, as the reference's float(exp(double))).
void launch_gauss_pass(const float *src, float *dst, Dims4 d, int nc, int s,
                       const float *wtab, int zero_border, cudaStream_t st);
// Separable variant (blurType 2): two axes of the 4x1D stencil with
// in-bounds normalisation, x then y (zt = 0, every cell) or z then t (zt = 1,
// interior cells; border_mode 1 zeros the one-cell ring, 2 leaves it alone);
// equal to the reference's blur up to rounding.
void launch_gauss_sep_pair(const float *src, float *dst, Dims4 d, int nc, int zt, int s,
                           const float *w1d, int border_mode, cudaStream_t st);

// Shared-memory slab versions (flof_stencil.cu) of the blur pass for radius
// 1 and 2 and of the extrapolation sweep; same results bit for bit.
// wsum_dev holds the in-bounds weight sums by clipping pattern
// ((S+1)^2 codes per axis, t-major).
bool gauss_slab_supported(int s, Dims4 d);
void launch_gauss_slab(const float *src, float *dst, Dims4 d, int nc, int s,
                       const float *wtab, const float *wsum_dev, int zero_border,
                       cudaStream_t st);
void launch_expol_slab(const float4 *in, float4 *out, const float *mark, Dims4 d,
                       cudaStream_t st);

// TMA-staged versions (flof_tma.cu) for Vec4 grids: same results bit for
// bit.  They return false when no tensor map can be built (the caller then
// uses the cp.async kernels).  A block whose bounded mbarrier wait runs out
// stores FLOF_DEV_ERR_TMA_TIMEOUT in *err and returns.
constexpr int FLOF_DEV_ERR_TMA_TIMEOUT = 1;
// a tensor-core convolution block whose bounded wait on its MMAs ran out
constexpr int FLOF_DEV_ERR_TC_TIMEOUT = 2;
bool launch_gauss_tma(const float4 *src, float4 *dst, Dims4 d, int s, const float *wtab,
                      const float *wsum_dev, int zero_border, int *err, cudaStream_t st);
// The TMA extrapolation sweep writes only the cells it updates (unmarked
// interior cells), so its output buffer must already hold the input's values
// at every other cell (a copy of the input made once per projection round).
// Which cells those are comes from a packed mask that launch_expol_mask
// builds from the marker once per round: expol_mask_words(d) 16-bit words.
size_t expol_mask_words(Dims4 d);
void launch_expol_mask(const float *mark, uint16_t *mask, Dims4 d, cudaStream_t st);
// The sweep walking t with three output planes' running sums in registers
// (every output adds its 81 taps in the reference's order); false when TMA
// is unavailable (the caller then uses launch_expol_slab).
bool launch_expol_tw(const float4 *in, float4 *out, const uint16_t *mask, Dims4 d, int *err,
                     cudaStream_t st);
// The sweep with its 3^4 box sum formed separably (blurType 2, flof_mg.cu):
// s2 (a Vec4 grid of d's size) receives the 3x3 (x,y) sums, out the 1/81 of
// their 3x3 (z,t) sums at unmarked interior cells.  Equal to the reference's
// 81-term sum up to rounding.
void launch_expol_sep(const float4 *in, float4 *out, float4 *s2, const float *mark, Dims4 d,
                      cudaStream_t s);
// The separable sweep in one TMA pass walking t, with the same sums in the
// same order as launch_expol_sep (equal bits); false when TMA is unavailable.
bool launch_expol_sep_tw(const float4 *in, float4 *out, const uint16_t *mask, Dims4 d, int *err,
                         cudaStream_t st);

// ---- projection correction ------------------------------------------------------
// knProjectCells in two kernels: the normals and the cells that finish
// without a search, then the searches of the others, taken from `queue`
// (project_queue_bytes(d) bytes: the whole box or a t slab of it at a time)
// by whichever lane is free.  `counters` is two unsigned ints, zero on entry.
void launch_project_cells(float4 *dst, const float4 *vel, const float *phiOrg,
                          const float *phiTarget, float *marker, Dims4 d,
                          float threshPhi, int maxIter, void *queue, unsigned int *counters,
                          cudaStream_t s);
size_t project_queue_bytes(Dims4 d);
// one knCvExpolBlur4d sweep fused with the copy: out = unmarked interior ?
// avg81(in) : in
void launch_expol_sweep(const float4 *in, float4 *out, const float *mark,
                        Dims4 d, cudaStream_t s);

// ---- input conditioning and output stage (flof_cond.cu) ---------------------
// repeatFrame4d: slices t0..t1 of the bnd box get phi interpolated at time
// srct; `slice` is scratch of X*Y*Z floats.
void launch_repeat_frame(float *phi, Dims4 d, float srct, int t0, int t1, int bnd, float *slice,
                         cudaStream_t s);
// extrap4dLsSimple steps; tmp holds X*Y*Z*T ints.
void launch_extrap_mark(const float *phi, int *tmp, Dims4 d, int inside, cudaStream_t s);
void launch_extrap_layer(int *tmp, Dims4 d, cudaStream_t s);
void launch_extrap_step(float *phi, int *tmp, Dims4 d, int dd, float direction, cudaStream_t s);
void launch_extrap_remaining(float *phi, const int *tmp, Dims4 d, float value, cudaStream_t s);
// one knSimpleBlurSpecial pass a -> tmp over a 3D (Z > 1) or 2D (Z == 1) grid
void launch_simple_blur_special(const float *a, float *tmp, int X, int Y, int Z, float thresh,
                                int bord, cudaStream_t s);
void launch_join(float *a, const float *b, long long n, cudaStream_t s);
void launch_set_bound3(float *a, int X, int Y, int Z, int nc, float4 v, int w, cudaStream_t s);
void launch_set_bound_neumann3(float *a, int X, int Y, int Z, int nc, int w, cudaStream_t s);
// knLoadPlaceGridIpol / knLoadPlaceGridRescale
void launch_place_slice(float *phi, Dims4 d, int slice, const float *src, const int sdims[3],
                        const float sf[3], const float off[3], float wc, cudaStream_t s);
void launch_rescale_slices(float *phi, Dims4 d, const float *w, cudaStream_t s);
// a += v over the bnd = 1 box of a 3D grid
void launch_add_inner3(float *a, int X, int Y, int Z, float v, cudaStream_t s);

// ---- learned warm start network (flof_net.cu) -----------------------------------
// Channels-last tensors over cubic 4D grids; 3^4 (pad 1) or 1^4 convolutions.
void net_conv_fwd(const float *in, const float *w, const float *b, float *out, int rin, int rout,
                  int cin, int cout, int ks, int stride, int relu, cudaStream_t s);
void net_conv_bwd_data(const float *dout, const float *w, float *din, int rin, int rout,
                       int cin, int cout, int ks, int stride, cudaStream_t s);
// dw = weight gradient; work holds net_conv_bwd_weight_work(...) floats
size_t net_conv_bwd_weight_work(int rout, int cin, int cout, int ks);
void net_conv_bwd_weight(const float *in, const float *dout, float *dw, float *work, int rin,
                         int rout, int cin, int cout, int ks, int stride, cudaStream_t s);
void net_relu_bwd(float *dy, const float *y, long long n, cudaStream_t s);
void net_upcat(const float *lo, const float *skip, float *out, int R, int c1, int c2,
               cudaStream_t s);
void net_upcat_bwd(const float *dout, float *dlo, float *dskip, int R, int c1, int c2,
                   cudaStream_t s);
void net_bias_grad(const float *d, float *db, long long V, int C, cudaStream_t s);
void net_mse(const float *pred, const float *target, float *dpred, long long n, double *partial,
             unsigned *counter, double *loss, cudaStream_t s);
void net_adam(float *w, float *wq, const float *g, float *m, float *v, long long n, float lr,
              int step, float gscale, cudaStream_t s);
void net_round_bf16(const float *w, float *wq, long long n, cudaStream_t s);
void net_input(const float *i0, const float *i1, float *x, long long V, float scale,
               cudaStream_t s);
void net_add_into(float *a, const float *b, long long n, cudaStream_t s);

// Tensor-core (tcgen05) versions of the 3^4 convolutions (flof_conv_tc.cu).
// The *_ok predicates name the shapes they take; the weights enter as BF16
// copies made by net_weights_tc: WB[tap][ci][co] (input gradient) and
// WT[co][kpad] (forward, rows of net_tc_kpad entries, zero tail).  `work`
// holds net_tc_work(...) floats; a block whose bounded wait runs out stores
// FLOF_DEV_ERR_TC_TIMEOUT in *err.
bool net_tc_fwd_ok(int cin, int cout, int ks);
bool net_tc_bwd_data_ok(int cin, int cout, int ks);
bool net_tc_bwd_weight_ok(int cin, int cout, int ks);
int net_tc_kpad(int cin, int ks);
size_t net_tc_work(int rin, int rout, int cin, int cout, int ks);
void net_weights_tc(const float *wq, uint16_t *wb, uint16_t *wt, int cin, int cout, int ks,
                    cudaStream_t s);
void net_tc_conv_fwd(const float *in, const uint16_t *wt, const float *b, float *out,
                     float *work, int rin, int rout, int cin, int cout, int stride, int relu,
                     int *err, cudaStream_t s);
void net_tc_conv_bwd_data(const float *dout, const uint16_t *wb, float *din, float *work,
                          int rin, int rout, int cin, int cout, int stride, int *err,
                          cudaStream_t s);
// Weight and bias gradient of the 1^4 output layer (16 -> 4 channels) over
// V voxels: dw receives the 64 weight entries then the 4 bias entries; work
// holds net_wgrad_1x1_work() floats.
bool net_wgrad_1x1_ok(int cin, int cout, int ks);
size_t net_wgrad_1x1_work();
void net_wgrad_1x1(const float *in, const float *dout, float *dw, float *work, long long V,
                   cudaStream_t s);
// dw receives 81 cin cout weight-gradient entries followed by the cout bias
// gradients
void net_tc_conv_bwd_weight(const float *in, const float *dout, float *dw, float *work, int rin,
                            int rout, int cin, int cout, int stride, int *err, cudaStream_t s);

}  // namespace flof
