// flof_model.cu -- the learned warm start: a 4D convolutional encoder-decoder
// (three levels, 16/32/64 channels) that maps the two coarsest-level inputs
// of the multiscale solve to that level's deformation.  The multiscale
// driver uses its prediction as the coarsest level's starting velocity
// (opticalFlowMultiscaleTemplate starts it at zero, optflow4d.cpp:936-1173);
// the plain PCG then refines every level as usual and the error metric
// decides: a prediction that leaves the coarse error above the zero start
// is dropped.  The network is trained on the GPU with the kernels of
// flof_net.cu (forward, input and weight gradients, Adam).
//
// Architecture at coarse extent R (a multiple of 4), channels-last:
//   E1 conv3 2->16 relu (R) | D1 conv3/2 16->32 relu (R/2) | E2 conv3 32->32 relu
//   D2 conv3/2 32->64 relu (R/4) | B conv3 64->64 relu
//   U2 [up(B), E2] conv3 96->32 relu (R/2) | U1 [up(U2), E1] conv3 48->16 relu (R)
//   O conv1 16->4 (the velocity, in coarse cells)
// Inputs are the coarse i0, i1 times INPUT_SCALE (the solver's lsFactor
// undone: SDF values in cells).
#include <algorithm>
#include <random>

#include "flof_internal.h"

using namespace flof;
using namespace fh;

namespace {

constexpr float INPUT_SCALE = -200.f;  // 1 / lsFactor (scenes/flof.py:319)

struct LayerDef {
  int cin, cout, ks, stride, relu, rin_div, rout_div;  // extents are R / div
};
// E1, D1, E2, D2, B, U2, U1, O
const LayerDef LAYERS[8] = {
    {2, 16, 3, 1, 1, 1, 1},  {16, 32, 3, 2, 1, 1, 2}, {32, 32, 3, 1, 1, 2, 2},
    {32, 64, 3, 2, 1, 2, 4}, {64, 64, 3, 1, 1, 4, 4}, {96, 32, 3, 1, 1, 2, 2},
    {48, 16, 3, 1, 1, 1, 1}, {16, 4, 1, 1, 0, 1, 1}};

}  // namespace

struct flof_model {
  flof_ctx *ctx = nullptr;
  int R = 16;
  long long nparams = 0;
  long long woff[8], boff[8], wsize[8];
  float *w = nullptr, *wq = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  float *scratch = nullptr;  // one layer's weight gradient
  float *work = nullptr;     // split-reduction slices of a convolution
  // BF16 weight copies of the tensor-core convolutions: WB (the weights'
  // own order) at woff, WT (transposed, rows of kpad) at wtoff
  uint16_t *wb = nullptr, *wt = nullptr;
  long long wtoff[8];
  int step = 0;
  // activations and their gradients
  float *x = nullptr, *a[7] = {}, *c5 = nullptr, *c6 = nullptr, *out = nullptr;
  float *da[7] = {}, *dc5 = nullptr, *dc6 = nullptr, *dout = nullptr, *tmp = nullptr;
  double *dloss = nullptr;  // device loss accumulator
  double *part = nullptr;
  unsigned *cnt = nullptr;
  double *hloss = nullptr;  // pinned
  std::vector<void *> allocs;

  long long V(int div) const {
    const long long r = R / div;
    return r * r * r * r;
  }
  float *alloc(size_t n) {
    void *p = nullptr;
    CK(cudaMalloc(&p, n * sizeof(float) > 0 ? n * sizeof(float) : 16));
    allocs.push_back(p);
    return (float *)p;
  }
};

namespace {

cudaStream_t S(flof_model *m) { return m->ctx->stream; }
int *E(flof_model *m) { return m->ctx->dev_err; }

// the BF16 weight copies follow every change of the working weights
void refresh_tc_weights(flof_model *m) {
  for (int l = 0; l < 8; ++l) {
    const LayerDef &L = LAYERS[l];
    net_weights_tc(m->wq + m->woff[l], m->wb + m->woff[l], m->wt + m->wtoff[l], L.cin, L.cout,
                   L.ks, S(m));
  }
}

void forward(flof_model *m, const float *i0, const float *i1, float *out) {
  const int R = m->R;
  cudaStream_t s = S(m);
  net_input(i0, i1, m->x, m->V(1), INPUT_SCALE, s);
  auto conv = [&](int l, const float *in, float *o) {
    const LayerDef &L = LAYERS[l];
    if (net_tc_fwd_ok(L.cin, L.cout, L.ks))
      net_tc_conv_fwd(in, m->wt + m->wtoff[l], m->wq + m->boff[l], o, m->work, R / L.rin_div,
                      R / L.rout_div, L.cin, L.cout, L.stride, L.relu, E(m), s);
    else
      net_conv_fwd(in, m->wq + m->woff[l], m->wq + m->boff[l], o, R / L.rin_div,
                   R / L.rout_div, L.cin, L.cout, L.ks, L.stride, L.relu, s);
  };
  conv(0, m->x, m->a[0]);
  conv(1, m->a[0], m->a[1]);
  conv(2, m->a[1], m->a[2]);
  conv(3, m->a[2], m->a[3]);
  conv(4, m->a[3], m->a[4]);
  net_upcat(m->a[4], m->a[2], m->c5, R / 2, 64, 32, s);
  conv(5, m->c5, m->a[5]);
  net_upcat(m->a[5], m->a[0], m->c6, R, 32, 16, s);
  conv(6, m->c6, m->a[6]);
  conv(7, m->a[6], out);
}

// gradient of layer l's weights and bias into the accumulators, and (when din
// is given) of its input
void layer_bwd(flof_model *m, int l, const float *in, const float *dy, float *din) {
  const LayerDef &L = LAYERS[l];
  const int R = m->R;
  cudaStream_t s = S(m);
  const int rin = R / L.rin_div, rout = R / L.rout_div;
  if (net_wgrad_1x1_ok(L.cin, L.cout, L.ks)) {
    net_wgrad_1x1(in, dy, m->scratch, m->work, (long long)rout * rout * rout * rout, s);
    net_add_into(m->grad + m->woff[l], m->scratch, m->wsize[l] + L.cout, s);
  } else if (net_tc_bwd_weight_ok(L.cin, L.cout, L.ks)) {
    // weights and bias in one pass; the bias follows the weights in grad
    net_tc_conv_bwd_weight(in, dy, m->scratch, m->work, rin, rout, L.cin, L.cout, L.stride,
                           E(m), s);
    net_add_into(m->grad + m->woff[l], m->scratch, m->wsize[l] + L.cout, s);
  } else {
    net_conv_bwd_weight(in, dy, m->scratch, m->work, rin, rout, L.cin, L.cout, L.ks, L.stride,
                        s);
    net_add_into(m->grad + m->woff[l], m->scratch, m->wsize[l], s);
    net_bias_grad(dy, m->scratch, (long long)rout * rout * rout * rout, L.cout, s);
    net_add_into(m->grad + m->boff[l], m->scratch, L.cout, s);
  }
  if (!din) return;
  if (net_tc_bwd_data_ok(L.cin, L.cout, L.ks))
    net_tc_conv_bwd_data(dy, m->wb + m->woff[l], din, m->work, rin, rout, L.cin, L.cout,
                         L.stride, E(m), s);
  else
    net_conv_bwd_data(dy, m->wq + m->woff[l], din, rin, rout, L.cin, L.cout, L.ks, L.stride, s);
}

// loss of one sample, gradients added to m->grad
void backward(flof_model *m, const float *target) {
  const int R = m->R;
  cudaStream_t s = S(m);
  const long long n = m->V(1) * 4;
  net_mse(m->out, target, m->dout, n, m->part, m->cnt, m->dloss, s);
  layer_bwd(m, 7, m->a[6], m->dout, m->da[6]);
  net_relu_bwd(m->da[6], m->a[6], m->V(1) * 16, s);
  layer_bwd(m, 6, m->c6, m->da[6], m->dc6);
  CK(cudaMemsetAsync(m->da[0], 0, m->V(1) * 16 * sizeof(float), s));
  net_upcat_bwd(m->dc6, m->da[5], m->da[0], R, 32, 16, s);
  net_relu_bwd(m->da[5], m->a[5], m->V(2) * 32, s);
  layer_bwd(m, 5, m->c5, m->da[5], m->dc5);
  CK(cudaMemsetAsync(m->da[2], 0, m->V(2) * 32 * sizeof(float), s));
  net_upcat_bwd(m->dc5, m->da[4], m->da[2], R / 2, 64, 32, s);
  net_relu_bwd(m->da[4], m->a[4], m->V(4) * 64, s);
  layer_bwd(m, 4, m->a[3], m->da[4], m->da[3]);
  net_relu_bwd(m->da[3], m->a[3], m->V(4) * 64, s);
  layer_bwd(m, 3, m->a[2], m->da[3], m->tmp);
  net_add_into(m->da[2], m->tmp, m->V(2) * 32, s);
  net_relu_bwd(m->da[2], m->a[2], m->V(2) * 32, s);
  layer_bwd(m, 2, m->a[1], m->da[2], m->da[1]);
  net_relu_bwd(m->da[1], m->a[1], m->V(2) * 32, s);
  layer_bwd(m, 1, m->a[0], m->da[1], m->tmp);
  net_add_into(m->da[0], m->tmp, m->V(1) * 16, s);
  net_relu_bwd(m->da[0], m->a[0], m->V(1) * 16, s);
  layer_bwd(m, 0, m->x, m->da[0], nullptr);
}

void need_model_grid(flof_model *m, const flof_grid *g, int elem, const char *name) {
  need_grid(g, name);
  need_elem(g, elem, name);
  need(g->dims[0] == m->R && g->dims[1] == m->R && g->dims[2] == m->R && g->dims[3] == m->R,
       std::string(name) + " must be a " + std::to_string(m->R) + "^4 grid");
}

}  // namespace

namespace fh {
// The warm start's prediction for the coarsest level (used by the driver).
void model_predict_raw(flof_model *m, const float *i0, const float *i1, float4 *vel) {
  forward(m, i0, i1, (float *)vel);
  CK(cudaGetLastError());
}
int model_res(const flof_model *m) { return m->R; }
void model_orphan(flof_model *m) {
  for (void *p : m->allocs) cudaFree(p);
  m->allocs.clear();
  if (m->hloss) cudaFreeHost(m->hloss);
  m->hloss = nullptr;
  m->ctx = nullptr;
}
}  // namespace fh

// ---- C ABI --------------------------------------------------------------------

FLOF_API int flof_model_create(flof_ctx *c, int res, flof_model **out) {
  flof_model *m = nullptr;
  const int st = guarded([&] {
    need(c != nullptr && out != nullptr, "NULL argument");
    need(res >= 4 && res % 4 == 0 && res <= 64, "res must be a multiple of 4 in [4, 64]");
    set_ctx_device(c);
    m = new flof_model();
    m->ctx = c;
    m->R = res;
    long long off = 0, maxw = 0;
    for (int l = 0; l < 8; ++l) {
      const LayerDef &L = LAYERS[l];
      const long long taps = L.ks == 3 ? 81 : 1;
      m->wsize[l] = taps * L.cin * L.cout;
      m->woff[l] = off;
      off += m->wsize[l];
      m->boff[l] = off;
      off += L.cout;
      maxw = m->wsize[l] > maxw ? m->wsize[l] : maxw;
    }
    m->nparams = off;
    m->w = m->alloc(off);
    m->wq = m->alloc(off);
    m->grad = m->alloc(off);
    m->m = m->alloc(off);
    m->v = m->alloc(off);
    m->scratch = m->alloc(maxw + 128);  // a weight gradient and its bias gradient
    size_t maxwork = 0;
    long long wtsize = 0;
    for (int l = 0; l < 8; ++l) {
      const LayerDef &L = LAYERS[l];
      const size_t wk = net_conv_bwd_weight_work(res / L.rout_div, L.cin, L.cout, L.ks);
      const size_t wt = net_tc_work(res / L.rin_div, res / L.rout_div, L.cin, L.cout, L.ks);
      maxwork = std::max(maxwork, std::max(std::max(wk, wt), net_wgrad_1x1_work()));
      m->wtoff[l] = wtsize;
      wtsize += (long long)L.cout * net_tc_kpad(L.cin, L.ks);
    }
    m->work = m->alloc(maxwork);
    m->wb = (uint16_t *)m->alloc((off + 1) / 2);
    m->wt = (uint16_t *)m->alloc((wtsize + 1) / 2);
    CK(cudaMemsetAsync(m->wt, 0, wtsize * sizeof(uint16_t), c->stream));
    const long long V1 = m->V(1), V2 = m->V(2), V4 = m->V(4);
    m->x = m->alloc(V1 * 2);
    const long long asz[7] = {V1 * 16, V2 * 32, V2 * 32, V4 * 64, V4 * 64, V2 * 32, V1 * 16};
    for (int q = 0; q < 7; ++q) {
      m->a[q] = m->alloc(asz[q]);
      m->da[q] = m->alloc(asz[q]);
    }
    m->c5 = m->alloc(V2 * 96);
    m->dc5 = m->alloc(V2 * 96);
    m->c6 = m->alloc(V1 * 48);
    m->dc6 = m->alloc(V1 * 48);
    m->out = m->alloc(V1 * 4);
    m->dout = m->alloc(V1 * 4);
    m->tmp = m->alloc(V1 * 16);
    m->dloss = (double *)m->alloc(2);
    m->part = (double *)m->alloc(2 * 4096);
    m->cnt = (unsigned *)m->alloc(1);
    CK(cudaMemsetAsync(m->cnt, 0, sizeof(unsigned), c->stream));
    CK(cudaMallocHost(&m->hloss, sizeof(double)));
    CK(cudaMemsetAsync(m->m, 0, off * sizeof(float), c->stream));
    CK(cudaMemsetAsync(m->v, 0, off * sizeof(float), c->stream));
    CK(cudaMemsetAsync(m->w, 0, off * sizeof(float), c->stream));
    CK(cudaMemsetAsync(m->wq, 0, off * sizeof(float), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->models.insert(m);
    *out = m;
  });
  if (st != FLOF_OK && m) {
    for (void *p : m->allocs) cudaFree(p);
    if (m->hloss) cudaFreeHost(m->hloss);
    delete m;
  }
  return st;
}

FLOF_API int flof_model_destroy(flof_model *m) {
  if (!m) return FLOF_OK;
  if (m->ctx) {
    cudaSetDevice(m->ctx->device);
    cudaStreamSynchronize(m->ctx->stream);
    if (m->ctx->model == m) m->ctx->model = nullptr;
    m->ctx->models.erase(m);
    model_orphan(m);
  }
  delete m;
  cudaGetLastError();
  return FLOF_OK;
}

FLOF_API int flof_model_num_params(const flof_model *m, long long *n) {
  return guarded_host([&] {
    need(m != nullptr && n != nullptr, "NULL argument");
    *n = m->nparams;
  });
}

// He-normal weights (std sqrt(2 / fan_in)), zero biases, from a seeded host RNG
FLOF_API int flof_model_init(flof_model *m, unsigned long long seed) {
  return guarded([&] {
    need(m != nullptr, "model is NULL");
    need(m->ctx != nullptr, "the model's context was destroyed");
    std::vector<float> h(m->nparams, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < 8; ++l) {
      const LayerDef &L = LAYERS[l];
      const double fan_in = (double)(L.ks == 3 ? 81 : 1) * L.cin;
      std::normal_distribution<double> nd(0.0, sqrt((l == 7 ? 1.0 : 2.0) / fan_in));
      for (long long q = 0; q < m->wsize[l]; ++q) h[m->woff[l] + q] = (float)nd(rng);
    }
    set_ctx_device(m->ctx);
    CK(cudaMemcpyAsync(m->w, h.data(), m->nparams * sizeof(float), cudaMemcpyHostToDevice,
                       S(m)));
    net_round_bf16(m->w, m->wq, m->nparams, S(m));
    refresh_tc_weights(m);
    CK(cudaMemsetAsync(m->m, 0, m->nparams * sizeof(float), S(m)));
    CK(cudaMemsetAsync(m->v, 0, m->nparams * sizeof(float), S(m)));
    m->step = 0;
    CK(cudaStreamSynchronize(S(m)));
  });
}

FLOF_API int flof_model_get_params(const flof_model *m, float *host) {
  return guarded([&] {
    need(m != nullptr && host != nullptr, "NULL argument");
    need(m->ctx != nullptr, "the model's context was destroyed");
    set_ctx_device(m->ctx);
    CK(cudaMemcpyAsync(host, m->w, m->nparams * sizeof(float), cudaMemcpyDeviceToHost,
                       m->ctx->stream));
    CK(cudaStreamSynchronize(m->ctx->stream));
  });
}

FLOF_API int flof_model_set_params(flof_model *m, const float *host) {
  return guarded([&] {
    need(m != nullptr && host != nullptr, "NULL argument");
    need(m->ctx != nullptr, "the model's context was destroyed");
    set_ctx_device(m->ctx);
    CK(cudaMemcpyAsync(m->w, host, m->nparams * sizeof(float), cudaMemcpyHostToDevice, S(m)));
    net_round_bf16(m->w, m->wq, m->nparams, S(m));
    refresh_tc_weights(m);
    CK(cudaStreamSynchronize(S(m)));
  });
}

FLOF_API int flof_model_predict(flof_model *m, const flof_grid *i0, const flof_grid *i1,
                                flof_grid *vel) {
  return guarded([&] {
    need(m != nullptr, "model is NULL");
    need(m->ctx != nullptr, "the model's context was destroyed");
    need_model_grid(m, i0, FLOF_REAL, "i0");
    need_model_grid(m, i1, FLOF_REAL, "i1");
    need_model_grid(m, vel, FLOF_VEC4, "vel");
    set_ctx_device(m->ctx);
    forward(m, i0->f(), i1->f(), vel->f());
    CK(cudaGetLastError());  // a refused launch of any network kernel
    CK(cudaStreamSynchronize(S(m)));
    check_device_errors(m->ctx);
  });
}

// Loss of one sample and (grad_host nullable) its gradient w.r.t. the
// parameters, as the network sees them (the BF16-rounded weights).
FLOF_API int flof_model_loss_grad(flof_model *m, const flof_grid *i0, const flof_grid *i1,
                                  const flof_grid *target, double *loss, float *grad_host) {
  return guarded([&] {
    need(m != nullptr, "model is NULL");
    need(m->ctx != nullptr, "the model's context was destroyed");
    need_model_grid(m, i0, FLOF_REAL, "i0");
    need_model_grid(m, i1, FLOF_REAL, "i1");
    need_model_grid(m, target, FLOF_VEC4, "target");
    set_ctx_device(m->ctx);
    CK(cudaMemsetAsync(m->grad, 0, m->nparams * sizeof(float), S(m)));
    CK(cudaMemsetAsync(m->dloss, 0, sizeof(double), S(m)));
    forward(m, i0->f(), i1->f(), m->out);
    backward(m, target->f());
    CK(cudaMemcpyAsync(m->hloss, m->dloss, sizeof(double), cudaMemcpyDeviceToHost, S(m)));
    if (grad_host)
      CK(cudaMemcpyAsync(grad_host, m->grad, m->nparams * sizeof(float), cudaMemcpyDeviceToHost,
                         S(m)));
    CK(cudaGetLastError());  // a refused launch of any network kernel
    CK(cudaStreamSynchronize(S(m)));
    check_device_errors(m->ctx);
    if (loss) *loss = *m->hloss;
  });
}

// One Adam step on the mean loss of n samples; loss (nullable) receives it.
FLOF_API int flof_model_train_step(flof_model *m, int n, const flof_grid *const *i0s,
                                   const flof_grid *const *i1s,
                                   const flof_grid *const *targets, float lr, double *loss) {
  return guarded([&] {
    need(m != nullptr, "model is NULL");
    need(m->ctx != nullptr, "the model's context was destroyed");
    need(n > 0 && i0s && i1s && targets, "empty batch");
    for (int q = 0; q < n; ++q) {
      need_model_grid(m, i0s[q], FLOF_REAL, "i0");
      need_model_grid(m, i1s[q], FLOF_REAL, "i1");
      need_model_grid(m, targets[q], FLOF_VEC4, "target");
    }
    need(lr > 0.f, "learning rate must be positive");
    set_ctx_device(m->ctx);
    CK(cudaMemsetAsync(m->grad, 0, m->nparams * sizeof(float), S(m)));
    CK(cudaMemsetAsync(m->dloss, 0, sizeof(double), S(m)));
    for (int q = 0; q < n; ++q) {
      forward(m, i0s[q]->f(), i1s[q]->f(), m->out);
      backward(m, targets[q]->f());
    }
    m->step++;
    net_adam(m->w, m->wq, m->grad, m->m, m->v, m->nparams, lr, m->step, 1.f / n, S(m));
    refresh_tc_weights(m);
    CK(cudaMemcpyAsync(m->hloss, m->dloss, sizeof(double), cudaMemcpyDeviceToHost, S(m)));
    CK(cudaGetLastError());  // a refused launch of any network kernel
    CK(cudaStreamSynchronize(S(m)));
    check_device_errors(m->ctx);
    if (loss) *loss = *m->hloss / n;
  });
}

FLOF_API int flof_ctx_set_model(flof_ctx *c, flof_model *m) {
  return guarded_host([&] {
    need(c != nullptr, "ctx is NULL");
    need(m == nullptr || m->ctx == c, "the model belongs to another context");
    c->model = m;
  });
}
