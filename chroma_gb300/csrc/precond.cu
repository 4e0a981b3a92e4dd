// Learned-preconditioner entry points: initialisation, training on the current gauge field,
// application, and the versioned weights file (the network kernels are in cnn.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>

#include "cnn.h"
#include "ctx.h"

namespace gbc {

static Cnn* net_of(gbc_ctx* c) { return static_cast<Cnn*>(c->precond); }

void precond_free(gbc_ctx* c) {
  if (!c || !c->precond) return;
  Cnn* n = net_of(c);
  n->release();
  delete n;
  c->precond = nullptr;
}

void precond_apply(gbc_ctx* c, const Spinor& in, const Spinor& out) {
  Cnn* n = net_of(c);
  if (!n) {
    blas_copy(c->g, out, in, c->stream);
    return;
  }
  cnn_apply_spinor(c, *n, in, out);
}

int precond_layers(gbc_ctx* c) { return c->precond ? net_of(c)->nlayers : 0; }
int precond_channels(gbc_ctx* c, int l, bool out) { return out ? net_of(c)->cout(l) : net_of(c)->cin(l); }

}  // namespace gbc

using namespace gbc;

namespace {

template <class F>
int guard(gbc_ctx* c, F&& f) {
  try {
    return f();
  } catch (const CudaError& e) {
    c->err = std::string(e.where) + ": " + cudaGetErrorString(e.e);
    return GBC_ERR_CUDA;
  } catch (const std::string& s) {
    c->err = s;
    return GBC_ERR_STATE;
  }
}

// |e|^2 over the odd sites of nb canonical host fields
std::vector<double> odd_norms(const gbc_ctx* c, const double* f, int nb) {
  std::vector<double> n(nb, 0.0);
  const long V = c->V;
  for (int b = 0; b < nb; ++b) {
    const double* p = f + (size_t)b * V * 24;
    double s = 0;
    for (long site = 0; site < V; ++site) {
      long r = site;
      int x = r % c->dims[0];
      r /= c->dims[0];
      int y = r % c->dims[1];
      r /= c->dims[1];
      int z = r % c->dims[2];
      int t = (int)(r / c->dims[2]);
      if (((x + y + z + t) & 1) == 0) continue;
      for (int k = 0; k < 24; ++k) s += p[site * 24 + k] * p[site * 24 + k];
    }
    n[b] = s;
  }
  return n;
}

}  // namespace

extern "C" {

int gbc_precond_init(gbc_ctx* c, int hidden, int layers, unsigned long long seed) {
  if (!c || (hidden != 4 && hidden != 12) || layers < 1 || layers > 8) return GBC_ERR_ARGS;
  precond_free(c);
  Cnn* n = new Cnn;
  n->init(hidden, layers, seed);
  c->precond = n;
  return GBC_OK;
}

int gbc_load_precond(gbc_ctx* c, const char* path) {
  if (!c || !path) return GBC_ERR_ARGS;
  Cnn* n = new Cnn;
  int rc = n->load(path);
  if (rc != GBC_OK) {
    delete n;
    c->err = std::string("cannot load network weights from ") + path + " (missing, truncated or checksum mismatch)";
    return rc;
  }
  precond_free(c);
  c->precond = n;
  return GBC_OK;
}

int gbc_precond_save(gbc_ctx* c, const char* path) {
  if (!c || !path || !c->precond) return GBC_ERR_ARGS;
  return net_of(c)->save(path) ? GBC_OK : GBC_ERR_ARGS;
}

// weights as interleaved (re, im) floats, layer after layer, W[l][(d*cout + o)*cin + i]
int gbc_precond_weights(gbc_ctx* c, float* out, int capacity, int* count) {
  if (!c || !c->precond) return GBC_ERR_STATE;
  Cnn* n = net_of(c);
  int total = 0;
  for (auto& w : n->W) total += (int)w.size() * 2;
  if (count) *count = total;
  if (!out) return GBC_OK;
  if (capacity < total) return GBC_ERR_ARGS;
  int k = 0;
  for (auto& w : n->W)
    for (auto& z : w) {
      out[k++] = z.real();
      out[k++] = z.imag();
    }
  return GBC_OK;
}

int gbc_precond_set_weights(gbc_ctx* c, const float* in, int count) {
  if (!c || !c->precond || !in) return GBC_ERR_STATE;
  Cnn* n = net_of(c);
  int total = 0;
  for (auto& w : n->W) total += (int)w.size() * 2;
  if (count != total) return GBC_ERR_ARGS;
  int k = 0;
  for (auto& w : n->W)
    for (auto& z : w) {
      z = std::complex<float>(in[k], in[k + 1]);
      k += 2;
    }
  n->dirty = true;
  return GBC_OK;
}

// out = K(in) for nrhs host canonical fields (odd sites read and written, even sites set to 0)
int gbc_precond_apply(gbc_ctx* c, int nrhs, double* out, const double* in) {
  if (!c || !out || !in || nrhs < 1) return GBC_ERR_ARGS;
  if (!c->precond) return GBC_ERR_PRECOND;
  if (!c->have_gauge) return GBC_ERR_STATE;
  return guard(c, [&]() {
    Cnn& n = *net_of(c);
    ensure_stage(c, nrhs);
    const size_t bytes = (size_t)nrhs * c->V * 24 * sizeof(double);
    GBC_CUDA(cudaMemcpyAsync(c->d_stage[0], in, bytes, cudaMemcpyHostToDevice, c->stream));
    n.ensure(c, nrhs);
    cnn_embed_canon(c, n, nrhs, c->d_stage[0], n.act[0]);
    n.forward(c, nrhs);
    cnn_extract_canon(c, n, nrhs, n.act[n.nlayers], c->d_stage[1]);
    GBC_CUDA(cudaMemcpyAsync(out, c->d_stage[1], bytes, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    return GBC_OK;
  });
}

// loss = sum_b |K(in_b) - target_b|^2 / |target_b|^2 over the odd sites, and its gradient with
// respect to the weights, dL/dRe W + i dL/dIm W, interleaved like gbc_precond_weights
int gbc_precond_loss_grad(gbc_ctx* c, int nb, const double* in, const double* target, double* loss, float* grad,
                          int capacity) {
  if (!c || !in || !target || !loss || nb < 1) return GBC_ERR_ARGS;
  if (!c->precond) return GBC_ERR_PRECOND;
  if (!c->have_gauge) return GBC_ERR_STATE;
  return guard(c, [&]() {
    Cnn& n = *net_of(c);
    ensure_stage(c, nb);
    const size_t bytes = (size_t)nb * c->V * 24 * sizeof(double);
    n.ensure(c, nb);
    std::vector<double> en = odd_norms(c, target, nb);
    double* d_en = nullptr;
    float2* tgt = nullptr;
    GBC_CUDA(cudaMalloc(&d_en, sizeof(double) * nb));
    GBC_CUDA(cudaMalloc(&tgt, sizeof(float2) * (size_t)nb * c->V * 12));
    GBC_CUDA(cudaMemcpyAsync(d_en, en.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, c->stream));
    GBC_CUDA(cudaMemcpyAsync(c->d_stage[0], in, bytes, cudaMemcpyHostToDevice, c->stream));
    GBC_CUDA(cudaMemcpyAsync(c->d_stage[1], target, bytes, cudaMemcpyHostToDevice, c->stream));
    cnn_embed_canon(c, n, nb, c->d_stage[0], n.act[0]);
    cnn_embed_canon(c, n, nb, c->d_stage[1], tgt);
    *loss = n.loss_and_grad(c, nb, tgt, d_en);
    cudaFree(d_en);
    cudaFree(tgt);
    if (grad) {
      std::vector<std::vector<std::complex<float>>> g;
      n.download_grad(c->stream, g);
      int k = 0;
      for (auto& w : g)
        for (auto& z : w) {
          if (k + 2 > capacity) return GBC_ERR_ARGS;
          grad[k++] = z.real();
          grad[k++] = z.imag();
        }
    }
    return GBC_OK;
  });
}

// Adam on minibatches of the nsamples (input, target) pairs, on the current gauge field.
// loss_per_epoch (may be NULL) receives the mean loss of each epoch.
int gbc_precond_train(gbc_ctx* c, int nsamples, const double* in, const double* target, int epochs, int batch,
                      double lr, unsigned long long seed, double* loss_per_epoch) {
  if (!c || !in || !target || nsamples < 1 || epochs < 1 || batch < 1) return GBC_ERR_ARGS;
  if (!c->precond) return GBC_ERR_PRECOND;
  if (!c->have_gauge) return GBC_ERR_STATE;
  return guard(c, [&]() {
    Cnn& n = *net_of(c);
    batch = std::min(batch, nsamples);
    const size_t per = (size_t)c->V * 24;
    ensure_stage(c, batch);
    n.ensure(c, batch);
    std::vector<double> en = odd_norms(c, target, nsamples);
    double* d_en = nullptr;
    float2* tgt = nullptr;
    GBC_CUDA(cudaMalloc(&d_en, sizeof(double) * batch));
    GBC_CUDA(cudaMalloc(&tgt, sizeof(float2) * (size_t)batch * c->V * 12));
    std::vector<int> order(nsamples);
    std::iota(order.begin(), order.end(), 0);
    std::mt19937_64 rng(seed);
    std::vector<double> hin(per * batch), htg(per * batch), hen(batch);
    for (int ep = 0; ep < epochs; ++ep) {
      std::shuffle(order.begin(), order.end(), rng);
      double tot = 0;
      for (int s0 = 0; s0 + batch <= nsamples; s0 += batch) {
        for (int b = 0; b < batch; ++b) {
          const int q = order[s0 + b];
          std::memcpy(&hin[per * b], in + per * q, per * sizeof(double));
          std::memcpy(&htg[per * b], target + per * q, per * sizeof(double));
          hen[b] = en[q];
        }
        GBC_CUDA(cudaMemcpyAsync(c->d_stage[0], hin.data(), per * batch * sizeof(double), cudaMemcpyHostToDevice,
                                 c->stream));
        GBC_CUDA(cudaMemcpyAsync(c->d_stage[1], htg.data(), per * batch * sizeof(double), cudaMemcpyHostToDevice,
                                 c->stream));
        GBC_CUDA(cudaMemcpyAsync(d_en, hen.data(), sizeof(double) * batch, cudaMemcpyHostToDevice, c->stream));
        n.upload(c->stream);
        cnn_embed_canon(c, n, batch, c->d_stage[0], n.act[0]);
        cnn_embed_canon(c, n, batch, c->d_stage[1], tgt);
        tot += n.loss_and_grad(c, batch, tgt, d_en);
        std::vector<std::vector<std::complex<float>>> g;
        n.download_grad(c->stream, g);
        for (auto& w : g)
          for (auto& z : w) z /= (float)batch;
        n.adam(g, lr);
      }
      if (loss_per_epoch) loss_per_epoch[ep] = tot / (nsamples / batch * batch);
    }
    n.upload(c->stream);
    cudaFree(d_en);
    cudaFree(tgt);
    return GBC_OK;
  });
}

}  // extern "C"
