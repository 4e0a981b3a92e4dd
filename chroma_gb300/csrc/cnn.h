// Learned preconditioner model (cnn.cu): weights on the host (FP32 master copy, Adam state),
// BF16 real-form weights and activations on the device.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <complex>
#include <string>
#include <vector>

#include "gbc_kernels.h"

struct gbc_ctx;

namespace gbc {

struct Cnn {
  int hidden = 12;
  int nlayers = 4;
  // W[l][(d * cout + o) * cin + i], d = 0 self, 1 + 2 mu (+mu hop), 2 + 2 mu (-mu hop)
  std::vector<std::vector<std::complex<float>>> W;
  std::vector<std::vector<float>> m1, m2;  // Adam moments (re, im interleaved)
  long step = 0;
  bool dirty = true;

  __nv_bfloat16* dW[8] = {nullptr};     // real form [npad(cout)][kpad(cin)]
  __nv_bfloat16* dWadj[8] = {nullptr};  // input-gradient form
  float* dG[8] = {nullptr};             // real-form weight gradients
  std::vector<float2*> act;             // activations per layer boundary, [batch][V][ch][3]
  float2* delta[2] = {nullptr, nullptr};
  int act_batch = 0;
  float2* links = nullptr;              // FP32 links, even-odd order [V][4][9]
  long links_version = -1;

  int cin(int l) const;
  int cout(int l) const;
  void init(int hidden, int layers, unsigned long long seed);
  void upload(cudaStream_t s);
  void ensure(gbc_ctx* c, int batch);
  void forward(gbc_ctx* c, int batch);
  // forward + backward of sum_b |y_b - e_b|^2 / |e_b|^2 (odd sites); gradients left in dG
  double loss_and_grad(gbc_ctx* c, int batch, const float2* target, const double* enorm2);
  void download_grad(cudaStream_t s, std::vector<std::vector<std::complex<float>>>& grad);
  void adam(const std::vector<std::vector<std::complex<float>>>& grad, double lr);
  bool save(const std::string& path) const;
  int load(const std::string& path);
  void release();
};

void cnn_apply_spinor(gbc_ctx* c, Cnn& net, const Spinor& in, const Spinor& out);
void cnn_embed_canon(gbc_ctx* c, Cnn& net, int batch, const double* canon_dev, float2* act);
void cnn_extract_canon(gbc_ctx* c, Cnn& net, int batch, const float2* act, double* canon_dev);

}  // namespace gbc
