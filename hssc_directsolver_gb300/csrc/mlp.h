// Rank-predictor MLP (see mlp.cu).
#pragma once

#include "common.cuh"

namespace hss {

constexpr int MLP_NIN_MAX = 16;
constexpr int MLP_H = 32;  // hidden width (compile time: the activations live in registers)

__host__ __device__ inline int mlp_nparams(int nin, int H) { return H * nin + H + H * H + H + H + 1; }

double host_uniform(unsigned long long seed, unsigned long long stream, unsigned long long i);

struct MLP {
  int nin, H;
  int step = 0;
  cudaStream_t stream = nullptr;
  DevBuf<float> p, m, v, g, part;
  MLP(int nin, int H, unsigned long long seed);
  ~MLP();
  void forward(const float* dX, float* dy, int B, cudaStream_t s);
  // gradient of 0.5*mean((y-t)^2) into g (g[np] = sum of squared errors); returns the loss when host_loss
  float grad(const float* dX, const float* dt, int B, float inv_batch, cudaStream_t s, bool host_loss);
  float train(const float* dX, const float* dt, int B, int epochs, int batch, float lr);
};

}  // namespace hss

struct hss_mlp {
  hss::MLP* impl;
};
