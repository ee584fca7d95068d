// Rank-predictor MLP: hand-written forward, backward and Adam kernels (FP32).
//
// nin -> H -> H -> 1, ReLU hidden layers, sigmoid output, mean-squared-error
// loss on the plain ID's rank fraction k/n.  It replaces the reference's
// hand-fitted rank table (HSS2D/predict_rank.m:5-23) with a network trained on
// the ranks the plain ID itself produces.  Parameters are one flat vector
// [W1 (H x nin), b1, W2 (H x H), b2, W3 (1 x H), b3]; gradients are reduced in
// a fixed order (per-warp shuffles, warps then blocks in index order), so a
// training run is bitwise reproducible.
#include "mlp.h"

#include <cmath>

namespace hss {

static __device__ __forceinline__ float wsum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct MlpView {
  const float *W1, *b1, *W2, *b2, *W3, *b3;
};

__device__ __forceinline__ MlpView mlp_view(const float* p, int nin, int H) {
  MlpView v;
  v.W1 = p;
  v.b1 = v.W1 + H * nin;
  v.W2 = v.b1 + H;
  v.b2 = v.W2 + H * H;
  v.W3 = v.b2 + H;
  v.b3 = v.W3 + H;
  return v;
}

constexpr int MLP_THREADS = 128;

template <int H>
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_forward(const float* __restrict__ params, const float* __restrict__ X,
                                                             float* __restrict__ y, int B, int nin) {
  extern __shared__ float sp[];
  const int np = mlp_nparams(nin, H);
  for (int e = threadIdx.x; e < np; e += blockDim.x) sp[e] = params[e];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const MlpView w = mlp_view(sp, nin, H);
  float x[MLP_NIN_MAX], a1[H];
#pragma unroll
  for (int f = 0; f < MLP_NIN_MAX; ++f) x[f] = (f < nin) ? X[(size_t)i * nin + f] : 0.f;
#pragma unroll
  for (int j = 0; j < H; ++j) {
    float z = w.b1[j];
#pragma unroll
    for (int f = 0; f < MLP_NIN_MAX; ++f)
      if (f < nin) z += w.W1[j * nin + f] * x[f];
    a1[j] = fmaxf(z, 0.f);
  }
  float z3 = w.b3[0];
#pragma unroll
  for (int j = 0; j < H; ++j) {
    float z = w.b2[j];
#pragma unroll
    for (int q = 0; q < H; ++q) z += w.W2[j * H + q] * a1[q];
    z3 += w.W3[j] * fmaxf(z, 0.f);
  }
  y[i] = 1.f / (1.f + expf(-z3));
}

// One sample per thread; per-parameter contributions are summed by warp
// shuffles and written per warp, then per block in warp order.
// part[blockIdx.x * (np + 1) + q]: gradient partials, last entry = sum of squared errors.
template <int H>
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_backward(const float* __restrict__ params, const float* __restrict__ X,
                                                              const float* __restrict__ t, int B, int nin,
                                                              float inv_batch, float* __restrict__ part) {
  extern __shared__ float sm[];
  const int np = mlp_nparams(nin, H);
  float* sp = sm;                   // np
  float* wacc = sm + np;            // (MLP_THREADS/32) x (np + 1)
  for (int e = threadIdx.x; e < np; e += blockDim.x) sp[e] = params[e];
  __syncthreads();
  const MlpView w = mlp_view(sp, nin, H);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < B;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float x[MLP_NIN_MAX], a1[H], a2[H];
#pragma unroll
  for (int f = 0; f < MLP_NIN_MAX; ++f) x[f] = (live && f < nin) ? X[(size_t)i * nin + f] : 0.f;
#pragma unroll
  for (int j = 0; j < H; ++j) {
    float z = w.b1[j];
#pragma unroll
    for (int f = 0; f < MLP_NIN_MAX; ++f)
      if (f < nin) z += w.W1[j * nin + f] * x[f];
    a1[j] = fmaxf(z, 0.f);
  }
  float z3 = w.b3[0];
#pragma unroll
  for (int j = 0; j < H; ++j) {
    float z = w.b2[j];
#pragma unroll
    for (int q = 0; q < H; ++q) z += w.W2[j * H + q] * a1[q];
    a2[j] = fmaxf(z, 0.f);
    z3 += w.W3[j] * a2[j];
  }
  const float y = 1.f / (1.f + expf(-z3));
  const float r = live ? (y - t[i]) : 0.f;
  const float dz3 = r * y * (1.f - y) * inv_batch;
  float* acc = wacc + (size_t)wid * (np + 1);
  const int oW1 = 0, ob1 = H * nin, oW2 = ob1 + H, ob2 = oW2 + H * H, oW3 = ob2 + H, ob3 = oW3 + H;
  // layer 3
#pragma unroll
  for (int j = 0; j < H; ++j) {
    const float v = wsum(dz3 * a2[j]);
    if (lane == 0) acc[oW3 + j] = v;
  }
  {
    const float v = wsum(dz3);
    if (lane == 0) acc[ob3] = v;
  }
  // dz2 (in a2's registers)
#pragma unroll
  for (int j = 0; j < H; ++j) a2[j] = (a2[j] > 0.f) ? dz3 * w.W3[j] : 0.f;
#pragma unroll
  for (int j = 0; j < H; ++j) {
#pragma unroll
    for (int q = 0; q < H; ++q) {
      const float v = wsum(a2[j] * a1[q]);
      if (lane == 0) acc[oW2 + j * H + q] = v;
    }
    const float v = wsum(a2[j]);
    if (lane == 0) acc[ob2 + j] = v;
  }
  // dz1
#pragma unroll
  for (int q = 0; q < H; ++q) {
    float d = 0.f;
#pragma unroll
    for (int j = 0; j < H; ++j) d += a2[j] * w.W2[j * H + q];
    const float dz1 = (a1[q] > 0.f) ? d : 0.f;
#pragma unroll
    for (int f = 0; f < MLP_NIN_MAX; ++f) {
      if (f >= nin) break;
      const float v = wsum(dz1 * x[f]);
      if (lane == 0) acc[oW1 + q * nin + f] = v;
    }
    const float v = wsum(dz1);
    if (lane == 0) acc[ob1 + q] = v;
  }
  {
    const float v = wsum(r * r);
    if (lane == 0) acc[np] = v;
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  for (int q = threadIdx.x; q <= np; q += blockDim.x) {
    float s = 0.f;
    for (int ww = 0; ww < nw; ++ww) s += wacc[(size_t)ww * (np + 1) + q];
    part[(size_t)blockIdx.x * (np + 1) + q] = s;
  }
}

__global__ void k_mlp_reduce(const float* __restrict__ part, int nblk, int np, float* __restrict__ g) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q <= np; q += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < nblk; ++b) s += part[(size_t)b * (np + 1) + q];
    g[q] = s;
  }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int np, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
    const float gq = g[q];
    const float mq = b1 * m[q] + (1.f - b1) * gq;
    const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
    m[q] = mq;
    v[q] = vq;
    p[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
  }
}

// ---------------------------------------------------------------------------
MLP::MLP(int nin_, int H_, unsigned long long seed) : nin(nin_), H(H_) {
  HSS_REQUIRE(nin >= 1 && nin <= MLP_NIN_MAX && H == MLP_H, HSS_ERR_ARG, "MLP: nin in 1..16 and 32 hidden units");
  HSS_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  const int np = mlp_nparams(nin, H);
  // He-uniform from the counter RNG (the oracle draws the same stream)
  std::vector<float> h(np, 0.f);
  int o = 0;
  const int fan[3] = {nin, H, H}, cnt[3] = {H * nin, H * H, H}, nb[3] = {H, H, 1};
  for (int l = 0; l < 3; ++l) {
    const double lim = std::sqrt(6.0 / fan[l]);
    for (int q = 0; q < cnt[l]; ++q) h[o + q] = (float)((host_uniform(seed, 0x4D4C50ULL, (unsigned long long)(o + q)) * 2.0 - 1.0) * lim);
    o += cnt[l] + nb[l];
  }
  p.upload(h, stream);
  m.alloc(np);
  v.alloc(np);
  g.alloc(np + 1);
  m.zero(stream);
  v.zero(stream);
  HSS_CUDA(cudaStreamSynchronize(stream));
}

MLP::~MLP() {
  if (stream) cudaStreamDestroy(stream);
}

double host_uniform(unsigned long long seed, unsigned long long stream, unsigned long long i) {
  unsigned long long z = seed ^ (stream * 0xD1B54A32D192ED03ULL);
  z += (i + 1ULL) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double)(z >> 11) * 0x1.0p-53;
}

static size_t bwd_smem(int np) { return ((size_t)np + (size_t)(MLP_THREADS / 32) * (np + 1)) * sizeof(float); }

void MLP::forward(const float* dX, float* dy, int B, cudaStream_t s) {
  if (B <= 0) return;
  const int np = mlp_nparams(nin, H);
  k_mlp_forward<MLP_H><<<ceil_div(B, MLP_THREADS), MLP_THREADS, np * sizeof(float), s>>>(p.p, dX, dy, B, nin);
  check_launch("k_mlp_forward");
}

float MLP::grad(const float* dX, const float* dt, int B, float inv_batch, cudaStream_t s, bool host_loss) {
  const int np = mlp_nparams(nin, H);
  const int nblk = ceil_div(B, MLP_THREADS);
  part.ensure((size_t)nblk * (np + 1));
  const size_t sm = bwd_smem(np);
  HSS_REQUIRE(sm <= 48 * 1024, HSS_ERR_ARG, "MLP too large for the backward kernel");
  k_mlp_backward<MLP_H><<<nblk, MLP_THREADS, sm, s>>>(p.p, dX, dt, B, nin, inv_batch, part.p);
  check_launch("k_mlp_backward");
  k_mlp_reduce<<<ceil_div(np + 1, 256), 256, 0, s>>>(part.p, nblk, np, g.p);
  check_launch("k_mlp_reduce");
  if (!host_loss) return 0.f;
  float l = 0.f;
  HSS_CUDA(cudaMemcpyAsync(&l, g.p + np, sizeof(float), cudaMemcpyDeviceToHost, s));
  HSS_CUDA(cudaStreamSynchronize(s));
  return 0.5f * l / (float)B;
}

float MLP::train(const float* dX, const float* dt, int B, int epochs, int batch, float lr) {
  const int np = mlp_nparams(nin, H);
  HSS_REQUIRE(B >= 1 && epochs >= 1 && batch >= 1, HSS_ERR_ARG, "bad training arguments");
  for (int e = 0; e < epochs; ++e) {
    for (int s0 = 0; s0 < B; s0 += batch) {
      const int nb = std::min(batch, B - s0);
      grad(dX + (size_t)s0 * nin, dt + s0, nb, 1.f / (float)nb, stream, false);
      ++step;
      const float c1 = 1.f - std::pow(0.9f, (float)step), c2 = 1.f - std::pow(0.999f, (float)step);
      k_adam<<<ceil_div(np, 256), 256, 0, stream>>>(p.p, g.p, m.p, v.p, np, lr, 0.9f, 0.999f, 1e-8f, c1, c2);
      check_launch("k_adam");
    }
  }
  return grad(dX, dt, B, 1.f / (float)B, stream, true);
}

}  // namespace hss
