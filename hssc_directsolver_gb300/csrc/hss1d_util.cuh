// Host helpers shared by the HSS1D translation units (hss1d.cu: compress, invert and the
// solve plans; hss1d_algebra.cu: transpose, scalar multiple, dense export, rectangular
// compress, sum and the low-rank compress).
#pragma once

#include <vector>

#include "hss1d.h"

namespace hss {

constexpr double RADIUS_REL = 1.75;  // HSS1D_compress_nsym.m:51
constexpr int NPROXY = 50;           // HSS1D_compress_nsym.m:52

// Proxy points of a box whose circumscribing circle has radius R, HSS1D_compress_nsym.m:111-114:
// 50, or for the Helmholtz kernel min(max(50, round(4 kh 1.75 R + 30)), ntot) (four points per
// wavelength on the ring); ntot = the problem's points.
inline int proxy_count(const hss_kernel_params& kp, double R, long long ntot) {
  if (kp.flag != HSS_SL_H_2D) return NPROXY;
  const long long r = std::lround(4.0 * kp.kh * RADIUS_REL * R + 30.0);
  return (int)std::min<long long>(std::max<long long>(NPROXY, r), ntot);
}

template <typename T>
inline T* upload_vec(DevBuf<T>& buf, const std::vector<T>& h, cudaStream_t s) {
  buf.alloc(std::max<size_t>(h.size(), 1));
  if (!h.empty()) HSS_CUDA(cudaMemcpyAsync(buf.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return buf.p;
}

// batched block moves, then a stream sync
void run_moves(const std::vector<MoveP>& mv, cudaStream_t s);
// batched products C = alpha op(A) op(B) + beta C in chunks of 65535, then a stream sync
void run_gemms(const std::vector<GemmP<double>>& P, bool tA, bool tB, double alpha, double beta, cudaStream_t s,
               bool skinny = false, bool df = false);
// LOCAL_get_circum_circle (HSS1D_compress_nsym.m:339-356) on the rows idx of X (6 per point)
void circum_circle(const std::vector<double>& X, const std::vector<int>& idx, double& xc, double& yc, double& R);

}  // namespace hss
