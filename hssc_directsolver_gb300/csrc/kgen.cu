// Kernel-matrix generation (Common/Kernel_Eval.m:29-96, custom slot :75-79).
//
// FP64 entries are formed without FMA contraction (explicit _rn intrinsics) so
// that the squared distance and the double-layer numerator round exactly as
// the reference's element-wise MATLAB expressions do.
#include "kgen.cuh"

#include <cmath>

namespace hss {

double modulation(double alpha, double x0, double y0, double isig, double px, double py) {
  if (alpha == 0.0) return 1.0;
  const double d1 = px - x0, d2 = py - y0;
  double s = d1 * d1 + d2 * d2;
  if (isig != 1.0) s = isig * s;
  return 1.0 + alpha * std::exp(-s);
}

void PointTable::upload(const std::vector<double>& hx, const std::vector<double>& hy,
                        const std::vector<double>& hnx, const std::vector<double>& hny,
                        const std::vector<double>& hw, const std::vector<double>& hkap,
                        const hss_kernel_params& kp, cudaStream_t s) {
  const size_t n = hx.size();
  std::vector<double> b(n), c(n);
  for (size_t i = 0; i < n; ++i) {
    b[i] = modulation(kp.b_alpha, kp.b_x0, kp.b_y0, kp.b_isig, hx[i], hy[i]);
    c[i] = modulation(kp.c_alpha, kp.c_x0, kp.c_y0, kp.c_isig, hx[i], hy[i]);
  }
  x.upload(hx, s); y.upload(hy, s); nx.upload(hnx, s); ny.upload(hny, s);
  w.upload(hw, s); kap.upload(hkap, s); bval.upload(b, s); cval.upload(c, s);
  count = (int)n;
  HSS_CUDA(cudaStreamSynchronize(s));
}

void PointTable::reserve(size_t n) {
  x.alloc(n); y.alloc(n); nx.alloc(n); ny.alloc(n); w.alloc(n); kap.alloc(n); bval.alloc(n); cval.alloc(n);
  count = (int)n;
}

void PointTable::upload_range(size_t first, size_t n, const double* hx, const double* hy, const double* hnx,
                              const double* hny, const double* hw, const double* hkap, const hss_kernel_params& kp,
                              cudaStream_t s) {
  HSS_REQUIRE(first + n <= (size_t)count, HSS_ERR_ARG, "point range outside the table");
  if (n == 0) return;
  std::vector<double> b(n), c(n);
  for (size_t i = 0; i < n; ++i) {
    b[i] = modulation(kp.b_alpha, kp.b_x0, kp.b_y0, kp.b_isig, hx[i], hy[i]);
    c[i] = modulation(kp.c_alpha, kp.c_x0, kp.c_y0, kp.c_isig, hx[i], hy[i]);
  }
  const size_t bytes = n * sizeof(double);
  const double* src[8] = {hx, hy, hnx, hny, hw, hkap, b.data(), c.data()};
  double* dst[8] = {x.p, y.p, nx.p, ny.p, w.p, kap.p, bval.p, cval.p};
  for (int a = 0; a < 8; ++a)
    HSS_CUDA(cudaMemcpyAsync(dst[a] + first, src[a], bytes, cudaMemcpyHostToDevice, s));
  HSS_CUDA(cudaStreamSynchronize(s));
}

__device__ __forceinline__ double kernel_entry(const KernelDev& k, const PointView& P, int t, int s) {
  const double dx = __dadd_rn(P.x[t], -P.x[s]);
  const double dy = __dadd_rn(P.y[t], -P.y[s]);
  const double den = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  const bool z = (den == 0.0);
  if (k.flag == HSS_SL_L_2D) {
    double v = __dmul_rn(k.h2half, P.bval[t]);
    v = __dmul_rn(v, log(z ? 1.0 : den));
    v = __dmul_rn(v, P.cval[s]);
    return __dadd_rn(v, z ? 1.0 : 0.0);
  }
  // double layer: w/(2 pi) n_y.(x-y)/|x-y|^2 ; diagonal -1/2 - w kappa/(4 pi)
  const double w = P.w[s];
  if (z) return __dadd_rn(-0.5, -__dmul_rn(__dmul_rn(w, P.kap[s]), 0.07957747154594767));
  const double num = __dadd_rn(__dmul_rn(P.nx[s], dx), __dmul_rn(P.ny[s], dy));
  return __ddiv_rn(__dmul_rn(__dmul_rn(w, 0.15915494309189535), num), den);
}

template <typename R>
__global__ void __launch_bounds__(256) k_kgen(const KgenP<R>* __restrict__ D, PointView P, KernelDev k) {
  const KgenP<R> d = D[blockIdx.y];
  const long long tot = (long long)d.m * d.n;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    int i, j;
    size_t o;
    if (!d.trans) { i = (int)(e % d.m); j = (int)(e / d.m); o = i + (size_t)j * d.ld; }
    else { j = (int)(e % d.n); i = (int)(e / d.n); o = j + (size_t)i * d.ld; }
    d.out[o] = (R)kernel_entry(k, P, d.ti[i], d.si[j]);
  }
}

template <typename R>
void kgen_batched(const KgenP<R>* dP, int batch, long long maxEntries, const PointView& pts,
                  const KernelDev& k, cudaStream_t s) {
  if (batch <= 0 || maxEntries <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "kgen batch too large");
  const int gx = std::max(1, std::min(ceil_div(maxEntries, 256), 2048));
  k_kgen<R><<<dim3(gx, batch), 256, 0, s>>>(dP, pts, k);
  check_launch("k_kgen");
}

template void kgen_batched<double>(const KgenP<double>*, int, long long, const PointView&,
                                   const KernelDev&, cudaStream_t);
template void kgen_batched<float>(const KgenP<float>*, int, long long, const PointView&,
                                  const KernelDev&, cudaStream_t);

}  // namespace hss
