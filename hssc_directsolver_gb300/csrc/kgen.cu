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

// Bump_function option 4 (Common/Bump_function.m:53-63): a product of two
// 0.5 tanh(10 (1 - shift - |x_d|)) + 0.5 ramps
static double bump4(double px, double py, double shift) {
  const double D = 1.0 / 0.1;
  const double f1 = 0.5 * std::tanh(D * (-std::fabs(px) + 1.0 - shift)) + 0.5;
  const double f2 = 0.5 * std::tanh(D * (-std::fabs(py) + 1.0 - shift)) + 0.5;
  return f1 * f2;
}

double modulation(const hss_kernel_params& kp, int which, double px, double py) {
  const int kind = which ? kp.c_kind : kp.b_kind;
  if (kind == HSS_MOD_BUMP) return bump4(px, py, 0.0);
  if (kind == HSS_MOD_SQRT_BUMP) return std::sqrt(bump4(px, py, 4.0 * kp.h));
  if (kind == HSS_MOD_GAUSS0) {
    // alpha exp(-isig |p - p0|^2), no constant term
    const double a = which ? kp.c_alpha : kp.b_alpha, x0 = which ? kp.c_x0 : kp.b_x0;
    const double y0 = which ? kp.c_y0 : kp.b_y0, is = which ? kp.c_isig : kp.b_isig;
    const double d1 = px - x0, d2 = py - y0;
    return a * std::exp(-is * (d1 * d1 + d2 * d2));
  }
  HSS_REQUIRE(kind == HSS_MOD_GAUSS, HSS_ERR_ARG, "unknown modulation form");
  return which ? modulation(kp.c_alpha, kp.c_x0, kp.c_y0, kp.c_isig, px, py)
               : modulation(kp.b_alpha, kp.b_x0, kp.b_y0, kp.b_isig, px, py);
}

HelmDev make_helm_dev(const hss_kernel_params& kp) {
  // Kernel_Eval.m:47-49 forms (h^2) kh^2 (0.25 i) and 1 + kh^2 (0.25 i) dr
  HelmDev k;
  k.kh = kp.kh;
  k.s = ((kp.h * kp.h) * (kp.kh * kp.kh)) * 0.25;
  const double q = (kp.kh * kp.kh) * 0.25;
  k.w_re = 1.0 - q * kp.dr_im;
  k.w_im = q * kp.dr_re;
  for (int j = 0; j <= kHankelNodes; ++j) {
    const double sj = j * kHankelStep;
    k.hw[j] = 2.0 * std::exp(-sj * sj);
  }
  return k;
}

void PointTable::upload(const std::vector<double>& hx, const std::vector<double>& hy,
                        const std::vector<double>& hnx, const std::vector<double>& hny,
                        const std::vector<double>& hw, const std::vector<double>& hkap,
                        const hss_kernel_params& kp, cudaStream_t s) {
  const size_t n = hx.size();
  std::vector<double> b(n), c(n);
  for (size_t i = 0; i < n; ++i) {
    b[i] = modulation(kp, 0, hx[i], hy[i]);
    c[i] = modulation(kp, 1, hx[i], hy[i]);
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
    b[i] = modulation(kp, 0, hx[i], hy[i]);
    c[i] = modulation(kp, 1, hx[i], hy[i]);
  }
  const size_t bytes = n * sizeof(double);
  const double* src[8] = {hx, hy, hnx, hny, hw, hkap, b.data(), c.data()};
  double* dst[8] = {x.p, y.p, nx.p, ny.p, w.p, kap.p, bval.p, cval.p};
  for (int a = 0; a < 8; ++a)
    HSS_CUDA(cudaMemcpyAsync(dst[a] + first, src[a], bytes, cudaMemcpyHostToDevice, s));
  HSS_CUDA(cudaStreamSynchronize(s));
}

// H0^(1)(x) = J0(x) + i Y0(x) for x > 0 to ~2e-16 absolute accuracy.
//  x < 3.5: the ascending series
//    J0 = sum_k (-1)^k q^k / (k!)^2,  Y0 = (2/pi) [(log(x/2) + gamma) J0 + sum_k (-1)^(k+1) H_k q^k / (k!)^2],
//    q = x^2 / 4, H_k the harmonic numbers.
//  x >= 3.5: Hankel's integral (Watson, Theory of Bessel Functions, sec. 7.2), for nu = 0
//    H0^(1)(x) = sqrt(2 / (pi x)) e^{i (x - pi/4)} / sqrt(pi) * int_{-inf}^{inf} e^{-s^2} (1 + i s^2 / (2x))^(-1/2) ds,
//  by the trapezoidal rule with step 0.3 on |s| <= 6.3, which converges geometrically for
//  this analytic integrand (Trefethen & Weideman, SIAM Review 56, 2014).  The factor
//  (1 + i v)^(-1/2) = r^(-1/2) (cos(t/2) - i sin(t/2)), r = |1 + i v|, t = arg(1 + i v),
//  with sin(t/2) = (v / r) / (2 cos(t/2)) to avoid cancellation at small v.
// hw: the trapezoid weights 2 exp(-(j step)^2) (HelmDev::hw), indexed with constants only
// (the loop below is unrolled) so they stay in the parameter bank.
__device__ __forceinline__ void hankel0(double x, const double (&hw)[kHankelNodes + 1], double& J, double& Y) {
  constexpr double kGamma = 0.57721566490153286061, kTwoOverPi = 0.63661977236758134308;
  if (x < 3.5) {
    const double q = 0.25 * x * x;
    double t = 1.0, j = 1.0, ys = 0.0, hk = 0.0;
    for (int k = 1; k < 40; ++k) {
      t *= -q / ((double)k * k);
      hk += 1.0 / k;
      j += t;
      ys -= t * hk;
      if (fabs(t) < 1e-18) break;
    }
    J = j;
    Y = kTwoOverPi * ((log(0.5 * x) + kGamma) * j + ys);
    return;
  }
  double ir = 1.0, ii = 0.0;
  const double i2x = 0.5 / x;
#pragma unroll
  for (int k = 1; k <= kHankelNodes; ++k) {
    const double sk = k * kHankelStep;
    const double v = sk * sk * i2x;
    const double r = sqrt(1.0 + v * v);
    const double ch = sqrt(0.5 * (1.0 + 1.0 / r));
    const double sh = (v / r) / (2.0 * ch);
    const double rs = 1.0 / sqrt(r);
    ir += hw[k] * (ch * rs);
    ii -= hw[k] * (sh * rs);
  }
  const double norm = kHankelStep * 0.56418958354775628695;  // step / sqrt(pi)
  ir *= norm;
  ii *= norm;
  double sx, cx;
  sincos(x, &sx, &cx);
  const double c = (cx + sx) * 0.70710678118654752440;  // cos(x - pi/4)
  const double sn = (sx - cx) * 0.70710678118654752440; // sin(x - pi/4)
  const double f = sqrt(kTwoOverPi / x);
  J = f * (c * ir - sn * ii);
  Y = f * (c * ii + sn * ir);
}

// Helmholtz entry (Kernel_Eval.m:44-49): w on the diagonal, else
// (0, s) * b(x) * (J0 + i Y0)(kh r) * c(y) with the products in MATLAB's order, which
// for the purely imaginary (0, s b) factor is Re = -((s b) Y0) c, Im = ((s b) J0) c.
__global__ void __launch_bounds__(256) k_kgen_complex(const KgenCP* __restrict__ D, PointView P, HelmDev k) {
  const KgenCP d = D[blockIdx.y];
  const long long tot = (long long)d.m * d.n;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int i = (int)(e % d.m), j = (int)(e / d.m);
    const int t = d.ti[i], s = d.si[j];
    const double dx = __dadd_rn(P.x[t], -P.x[s]);
    const double dy = __dadd_rn(P.y[t], -P.y[s]);
    const double den = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    double re, im;
    if (den == 0.0) {
      re = k.w_re;
      im = k.w_im;
    } else {
      const double x = __dmul_rn(k.kh, sqrt(den));
      const double sb = __dmul_rn(k.s, P.bval[t]);
      double hj, hy;
      hankel0(x, k.hw, hj, hy);
      re = -__dmul_rn(__dmul_rn(sb, hy), P.cval[s]);
      im = __dmul_rn(__dmul_rn(sb, hj), P.cval[s]);
    }
    const size_t o = 2 * ((size_t)i + (size_t)j * d.ld);
    d.out[o] = re;
    d.out[o + 1] = im;
  }
}

// Complex Helmholtz entry K(t, s) of the point table (the operations of k_kgen_complex).
__device__ __forceinline__ void helm_entry(const HelmDev& k, const PointView& P, int t, int s, double& re,
                                           double& im) {
  const double dx = __dadd_rn(P.x[t], -P.x[s]);
  const double dy = __dadd_rn(P.y[t], -P.y[s]);
  const double den = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  if (den == 0.0) {
    re = k.w_re;
    im = k.w_im;
    return;
  }
  const double x = __dmul_rn(k.kh, sqrt(den));
  const double sb = __dmul_rn(k.s, P.bval[t]);
  double hj, hy;
  hankel0(x, k.hw, hj, hy);
  re = -__dmul_rn(__dmul_rn(sb, hy), P.cval[s]);
  im = __dmul_rn(__dmul_rn(sb, hj), P.cval[s]);
}

// entry (a, b) of the real 2 x 2 embedding [[re, -im], [im, re]]
__device__ __forceinline__ double emb_entry(double re, double im, int a, int b) {
  return (a == b) ? re : (a ? im : -im);
}

__device__ __forceinline__ double kernel_entry(const KernelDev& k, const PointView& P, int t, int s) {
  const double dx = __dadd_rn(P.x[t], -P.x[s]);
  const double dy = __dadd_rn(P.y[t], -P.y[s]);
  const double den = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  const bool z = (den == 0.0);
  if (k.flag == HSS_SL_H_2D) {  // embedded complex entry
    double re, im;
    helm_entry(k.helm, P, t & ~1, s & ~1, re, im);
    return emb_entry(re, im, t & 1, s & 1);
  }
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

// Embedded Helmholtz blocks: one thread per complex entry (index pairs 2i, 2i + 1 of ti and
// si address the two components of one point), the four real entries of its 2 x 2 block
// written together; m and n are even.
template <typename R>
__global__ void __launch_bounds__(256) k_kgen_emb(const KgenP<R>* __restrict__ D, PointView P, HelmDev k) {
  const KgenP<R> d = D[blockIdx.y];
  const int mc = d.m / 2, nc = d.n / 2;
  const long long tot = (long long)mc * nc;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int i = (int)(e % mc), j = (int)(e / mc);
    double re, im;
    helm_entry(k, P, d.ti[2 * i], d.si[2 * j], re, im);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const int r = 2 * i + a, c = 2 * j + b;
        const size_t o = d.trans ? (c + (size_t)r * d.ld) : (r + (size_t)c * d.ld);
        d.out[o] = (R)emb_entry(re, im, a, b);
      }
  }
}

void kgen_complex_batched(const KgenCP* dP, int batch, long long maxEntries, const PointView& pts,
                          const HelmDev& k, cudaStream_t s) {
  if (batch <= 0 || maxEntries <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "kgen batch too large");
  const int gx = std::max(1, std::min(ceil_div(maxEntries, 256), 4096));
  k_kgen_complex<<<dim3(gx, batch), 256, 0, s>>>(dP, pts, k);
  check_launch("k_kgen_complex");
}

template <typename R>
void kgen_batched(const KgenP<R>* dP, int batch, long long maxEntries, const PointView& pts,
                  const KernelDev& k, cudaStream_t s) {
  if (batch <= 0 || maxEntries <= 0) return;
  HSS_REQUIRE(batch <= 65535, HSS_ERR_ARG, "kgen batch too large");
  if (k.flag == HSS_SL_H_2D) {
    const int gx = std::max(1, std::min(ceil_div(maxEntries / 4, 256), 2048));
    k_kgen_emb<R><<<dim3(gx, batch), 256, 0, s>>>(dP, pts, k.helm);
    check_launch("k_kgen_emb");
    return;
  }
  const int gx = std::max(1, std::min(ceil_div(maxEntries, 256), 2048));
  k_kgen<R><<<dim3(gx, batch), 256, 0, s>>>(dP, pts, k);
  check_launch("k_kgen");
}

// One thread per target; the target's data and h^2/2 b(x) are held in registers, every
// entry is formed with kernel_entry's operations in kernel_entry's order.
template <int NR>
__global__ void __launch_bounds__(256) k_kmatvec(const KmvP* __restrict__ D, PointView P, KernelDev k, int nsplit,
                                                 double* __restrict__ part, int mmax, int nrhs) {
  const KmvP d = D[blockIdx.z];
  if ((int)blockIdx.x * 256 >= d.m) return;
  const int i = blockIdx.x * 256 + threadIdx.x;
  const int per = (d.n + nsplit - 1) / nsplit;
  const int jb = blockIdx.y * per, je = min(d.n, jb + per);
  double acc[NR];
#pragma unroll
  for (int c = 0; c < NR; ++c) acc[c] = 0.0;
  if (i < d.m) {
    const int t = d.t0 + i;
    const double tx = P.x[t], ty = P.y[t];
    const double hb = __dmul_rn(k.h2half, P.bval[t]);
    for (int j = jb; j < je; ++j) {
      const int sj = d.s0 + j;
      const double dx = __dadd_rn(tx, -P.x[sj]);
      const double dy = __dadd_rn(ty, -P.y[sj]);
      const double den = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      const bool z = (den == 0.0);
      double v;
      if (k.flag == HSS_SL_L_2D) {
        v = __dmul_rn(__dmul_rn(hb, log(z ? 1.0 : den)), P.cval[sj]);
        v = __dadd_rn(v, z ? 1.0 : 0.0);
      } else {
        const double w = P.w[sj];
        if (z) {
          v = __dadd_rn(-0.5, -__dmul_rn(__dmul_rn(w, P.kap[sj]), 0.07957747154594767));
        } else {
          const double num = __dadd_rn(__dmul_rn(P.nx[sj], dx), __dmul_rn(P.ny[sj], dy));
          v = __ddiv_rn(__dmul_rn(__dmul_rn(w, 0.15915494309189535), num), den);
        }
      }
      const double* qj = d.q + j;
#pragma unroll
      for (int c = 0; c < NR; ++c)
        if (c < nrhs) acc[c] = fma(v, qj[(size_t)c * d.ldq], acc[c]);
    }
    double* pp = part + (((size_t)blockIdx.z * nsplit + blockIdx.y) * mmax + i) * NR;
#pragma unroll
    for (int c = 0; c < NR; ++c) pp[c] = acc[c];
  }
}

// Embedded complex kernel (HSS_SL_H_2D): one thread per complex target (real rows 2i, 2i + 1
// of the embedded system), each complex entry formed once and applied to the interleaved
// (re, im) source vector: complex128 arithmetic.
template <int NR>
__global__ void __launch_bounds__(256) k_kmatvec_c(const KmvP* __restrict__ D, PointView P, HelmDev k, int nsplit,
                                                   double* __restrict__ part, int mmax, int nrhs) {
  const KmvP d = D[blockIdx.z];
  const int mc = d.m / 2, nc = d.n / 2;
  if ((int)blockIdx.x * 256 >= mc) return;
  const int i = blockIdx.x * 256 + threadIdx.x;
  const int per = (nc + nsplit - 1) / nsplit;
  const int jb = blockIdx.y * per, je = min(nc, jb + per);
  double ar[NR], ai[NR];
#pragma unroll
  for (int c = 0; c < NR; ++c) ar[c] = ai[c] = 0.0;
  if (i < mc) {
    const int t = d.t0 + 2 * i;
    for (int j = jb; j < je; ++j) {
      double re, im;
      helm_entry(k, P, t, d.s0 + 2 * j, re, im);
      const double* qj = d.q + 2 * j;
#pragma unroll
      for (int c = 0; c < NR; ++c)
        if (c < nrhs) {
          const double xr = qj[(size_t)c * d.ldq], xi = qj[(size_t)c * d.ldq + 1];
          ar[c] = fma(re, xr, fma(-im, xi, ar[c]));
          ai[c] = fma(re, xi, fma(im, xr, ai[c]));
        }
    }
    double* pp = part + (((size_t)blockIdx.z * nsplit + blockIdx.y) * mmax + 2 * i) * NR;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
      pp[c] = ar[c];
      pp[NR + c] = ai[c];
    }
  }
}

template <int NR>
__global__ void k_kmatvec_reduce(const KmvP* __restrict__ D, int nsplit, const double* __restrict__ part, int mmax,
                                 int nrhs) {
  const KmvP d = D[blockIdx.y];
  const int tot = d.m * nrhs;
  for (int e = blockIdx.x * 256 + threadIdx.x; e < tot; e += gridDim.x * 256) {
    const int i = e % d.m, c = e / d.m;
    double s = 0.0;
    for (int y = 0; y < nsplit; ++y) s += part[(((size_t)blockIdx.y * nsplit + y) * mmax + i) * NR + c];
    d.u[i + (size_t)c * d.ldu] = s;
  }
}

void kernel_matvec(const KmvP* dP, int batch, int maxM, int maxN, int nrhs, const PointView& pts, const KernelDev& k,
                   DevBuf<double>& part, cudaStream_t s) {
  if (batch <= 0 || maxM <= 0) return;
  HSS_REQUIRE(batch <= 65535 && nrhs >= 1 && nrhs <= 8, HSS_ERR_ARG, "kernel matvec: batch <= 65535, 1..8 columns");
  const bool cplx = (k.flag == HSS_SL_H_2D);
  const int tiles = ceil_div(cplx ? maxM / 2 : maxM, 256);
  const int nsplit = std::max(1, std::min(64, std::min(ceil_div(1216, (long long)tiles * batch), std::max(1, maxN / 256))));
  const int NR = nrhs <= 4 ? 4 : 8;
  part.ensure((size_t)batch * nsplit * maxM * NR);
  const dim3 grid(tiles, nsplit, batch);
  if (cplx) {
    if (NR == 4) k_kmatvec_c<4><<<grid, 256, 0, s>>>(dP, pts, k.helm, nsplit, part.p, maxM, nrhs);
    else k_kmatvec_c<8><<<grid, 256, 0, s>>>(dP, pts, k.helm, nsplit, part.p, maxM, nrhs);
  } else if (NR == 4) {
    k_kmatvec<4><<<grid, 256, 0, s>>>(dP, pts, k, nsplit, part.p, maxM, nrhs);
  } else {
    k_kmatvec<8><<<grid, 256, 0, s>>>(dP, pts, k, nsplit, part.p, maxM, nrhs);
  }
  check_launch("k_kmatvec");
  const int gx = std::max(1, std::min(ceil_div((long long)maxM * nrhs, 256), 256));
  if (NR == 4) k_kmatvec_reduce<4><<<dim3(gx, batch), 256, 0, s>>>(dP, nsplit, part.p, maxM, nrhs);
  else k_kmatvec_reduce<8><<<dim3(gx, batch), 256, 0, s>>>(dP, nsplit, part.p, maxM, nrhs);
  check_launch("k_kmatvec_reduce");
}

template void kgen_batched<double>(const KgenP<double>*, int, long long, const PointView&,
                                   const KernelDev&, cudaStream_t);
template void kgen_batched<float>(const KgenP<float>*, int, long long, const PointView&,
                                  const KernelDev&, cudaStream_t);

}  // namespace hss
