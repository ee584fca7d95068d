// Preconditioned BiCGSTAB over compressed HSS2D operators.
//
// The reference's iterative solution (HSS2D/Test/Test_HSS2D_InverseCompression.m:201-228)
// runs MATLAB's bicgstab(Mapp, f, tol, maxit, Iapp): Mapp = the forward apply of the
// compressed operator, Iapp = the inverse apply of a second (translation-invariant)
// compressed operator used as the preconditioner.  This is the same iteration (van der
// Vorst's preconditioned BiCGSTAB with preconditioned directions and the recursive
// residual; the true residual f - A x is recomputed for the reported relres), run for
// every right-hand side in lockstep: the vectors stay on the device, the per-column
// scalars (rho, alpha, omega) are reduced on the device in a fixed order and combined on
// the host.
#include <cmath>
#include <vector>

#include "hss2d.h"

namespace hss {

namespace {

constexpr int KR_BLOCKS = 256;

// part[(b * r + c) * 2 + {0,1}] = block partials of x_c . y_c and y_c . y_c
__global__ void k_dot2(long long N, int r, const double* __restrict__ X, const double* __restrict__ Y,
                       double* __restrict__ part) {
  __shared__ double sa[256], sb[256];
  for (int c = 0; c < r; ++c) {
    double a = 0.0, b = 0.0;
    for (long long i = blockIdx.x * 256LL + threadIdx.x; i < N; i += (long long)gridDim.x * 256) {
      const double x = X[i + c * N], y = Y[i + c * N];
      a += x * y;
      b += y * y;
    }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) {
        sa[threadIdx.x] += sa[threadIdx.x + o];
        sb[threadIdx.x] += sb[threadIdx.x + o];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      part[((size_t)blockIdx.x * r + c) * 2] = sa[0];
      part[((size_t)blockIdx.x * r + c) * 2 + 1] = sb[0];
    }
    __syncthreads();
  }
}

// Z_c = X_c + a_c Y_c + b_c W_c   (column scalars on the device; W may be null; Z may be
// X or Y: every element is read before it is written by the same thread)
__global__ void k_comb(long long N, int r, double* Z, const double* X, const double* Y, const double* W,
                       const double* __restrict__ ab) {
  const long long tot = N * r;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int c = (int)(e / N);
    double v = X[e] + ab[2 * c] * Y[e];
    if (W) v += ab[2 * c + 1] * W[e];
    Z[e] = v;
  }
}

}  // namespace

struct Krylov {
  cudaStream_t s;
  long long N;
  int r;
  DevBuf<double> part, sc;
  Krylov(cudaStream_t st, long long n, int nr) : s(st), N(n), r(nr), part((size_t)KR_BLOCKS * nr * 2), sc(2 * nr) {}
  // per column (x.y, y.y)
  void dots(const double* X, const double* Y, std::vector<double>& xy, std::vector<double>& yy) {
    k_dot2<<<KR_BLOCKS, 256, 0, s>>>(N, r, X, Y, part.p);
    check_launch("k_dot2");
    std::vector<double> h;
    download(h, part.p, (size_t)KR_BLOCKS * r * 2, s);
    HSS_CUDA(cudaStreamSynchronize(s));
    xy.assign(r, 0.0);
    yy.assign(r, 0.0);
    for (int b = 0; b < KR_BLOCKS; ++b)
      for (int c = 0; c < r; ++c) {
        xy[c] += h[((size_t)b * r + c) * 2];
        yy[c] += h[((size_t)b * r + c) * 2 + 1];
      }
  }
  void comb(double* Z, const double* X, const double* Y, const double* W, const std::vector<double>& a,
            const std::vector<double>& b) {
    std::vector<double> ab(2 * r);
    for (int c = 0; c < r; ++c) { ab[2 * c] = a[c]; ab[2 * c + 1] = W ? b[c] : 0.0; }
    HSS_CUDA(cudaMemcpyAsync(sc.p, ab.data(), 2 * r * sizeof(double), cudaMemcpyHostToDevice, s));
    const int gx = std::max(1, std::min(ceil_div(N * r, 256), 4096));
    k_comb<<<gx, 256, 0, s>>>(N, r, Z, X, Y, W, sc.p);
    check_launch("k_comb");
    HSS_CUDA(cudaStreamSynchronize(s));  // ab is a host temporary
  }
};

// x = A^-1 f by BiCGSTAB with preconditioner M^-1 (M == nullptr: none).  f, x: device,
// N x nrhs column-major.  relres: max over columns of ||f - A x|| / ||f||; iters: the
// iterations of the slowest column.
void bicgstab_device(HSS2D& A, HSS2D* M, const double* f, double* x, int nrhs, double tol, int maxit,
                     double* relres, int* iters) {
  HSS_REQUIRE(A.compressed, HSS_ERR_STATE, "bicgstab: the operator must be compressed");
  HSS_REQUIRE(!M || M->inverted, HSS_ERR_STATE, "bicgstab: the preconditioner must be inverted");
  HSS_REQUIRE(!M || M->geo.N == A.geo.N, HSS_ERR_ARG, "bicgstab: operator and preconditioner sizes differ");
  HSS_REQUIRE(nrhs >= 1 && maxit >= 1 && tol > 0, HSS_ERR_ARG, "bicgstab: bad arguments");
  const long long N = A.geo.N;
  const int r = nrhs;
  const cudaStream_t s = A.stream;
  const size_t cnt = (size_t)N * r;
  DevBuf<double> R(cnt), Rh(cnt), P(cnt), V(cnt), Ph(cnt), Sv(cnt), Sh(cnt), T(cnt);
  Krylov K(s, N, r);
  auto precond = [&](const double* in, double* out) {
    if (M) M->applyinv_device(in, out, r, s);
    else HSS_CUDA(cudaMemcpyAsync(out, in, cnt * sizeof(double), cudaMemcpyDeviceToDevice, s));
  };
  std::vector<double> m1(r, -1.0), tmp, fn2, rn2;
  // x0 = 0: r = f
  HSS_CUDA(cudaMemsetAsync(x, 0, cnt * sizeof(double), s));
  HSS_CUDA(cudaMemcpyAsync(R.p, f, cnt * sizeof(double), cudaMemcpyDeviceToDevice, s));
  HSS_CUDA(cudaMemcpyAsync(Rh.p, f, cnt * sizeof(double), cudaMemcpyDeviceToDevice, s));
  HSS_CUDA(cudaMemsetAsync(P.p, 0, cnt * sizeof(double), s));
  HSS_CUDA(cudaMemsetAsync(V.p, 0, cnt * sizeof(double), s));
  K.dots(f, f, tmp, fn2);
  std::vector<double> rho_prev(r, 1.0), alpha(r, 1.0), omega(r, 1.0), res(r, 0.0);
  std::vector<char> done(r, 0);
  for (int c = 0; c < r; ++c) {
    HSS_REQUIRE(std::isfinite(fn2[c]), HSS_ERR_NONFINITE, "bicgstab: non-finite right-hand side");
    if (fn2[c] == 0.0) done[c] = 1;
  }
  int it = 0;
  double worst = 0.0;
  auto zero_done = [&](std::vector<double>& v) {
    for (int c = 0; c < r; ++c)
      if (done[c]) v[c] = 0.0;
  };
  for (it = 1; it <= maxit; ++it) {
    std::vector<double> rho, beta(r), na(r);
    K.dots(Rh.p, R.p, rho, tmp);
    for (int c = 0; c < r; ++c) {
      beta[c] = (rho[c] / rho_prev[c]) * (alpha[c] / omega[c]);
      if (!std::isfinite(beta[c])) beta[c] = 0.0;
      na[c] = -beta[c] * omega[c];
    }
    zero_done(beta);
    zero_done(na);
    K.comb(P.p, R.p, P.p, V.p, beta, na);  // p = r + beta p - beta omega v
    precond(P.p, Ph.p);
    A.apply_device(Ph.p, V.p, r, s);
    std::vector<double> rv;
    K.dots(Rh.p, V.p, rv, tmp);
    std::vector<double> mal(r);
    for (int c = 0; c < r; ++c) {
      alpha[c] = rho[c] / rv[c];
      if (!std::isfinite(alpha[c]) || done[c]) alpha[c] = 0.0;
      mal[c] = -alpha[c];
    }
    K.comb(Sv.p, R.p, V.p, nullptr, mal, mal);  // s = r - alpha v
    precond(Sv.p, Sh.p);
    A.apply_device(Sh.p, T.p, r, s);
    std::vector<double> ts, tt;
    K.dots(Sv.p, T.p, ts, tt);
    std::vector<double> mom(r);
    for (int c = 0; c < r; ++c) {
      omega[c] = (tt[c] > 0.0) ? ts[c] / tt[c] : 0.0;
      if (done[c]) omega[c] = 0.0;
      mom[c] = -omega[c];
    }
    K.comb(x, x, Ph.p, Sh.p, alpha, omega);  // x += alpha p^ + omega s^
    K.comb(R.p, Sv.p, T.p, nullptr, mom, mom);  // r = s - omega t
    K.dots(R.p, R.p, tmp, rn2);
    worst = 0.0;
    bool all = true;
    for (int c = 0; c < r; ++c) {
      res[c] = (fn2[c] > 0.0) ? std::sqrt(rn2[c] / fn2[c]) : 0.0;
      HSS_REQUIRE(std::isfinite(res[c]), HSS_ERR_NONFINITE, "bicgstab: non-finite residual");
      if (res[c] <= tol) done[c] = 1;
      all = all && done[c];
      worst = std::max(worst, res[c]);
      rho_prev[c] = rho[c];
      if (omega[c] == 0.0 && !done[c]) done[c] = 1;  // breakdown: keep the current iterate
    }
    if (all) break;
  }
  // report the true residual f - A x (the iteration tracks the recursive one)
  A.apply_device(x, T.p, r, s);
  K.comb(R.p, f, T.p, nullptr, m1, m1);
  K.dots(R.p, R.p, tmp, rn2);
  worst = 0.0;
  for (int c = 0; c < r; ++c) worst = std::max(worst, (fn2[c] > 0.0) ? std::sqrt(rn2[c] / fn2[c]) : 0.0);
  if (relres) *relres = worst;
  if (iters) *iters = std::min(it, maxit);
}

}  // namespace hss
