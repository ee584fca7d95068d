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
#include <complex>
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

// Entries of the Krylov vectors: complex (interleaved re, im pairs of the embedded system)
// or real.  A vector set is nv vectors of N x r doubles, vector i at V + i * N * r.
// part[((b * nv + i) * r + c) * 2 + {0,1}] = block partial of <V_i, W>_c (complex: sum conj(v) w)
template <bool C>
__global__ void k_gm_dots(long long N, int r, int nv, const double* __restrict__ V, const double* __restrict__ W,
                          double* __restrict__ part) {
  __shared__ double sa[256], sb[256];
  const long long step = C ? 2 : 1, ne = N / step;
  for (int i = 0; i < nv; ++i)
    for (int c = 0; c < r; ++c) {
      const double* v = V + ((size_t)i * r + c) * N;
      const double* w = W + (size_t)c * N;
      double a = 0.0, b = 0.0;
      for (long long e = blockIdx.x * 256LL + threadIdx.x; e < ne; e += (long long)gridDim.x * 256) {
        if (C) {
          const double vr = v[2 * e], vi = v[2 * e + 1], wr = w[2 * e], wi = w[2 * e + 1];
          a = fma(vr, wr, fma(vi, wi, a));
          b = fma(vr, wi, fma(-vi, wr, b));
        } else {
          a = fma(v[e], w[e], a);
        }
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
        part[(((size_t)blockIdx.x * nv + i) * r + c) * 2] = sa[0];
        part[(((size_t)blockIdx.x * nv + i) * r + c) * 2 + 1] = sb[0];
      }
      __syncthreads();
    }
}

// W_c += sum_i h[i, c] V_i,c   (h complex: h[(i * r + c) * 2 + {0,1}]; real vectors use Re h)
template <bool C>
__global__ void k_gm_axpy(long long N, int r, int nv, const double* __restrict__ V, const double* __restrict__ h,
                          double* __restrict__ W) {
  const long long step = C ? 2 : 1, ne = N / step, tot = ne * r;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256) {
    const int c = (int)(e / ne);
    const long long q = e % ne;
    double* w = W + (size_t)c * N;
    if (C) {
      double wr = w[2 * q], wi = w[2 * q + 1];
      for (int i = 0; i < nv; ++i) {
        const double* v = V + ((size_t)i * r + c) * N;
        const double hr = h[(i * r + c) * 2], hi = h[(i * r + c) * 2 + 1];
        const double vr = v[2 * q], vi = v[2 * q + 1];
        wr = fma(hr, vr, fma(-hi, vi, wr));
        wi = fma(hr, vi, fma(hi, vr, wi));
      }
      w[2 * q] = wr;
      w[2 * q + 1] = wi;
    } else {
      double wv = w[q];
      for (int i = 0; i < nv; ++i) wv = fma(h[(i * r + c) * 2], V[((size_t)i * r + c) * N + q], wv);
      w[q] = wv;
    }
  }
}

// Z_c = a_c X_c (real scale per column; Z may be X)
__global__ void k_gm_scale(long long N, int r, const double* X, const double* __restrict__ a, double* Z) {
  const long long tot = N * r;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < tot; e += (long long)gridDim.x * 256)
    Z[e] = a[e / N] * X[e];
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

// Restarted GMRES(m) with right preconditioner M^-1 (Saad & Schultz, SIAM J. Sci. Stat.
// Comput. 7, 1986): Arnoldi with classical Gram-Schmidt applied twice (one batched product
// and one batched update per pass instead of a dependent chain of j dot products), Givens
// rotations on the Hessenberg matrix, x = x0 + Z y with Z = M^-1 V.  Complex arithmetic
// (complex128) on the interleaved vectors of a complex tree.  Every column keeps its own
// Krylov space, rotations and stopping point; the operator and preconditioner applies act on
// all columns at once.
void gmres_device(HSS2D& A, HSS2D* M, const double* f, double* x, int nrhs, double tol, int restart, int maxit,
                  double* relres, int* iters) {
  using cd = std::complex<double>;
  HSS_REQUIRE(A.compressed, HSS_ERR_STATE, "gmres: the operator must be compressed");
  HSS_REQUIRE(!M || M->inverted, HSS_ERR_STATE, "gmres: the preconditioner must be inverted");
  HSS_REQUIRE(!M || (M->geo.N == A.geo.N && M->cplx == A.cplx), HSS_ERR_ARG,
              "gmres: operator and preconditioner sizes differ");
  HSS_REQUIRE(nrhs >= 1 && maxit >= 1 && restart >= 1 && tol > 0, HSS_ERR_ARG, "gmres: bad arguments");
  const bool C = A.cplx;
  const long long N = A.geo.N;
  const int r = nrhs, m = std::min(restart, maxit);
  const cudaStream_t s = A.stream;
  const size_t cnt = (size_t)N * r;
  DevBuf<double> V((size_t)(m + 1) * cnt), Z((size_t)m * cnt), Wv(cnt), part((size_t)KR_BLOCKS * (m + 1) * r * 2),
      hd((size_t)(m + 1) * r * 2), sc(r);
  const int gx = std::max(1, std::min(ceil_div((long long)cnt, 256), 4096));
  auto dots = [&](const double* Vs, int nv, const double* W, std::vector<cd>& out) {
    if (C) k_gm_dots<true><<<KR_BLOCKS, 256, 0, s>>>(N, r, nv, Vs, W, part.p);
    else k_gm_dots<false><<<KR_BLOCKS, 256, 0, s>>>(N, r, nv, Vs, W, part.p);
    check_launch("k_gm_dots");
    std::vector<double> h;
    download(h, part.p, (size_t)KR_BLOCKS * nv * r * 2, s);
    HSS_CUDA(cudaStreamSynchronize(s));
    out.assign((size_t)nv * r, cd(0.0, 0.0));
    for (int b = 0; b < KR_BLOCKS; ++b)
      for (int q = 0; q < nv * r; ++q)
        out[q] += cd(h[((size_t)b * nv * r + q) * 2], h[((size_t)b * nv * r + q) * 2 + 1]);
  };
  // W += sum_i coef[i, c] Vs_i
  auto axpy = [&](const double* Vs, int nv, const std::vector<cd>& coef, double* W) {
    std::vector<double> h((size_t)nv * r * 2);
    for (int q = 0; q < nv * r; ++q) { h[2 * q] = coef[q].real(); h[2 * q + 1] = coef[q].imag(); }
    HSS_CUDA(cudaMemcpyAsync(hd.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    if (C) k_gm_axpy<true><<<gx, 256, 0, s>>>(N, r, nv, Vs, hd.p, W);
    else k_gm_axpy<false><<<gx, 256, 0, s>>>(N, r, nv, Vs, hd.p, W);
    check_launch("k_gm_axpy");
    HSS_CUDA(cudaStreamSynchronize(s));  // h is a host temporary
  };
  auto scale = [&](const double* X, const std::vector<double>& a, double* Zo) {
    HSS_CUDA(cudaMemcpyAsync(sc.p, a.data(), r * sizeof(double), cudaMemcpyHostToDevice, s));
    k_gm_scale<<<gx, 256, 0, s>>>(N, r, X, sc.p, Zo);
    check_launch("k_gm_scale");
    HSS_CUDA(cudaStreamSynchronize(s));
  };
  auto norms = [&](const double* X, std::vector<double>& nv) {
    std::vector<cd> d;
    dots(X, 1, X, d);
    nv.resize(r);
    for (int c = 0; c < r; ++c) nv[c] = std::sqrt(std::max(0.0, d[c].real()));
  };
  auto precond = [&](const double* in, double* out) {
    if (M) M->applyinv_device(in, out, r, s);
    else HSS_CUDA(cudaMemcpyAsync(out, in, cnt * sizeof(double), cudaMemcpyDeviceToDevice, s));
  };
  // residual R = f - A x into V_0; beta per column
  std::vector<double> fn, beta;
  norms(f, fn);
  for (int c = 0; c < r; ++c) HSS_REQUIRE(std::isfinite(fn[c]), HSS_ERR_NONFINITE, "gmres: non-finite right-hand side");
  HSS_CUDA(cudaMemsetAsync(x, 0, cnt * sizeof(double), s));
  auto residual = [&]() {
    A.apply_device(x, Wv.p, r, s);
    HSS_CUDA(cudaMemcpyAsync(V.p, f, cnt * sizeof(double), cudaMemcpyDeviceToDevice, s));
    // V_0 = f - A x: the A x part through the batched update with coefficient -1
    std::vector<double> h((size_t)r * 2);
    for (int c = 0; c < r; ++c) { h[2 * c] = -1.0; h[2 * c + 1] = 0.0; }
    HSS_CUDA(cudaMemcpyAsync(hd.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    if (C) k_gm_axpy<true><<<gx, 256, 0, s>>>(N, r, 1, Wv.p, hd.p, V.p);
    else k_gm_axpy<false><<<gx, 256, 0, s>>>(N, r, 1, Wv.p, hd.p, V.p);
    check_launch("k_gm_axpy");
    norms(V.p, beta);
  };
  residual();
  std::vector<double> res(r);
  auto rel = [&](int c) { return fn[c] > 0.0 ? beta[c] / fn[c] : 0.0; };
  int its = 0;
  for (int c = 0; c < r; ++c) res[c] = rel(c);
  auto worst_res = [&]() {
    double w = 0.0;
    for (int c = 0; c < r; ++c) w = std::max(w, res[c]);
    return w;
  };
  while (worst_res() > tol && its < maxit) {
    const int mm = std::min(m, maxit - its);
    std::vector<double> inv(r);
    for (int c = 0; c < r; ++c) inv[c] = beta[c] > 0.0 ? 1.0 / beta[c] : 0.0;
    scale(V.p, inv, V.p);
    std::vector<std::vector<cd>> H(r, std::vector<cd>((size_t)(mm + 1) * mm, cd(0.0, 0.0)));
    std::vector<std::vector<cd>> cs(r, std::vector<cd>(mm)), sn(r, std::vector<cd>(mm)), g(r, std::vector<cd>(mm + 1));
    std::vector<int> kc(r, 0);
    std::vector<char> active(r, 0);
    for (int c = 0; c < r; ++c) {
      g[c][0] = beta[c];
      active[c] = (res[c] > tol && beta[c] > 0.0);
    }
    int j = 0;
    for (; j < mm; ++j) {
      bool any = false;
      for (int c = 0; c < r; ++c) any = any || active[c];
      if (!any) break;
      double* Zj = Z.p + (size_t)j * cnt;
      double* Vj1 = V.p + (size_t)(j + 1) * cnt;
      precond(V.p + (size_t)j * cnt, Zj);
      A.apply_device(Zj, Vj1, r, s);
      // two passes of classical Gram-Schmidt against V_0..V_j
      std::vector<cd> h1, h2;
      dots(V.p, j + 1, Vj1, h1);
      std::vector<cd> neg(h1.size());
      for (size_t q = 0; q < h1.size(); ++q) neg[q] = -h1[q];
      axpy(V.p, j + 1, neg, Vj1);
      dots(V.p, j + 1, Vj1, h2);
      for (size_t q = 0; q < h2.size(); ++q) neg[q] = -h2[q];
      axpy(V.p, j + 1, neg, Vj1);
      std::vector<double> hn;
      norms(Vj1, hn);
      std::vector<double> sinv(r);
      ++its;
      for (int c = 0; c < r; ++c) {
        sinv[c] = (active[c] && hn[c] > 0.0) ? 1.0 / hn[c] : 0.0;
        if (!active[c]) continue;
        std::vector<cd>& Hc = H[c];
        auto Hat = [&](int row, int col) -> cd& { return Hc[(size_t)row + (size_t)col * (mm + 1)]; };
        for (int i = 0; i <= j; ++i) Hat(i, j) = h1[(size_t)i * r + c] + h2[(size_t)i * r + c];
        Hat(j + 1, j) = hn[c];
        for (int i = 0; i < j; ++i) {  // rotation i on rows (i, i + 1): [[conj c, conj s], [-s, c]]
          const cd t = std::conj(cs[c][i]) * Hat(i, j) + std::conj(sn[c][i]) * Hat(i + 1, j);
          Hat(i + 1, j) = -sn[c][i] * Hat(i, j) + cs[c][i] * Hat(i + 1, j);
          Hat(i, j) = t;
        }
        const double den = std::sqrt(std::norm(Hat(j, j)) + std::norm(Hat(j + 1, j)));
        cs[c][j] = den > 0.0 ? Hat(j, j) / den : cd(1.0, 0.0);
        sn[c][j] = den > 0.0 ? Hat(j + 1, j) / den : cd(0.0, 0.0);
        Hat(j, j) = den;
        Hat(j + 1, j) = 0.0;
        g[c][j + 1] = -sn[c][j] * g[c][j];
        g[c][j] = std::conj(cs[c][j]) * g[c][j];
        kc[c] = j + 1;
        res[c] = fn[c] > 0.0 ? std::abs(g[c][j + 1]) / fn[c] : 0.0;
        if (res[c] <= tol || hn[c] == 0.0) active[c] = 0;
      }
      scale(Vj1, sinv, Vj1);
    }
    // x += Z y per column, y = H(0:k, 0:k) \ g(0:k)
    const int kmax = *std::max_element(kc.begin(), kc.end());
    if (kmax > 0) {
      std::vector<cd> y((size_t)kmax * r, cd(0.0, 0.0));
      for (int c = 0; c < r; ++c) {
        const int k = kc[c];
        auto Hat = [&](int row, int col) { return H[c][(size_t)row + (size_t)col * (mm + 1)]; };
        for (int i = k - 1; i >= 0; --i) {
          cd t = g[c][i];
          for (int q = i + 1; q < k; ++q) t -= Hat(i, q) * y[(size_t)q * r + c];
          y[(size_t)i * r + c] = t / Hat(i, i);
        }
      }
      for (auto& v : y) HSS_REQUIRE(std::isfinite(v.real()) && std::isfinite(v.imag()), HSS_ERR_NONFINITE,
                                    "gmres: non-finite update");
      axpy(Z.p, kmax, y, x);
    }
    residual();
    for (int c = 0; c < r; ++c) res[c] = rel(c);
    if (kmax == 0) break;
  }
  if (relres) *relres = worst_res();
  if (iters) *iters = its;
}

}  // namespace hss
