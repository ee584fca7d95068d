// Duan–Rokhlin diagonal corrections of the Helmholtz (Lippmann–Schwinger) kernel on a
// uniform grid: DR_stencil (Common/DR_stencil.m:1-53) and the corr0 / corr1 outputs of
// its external Fortran program (Common/FORTRAN_get_DR_weights.f:85-, corr_hank).
//
// The reference interpolates tabulated coefficient lists.  This file derives the same
// numbers from the asymptotics of the punctured trapezoidal rule instead.  On the lattice
// h Z^2, for smooth compactly supported f and G(y) = H0^(1)(k |y|):
//
//   int G f dy = h^2 sum_{j != 0} G(jh) f(jh) + corr0 f(0) + (corr1 / 2) lap f(0) + ...
//
// Split H0(k r) = i (2/pi) log(r) J0(k r) + R(r) with R smooth and
// R(0) = 1 + i (2/pi) (log(k/2) + gamma).  The smooth part contributes h^2 R(0) f(0) (the
// rule is spectrally accurate apart from the missing origin).  For the logarithmic part
// the zeta-regularised Euler–Maclaurin expansion of the lattice sum gives, for every
// m >= 0,
//
//   int |y|^(2m) log|y| g - h^2 sum' |jh|^(2m) log|jh| g(jh)
//       = h^(2+2m) (Z'(-2m) - log(h) Z(-2m)) g(0) + ...,
//
// with Z(s) = sum'_{j in Z^2} |j|^(-s) = 4 zeta(s/2) beta(s/2) (beta: Dirichlet beta),
// Z(0) = -1 and Z(-2m) = 0 for m >= 1.  Expanding J0(k r) = sum_m c_m r^(2m),
// c_m = (-1)^m (k/2)^(2m) / (m!)^2, and the isotropic second-order Taylor term of f
// ((lap f(0) / 4) |y|^2):
//
//   corr0 = h^2 [1 + i (2/pi)(log(k h / 2) + gamma + Z'(0))] + i (2/pi) sum_{m>=1} c_m h^(2+2m) Z'(-2m)
//   corr1 = i (1/pi) sum_{m>=0} c_m h^(4+2m) Z'(-2m-2)
//
// Closed forms used for Z'(-2m) (Z'(s) = 2 [zeta'(s/2) beta(s/2) + zeta(s/2) beta'(s/2)]):
//   Z'(0)       = -log(2 pi)/2 - log(Gamma(1/4)^2 / (2 pi sqrt 2))
//   m = 2n > 0  : Z'(-2m) = 2 zeta'(-2n) beta(-2n),
//                 zeta'(-2n) = (-1)^n (2n)! zeta(2n+1) / (2 (2 pi)^(2n)),  beta(-2n) = E_2n / 2
//   m = 2n + 1  : Z'(-2m) = 2 zeta(-m) beta'(-m),
//                 zeta(-m) = -B_(m+1) / (m+1),  beta'(-m) = (-1)^n (2/pi)^m m! beta(m+1)
// (E: Euler numbers, B: Bernoulli numbers).  The series converge geometrically for
// |k h| < 2 pi.  corr2..corr5 (the fourth- and sixth-order anisotropic lattice moments,
// needed only by the order-8 and order-10 stencils) are not derived.
#include <cmath>
#include <complex>
#include <vector>

#include "common.cuh"

namespace hss {

namespace {

using cd = std::complex<double>;

constexpr double kPi = 3.14159265358979323846;
constexpr double kEulerGamma = 0.57721566490153286061;
constexpr double kCatalan = 0.91596559417721901505;  // beta(2)

// Bernoulli numbers B_0..B_n (B_1 = -1/2) by the standard recurrence (used only for the
// few Euler–Maclaurin coefficients, where it is exact enough)
std::vector<double> bernoulli(int n) {
  std::vector<double> B(n + 1, 0.0);
  B[0] = 1.0;
  for (int m = 1; m <= n; ++m) {
    double s = 0.0, binom = 1.0;  // binom = C(m+1, k)
    for (int k = 0; k < m; ++k) {
      s += binom * B[k];
      binom = binom * (m + 1 - k) / (k + 1);
    }
    B[m] = -s / (m + 1);
  }
  return B;
}

// Hurwitz zeta(s, q), real s > 1, q > 0, by Euler–Maclaurin summation
double hurwitz(double s, double q) {
  const int K = 12;
  double sum = 0.0;
  for (int k = 0; k < K; ++k) sum += std::pow(k + q, -s);
  const double a = K + q;
  sum += std::pow(a, 1.0 - s) / (s - 1.0) + 0.5 * std::pow(a, -s);
  static const std::vector<double> B = bernoulli(24);
  double fact = 1.0;   // (2j)!
  double rising = s;   // s (s+1) ... (s+2j-2)
  double powa = std::pow(a, -s - 1.0);
  for (int j = 1; j <= 12; ++j) {
    fact *= (2.0 * j - 1.0) * (2.0 * j);
    sum += B[2 * j] / fact * rising * powa;
    rising *= (s + 2.0 * j - 1.0) * (s + 2.0 * j);
    powa /= a * a;
  }
  return sum;
}

double zeta_pos(double s) { return hurwitz(s, 1.0); }
double beta_pos(double s) {
  if (s == 2.0) return kCatalan;
  return std::pow(4.0, -s) * (hurwitz(s, 0.25) - hurwitz(s, 0.75));
}

// Z'(-2m) of the square-lattice zeta function Z(s) = 4 zeta(s/2) beta(s/2).  The Euler
// and Bernoulli numbers enter through their zeta / beta forms (stable for large m):
//   E_2n = (-1)^n 2^(2n+2) (2n)! beta(2n+1) / pi^(2n+1),
//   B_2n = (-1)^(n+1) 2 (2n)! zeta(2n) / (2 pi)^(2n).
double lattice_zeta_deriv(int m) {
  if (m == 0) {
    const double g = std::tgamma(0.25);
    return -0.5 * std::log(2.0 * kPi) - std::log(g * g / (2.0 * kPi * std::sqrt(2.0)));
  }
  if (m % 2 == 0) {
    // 2 zeta'(-2n) beta(-2n) = 2 [(-1)^n (2n)! zeta(2n+1) / (2 (2pi)^2n)] [E_2n / 2]
    const int n = m / 2;
    const double f2n = std::tgamma(2.0 * n + 1.0);
    const double zp = ((n % 2) ? -1.0 : 1.0) * f2n * zeta_pos(2.0 * n + 1.0) / (2.0 * std::pow(2.0 * kPi, 2.0 * n));
    const double E = ((n % 2) ? -1.0 : 1.0) * std::pow(2.0, 2.0 * n + 2.0) * f2n * beta_pos(2.0 * n + 1.0) /
                     std::pow(kPi, 2.0 * n + 1.0);
    return 2.0 * zp * (0.5 * E);
  }
  // 2 zeta(-m) beta'(-m) with zeta(-m) = -B_(m+1) / (m+1), m + 1 = 2n + 2
  const int n = (m - 1) / 2;
  const int q = n + 1;  // B_2q
  const double B = ((q % 2) ? 1.0 : -1.0) * 2.0 * std::tgamma(2.0 * q + 1.0) * zeta_pos(2.0 * q) /
                   std::pow(2.0 * kPi, 2.0 * q);
  const double zm = -B / (m + 1);
  const double bp = ((n % 2) ? -1.0 : 1.0) * std::pow(2.0 / kPi, (double)m) * std::tgamma(m + 1.0) *
                    beta_pos(m + 1.0);
  return 2.0 * zm * bp;
}

}  // namespace

// corr0 and corr1 of the Duan–Rokhlin correction for grid spacing h and wavenumber k
void dr_corrections(double h, cd k, cd& corr0, cd& corr1) {
  HSS_REQUIRE(h > 0 && std::isfinite(h), HSS_ERR_ARG, "DR weights: h must be positive");
  HSS_REQUIRE(std::abs(k) > 0 && std::isfinite(k.real()) && std::isfinite(k.imag()), HSS_ERR_ARG,
              "DR weights: the wavenumber must be finite and non-zero");
  HSS_REQUIRE(std::abs(k) * h < 2.0 * kPi, HSS_ERR_ARG, "DR weights: |k| h must be below 2 pi");
  const cd I(0.0, 1.0);
  const double tpi = 2.0 / kPi;
  corr0 = h * h * (1.0 + I * tpi * (std::log(k * h / 2.0) + kEulerGamma + lattice_zeta_deriv(0)));
  corr1 = 0.0;
  const cd q = (k / 2.0) * (k / 2.0);
  cd cm = 1.0;  // c_m = (-1)^m (k/2)^(2m) / (m!)^2
  for (int m = 0; m <= 60; ++m) {
    if (m > 0) cm *= -q / ((double)m * m);
    const cd t0 = (m > 0) ? I * tpi * cm * std::pow(h, 2.0 + 2.0 * m) * lattice_zeta_deriv(m) : cd(0.0);
    const cd t1 = I * (1.0 / kPi) * cm * std::pow(h, 4.0 + 2.0 * m) * lattice_zeta_deriv(m + 1);
    corr0 += t0;
    corr1 += t1;
    if (m > 2 && std::abs(t0) <= 1e-18 * std::abs(corr0) && std::abs(t1) <= 1e-18 * std::abs(corr1)) break;
  }
}

// DR_stencil(h, rk, n, order) for order 0, 4 and 6: count entries of (J, weight, stencil
// column); J = i2 + n i1 (Common/DR_stencil.m:18-32).
void dr_stencil(double h, cd k, long long n, int order, std::vector<long long>& J, std::vector<cd>& w,
                std::vector<int>& stencil) {
  J.clear();
  w.clear();
  stencil.clear();
  if (order == 0) {
    J.push_back(0);
    w.push_back(0.0);
    stencil.insert(stencil.end(), {0, 0, 1});
    return;
  }
  HSS_REQUIRE(order == 4 || order == 6, HSS_ERR_ARG,
              "DR_stencil: orders 0, 4 and 6 are supported (8 and 10 need corr2..corr5)");
  cd c0, c1;
  dr_corrections(h, k, c0, c1);
  if (order == 4) {
    J.push_back(0);
    w.push_back(c0);
    stencil.insert(stencil.end(), {0, 0, 1});
    return;
  }
  // order 6: the centre and its four lattice neighbours, DVEC_scaled = corr .* [1; 1/h^2]
  const cd s0 = c0, s1 = c1 / (h * h);
  const cd dr6[2] = {s0 - 2.0 * s1, 0.5 * s1};
  const int ist[3][5] = {{0, 0, 1, 0, -1}, {0, -1, 0, 1, 0}, {1, 2, 2, 2, 2}};
  for (int e = 0; e < 5; ++e) {
    J.push_back(ist[1][e] + n * ist[0][e]);
    w.push_back(dr6[ist[2][e] - 1]);
    stencil.insert(stencil.end(), {ist[0][e], ist[1][e], ist[2][e]});
  }
}

}  // namespace hss
