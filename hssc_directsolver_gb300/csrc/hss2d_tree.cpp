// HSS2D tree geometry on the host: uniform alternating-bisection tree,
// preset 'bdry' skeletons and 'bdry' box proxies.  Integer and sorting work
// only; every floating-point comparison is formed in the same order as the
// reference's MATLAB expressions.
//
//   tree / centres     HSS2D/HSS2D_build_tree_nsym.m:145-277, bisect_level :1183-1240
//   leaf sources       Build_I_source_unif :1097-1124
//   skeletons          LOCAL_Preset_Skeleton_Info 'bdry' :732-792, orient :794-811
//   proxies            HSS2D/build_box_proxy.m:52-88 via LOCAL_Build_Proxy :945-949
//   proxy layers       :360-368
//   'rand' proxies     LOCAL_Build_Proxy :883-905, LOCAL_random_sampler :964-1001
//   'wdec' proxies     :877-881, Common/Whitney_decomposition_1Dcurve.m
//   ID skeletons       :399-412, LOCAL_Non_Preset_Skeleton_Info :614-657 (kh > 0)
#include "hss2d_tree.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <numeric>
#include <random>

namespace hss {

static void box_radii(int lev, double& colrad, double& rowrad) {
  const int scl = lev / 2;
  rowrad = std::ldexp(1.0, -scl);
  colrad = rowrad / (double)(1 << (lev % 2));
}

static std::vector<double> colon(double a, double step, double b) {
  const int n = (int)std::floor((b - a) / step + 1e-9) + 1;
  std::vector<double> v;
  for (int i = 0; i < n; ++i) v.push_back(a + step * (double)i);
  return v;
}

static void stable_argsort(const std::vector<double>& key, std::vector<int>& idx) {
  idx.resize(key.size());
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return key[a] < key[b]; });
}

void box_proxy(double cx, double cy, double colrad, double rowrad, int layers, double h,
               std::vector<double>& px, std::vector<double>& py) {
  const double width = ((double)layers - 0.5) * h;
  struct P { double x, y; };
  std::vector<P> X1, X2, X3, X4;
  {
    auto xs = colon(cx - colrad - width, h, cx - colrad - h / 2);
    auto ys = colon(cy - rowrad - width, h, cy + rowrad + width);
    for (double y : ys) for (double x : xs) X1.push_back({x, y});
  }
  {
    auto xs = colon(cx - colrad + h / 2, h, cx + colrad - h / 2);
    auto ys = colon(cy + rowrad + width, -h, cy + rowrad + h / 2);
    for (double x : xs) for (double y : ys) X2.push_back({x, y});
  }
  {
    auto xs = colon(cx + colrad + h / 2, h, cx + colrad + width);
    auto ys = colon(cy + rowrad + width, -h, cy - rowrad - width);
    for (double y : ys) for (double x : xs) X3.push_back({x, y});
  }
  {
    auto xs = colon(cx + colrad - h / 2, -h, cx - colrad + h / 2);
    auto ys = colon(cy - rowrad - h / 2, -h, cy - rowrad - width);
    for (double x : xs) for (double y : ys) X4.push_back({x, y});
  }
  const double r1 = (double)(layers * layers) - 0.5, r2 = (double)(layers * layers) + 0.5;
  const double W = rowrad + width, V = colrad + width;
  auto m1 = [&](const P& p) {
    return ((std::fabs(p.x - cx) > (V - h / 2)) && ((p.y - cy > (W - r1 * h)) || (p.y - cy < -(W - r2 * h)))) ||
           (std::fabs(p.y - cy) > (W - h / 2));
  };
  auto m2 = [&](const P& p) {
    return (std::fabs(p.y - cy) > (W - h / 2)) && ((p.x - cx > (V - r1 * h)) || (p.x - cx < -(V - r2 * h)));
  };
  auto m3 = [&](const P& p) {
    return ((std::fabs(p.x - cx) > (V - h / 2)) && ((p.y - cy > (W - r2 * h)) || (p.y - cy < -(W - r1 * h)))) ||
           (std::fabs(p.y - cy) > (W - h / 2));
  };
  auto m4 = [&](const P& p) {
    return (std::fabs(p.y - cy) > (W - h / 2)) && ((p.x - cx > (V - r2 * h)) || (p.x - cx < -(V - r1 * h)));
  };
  px.clear();
  py.clear();
  for (int pass = 0; pass < 2; ++pass) {
    const bool want = (pass == 1);
    for (auto& p : X1) if (m1(p) == want) { px.push_back(p.x); py.push_back(p.y); }
    for (auto& p : X2) if (m2(p) == want) { px.push_back(p.x); py.push_back(p.y); }
    for (auto& p : X3) if (m3(p) == want) { px.push_back(p.x); py.push_back(p.y); }
    for (auto& p : X4) if (m4(p) == want) { px.push_back(p.x); py.push_back(p.y); }
  }
}

// LOCAL_orient_residual (:805-811): order of points (x[i], y[i]) by the normal coordinate,
// then stably by the negated tangential one
static std::vector<int> orient_residual(const std::vector<double>& x, const std::vector<double>& y, int nrm) {
  const std::vector<double>& a = nrm == 0 ? x : y;
  const std::vector<double>& b = nrm == 0 ? y : x;
  std::vector<int> J1, J2;
  stable_argsort(a, J1);
  std::vector<double> key2(J1.size());
  for (size_t i = 0; i < J1.size(); ++i) key2[i] = -b[J1[i]];
  stable_argsort(key2, J2);
  std::vector<int> out(J1.size());
  for (size_t i = 0; i < J1.size(); ++i) out[i] = J1[J2[i]];
  return out;
}

// LOCAL_orient_skeleton (:794-802): polar order around (cx, cy) from angle th0, ties by radius
static std::vector<int> orient_skeleton(const std::vector<double>& x, const std::vector<double>& y, double cx,
                                        double cy, double th0) {
  const size_t n = x.size();
  std::vector<double> th(n), rho(n);
  for (size_t i = 0; i < n; ++i) {
    const double dx = x[i] - cx, dy = y[i] - cy;
    double t = std::atan2(dy, dx);
    if (t < th0) t = t + 2.0 * M_PI;
    th[i] = t;
    rho[i] = std::hypot(dx, dy);
  }
  std::vector<int> J1, J2;
  stable_argsort(rho, J1);
  std::vector<double> th1(n);
  for (size_t i = 0; i < n; ++i) th1[i] = th[J1[i]];
  stable_argsort(th1, J2);
  std::vector<int> out(n);
  for (size_t i = 0; i < n; ++i) out[i] = J1[J2[i]];
  return out;
}

static void level_orientation(int lev, int& nrm, double& th0) {
  if (lev % 2 == 0) { nrm = 0; th0 = M_PI / 2; }
  else { nrm = 1; th0 = 0.0; }
}

// J (local permutation, skeleton first) and k of one box.
static void preset_skeleton(const std::vector<double>& X, const std::vector<int>& I_src, double cx,
                            double cy, int lev, double colrad, double rowrad, int layers, double h,
                            std::vector<int>& J, int& k) {
  const int n = (int)I_src.size();
  const double width = layers * h;
  std::vector<int> sk, rs;
  for (int i = 0; i < n; ++i) {
    const double x = X[2 * (size_t)I_src[i]], y = X[2 * (size_t)I_src[i] + 1];
    const bool b = (std::fabs(x - cx) > (colrad - width)) || (std::fabs(y - cy) > (rowrad - width));
    (b ? sk : rs).push_back(i);
  }
  int nrm;
  double th0;
  level_orientation(lev, nrm, th0);
  std::vector<double> rx(rs.size()), ry(rs.size()), sx(sk.size()), sy(sk.size());
  for (size_t i = 0; i < rs.size(); ++i) { rx[i] = X[2 * (size_t)I_src[rs[i]]]; ry[i] = X[2 * (size_t)I_src[rs[i]] + 1]; }
  for (size_t i = 0; i < sk.size(); ++i) { sx[i] = X[2 * (size_t)I_src[sk[i]]]; sy[i] = X[2 * (size_t)I_src[sk[i]] + 1]; }
  const std::vector<int> Jr = orient_residual(rx, ry, nrm);
  const std::vector<int> Js = orient_skeleton(sx, sy, cx, cy, th0);
  J.clear();
  for (int v : Js) J.push_back(sk[v]);
  k = (int)sk.size();
  for (int v : Jr) J.push_back(rs[v]);
}

// LOCAL_random_sampler (:964-1001): points within lay h of the box are kept, the others with
// probability 2^(-lam l) by dyadic distance band l.  The reference resets MATLAB's generator
// (the Mersenne Twister with its default seed 5489) on every call; the uniforms are that
// generator's 53-bit doubles (two 32-bit draws, a >> 5 and b >> 6, (a 2^26 + b) 2^-53).
static std::vector<char> sampler_mask(const std::vector<double>& px, const std::vector<double>& py, double cx,
                                      double cy, double colrad, double rowrad, double lam, int lay, double h) {
  const size_t n = px.size();
  std::vector<char> keep(n, 0);
  if (n == 0) return keep;
  std::vector<double> D(n);
  double rad = 0.0;
  for (size_t i = 0; i < n; ++i) {
    D[i] = std::fabs(std::min(colrad - std::fabs(px[i] - cx), rowrad - std::fabs(py[i] - cy)));
    rad = std::max(rad, D[i]);
  }
  const double width = lay * h;
  const int sz = -(int)std::floor(std::log2(width / rad)) + 1;
  for (size_t i = 0; i < n; ++i) keep[i] = D[i] < width;
  if (sz > 0) {
    std::mt19937 gen(5489u);
    for (size_t i = 0; i < n; ++i) {
      double Ld;
      if (D[i] < width) Ld = sz;
      else Ld = std::min(-std::ceil(std::log2(D[i] / rad)), (double)(sz - 2)) + 1.0;
      const double P = std::pow(2.0, -lam * (double)(sz - (int)Ld));  // prob(Ld) of :985-990
      const uint32_t a = gen() >> 5, b = gen() >> 6;
      const double u = ((double)a * 67108864.0 + (double)b) * (1.0 / 9007199254740992.0);
      keep[i] = u < P;
    }
  }
  return keep;
}

static void random_sampler(std::vector<double>& px, std::vector<double>& py, double cx, double cy, double colrad,
                           double rowrad, double lam, int lay, double h) {
  const std::vector<char> keep = sampler_mask(px, py, cx, cy, colrad, rowrad, lam, lay, h);
  size_t o = 0;
  for (size_t i = 0; i < px.size(); ++i)
    if (keep[i]) { px[o] = px[i]; py[o] = py[i]; ++o; }
  px.resize(o);
  py.resize(o);
}

// LOCAL_Preset_Skeleton_Info 'rand' (:703-730): the box's own points sampled (each retry on
// the full set with 0.9 lambda) until the sample reaches k0 / 1.1, k0 = ceil(2/3 n) (even
// levels) or ceil(3/4 n); ordered as the 'bdry' rule orders its sets.
static void random_skeleton(const std::vector<double>& X, const std::vector<int>& I_src, double cx, double cy,
                            int lev, double colrad, double rowrad, int layers, double h, double lambda,
                            std::vector<int>& J, int& k) {
  const int n = (int)I_src.size();
  std::vector<double> x(n), y(n);
  for (int i = 0; i < n; ++i) { x[i] = X[2 * (size_t)I_src[i]]; y[i] = X[2 * (size_t)I_src[i] + 1]; }
  const int k0 = (lev % 2 == 0) ? (int)std::ceil((2.0 / 3.0) * n) : (int)std::ceil((3.0 / 4.0) * n);
  double lam = lambda;
  int kk = 0;
  std::vector<char> keep(n, 0);
  while (k0 > 1.1 * kk) {
    keep = sampler_mask(x, y, cx, cy, colrad, rowrad, lam, layers, h);
    kk = 0;
    for (char c : keep) kk += c ? 1 : 0;
    if (k0 > 1.1 * kk) lam = 0.9 * lam;
  }
  std::vector<int> sk, rs;
  for (int i = 0; i < n; ++i) (keep[i] ? sk : rs).push_back(i);
  int nrm;
  double th0;
  level_orientation(lev, nrm, th0);
  std::vector<double> rx(rs.size()), ry(rs.size()), sx(sk.size()), sy(sk.size());
  for (size_t i = 0; i < rs.size(); ++i) { rx[i] = x[rs[i]]; ry[i] = y[rs[i]]; }
  for (size_t i = 0; i < sk.size(); ++i) { sx[i] = x[sk[i]]; sy[i] = y[sk[i]]; }
  const std::vector<int> Jr = orient_residual(rx, ry, nrm);
  const std::vector<int> Js = orient_skeleton(sx, sy, cx, cy, th0);
  J.clear();
  for (int v : Js) J.push_back(sk[v]);
  k = (int)sk.size();
  for (int v : Jr) J.push_back(rs[v]);
}

// LOCAL_Preset_Skeleton_Info 'wdec' (:668-701) over Common/Whitney_decomposition.m: on the
// box's integer grid coordinates, the full boundary layers, then for each finer dyadic scale
// i the lines at distance c_i from the box edges sampled every 2^max(i - ceil(layers/2), 0)
// points (c_i a power of two below Ng, or Ng times one: the Ng x Ng panel grid).
static void whitney_skeleton(const std::vector<double>& X, const std::vector<int>& I_src, double cx, double cy,
                             int lev, double colrad, double rowrad, int layers, double h, int Ng,
                             std::vector<int>& J, int& k) {
  const int n = (int)I_src.size();
  std::vector<long long> c1(n), c2(n);
  long long max1 = 0, max2 = 0;
  for (int i = 0; i < n; ++i) {
    c1[i] = (long long)std::round((-cx + (colrad - h / 2) + X[2 * (size_t)I_src[i]]) / h);
    c2[i] = (long long)std::round((-cy + (rowrad - h / 2) + X[2 * (size_t)I_src[i] + 1]) / h);
    max1 = std::max(max1, c1[i]);
    max2 = std::max(max2, c2[i]);
  }
  const long long dmax = std::max(max1, max2);
  const int depth = (int)std::ceil(std::log2((double)dmax)) + 1;
  const int freq = (layers + 1) / 2;
  const int lNg = (int)std::ceil(std::log2((double)Ng));
  std::vector<char> keep(n);
  for (int i = 0; i < n; ++i)
    keep[i] = c1[i] < layers || max1 - c1[i] < layers || c2[i] < layers || max2 - c2[i] < layers;
  for (int d = 2; d <= depth; ++d) {
    long long ci, mi;
    if ((1LL << (d - 1)) < Ng) {
      ci = 1LL << (d - 1);
      mi = Ng;
    } else {
      ci = (long long)Ng << (d - 1 - lNg);
      mi = 2 * ci;
    }
    const long long e = 1LL << std::max(d - freq, 0);
    for (int i = 0; i < n; ++i) {
      const bool a = (c1[i] == ci || c1[i] == max1 - ci) && (((c2[i] % mi) % e) == 0 || c2[i] == max2 - ci);
      const bool b = (c2[i] == ci || c2[i] == max2 - ci) && (((c1[i] % mi) % e) == 0 || c1[i] == max1 - ci);
      if (a || b) keep[i] = 1;
    }
  }
  std::vector<int> sk, rs;
  for (int i = 0; i < n; ++i) (keep[i] ? sk : rs).push_back(i);
  int nrm;
  double th0;
  level_orientation(lev, nrm, th0);
  std::vector<double> rx(rs.size()), ry(rs.size()), sx(sk.size()), sy(sk.size());
  for (size_t i = 0; i < rs.size(); ++i) { rx[i] = X[2 * (size_t)I_src[rs[i]]]; ry[i] = X[2 * (size_t)I_src[rs[i]] + 1]; }
  for (size_t i = 0; i < sk.size(); ++i) { sx[i] = X[2 * (size_t)I_src[sk[i]]]; sy[i] = X[2 * (size_t)I_src[sk[i]] + 1]; }
  const std::vector<int> Jr = orient_residual(rx, ry, nrm);
  const std::vector<int> Js = orient_skeleton(sx, sy, cx, cy, th0);
  J.clear();
  for (int v : Js) J.push_back(sk[v]);
  k = (int)sk.size();
  for (int v : Jr) J.push_back(rs[v]);
}

// LOCAL_Build_Proxy 'rand' (:883-905): the box's proxy layers sampled until at least
// k0 = ceil(2/3 n) (even levels) or ceil(3/4 n) (odd) points remain, each retry sampling the
// previous sample again with 0.9 lambda.
static void random_proxy(std::vector<double>& px, std::vector<double>& py, int n_src, double cx, double cy,
                         double colrad, double rowrad, int lev, int layers, double h, double lambda) {
  int k0 = (lev % 2 == 0) ? (int)std::ceil((2.0 / 3.0) * n_src) : (int)std::ceil((3.0 / 4.0) * n_src);
  k0 = std::min(k0, (int)px.size());
  double lam = lambda;
  int k = 0, c = 0;
  while (k0 > k && c < 10) {
    random_sampler(px, py, cx, cy, colrad, rowrad, lam, layers, h);
    k = (int)px.size();
    if (k0 > k) lam = 0.9 * lam;
    ++c;
  }
}

// Common/Whitney_decomposition_1Dcurve.m with C = (0, 0), R = (1, 1) (its only call, the
// 'wdec' proxy rule of LOCAL_Build_Proxy :877-881): a quadtree over [-1, 1]^2 refines every
// box that holds more than one point and lies within freq 1.5 rad of the box boundary
// (freq = min(ceil(layers / 2), 2)), marking the points of least and largest integer
// coordinate in each direction (first on ties) of every box it splits; the points within
// layers h of the box boundary are added.  Keeps the marked points of (px, py).
static void whitney_curve(std::vector<double>& px, std::vector<double>& py, double cx, double cy, double colrad,
                          double rowrad, int layers, double h) {
  const int N = (int)px.size();
  if (N == 0) return;
  std::vector<long long> c1(N), c2(N);
  long long mn1 = LLONG_MAX, mx1 = LLONG_MIN, mn2 = LLONG_MAX, mx2 = LLONG_MIN;
  for (int i = 0; i < N; ++i) {
    c1[i] = (long long)std::round((0.0 + (1.0 - h / 2) + px[i]) / h);
    c2[i] = (long long)std::round((0.0 + (1.0 - h / 2) + py[i]) / h);
    mn1 = std::min(mn1, c1[i]); mx1 = std::max(mx1, c1[i]);
    mn2 = std::min(mn2, c2[i]); mx2 = std::max(mx2, c2[i]);
  }
  const long long dmax = std::max(mx1 - mn1, mx2 - mn2);
  const int depth = dmax > 0 ? (int)std::ceil(std::log2((double)dmax)) : 0;
  const int freq = std::min((layers + 1) / 2, 2);
  const double rB[2] = {colrad, rowrad}, cB[2] = {cx, cy};
  std::vector<char> keep(N, 0);
  struct Box { double c0, c1; std::vector<int> J; };
  std::vector<Box> level(1);
  level[0].c0 = 0.0;
  level[0].c1 = 0.0;
  level[0].J.resize(N);
  std::iota(level[0].J.begin(), level[0].J.end(), 0);
  const double cta[4][2] = {{-0.5, -0.5}, {-0.5, 0.5}, {0.5, -0.5}, {0.5, 0.5}};
  for (int lev = 0; lev < depth; ++lev) {
    std::vector<Box> nxt;
    for (const Box& bx : level) {
      const int n = (int)bx.J.size();
      if (n == 0) continue;
      int imn[2] = {0, 0}, imx[2] = {0, 0};
      for (int q = 1; q < n; ++q) {
        if (c1[bx.J[q]] < c1[bx.J[imn[0]]]) imn[0] = q;
        if (c2[bx.J[q]] < c2[bx.J[imn[1]]]) imn[1] = q;
        if (c1[bx.J[q]] > c1[bx.J[imx[0]]]) imx[0] = q;
        if (c2[bx.J[q]] > c2[bx.J[imx[1]]]) imx[1] = q;
      }
      const double d0 = std::fabs(bx.c0 - cB[0]), d1 = std::fabs(bx.c1 - cB[1]);
      const int i = (d1 > d0) ? 1 : 0;
      const double dist = std::fabs(rB[i] - (i ? d1 : d0));
      const double rad = std::ldexp(1.0, -lev);
      if (n > 1 && dist < freq * 1.5 * rad) {
        const long long rowmid = (long long)std::round((0.0 + (1.0 - h / 2) + bx.c0) / h);
        const long long colmid = (long long)std::round((0.0 + (1.0 - h / 2) + bx.c1) / h);
        for (int j = 0; j < 4; ++j) {
          Box ch;
          ch.c0 = bx.c0 + rad * cta[j][0];
          ch.c1 = bx.c1 + rad * cta[j][1];
          for (int q : bx.J) {
            const bool lo1 = c1[q] < rowmid, lo2 = c2[q] < colmid;
            const bool in = (j == 0) ? (lo1 && lo2) : (j == 1) ? (lo1 && !lo2) : (j == 2) ? (!lo1 && lo2) : (!lo1 && !lo2);
            if (in) ch.J.push_back(q);
          }
          nxt.push_back(std::move(ch));
        }
        keep[bx.J[imn[0]]] = keep[bx.J[imn[1]]] = keep[bx.J[imx[0]]] = keep[bx.J[imx[1]]] = 1;
      }
    }
    level.swap(nxt);
  }
  size_t o = 0;
  for (int q = 0; q < N; ++q) {
    const double a0 = std::fabs(px[q] - cx), a1 = std::fabs(py[q] - cy);
    const double dist = std::min(std::fabs(colrad - a0), std::fabs(rowrad - a1));
    const bool bdry = dist < layers * h && a0 < colrad + layers * h && a1 < rowrad + layers * h;
    if (keep[q] || bdry) { px[o] = px[q]; py[o] = py[q]; ++o; }
  }
  px.resize(o);
  py.resize(o);
}

// proxy layers of a level (:360-368): layers + 1 for the Laplace kernel, 2 round(min radius / h)
// for kh > 0; the root keeps params.layers
static int proxy_layers(const hss2d_params& prm, int lev, double colrad, double rowrad, double h) {
  if (lev == 0) return prm.layers;
  if (prm.kp.flag == HSS_SL_H_2D) return 2 * (int)std::lround(std::min(colrad, rowrad) / h);
  return prm.layers + 1;
}

void level_proxy(const hss2d_params& prm, int lev, double cx, double cy, int n_src, std::vector<double>& px,
                 std::vector<double>& py) {
  double colrad, rowrad;
  box_radii(lev, colrad, rowrad);
  const double h = 2.0 / (double)(prm.Ng * prm.npan);
  box_proxy(cx, cy, colrad, rowrad, proxy_layers(prm, lev, colrad, rowrad, h), h, px, py);
  if (prm.proxy_rule == HSS_PROXY_RAND)
    random_proxy(px, py, n_src, cx, cy, colrad, rowrad, lev, prm.layers, h, prm.lambda > 0 ? prm.lambda : 2.0);
  else if (prm.proxy_rule == HSS_PROXY_WDEC)
    whitney_curve(px, py, cx, cy, colrad, rowrad, 2 * prm.layers, h);
}

void build_tree_geometry(const hss2d_params& prm, Tree2D& T, const IdLevelFn& id_level) {
  HSS_REQUIRE(prm.Ng > 0 && prm.npan > 1 && (prm.npan & (prm.npan - 1)) == 0, HSS_ERR_ARG,
              "npan must be a power of two >= 2 and Ng > 0");
  HSS_REQUIRE(prm.layers >= 1, HSS_ERR_ARG, "layers must be >= 1");
  HSS_REQUIRE(prm.kp.flag == HSS_SL_L_2D || prm.kp.flag == HSS_SL_H_2D, HSS_ERR_ARG,
              "HSS2D takes the SL_L_2D and SL_H_2D kernels");
  HSS_REQUIRE(prm.proxy_rule == HSS_PROXY_BDRY || prm.proxy_rule == HSS_PROXY_RAND || prm.proxy_rule == HSS_PROXY_WDEC,
              HSS_ERR_ARG, "unknown proxy rule");
  HSS_REQUIRE(prm.skel_rule == HSS_SKEL_BDRY || prm.skel_rule == HSS_SKEL_RAND || prm.skel_rule == HSS_SKEL_ID ||
                  prm.skel_rule == HSS_SKEL_WDEC,
              HSS_ERR_ARG, "unknown skeleton rule");
  HSS_REQUIRE(prm.skel_rule != HSS_SKEL_ID || prm.kp.flag == HSS_SL_H_2D, HSS_ERR_ARG,
              "the 'ID' skeleton rule is built for kh > 0 trees");
  const int Ng = prm.Ng, np = prm.npan;
  const double hh = 2.0 / (double)(Ng * np);
  const double hp = 2.0 / (double)np;
  const int nlevels = (int)std::lround(2.0 * (std::log((double)np) / std::log(2.0) - 1.0) + 3.0);
  T.depth = nlevels - 1;
  T.h = hh;
  T.N = (long long)np * np * Ng * Ng;
  const int depth = T.depth;
  const int nb = (1 << (depth + 1)) - 1;
  T.nboxes = nb;
  // X_source (HSS_tree_parameters.m:141-162): panel-major, y fastest in a panel
  std::vector<double> z(Ng);
  for (int i = 0; i < Ng; ++i) {
    // linspace(0.5h, Ng h - 0.5h, Ng)
    const double a = 0.5 * hh, b = Ng * hh - 0.5 * hh;
    z[i] = (Ng == 1) ? b : (i == Ng - 1 ? b : a + (double)i * ((b - a) / (double)(Ng - 1)));
  }
  T.X.resize(2 * (size_t)T.N);
  const int J = Ng * Ng;
  for (int pi = 0; pi < np * np; ++pi) {
    const double px = -1.0 + (double)(pi / np) * hp, py = -1.0 + (double)(pi % np) * hp;
    for (int q = 0; q < J; ++q) {
      const int jx = q / Ng, jy = q % Ng;
      T.X[2 * ((size_t)J * pi + q)] = px + z[jx];
      T.X[2 * ((size_t)J * pi + q) + 1] = py + z[jy];
    }
  }
  // centres
  T.cent.assign(2 * (size_t)nb, 0.0);
  for (int lev = 0; lev < depth; ++lev) {
    const double d = 0.5 * std::ldexp(1.0, -(lev / 2));
    for (int b = (1 << lev) - 1; b < (1 << (lev + 1)) - 1; ++b) {
      const double cx = T.cent[2 * b], cy = T.cent[2 * b + 1];
      if (lev % 2 == 0) {
        T.cent[2 * (2 * b + 1)] = cx - d; T.cent[2 * (2 * b + 1) + 1] = cy;
        T.cent[2 * (2 * b + 2)] = cx + d; T.cent[2 * (2 * b + 2) + 1] = cy;
      } else {
        T.cent[2 * (2 * b + 1)] = cx; T.cent[2 * (2 * b + 1) + 1] = cy + d;
        T.cent[2 * (2 * b + 2)] = cx; T.cent[2 * (2 * b + 2) + 1] = cy - d;
      }
    }
  }
  // leaf of each panel: descend from the root with the first point of the panel
  T.leaf_panel.assign(nb, -1);
  for (int pi = 0; pi < np * np; ++pi) {
    const double px = T.X[2 * ((size_t)J * pi)], py = T.X[2 * ((size_t)J * pi) + 1];
    int b = 0;
    for (int lev = 0; lev < depth; ++lev) {
      const double cx = T.cent[2 * b], cy = T.cent[2 * b + 1];
      if (lev % 2 == 0) b = (px < cx) ? 2 * b + 1 : 2 * b + 2;
      else b = (py > cy) ? 2 * b + 1 : 2 * b + 2;
    }
    HSS_REQUIRE(T.leaf_panel[b] < 0, HSS_ERR_ARG, "two panels map to one leaf");
    T.leaf_panel[b] = pi;
  }
  // upward skeleton pass
  const bool helm = (prm.kp.flag == HSS_SL_H_2D);
  T.levels.assign(depth + 1, Level2Geom{});
  std::vector<std::vector<int>> I_sk(nb);
  std::vector<std::vector<int>> I_src(nb);
  long long proxy_base = T.N;
  T.proxy_x.clear();
  T.proxy_y.clear();
  for (int lev = depth; lev >= 0; --lev) {
    Level2Geom& L = T.levels[lev];
    L.lev = lev;
    L.nb = 1 << lev;
    box_radii(lev, L.colrad, L.rowrad);
    L.lay_prox = proxy_layers(prm, lev, L.colrad, L.rowrad, hh);
    const int b0 = (1 << lev) - 1;
    std::vector<std::vector<double>> PX(L.nb), PY(L.nb);
    std::vector<std::vector<int>> Jall(L.nb);
    std::vector<int> kall(L.nb, 0);
    for (int i = 0; i < L.nb; ++i) {
      const int b = b0 + i;
      if (lev == depth) {
        const int pi = T.leaf_panel[b];
        HSS_REQUIRE(pi >= 0, HSS_ERR_ARG, "leaf without panel");
        I_src[b].resize(J);
        for (int q = 0; q < J; ++q) I_src[b][q] = J * pi + q;
      } else {
        I_src[b] = I_sk[2 * b + 1];
        I_src[b].insert(I_src[b].end(), I_sk[2 * b + 2].begin(), I_sk[2 * b + 2].end());
      }
      level_proxy(prm, lev, T.cent[2 * b], T.cent[2 * b + 1], (int)I_src[b].size(), PX[i], PY[i]);
    }
    // kh > 0: the two finest levels take their skeletons from the ID of K(proxies, box)
    L.id_level = helm && (lev >= depth - 1 || prm.skel_rule == HSS_SKEL_ID);
    if (L.id_level) {
      HSS_REQUIRE(id_level != nullptr, HSS_ERR_ARG, "kh > 0 tree without an ID step");
      std::vector<std::vector<int>> boxes(I_src.begin() + b0, I_src.begin() + b0 + L.nb);
      std::vector<std::vector<int>> perm;
      std::vector<int> kb;
      id_level(lev, boxes, PX, PY, perm, kb);
      HSS_REQUIRE((int)perm.size() == L.nb && (int)kb.size() == L.nb, HSS_ERR_ARG, "ID step: one result per box");
      const int kl = *std::max_element(kb.begin(), kb.end());
      int nrm;
      double th0;
      level_orientation(lev, nrm, th0);
      for (int i = 0; i < L.nb; ++i) {
        const int b = b0 + i, n = (int)I_src[b].size(), k = kb[i];
        HSS_REQUIRE((int)perm[i].size() == n && k >= 0 && kl <= n, HSS_ERR_ARG, "ID permutation size");
        const double cx = T.cent[2 * b], cy = T.cent[2 * b + 1];
        auto X_of = [&](int pos, int dim) { return T.X[2 * (size_t)I_src[b][perm[i][pos]] + dim]; };
        // the uniform level layout: the kl - k residual points nearest the boundary join the
        // skeleton with zero rows of T (ties in the ID's residual order)
        std::vector<double> d(n - k);
        for (int q = k; q < n; ++q)
          d[q - k] = std::min(L.colrad - std::fabs(X_of(q, 0) - cx), L.rowrad - std::fabs(X_of(q, 1) - cy));
        std::vector<int> o;
        stable_argsort(d, o);
        std::vector<char> take(n - k, 0);
        std::vector<int> skp, rsp;  // positions in perm
        std::vector<int> rows, cols;  // raw T row / column of each
        for (int q = 0; q < k; ++q) { skp.push_back(q); rows.push_back(q); }
        for (int q = 0; q < kl - k; ++q) { take[o[q]] = 1; skp.push_back(k + o[q]); rows.push_back(-1); }
        for (int q = 0; q < n - k; ++q)
          if (!take[q]) { rsp.push_back(k + q); cols.push_back(q); }
        // LOCAL_Non_Preset_Skeleton_Info :629-656: skeleton points around the centre,
        // residual points along the interface; T = T(Js, Jr)
        std::vector<double> sx(kl), sy(kl), rx(n - kl), ry(n - kl);
        for (int q = 0; q < kl; ++q) { sx[q] = X_of(skp[q], 0); sy[q] = X_of(skp[q], 1); }
        for (int q = 0; q < n - kl; ++q) { rx[q] = X_of(rsp[q], 0); ry[q] = X_of(rsp[q], 1); }
        const std::vector<int> Js = orient_skeleton(sx, sy, cx, cy, th0);
        const std::vector<int> Jr = orient_residual(rx, ry, nrm);
        for (int v : Js) { Jall[i].push_back(perm[i][skp[v]]); L.id_rows.push_back(rows[v]); }
        for (int v : Jr) { Jall[i].push_back(perm[i][rsp[v]]); L.id_cols.push_back(cols[v]); }
        kall[i] = kl;
      }
    } else {
      for (int i = 0; i < L.nb; ++i) {
        const int b = b0 + i;
        if (prm.transinv && i > 0) {
          // translation-invariant mode: every box of the level uses box 0's J and k
          // (INFO_TREE.LEV(l) of HSS2D_build_tree_nsym.m:438-449, 499-540)
          Jall[i] = Jall[0];
          kall[i] = kall[0];
        } else if (prm.skel_rule == HSS_SKEL_WDEC) {
          whitney_skeleton(T.X, I_src[b], T.cent[2 * b], T.cent[2 * b + 1], lev, L.colrad, L.rowrad, prm.layers,
                           hh, prm.Ng, Jall[i], kall[i]);
        } else if (prm.skel_rule == HSS_SKEL_RAND) {
          random_skeleton(T.X, I_src[b], T.cent[2 * b], T.cent[2 * b + 1], lev, L.colrad, L.rowrad, prm.layers,
                          hh, prm.lambda > 0 ? prm.lambda : 2.0, Jall[i], kall[i]);
        } else {
          preset_skeleton(T.X, I_src[b], T.cent[2 * b], T.cent[2 * b + 1], lev, L.colrad, L.rowrad, prm.layers,
                          hh, Jall[i], kall[i]);
        }
      }
      // above the ID levels of a kh > 0 tree the boundary-layer counts differ from box to
      // box; every box takes the level's largest count, promoting the residual points
      // nearest its boundary (ties in the residual order), then both sets are ordered as the
      // preset rule orders them
      const int kl = *std::max_element(kall.begin(), kall.end());
      int nrm;
      double th0;
      level_orientation(lev, nrm, th0);
      for (int i = 0; i < L.nb; ++i) {
        if (kall[i] == kl) continue;
        const int b = b0 + i, kb = kall[i], n = (int)I_src[b].size();
        HSS_REQUIRE(n >= kl, HSS_ERR_ARG, "box smaller than its level's skeleton");
        const double cx = T.cent[2 * b], cy = T.cent[2 * b + 1];
        std::vector<int> rs(Jall[i].begin() + kb, Jall[i].end());
        std::vector<double> d(rs.size());
        for (size_t q = 0; q < rs.size(); ++q) {
          const size_t g = (size_t)I_src[b][rs[q]];
          d[q] = std::min(L.colrad - std::fabs(T.X[2 * g] - cx), L.rowrad - std::fabs(T.X[2 * g + 1] - cy));
        }
        std::vector<int> o;
        stable_argsort(d, o);
        std::vector<char> take(rs.size(), 0);
        std::vector<int> sk(Jall[i].begin(), Jall[i].begin() + kb), rest;
        for (int q = 0; q < kl - kb; ++q) {
          take[o[q]] = 1;
          sk.push_back(rs[o[q]]);
        }
        for (size_t q = 0; q < rs.size(); ++q)
          if (!take[q]) rest.push_back(rs[q]);
        auto coords = [&](const std::vector<int>& v, std::vector<double>& x, std::vector<double>& y) {
          x.resize(v.size());
          y.resize(v.size());
          for (size_t q = 0; q < v.size(); ++q) {
            x[q] = T.X[2 * (size_t)I_src[b][v[q]]];
            y[q] = T.X[2 * (size_t)I_src[b][v[q]] + 1];
          }
        };
        std::vector<double> x, y;
        coords(sk, x, y);
        const std::vector<int> Js = orient_skeleton(x, y, cx, cy, th0);
        coords(rest, x, y);
        const std::vector<int> Jr = orient_residual(x, y, nrm);
        Jall[i].clear();
        for (int v : Js) Jall[i].push_back(sk[v]);
        for (int v : Jr) Jall[i].push_back(rest[v]);
        kall[i] = kl;
      }
    }
    L.poff.assign(1, 0);
    for (int i = 0; i < L.nb; ++i) {
      const int b = b0 + i;
      const std::vector<int>& Jb = Jall[i];
      const int kb = kall[i];
      const int n = (int)I_src[b].size();
      if (i == 0) { L.n = n; L.k = kb; L.p = 0; }
      HSS_REQUIRE(n == L.n && kb == L.k, HSS_ERR_ARG, "non-uniform level sizes");
      I_sk[b].resize(kb);
      for (int q = 0; q < kb; ++q) I_sk[b][q] = I_src[b][Jb[q]];
      for (int q = 0; q < n; ++q) {
        L.J.push_back(Jb[q]);
        L.Isrc.push_back(I_src[b][q]);
        L.IsrcJ.push_back(I_src[b][Jb[q]]);
      }
      const std::vector<double>& px = PX[i];
      const std::vector<double>& py = PY[i];
      L.p = std::max(L.p, (int)px.size());
      L.poff.push_back(L.poff.back() + (int)px.size());
      for (size_t q = 0; q < px.size(); ++q) {
        L.proxy.push_back((int)(proxy_base + (long long)T.proxy_x.size()));
        T.proxy_x.push_back(px[q]);
        T.proxy_y.push_back(py[q]);
      }
    }
    L.p_uniform = true;
    for (int i = 0; i < L.nb; ++i) L.p_uniform = L.p_uniform && (L.poff[i + 1] - L.poff[i] == L.p);
  }
  HSS_REQUIRE(proxy_base + (long long)T.proxy_x.size() < (1LL << 31), HSS_ERR_ARG,
              "point table exceeds 2^31 entries");
}

}  // namespace hss
