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
#include "hss2d_tree.h"

#include <algorithm>
#include <cmath>
#include <numeric>

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
  int nrm, tan;
  double th0;
  if (lev % 2 == 0) { nrm = 0; tan = 1; th0 = M_PI / 2; }
  else { nrm = 1; tan = 0; th0 = 0.0; }
  // residual: sort by normal coordinate, then stably by -tangential
  std::vector<int> J1, J2;
  {
    std::vector<double> key(rs.size());
    for (size_t i = 0; i < rs.size(); ++i) key[i] = X[2 * (size_t)I_src[rs[i]] + nrm];
    stable_argsort(key, J1);
    std::vector<double> key2(rs.size());
    for (size_t i = 0; i < rs.size(); ++i) key2[i] = -X[2 * (size_t)I_src[rs[J1[i]]] + tan];
    stable_argsort(key2, J2);
  }
  std::vector<int> rs_sorted(rs.size());
  for (size_t i = 0; i < rs.size(); ++i) rs_sorted[i] = rs[J1[J2[i]]];
  // skeleton: polar sort around the centre
  std::vector<double> th(sk.size()), rho(sk.size());
  for (size_t i = 0; i < sk.size(); ++i) {
    const double dx = X[2 * (size_t)I_src[sk[i]]] - cx, dy = X[2 * (size_t)I_src[sk[i]] + 1] - cy;
    double t = std::atan2(dy, dx);
    if (t < th0) t = t + 2.0 * M_PI;
    th[i] = t;
    rho[i] = std::hypot(dx, dy);
  }
  stable_argsort(rho, J1);
  std::vector<double> th1(sk.size());
  for (size_t i = 0; i < sk.size(); ++i) th1[i] = th[J1[i]];
  stable_argsort(th1, J2);
  J.clear();
  for (size_t i = 0; i < sk.size(); ++i) J.push_back(sk[J1[J2[i]]]);
  k = (int)sk.size();
  for (int v : rs_sorted) J.push_back(v);
}

void build_tree_geometry(const hss2d_params& prm, Tree2D& T) {
  HSS_REQUIRE(prm.Ng > 0 && prm.npan > 1 && (prm.npan & (prm.npan - 1)) == 0, HSS_ERR_ARG,
              "npan must be a power of two >= 2 and Ng > 0");
  HSS_REQUIRE(prm.layers >= 1, HSS_ERR_ARG, "layers must be >= 1");
  HSS_REQUIRE(prm.kp.flag == HSS_SL_L_2D, HSS_ERR_ARG, "HSS2D supports the SL_L_2D kernel family");
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
    int lay = prm.layers;
    if (lev > 0) lay = prm.layers + 1;  // SL_L_2D rule of :360-368
    L.lay_prox = lay;
    const int b0 = (1 << lev) - 1;
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
      std::vector<int> Jb;
      int kb = 0;
      if (prm.transinv && i > 0) {
        // translation-invariant mode: every box of the level uses box 0's J and k
        // (INFO_TREE.LEV(l) of HSS2D_build_tree_nsym.m:438-449, 499-540)
        Jb.assign(L.J.begin(), L.J.begin() + L.n);
        kb = L.k;
      } else {
        preset_skeleton(T.X, I_src[b], T.cent[2 * b], T.cent[2 * b + 1], lev, L.colrad, L.rowrad,
                        prm.layers, hh, Jb, kb);
      }
      const int n = (int)I_src[b].size();
      if (i == 0) { L.n = n; L.k = kb; }
      HSS_REQUIRE(n == L.n && kb == L.k, HSS_ERR_ARG, "non-uniform level sizes");
      I_sk[b].resize(kb);
      for (int q = 0; q < kb; ++q) I_sk[b][q] = I_src[b][Jb[q]];
      for (int q = 0; q < n; ++q) {
        L.J.push_back(Jb[q]);
        L.Isrc.push_back(I_src[b][q]);
        L.IsrcJ.push_back(I_src[b][Jb[q]]);
      }
      std::vector<double> px, py;
      box_proxy(T.cent[2 * b], T.cent[2 * b + 1], L.colrad, L.rowrad, lay, hh, px, py);
      if (i == 0) L.p = (int)px.size();
      HSS_REQUIRE((int)px.size() == L.p, HSS_ERR_ARG, "non-uniform proxy sizes");
      for (size_t q = 0; q < px.size(); ++q) {
        L.proxy.push_back((int)(proxy_base + (long long)T.proxy_x.size()));
        T.proxy_x.push_back(px[q]);
        T.proxy_y.push_back(py[q]);
      }
    }
  }
  HSS_REQUIRE(proxy_base + (long long)T.proxy_x.size() < (1LL << 31), HSS_ERR_ARG,
              "point table exceeds 2^31 entries");
}

}  // namespace hss
