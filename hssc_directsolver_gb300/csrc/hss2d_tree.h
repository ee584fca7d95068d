// HSS2D tree geometry (host side): see hss2d_tree.cpp.
#pragma once

#include <vector>

#include "common.cuh"

namespace hss {

// One tree level.  Every box of a level has the same n, k and proxy count on
// the uniform grid; arrays are box-major (box i of the level at i*n).
struct Level2Geom {
  int lev = 0, nb = 0, n = 0, k = 0, p = 0, lay_prox = 0;
  double colrad = 0, rowrad = 0;
  std::vector<int> J;      // local permutation [I_sk I_rs], nb*n
  std::vector<int> Isrc;   // global ids of I_src (reference order), nb*n
  std::vector<int> IsrcJ;  // global ids in J order, nb*n
  std::vector<int> proxy;  // point-table ids of the box proxies, nb*p
};

struct Tree2D {
  int depth = 0, nboxes = 0;
  long long N = 0;
  double h = 0;
  std::vector<double> X;       // N x 2 row-major (x, y)
  std::vector<double> cent;    // nboxes x 2
  std::vector<int> leaf_panel; // panel id of each leaf box (-1 for parents)
  std::vector<Level2Geom> levels;
  std::vector<double> proxy_x, proxy_y;  // point-table entries N.. (proxies)
};

void build_tree_geometry(const hss2d_params& prm, Tree2D& T);
void box_proxy(double cx, double cy, double colrad, double rowrad, int layers, double h,
               std::vector<double>& px, std::vector<double>& py);

}  // namespace hss
