// HSS2D tree geometry (host side): see hss2d_tree.cpp.
#pragma once

#include <functional>
#include <vector>

#include "common.cuh"

namespace hss {

// One tree level.  Every box of a level has the same n and k on the uniform grid (and the
// same proxy count with 'bdry' proxies); arrays are box-major (box i of the level at i*n).
struct Level2Geom {
  int lev = 0, nb = 0, n = 0, k = 0, p = 0, lay_prox = 0;
  double colrad = 0, rowrad = 0;
  std::vector<int> J;      // local permutation [I_sk I_rs], nb*n
  std::vector<int> Isrc;   // global ids of I_src (reference order), nb*n
  std::vector<int> IsrcJ;  // global ids in J order, nb*n
  std::vector<int> proxy;  // point-table ids of the box proxies, box i at poff[i]..poff[i+1]
  std::vector<int> poff;   // nb + 1 offsets into proxy; p = the largest count
  bool p_uniform = true;   // every box has p proxies
  // kh > 0: skeletons from the ID (the two finest levels).  Row r of box i's T is row
  // id_rows[i k + r] of the ID's T (-1: a zero row, a point promoted to the level's rank),
  // column c is its column id_cols[i (n-k) + c] (complex points)
  bool id_level = false;
  std::vector<int> id_rows, id_cols;
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

// The ID step of the kh > 0 levels (HSS2D_build_tree_nsym.m:614-627): for the level's boxes
// (source point ids) and proxies (coordinates), the ID's column order per box (local indices,
// skeleton first) and its rank per box.
using IdLevelFn = std::function<void(int lev, const std::vector<std::vector<int>>& I_src,
                                     const std::vector<std::vector<double>>& px,
                                     const std::vector<std::vector<double>>& py,
                                     std::vector<std::vector<int>>& perm, std::vector<int>& k)>;
void build_tree_geometry(const hss2d_params& prm, Tree2D& T, const IdLevelFn& id_level = nullptr);
// LOCAL_Build_Proxy of one box of level lev centred at (cx, cy) with n_src sources
void level_proxy(const hss2d_params& prm, int lev, double cx, double cy, int n_src, std::vector<double>& px,
                 std::vector<double>& py);
void box_proxy(double cx, double cy, double colrad, double rowrad, int layers, double h,
               std::vector<double>& px, std::vector<double>& py);

}  // namespace hss
