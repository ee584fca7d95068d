// HSS1D solver state.  See hss1d.cu.
#pragma once

#include <vector>

#include "dense.cuh"
#include "kgen.cuh"

namespace hss {

// Generic small block move: mode 0 row gather dst(i,c) = src(idx[i], c);
// mode 1 column gather dst(i,c) = src(i, idx[c]); mode 2 row scatter
// dst(idx[i], c) (+)= src(i, c).  idx == nullptr means identity.
struct MoveP {
  const double* src;
  double* dst;
  const int* idx;
  int nrows, ncols, lds, ldd, mode, accumulate;
};
void move_batched(const MoveP* dP, int batch, cudaStream_t s);

struct HSS1D {
  // tree (box_constants.m rows LEVEL..END2)
  long long N = 0;
  int nboxes = 0, leaf = 0, maxlev = 0;
  double acc = 0;
  unsigned long long seed = 0;
  std::vector<int> level, parent, c1, c2, off, cnt;
  // skeletons (host copies, 0-based)
  std::vector<int> nskel, kskel;
  std::vector<std::vector<int>> I_SKUP, I_SKDN, J_UP, J_DN;
  std::vector<double> X;  // N x 6 row-major
  hss_kernel_params kp{};
  KernelDev kdev{};
  PointTable pts;
  cudaStream_t stream = nullptr;
  // device arenas with per-box offsets
  DevBuf<double> T_UP, T_DN, TDNT, M_SELF, M_SIB;
  std::vector<long long> oT, oSelf, oSib;
  DevBuf<int> JUPd, JDNd;
  std::vector<long long> oJ;
  // inverse factors
  DevBuf<double> Linv, Rinv, Dinv, Einv, FTinv;
  std::vector<long long> oL, oR, oD, oE;
  int ktop = 0;
  bool inverted = false;
  // solve workspaces: per-box vectors (k x 8) for up/down passes
  DevBuf<double> v1, v2, v3, qs, ys;
  std::vector<long long> oV;  // per-level stacked offsets (rows), by box

  HSS1D();
  ~HSS1D();
  void compress(const double* Xh, long long N, long long ldx, int leaf, double acc, const hss_kernel_params& kp,
                unsigned long long seed);
  void invert();
  void applyinv_device(const double* dX, double* dY, int nrhs);
  void apply_device(const double* dX, double* dY, int nrhs);
  bool is_leaf(int b) const { return c1[b] < 0 && c2[b] < 0; }
};

}  // namespace hss

struct hss1d_matrix {
  hss::HSS1D* impl;
};
