// Kernel-matrix generation (Common/Kernel_Eval.m) into batched blocks.
#pragma once

#include "common.cuh"

namespace hss {

// Block b: out[i + j*ld] = K(target ti[i], source si[j])   (trans = 0)
//          out[j + i*ld] = K(target ti[i], source si[j])   (trans = 1)
// Indices address the device point table.
template <typename R>
struct KgenP {
  const int* ti;
  const int* si;
  int m, n;
  R* out;
  int ld;
  int trans;
};

// Point table: coordinates plus the per-point modulation values b(p), c(p)
// and the double-layer source data.
struct PointTable {
  DevBuf<double> x, y, nx, ny, w, kap, bval, cval;
  int count = 0;
  void upload(const std::vector<double>& hx, const std::vector<double>& hy,
              const std::vector<double>& hnx, const std::vector<double>& hny,
              const std::vector<double>& hw, const std::vector<double>& hkap,
              const hss_kernel_params& kp, cudaStream_t s);
  // allocate n entries (contents undefined), then fill entries [first, first+n) piecewise
  void reserve(size_t n);
  void upload_range(size_t first, size_t n, const double* hx, const double* hy, const double* hnx,
                    const double* hny, const double* hw, const double* hkap, const hss_kernel_params& kp,
                    cudaStream_t s);
};

struct PointView {
  const double *x, *y, *nx, *ny, *w, *kap, *bval, *cval;
};

inline PointView view(const PointTable& t) {
  return PointView{t.x.p, t.y.p, t.nx.p, t.ny.p, t.w.p, t.kap.p, t.bval.p, t.cval.p};
}

// modulation f(p) = 1 + alpha*exp(-isig*|p-p0|^2) evaluated on the host
double modulation(double alpha, double x0, double y0, double isig, double px, double py);
// b(p) (which = 0) or c(p) (which = 1) of the kernel parameters, any HSS_MOD_* form
double modulation(const hss_kernel_params& kp, int which, double px, double py);

// Complex blocks (HSS_SL_H_2D): out[2 (i + j ld)] = Re, [+1] = Im of K(ti[i], si[j])
struct KgenCP {
  const int* ti;
  const int* si;
  int m, n;
  double* out;
  long long ld;
};
void kgen_complex_batched(const KgenCP* dP, int batch, long long maxEntries, const PointView& pts,
                          const HelmDev& k, cudaStream_t s);

template <typename R>
void kgen_batched(const KgenP<R>* dP, int batch, long long maxEntries, const PointView& pts,
                  const KernelDev& k, cudaStream_t s);

// Kernel matrix times vectors without forming the matrix, in FP64 (the refinement residual
// of Common/Iterative_Refinement.m:20-35 against the kernel matrix itself): problem b
// computes u(i, c) = sum_j K(t0 + i, s0 + j) q(j, c), i < m, j < n, c < nrhs (<= 8), over
// the point table, with the entries of kernel_entry (SL_L_2D or DL_L_2D).  The sources are
// split over blocks; the partial sums are added in a fixed order.  HSS_SL_H_2D: rows and
// columns count embedded (real) entries, m, n, t0 and s0 even, q and u interleaved complex.
struct KmvP {
  int t0, m, s0, n;
  const double* q;
  int ldq;
  double* u;
  int ldu;
};
void kernel_matvec(const KmvP* dP, int batch, int maxM, int maxN, int nrhs, const PointView& pts, const KernelDev& k,
                   DevBuf<double>& part, cudaStream_t s);

}  // namespace hss
