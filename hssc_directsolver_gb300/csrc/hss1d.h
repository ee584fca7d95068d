// HSS1D solver state.  See hss1d.cu.
//
// A handle holds a forest: one or many independent curves ("problems") whose
// trees share one global box numbering, one point table and one set of device
// arenas, so every level of every problem is processed by the same launches.
#pragma once

#include <array>
#include <map>
#include <vector>

#include "dense.cuh"
#include "kgen.cuh"
#include "mlp.h"

namespace hss {

// Generic small block move: mode 0 row gather dst(i,c) = src(idx[i], c);
// mode 1 column gather dst(i,c) = src(i, idx[c]); mode 2 row scatter
// dst(idx[i], c) (+)= src(i, c); mode 3 transpose dst(c,i) = src(i,c); on real 2 x 2
// embeddings of complex blocks, mode 4 the conjugate and mode 5 the plain transpose
// (dst(c,i) = (-1)^(i+c) src(i,c)).
// idx == nullptr means identity.
struct MoveP {
  const double* src;
  double* dst;
  const int* idx;
  int nrows, ncols, lds, ldd, mode, accumulate;
};
void move_batched(const MoveP* dP, int batch, cudaStream_t s);

// A fixed sequence of batched skinny products and block moves (one inverse or
// forward apply for a given number of right-hand sides); descriptors stay on the
// device so the sequence can be replayed as a CUDA graph.
struct Plan1 {
  struct Step {
    bool move = false;
    DevBuf<GemmP<double>> g;
    DevBuf<MoveP> m;
    DevBuf<double> part;
    int batch = 0, maxM = 0, maxN = 0, ksplit = 1;
    double alpha = 1.0, beta = 0.0;
  };
  std::vector<Step> steps;
  bool df = false;  // operands stored as float pairs, products on the FP32 pipes
  void gemm(const std::vector<GemmP<double>>& P, double alpha, double beta, cudaStream_t s);
  void moves(const std::vector<MoveP>& mv, cudaStream_t s);
  void run(cudaStream_t s) const;
  int launches() const;
};

struct HSS1D {
  // forest: global box ids; box_constants.m rows LEVEL..END2 per box
  long long Ntot = 0;
  int nprob = 0, nboxes = 0, leaf = 0, maxlev = 0;
  double acc = 0;
  bool sym = false;  // fsym compression: one ID per box, incoming skeletons = outgoing
  // rectangular K(Xin, Xout) (HSS1D_compress_rectangular_nsym): the columns follow the tree
  // of off/cnt over the Ntot points of Xout, the rows a tree of the same shape with
  // off_in/cnt_in over the Mtot points of Xin (K_HSS rows 16:17) and row-side skeleton sizes
  // nskel_in/kskel_in (rows 18:19).  In the point table Xin follows Xout, so I_SKDN holds
  // Ntot + (row index).  Square handles keep these empty and read the column side.
  bool rect = false;
  long long Mtot = 0;
  std::vector<int> off_in, cnt_in, nskel_in, kskel_in;
  std::vector<long long> oTd, oJd;  // T_DN / TDNT and J_DN arena offsets of the row side
  const std::vector<int>& rk() const { return rect ? kskel_in : kskel; }
  const std::vector<int>& rn() const { return rect ? nskel_in : nskel; }
  const std::vector<int>& roff() const { return rect ? off_in : off; }
  const std::vector<int>& rcnt() const { return rect ? cnt_in : cnt; }
  const std::vector<long long>& roT() const { return rect ? oTd : oT; }
  const std::vector<long long>& roJ() const { return rect ? oJd : oJ; }
  long long rows() const { return rect ? Mtot : Ntot; }
  bool id_df = false;  // the IDs' pivoted QR in double-float arithmetic (k_id_adaptive_df)
  bool id_step_test = false;  // every ID's pivoted QR tests the truncation rule at every step
  bool kernel_op = false;  // the handle compresses the kernel matrix of its point table (compress)
  // complex (HSS_SL_H_2D) matrix held as its real 2 x 2 embedding: point i is unknowns 2i, 2i + 1
  // (re, im), and Ntot, off, cnt, nskel, kskel, the skeleton sets and J count unknowns; T_DN
  // holds the embedding of conj(T_DN), so that the real L = [I; T_DN^T] is the embedding of
  // the complex L = [I; T_DN.'] (HSS1D_invert_nsym.m:70-72)
  bool cplx = false;
  std::vector<long long> pN, pbase;   // points per problem, first global point
  std::vector<int> proot;              // root box of each problem
  std::vector<unsigned long long> pseed;
  std::vector<int> prob, level, parent, c1, c2, off, cnt;  // off = global point index
  // skeletons (host copies, global point indices)
  std::vector<int> nskel, kskel;
  std::vector<std::vector<int>> I_SKUP, I_SKDN, J_UP, J_DN;
  std::vector<double> X;  // Ntot x 6 row-major
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
  std::vector<long long> oL, oR, oD, oE, oFT;
  std::vector<int> ktop;
  bool inverted = false;
  // solve workspaces, staging (Ntot x 8) and cached plans / graphs per RHS count
  DevBuf<double> v1, v2, v3, Xs, Ys, ir_y, ir_res, ir_dd;
  // host-buffer entry points: device copies of the caller's vectors; refinement partials
  DevBuf<double> io_in, io_out, ir_part;
  PinnedBuf ir_host;
  std::map<int, Plan1> inv_plans, fwd_plans;
  GraphCache g_inv, g_fwd;
  bool use_graphs = true;
  // HSS_PREC_DFLOAT: solve products in double-float arithmetic on float-pair copies
  int precision = HSS_PREC_FP64;
  DevBuf<double> Linv_df, Rinv_df, Dinv_df, FTinv_df, T_UP_df, TDNT_df, M_SELF_df, M_SIB_df;
  void set_precision(int prec);
  void make_df();
  bool dfm() const { return precision == HSS_PREC_DFLOAT || precision == HSS_PREC_DFLOAT_INV; }
  bool dfinv() const { return precision == HSS_PREC_DFLOAT_INV; }
  void clear_plans() {
    g_inv.clear();
    g_fwd.clear();
    inv_plans.clear();
    fwd_plans.clear();
  }
  Plan1& inv_plan(int r);
  Plan1& fwd_plan(int r);
  void ensure_work();
  // ID problem shapes of the last compress: (m_out, m_in, n, k) per non-root box
  std::vector<int> census;
  // rank-predictor features per box (NFEAT floats, known before the box's ID)
  static constexpr int NFEAT = 8;
  std::vector<float> feat;
  // learned-rank statistics: QR steps done, QR steps a full factorization takes, full reruns
  long long qr_steps = 0, qr_steps_full = 0;
  int reruns = 0;
  // host wall seconds of the last compress: setup (trees, neighbours, points), level
  // geometry, level uploads + launches, level GPU work up to the sync, level bookkeeping,
  // final blocks
  static constexpr int NPHASE = 6;
  double phase_s[NPHASE] = {};

  HSS1D();
  ~HSS1D();
  // problem p: X_p is an N_p x 6 column-major block [x y nx ny w kappa] (ld ldx_p)
  void compress(int nprob, const long long* N, const double* const* Xp, const long long* ldx, int leaf, double acc,
                const hss_kernel_params& kp, const unsigned long long* seeds, MLP* mlp = nullptr, bool sym = false);
  void invert();
  // the M x N matrix K(Xin, Xout) (HSS1D_compress_rectangular_nsym); Xin / Xout are M x 6 /
  // N x 6 column-major blocks [x y nx ny w kappa]
  void append_tree(int p, int base, int n);
  void compress_rect(long long M, const double* Xin, long long ldin, long long N, const double* Xout,
                     long long ldout, int leaf, double acc, const hss_kernel_params& kp, unsigned long long seed);
  // U V^T (U, V: N x r column-major) on the halving tree (HSS1D_compressLR_nsym)
  void compress_lr(long long N, int r, const double* U, long long ldu, const double* V, long long ldv, int leaf,
                   double acc, unsigned long long seed);
  void pack_T(const std::vector<DevBuf<double>>& Tkeep, const std::vector<std::array<long long, 2>>& Toff,
              const std::vector<int>& Tlev);
  // *this = A + B for two square handles on one forest (HSS1D_sum_nsym)
  void sum(const HSS1D& A, const HSS1D& B, double acc);
  // *this = A with its ranks reduced to acc (HSS1D_recompress_nsym)
  void recompress(const HSS1D& A, double acc);
  // K = the inverse in compressed format (HSS1D_transforminv_nsym)
  void transforminv(HSS1D& K);
  // K = the transpose in compressed format (HSS1D_transpose)
  void transpose(HSS1D& K) const;
  // M_SELF and M_SIB scaled by c in place (HSS1D_scalarmult); the inverse is dropped
  void scalarmult(double c);
  // the dense N_p x N_p matrix of problem p, column-major host array (HSS1D_dense_matrix)
  void dense_matrix(int p, double* Kd);
  void applyinv_device(const double* dX, double* dY, int nrhs);
  void apply_device(const double* dX, double* dY, int nrhs);
  void solve_device(const double* df, double* dx, int nrhs, double tol, int maxit, double* relres, int* iters);
  bool is_leaf(int b) const { return c1[b] < 0 && c2[b] < 0; }
};

}  // namespace hss

struct hss1d_matrix {
  hss::HSS1D* impl;
};
