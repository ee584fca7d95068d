// HSS2D solver state (device side).  See hss2d.cu.
#pragma once

#include <map>
#include <memory>
#include <type_traits>
#include <vector>

#include "dense.cuh"
#include "hss2d_tree.h"
#include "kgen.cuh"
#include "skinny_tc.cuh"

namespace hss {

// A fixed sequence of batched skinny products (one inverse or forward apply
// pass for a given number of right-hand sides); descriptors stay on the device.
template <typename R>
struct SolvePlan {
  struct Step {
    DevBuf<GemmP<R>> d;
    DevBuf<SegGemmP> dseg;  // segmented products (df plans only)
    DevBuf<R> part;  // split-K partial sums
    int batch = 0, maxM = 0, maxN = 0, maxK = 0, ksplit = 1;
    R alpha = R(1), beta = R(0);
    int side = 0;          // with streams: 0 the critical stream, 1 the side stream
    std::vector<int> deps; // earlier steps (indices) this one waits for
    bool rec = false;      // a later step waits for this one
  };
  std::vector<Step> steps;
  // set: the steps are issued on two streams (fork from and join back to run()'s stream)
  std::shared_ptr<PlanStreams> streams;
  std::vector<TcStep> tc_steps;  // tensor-core products (HSS_PREC_TC inverse applies)
  bool df = false;  // FP64 operands stored as float pairs, products on the FP32 pipes
  void run_step(const Step& st, cudaStream_t s) const;
  // time each step at K-split counts around the heuristic's and keep the fastest
  // (a step must run at least 2% faster than the heuristic's choice to replace it)
  void tune(cudaStream_t s);
  void add(const std::vector<GemmP<R>>& P, R alpha, R beta, cudaStream_t s);
  // C = alpha * sum_s sign_s A_s B_s + beta * C in one launch (df plans only)
  void add_seg(const std::vector<SegGemmP>& P, R alpha, R beta, cudaStream_t s);
  void run(cudaStream_t s) const;
  int launches() const {
    int n = 0;
    for (auto& st : steps) n += (st.ksplit > 1) ? 2 : 1;
    for (auto& st : tc_steps) n += st.launches();
    return n;
  }
};

struct Level2Dev {
  DevBuf<int> J, Isrc, IsrcJ, proxy;
  // forward operator, FP64
  DevBuf<double> Tup, Tdn, TdnT;  // k x (n-k) (ld k), k x (n-k), (n-k) x k
  DevBuf<double> Bself;           // leaves: n x n
  DevBuf<double> B12, B21;        // parents: kc x kc
  // inverse factors: 0 FI (n x n), 1 E (k x k), 2 U (k x n), 3 G (n x k), 4 GE (n x k)
  DevBuf<double> fd[5];
  DevBuf<float> ff[5];
  // HSS_PREC_DFLOAT: the same FP64 factors and forward blocks as float pairs (8 bytes each)
  DevBuf<double> fdf[5];
  DevBuf<double> Tup_df, TdnT_df, Bself_df, B12_df, B21_df;
  // HSS_PREC_TC: bf16 digit slices (tc_pack) of U (upward products) and of
  // [FI, -G, GE] (downward products, FI alone at the root), per factor box, with row exponents
  DevBuf<unsigned char> tcU, tcD;
  DevBuf<int> tcUe, tcDe;
  size_t tcU_box = 0, tcD_box = 0;  // packed bytes per factor box
  // inverse-apply vectors: 0 phi_up, 1 phi_dn (nb*k x 8)
  DevBuf<double> vd[2];
  DevBuf<float> vf[2];
  // forward-apply vectors (FP64)
  DevBuf<double> upF, dnF, rsF, tmF;
  double rdiag_min = 0, rdiag_max = 0;

  template <typename R>
  DevBuf<R>& fac(int i) {
    if constexpr (std::is_same<R, double>::value) return fd[i];
    else return ff[i];
  }
  template <typename R>
  DevBuf<R>& vec(int i) {
    if constexpr (std::is_same<R, double>::value) return vd[i];
    else return vf[i];
  }
};

struct FwdPlan {
  std::vector<SolvePlan<double>> up, lam, eta;
  // two streams: events 0..depth after each level's upward product, depth+1.. after each
  // level's sibling (leaf: self) products
  std::shared_ptr<PlanStreams> streams;
};

struct HSS2D {
  hss2d_params prm;
  Tree2D geo;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  PointTable pts;
  KernelDev kdev{};
  std::vector<Level2Dev> L;
  bool tree_built = false, compressed = false, inverted = false;
  // staging (N x 8): FP64 in/out, FP32 in/out, residual, correction
  DevBuf<double> Xd, Yd, Rd, Dd;
  // host-buffer entry points: device copies of the caller's vectors; refinement partials
  DevBuf<double> io_in, io_out, ir_part;
  PinnedBuf ir_host;
  DevBuf<float> Xf, Yf;
  std::map<int, SolvePlan<double>> inv_plans_d;
  std::map<int, SolvePlan<float>> inv_plans_f;
  std::map<int, FwdPlan> fwd_plans;
  GraphCache g_inv_d, g_inv_f, g_fwd;
  bool use_graphs = true;
  bool autotune = false;  // tune the K split of every solve-plan step when the plan is built
  void set_autotune(bool on);
  // double-float solve products (the inverse apply when its factors are FP64, the
  // forward apply of the refinement always in these modes)
  bool dfm() const {
    return prm.precision == HSS_PREC_DFLOAT || prm.precision == HSS_PREC_DFLOAT_INV ||
           prm.precision == HSS_PREC_MIXED || prm.precision == HSS_PREC_TC;
  }
  // inverse apply on the tensor cores over digit slices of the FP64 factors
  bool tcm() const { return prm.precision == HSS_PREC_TC; }
  void make_tc_inverse();
  void ensure_tc_err();
  DevBuf<int> tc_err;           // error word of the tensor-core products (0: none)
  int* tc_err_host = nullptr;   // pinned copy, read with the refinement's residual
  // double-float Gauss-Jordan updates of the block inverses
  bool dfinv() const { return prm.precision == HSS_PREC_DFLOAT_INV; }
  // double-float products of the inversion (E, U, G, GE)
  bool dfgemm() const { return prm.precision == HSS_PREC_DFLOAT_INV; }
  // least squares for T with double-float trailing updates: the forward operator and the
  // inverse factors share the same T, so the solve's refinement is unaffected
  bool dftree() const { return prm.precision != HSS_PREC_FP64; }
  void make_df_forward();
  void make_df_inverse();

  explicit HSS2D(const hss2d_params& p);
  ~HSS2D();

  // low-rank interpolation ('lowrank' INTERform): widest T.U per level (q(lev+1) of the
  // reference), the randomized ranks of T_up / T_dn per factor box of a level (empty on
  // dense levels)
  // host wall seconds: tree geometry, point/index uploads, interpolation operators (GPU),
  // compress, invert
  double phase_s[5] = {};
  std::vector<int> qlev;
  std::vector<std::vector<int>> qrank_up, qrank_dn;

  // complex (HSS_SL_H_2D) tree: every block in the real 2 x 2 embedding, vectors interleaved
  bool cplx = false;
  int ng_pts = 0;  // vector rows of one leaf panel (Ng^2, twice that for a complex tree)
  // raw ID T per level while the tree is built (box i at id_Toff[lev][i], 2k x 2(n - k))
  std::map<int, std::vector<double>> id_T;
  std::map<int, std::vector<long long>> id_Toff;
  void id_level(int lev, const std::vector<std::vector<int>>& boxes, const std::vector<std::vector<double>>& px,
                const std::vector<std::vector<double>>& py, std::vector<std::vector<int>>& perm, std::vector<int>& k);
  void id_T_level(int lev);
  void lstsq_tsqr(const std::vector<QrP<double>>& qp, int n, int k);
  void build_tree();
  void compute_T(int lev);
  bool uses_lowrank(int lev) const;
  void sample_guess(int lev, int m, int n, bool up, int& k0, int& C) const;
  void lowrank_T(int lev, const double* A, DevBuf<double>& Vw, DevBuf<double>& Tf, DevBuf<double>& diag);
  void compress();
  void invert();
  void applyinv_device(const double* dX, double* dY, int nrhs, cudaStream_t user);
  void apply_device(const double* dX, double* dY, int nrhs, cudaStream_t user);
  void solve_device(const double* df, double* dx, int nrhs, double tol, int maxit, double* relres, int* iters,
                    cudaStream_t user);
  long long solve_bytes() const;
  // Translation-invariant mode keeps one factor set per level: nf() boxes
  // carry factors, box i of a level uses factor box fo(i).
  int nf(const Level2Geom& g) const { return prm.transinv ? 1 : g.nb; }
  size_t fo(int i) const { return prm.transinv ? 0 : (size_t)i; }
  int solve_launches(int nrhs) const;

  template <typename R>
  void invert_impl();
  template <typename R>
  void invert_level(R* A, int n, int nb);
  template <typename R>
  void invert_level_schur(R* A, int n, int nb);
  template <typename R>
  void invert_level_ld(R* A, int n, int lda, int nb, size_t bs);
  template <typename R>
  SolvePlan<R>& inv_plan(int r);
  template <typename R>
  void applyinv_stage(int r);
  void apply_stage(int r);
  void apply_stage_body(int r);
  void fwd_prepare(int r);
  void solve_once(const double* f, double* x, int r);
  void ensure_stage();
  void sync_from(cudaStream_t user);
  void sync_to(cudaStream_t user);

  template <typename R>
  GraphCache& inv_graphs() {
    if constexpr (std::is_same<R, double>::value) return g_inv_d;
    else return g_inv_f;
  }
  template <typename R>
  std::map<int, SolvePlan<R>>& plan_cache() {
    if constexpr (std::is_same<R, double>::value) return inv_plans_d;
    else return inv_plans_f;
  }
  template <typename R>
  DevBuf<R>& stage_in() {
    if constexpr (std::is_same<R, double>::value) return Xd;
    else return Xf;
  }
  template <typename R>
  DevBuf<R>& stage_out() {
    if constexpr (std::is_same<R, double>::value) return Yd;
    else return Yf;
  }
};

// x = A^-1 f by restarted GMRES right-preconditioned with M^-1 (krylov.cu); complex on a
// complex tree
void gmres_device(HSS2D& A, HSS2D* M, const double* f, double* x, int nrhs, double tol, int restart, int maxit,
                  double* relres, int* iters);
// x = A^-1 f by BiCGSTAB preconditioned with M^-1 (krylov.cu)
void bicgstab_device(HSS2D& A, HSS2D* M, const double* f, double* x, int nrhs, double tol, int maxit,
                     double* relres, int* iters);

}  // namespace hss

// opaque C handle
struct hss2d_matrix {
  hss::HSS2D* impl;
};
