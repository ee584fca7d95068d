// Low-rank interpolation operators of HSS2D ('lowrank' INTERform).
//
// interpolation_operator.m:79-131 with lr = 1: on the levels above the leaves'
// parents with k < k_cut (LOCAL_Interpolation_Operators, HSS2D_build_tree_nsym.m:842-846)
// the residual block K21 (p x nr: K(Xp, X_rs) for T_up, K(X_rs, Xp)^T for T_dn) is
// compressed as U V^T by the randomized ID (LRID_rand.m:20-39 over ID_rand.m:26-49 and
// QR_findrank.m:45-91), then T.U = K11 \ U and T.V = V.  The product T = T.U T.V^T is
// stored in the dense T arrays, so compress, invert and the applies read one T format.
//
// Every step runs batched over all 2*nb ID problems of the level:
//   sample 0  G (p x k0) Gaussian, Y = K21^T G, pivoted QR of Y -> Q, |diag R|
//   sample s  problems whose last |R_jj| still exceeds acc draw C more columns:
//             Ynew = K21^T G, M = Ynew - Q Q^T Ynew, pivoted QR of M -> Qc,
//             Qc -= Q Q^T Qc, Q = [Q Qc]  (the host counts |R_jj| > acc per problem)
//   then      pivoted QR of Z = Y(:,1:q)^T and the fixed-rank ID (1e-12 pseudo-inverse cut),
//             U = K21(:, J(1:q)), T.U = K11 \ U (Householder least squares),
//             V(J,:) = [I T_id]^T, T = T.U V^T.
#include <algorithm>
#include <cmath>

#include "hss1d.h"  // MoveP, move_batched
#include "hss2d.h"

namespace hss {

namespace {

void run_gemm_list(const std::vector<GemmP<double>>& P, bool tA, bool tB, double alpha, double beta,
                   cudaStream_t s) {
  if (P.empty()) return;
  int maxM = 0, maxN = 0;
  for (auto& g : P) { maxM = std::max(maxM, g.M); maxN = std::max(maxN, g.N); }
  DevBuf<GemmP<double>> d;
  d.upload(P, s);
  for (size_t o = 0; o < P.size(); o += 65535) {
    const int cnt = (int)std::min<size_t>(65535, P.size() - o);
    gemm_batched<double>(d.p + o, cnt, maxM, maxN, tA, tB, alpha, beta, s);
  }
  HSS_CUDA(cudaStreamSynchronize(s));
}

void run_move_list(const std::vector<MoveP>& mv, cudaStream_t s) {
  if (mv.empty()) return;
  DevBuf<MoveP> d;
  d.upload(mv, s);
  move_batched(d.p, (int)mv.size(), s);
  HSS_CUDA(cudaStreamSynchronize(s));
}

// V (nr x q, ld nr): V(perm[i], i) = 1 for i < q, V(perm[q+r], c) = T(c, r) (T ld ldt)
struct LrvP {
  double* V;
  const int* perm;
  const double* T;
  int nr, q, ldt;
};

__global__ void k_lr_v(const LrvP* __restrict__ P) {
  const LrvP p = P[blockIdx.y];
  const long long cnt = (long long)p.nr * p.q;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e % p.nr), c = (int)(e / p.nr);  // r: position in J order
    double v;
    if (r < p.q) v = (r == c) ? 1.0 : 0.0;
    else v = p.T[c + (size_t)(r - p.q) * p.ldt];
    p.V[p.perm[r] + (size_t)c * p.nr] = v;
  }
}

}  // namespace

bool HSS2D::uses_lowrank(int lev) const {
  const auto& g = geo.levels[lev];
  const int kcut = prm.k_cut > 0 ? prm.k_cut : 2500;
  return prm.interform == HSS_INTER_LOWRANK && lev >= 1 && lev < geo.depth - 1 && g.k > 0 && g.k < kcut &&
         g.n - g.k > 0;
}

// First sample count k0 and block size C (interpolation_operator.m:98-116 box_2_proxy,
// :143-152 proxy_2_box).  All boxes of a level are processed together, so the
// same-level guess q(lev+1)+1 of the reference's box-by-box loop is never available and
// every box takes the finer-level guess.  qlev[l] = widest T.U of level l (0 if none).
void HSS2D::sample_guess(int lev, int m, int n, bool up, int& k0, int& C) const {
  const int mn = std::min(m, n);
  int have = 0;
  for (int v : qlev) have += (v > 0) ? 1 : 0;
  if (have < 5) {
    k0 = std::min((int)std::ceil(9.0 * std::log2((double)mn) - 20.0), mn);
    C = 5;
  } else {
    const int a = qlev[lev + 2], b = qlev[lev + 4];
    if (up) {
      k0 = std::min(std::max((int)std::ceil(2.0 * a - b + 2.0), a), mn);
      C = (int)std::ceil(std::abs(a - b) / 2.0) + 1;
    } else {
      k0 = std::min((int)std::ceil(2.0 * a - b + 2.0), mn);
      C = (int)std::ceil(a - b / 2.0) + 1;
    }
  }
  k0 = std::max(1, std::min(k0, mn));  // the guess is below 1 only for blocks of <= 4 columns
}

// A: the level's kernel blocks [K11 | K21] (p x n, ld p) of the 2*nb problems;
// writes T_up (even problems) and T_dn (odd) into L[lev].Tup / Tdn.
void HSS2D::lowrank_T(int lev, const double* A, DevBuf<double>& Vw, DevBuf<double>& Tf, DevBuf<double>& diag) {
  auto& g = geo.levels[lev];
  auto& d = L[lev];
  const int nb = nf(g), n = g.n, k = g.k, p = g.p, nr = n - k, batch = 2 * nb;
  const int mn = std::min(p, nr);
  HSS_REQUIRE(nr <= 4096, HSS_ERR_ARG, "low-rank interpolation: more than 4096 residual points in a box");
  int k0[2], C[2];
  sample_guess(lev, p, nr, true, k0[0], C[0]);
  sample_guess(lev, p, nr, false, k0[1], C[1]);
  const int k0max = std::max(k0[0], k0[1]);
  const int cmax = std::max(1, std::max(C[0], C[1]));
  const int gcap = std::max(k0max, std::min(cmax, mn));
  const int qcap = k0max + mn + cmax;
  const double tol = prm.acc;
  const unsigned long long seed = prm.seed;
  const cudaStream_t st = stream;
  DevBuf<double> Y((size_t)batch * nr * mn), Q((size_t)batch * nr * qcap), G((size_t)batch * p * gcap),
      M((size_t)batch * nr * gcap), T1((size_t)batch * qcap * gcap), tau((size_t)batch * gcap),
      D((size_t)batch * gcap);
  auto Yp = [&](int b) { return Y.p + (size_t)b * nr * mn; };
  auto Qp = [&](int b) { return Q.p + (size_t)b * nr * qcap; };
  auto Gp = [&](int b) { return G.p + (size_t)b * p * gcap; };
  auto Mp = [&](int b) { return M.p + (size_t)b * nr * gcap; };
  auto T1p = [&](int b) { return T1.p + (size_t)b * qcap * gcap; };
  auto A2 = [&](int b) { return A + (size_t)b * p * n + (size_t)k * p; };
  auto problem = [&](int b) { return 2 * ((1 << lev) - 1 + b / 2) + (b & 1); };
  std::vector<int> krank(batch, 0), qc(batch, 0), draw(batch, 0), num(batch, 0);
  std::vector<char> active(batch, 1);
  for (int round = 0;; ++round) {
    std::vector<int> act;
    for (int b = 0; b < batch; ++b) {
      if (!active[b]) continue;
      num[b] = (round == 0) ? k0[b & 1] : std::min(C[b & 1], mn - krank[b]);
      if (num[b] <= 0) { active[b] = 0; continue; }  // an empty block: residual 0, stop
      HSS_REQUIRE(qc[b] + num[b] <= qcap, HSS_ERR_RANK, "randomized range finder exceeded its sample bound");
      act.push_back(b);
    }
    if (act.empty()) break;
    // G, then Ynew = K21^T G into Y(:, krank : krank+num)
    std::vector<GaussP> gp;
    long long maxe = 0;
    for (int b : act) {
      const unsigned long long strm = ((unsigned long long)problem(b) << 8) | (unsigned)(draw[b] & 0xFF);
      gp.push_back(GaussP{Gp(b), p, num[b], p, seed, strm});
      maxe = std::max(maxe, (long long)p * num[b]);
      ++draw[b];
    }
    {
      DevBuf<GaussP> dg;
      dg.upload(gp, st);
      gauss_batched(dg.p, (int)gp.size(), maxe, st);
      HSS_CUDA(cudaStreamSynchronize(st));
    }
    std::vector<GemmP<double>> gs;
    for (int b : act)
      gs.push_back(GemmP<double>{A2(b), Gp(b), Yp(b) + (size_t)krank[b] * nr, nr, num[b], p, p, p, nr});
    run_gemm_list(gs, true, false, 1.0, 0.0, st);
    // M = Ynew (first sample block) or Ynew - Q Q^T Ynew
    std::vector<MoveP> mv;
    for (int b : act)
      mv.push_back(MoveP{Yp(b) + (size_t)krank[b] * nr, Mp(b), nullptr, nr, num[b], nr, nr, 0, 0});
    run_move_list(mv, st);
    if (round > 0) {
      std::vector<GemmP<double>> g1, g2;
      for (int b : act) {
        g1.push_back(GemmP<double>{Qp(b), Mp(b), T1p(b), qc[b], num[b], nr, nr, nr, qc[b]});
        g2.push_back(GemmP<double>{Qp(b), T1p(b), Mp(b), nr, num[b], qc[b], nr, qc[b], nr});
      }
      run_gemm_list(g1, true, false, 1.0, 0.0, st);
      run_gemm_list(g2, false, false, -1.0, 1.0, st);
    }
    // pivoted QR of M; its thin Q lands in Q(:, qc : qc+num)
    std::vector<PqrP> pq;
    for (int b : act)
      pq.push_back(PqrP{Mp(b), nr, num[b], nr, tau.p + (size_t)b * gcap, Qp(b) + (size_t)qc[b] * nr, nr,
                        D.p + (size_t)b * gcap});
    {
      DevBuf<PqrP> dq;
      dq.upload(pq, st);
      pqr_q_batched(dq.p, (int)pq.size(), st);
    }
    if (round > 0) {  // Qc -= Q Q^T Qc
      std::vector<GemmP<double>> g1, g2;
      for (int b : act) {
        double* Qc = Qp(b) + (size_t)qc[b] * nr;
        g1.push_back(GemmP<double>{Qp(b), Qc, T1p(b), qc[b], num[b], nr, nr, nr, qc[b]});
        g2.push_back(GemmP<double>{Qp(b), T1p(b), Qc, nr, num[b], qc[b], nr, qc[b], nr});
      }
      run_gemm_list(g1, true, false, 1.0, 0.0, st);
      run_gemm_list(g2, false, false, -1.0, 1.0, st);
    }
    std::vector<double> hD;
    download(hD, D.p, (size_t)batch * gcap, st);
    HSS_CUDA(cudaStreamSynchronize(st));
    for (int b : act) {
      const int l = std::min(nr, num[b]);
      int cnt = 0;
      for (int j = 0; j < l; ++j) cnt += (hD[(size_t)b * gcap + j] > tol) ? 1 : 0;
      HSS_REQUIRE(std::isfinite(hD[(size_t)b * gcap]), HSS_ERR_NONFINITE, "non-finite sample in the randomized ID");
      const double residual = (l > 0) ? hD[(size_t)b * gcap + l - 1] : 0.0;
      krank[b] += cnt;
      qc[b] += l;
      active[b] = (residual > tol && krank[b] < mn) ? 1 : 0;
    }
  }
  // ID of Z = Y(:, 1:q)^T (q x nr) at fixed rank q
  int qmax = 0;
  for (int b = 0; b < batch; ++b) qmax = std::max(qmax, krank[b]);
  qlev[lev] = qmax;
  qrank_up[lev].assign(nb, 0);
  qrank_dn[lev].assign(nb, 0);
  for (int b = 0; b < batch; ++b) ((b & 1) ? qrank_dn[lev] : qrank_up[lev])[b / 2] = krank[b];
  const size_t zsz = (size_t)std::max(qmax, 1) * nr;
  DevBuf<double> Z((size_t)batch * zsz), Zw((size_t)batch * zsz), Tid((size_t)batch * nr * nr),
      SW((size_t)batch * std::max(qmax, 1) * std::max(qmax, 1)), SV((size_t)batch * std::max(qmax, 1) * std::max(qmax, 1)),
      xw((size_t)batch * 2 * nr), yw((size_t)batch * (std::max(qmax, 1) + nr)), Uu((size_t)batch * k * std::max(qmax, 1)),
      Vv((size_t)batch * nr * std::max(qmax, 1)), LS((size_t)batch * p * (k + std::max(qmax, 1)));
  DevBuf<int> perm((size_t)batch * nr), rank(batch);
  std::vector<MoveP> mv;
  std::vector<IdP> ip;
  for (int b = 0; b < batch; ++b) {
    const int q = krank[b];
    if (q == 0) continue;
    mv.push_back(MoveP{Yp(b), Z.p + (size_t)b * zsz, nullptr, nr, q, nr, q, 3, 0});  // Z = Y(:,1:q)^T
    ip.push_back(IdP{Z.p + (size_t)b * zsz, Zw.p + (size_t)b * zsz, q, nr, perm.p + (size_t)b * nr, rank.p + b,
                     Tid.p + (size_t)b * nr * nr, q, SW.p + (size_t)b * qmax * qmax, SV.p + (size_t)b * qmax * qmax,
                     xw.p + (size_t)b * 2 * nr, yw.p + (size_t)b * (qmax + nr), problem(b), ID_QR_ONLY, seed,
                     nullptr});
  }
  run_move_list(mv, st);
  if (!ip.empty()) {
    DevBuf<IdP> di;
    di.upload(ip, st);
    id_adaptive_batched(di.p, (int)ip.size(), tol, st);
    id_fixed_batched(di.p, (int)ip.size(), st);
    HSS_CUDA(cudaStreamSynchronize(st));
  }
  // U = K21(:, J(1:q)) next to K11: [K11 | U] (p x (k+q)); V from J and T_id
  mv.clear();
  std::vector<LrvP> lv;
  for (int b = 0; b < batch; ++b) {
    const int q = krank[b];
    if (q == 0) continue;
    double* ls = LS.p + (size_t)b * p * (k + qmax);
    mv.push_back(MoveP{A + (size_t)b * p * n, ls, nullptr, p, k, p, p, 0, 0});
    mv.push_back(MoveP{A2(b), ls + (size_t)k * p, perm.p + (size_t)b * nr, p, q, p, p, 1, 0});
    lv.push_back(LrvP{Vv.p + (size_t)b * nr * qmax, perm.p + (size_t)b * nr, Tid.p + (size_t)b * nr * nr, nr, q, nr});
  }
  run_move_list(mv, st);
  if (!lv.empty()) {
    DevBuf<LrvP> dl;
    dl.upload(lv, st);
    const long long tot = (long long)nr * qmax;
    k_lr_v<<<dim3(std::max(1, std::min(ceil_div(tot, 256), 1024)), (unsigned)lv.size()), 256, 0, st>>>(dl.p);
    check_launch("k_lr_v");
    HSS_CUDA(cudaStreamSynchronize(st));
  }
  // T.U = K11 \ U (k x q), then T = T.U V^T; a rank-0 box has T = 0
  HSS_CUDA(cudaMemsetAsync(d.Tup.p, 0, (size_t)nb * k * nr * sizeof(double), st));
  HSS_CUDA(cudaMemsetAsync(d.Tdn.p, 0, (size_t)nb * k * nr * sizeof(double), st));
  std::vector<QrP<double>> qp;
  std::vector<GemmP<double>> gt;
  for (int b = 0; b < batch; ++b) {
    const int q = krank[b];
    if (q == 0) continue;
    qp.push_back(QrP<double>{LS.p + (size_t)b * p * (k + qmax), p, k + q, k, p, Vw.p + (size_t)b * p * QR_NB,
                             Tf.p + (size_t)b * QR_NB * QR_NB, diag.p + (size_t)b * k,
                             Uu.p + (size_t)b * k * qmax, k});
    double* T = ((b & 1) ? d.Tdn.p : d.Tup.p) + (size_t)(b / 2) * k * nr;
    gt.push_back(GemmP<double>{Uu.p + (size_t)b * k * qmax, Vv.p + (size_t)b * nr * qmax, T, k, nr, q, k, nr, k});
  }
  if (!qp.empty()) {
    DevBuf<QrP<double>> dq;
    dq.upload(qp, st);
    lstsq_batched<double>(dq.p, (int)qp.size(), p, k + qmax, k, st, dftree());
    HSS_CUDA(cudaStreamSynchronize(st));
  }
  run_gemm_list(gt, false, true, 1.0, 0.0, st);
}

}  // namespace hss
