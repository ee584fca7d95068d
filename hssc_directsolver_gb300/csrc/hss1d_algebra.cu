// HSS1D algebra on compressed matrices, FP64:
//
//  transpose     : HSS1D/HSS1D_transpose.m:24-50.
//  scalarmult    : HSS1D/HSS1D_scalarmult.m.
//  dense_matrix  : HSS1D/HSS1D_dense_matrix.m (through the forward apply).
//  compress_rect : HSS1D/HSS1D_compress_rectangular_nsym.m:70-266 (apply: the forward
//                  plan of hss1d.cu on the row tree, HSS1D_apply_rect_nsym.m).
//  sum           : HSS1D/HSS1D_sum_nsym.m:30-160.
//  compress_lr   : HSS1D/HSS1D_compressLR_nsym.m:25-88.
#include "hss1d.h"
#include "hss1d_util.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <numeric>

namespace hss {

__global__ void k_add_into(long long n, const double* __restrict__ d, double* __restrict__ x) {
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < n; e += (long long)gridDim.x * 256) x[e] += d[e];
}

// ---------------------------------------------------------------------------
// HSS1D algebra (HSS1D/HSS1D_transpose.m, HSS1D_scalarmult.m, HSS1D_dense_matrix.m)
// ---------------------------------------------------------------------------
// A^T in the same format: the up and down skeletons and interpolation matrices trade
// places, every leaf's M_SELF is transposed, and each sibling pair's M_SIB blocks are
// swapped and transposed (HSS1D_transpose.m:24-50).
void HSS1D::transpose(HSS1D& K) const {
  HSS_REQUIRE(!cplx, HSS_ERR_ARG, "the transpose of a complex handle is not built (real handles only)");
  HSS_REQUIRE(!rect, HSS_ERR_ARG, "transpose is defined for square handles only");
  K.Ntot = Ntot; K.nprob = nprob; K.nboxes = nboxes; K.leaf = leaf; K.maxlev = maxlev; K.acc = acc; K.sym = sym;
  K.pN = pN; K.pbase = pbase; K.proot = proot; K.pseed = pseed;
  K.prob = prob; K.level = level; K.parent = parent; K.c1 = c1; K.c2 = c2; K.off = off; K.cnt = cnt;
  K.nskel = nskel; K.kskel = kskel;
  K.I_SKUP = I_SKDN; K.I_SKDN = I_SKUP;
  K.J_UP = J_DN; K.J_DN = J_UP;
  K.X = X; K.kp = kp; K.kdev = kdev; K.census = census;
  K.oT = oT; K.oSelf = oSelf; K.oSib = oSib; K.oJ = oJ;
  K.inverted = false;
  const cudaStream_t st = stream;
  auto copy = [&](DevBuf<double>& dst, const DevBuf<double>& src) {
    dst.alloc(std::max<size_t>(src.n, 1));
    if (src.n) HSS_CUDA(cudaMemcpyAsync(dst.p, src.p, src.n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  };
  copy(K.T_UP, T_DN);
  copy(K.T_DN, T_UP);
  K.TDNT.alloc(std::max<size_t>(TDNT.n, 1));
  K.M_SELF.alloc(std::max<size_t>(M_SELF.n, 1));
  K.M_SIB.alloc(std::max<size_t>(M_SIB.n, 1));
  K.JUPd.alloc(std::max<size_t>(JDNd.n, 1));
  K.JDNd.alloc(std::max<size_t>(JUPd.n, 1));
  if (JDNd.n) HSS_CUDA(cudaMemcpyAsync(K.JUPd.p, JDNd.p, JDNd.n * sizeof(int), cudaMemcpyDeviceToDevice, st));
  if (JUPd.n) HSS_CUDA(cudaMemcpyAsync(K.JDNd.p, JUPd.p, JUPd.n * sizeof(int), cudaMemcpyDeviceToDevice, st));
  std::vector<MoveP> mv;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] >= 0) {
      const int n = nskel[b], k = kskel[b];
      // the transposed operator's T_DN^T is this operator's T_UP^T
      if (k > 0 && n - k > 0) mv.push_back(MoveP{T_UP.p + oT[b], K.TDNT.p + oT[b], nullptr, k, n - k, k, n - k, 3, 0});
      if (is_leaf(b)) mv.push_back(MoveP{M_SELF.p + oSelf[b], K.M_SELF.p + oSelf[b], nullptr, cnt[b], cnt[b], cnt[b],
                                         cnt[b], 3, 0});
    }
    if (c1[b] >= 0 && c2[b] >= 0) {
      const int s1 = c1[b], s2 = c2[b], k1 = kskel[s1], k2 = kskel[s2];
      if (k1 > 0 && k2 > 0) {
        mv.push_back(MoveP{M_SIB.p + oSib[s2], K.M_SIB.p + oSib[s1], nullptr, k2, k1, k2, k1, 3, 0});
        mv.push_back(MoveP{M_SIB.p + oSib[s1], K.M_SIB.p + oSib[s2], nullptr, k1, k2, k1, k2, 3, 0});
      }
    }
  }
  run_moves(mv, st);
  HSS_CUDA(cudaStreamSynchronize(st));
}

// E(row0 + c, c) = 1 for c < r (E: ld x r, zeroed)
__global__ void k_unit_cols(double* __restrict__ E, long long ld, long long row0, int r) {
  for (int c = threadIdx.x; c < r; c += blockDim.x) E[(size_t)c * ld + row0 + c] = 1.0;
}

__global__ void k_scale(double* __restrict__ p, long long n, double c) {
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < n; i += (long long)gridDim.x * 256) p[i] *= c;
}

// c * A: the leaf self blocks and the sibling blocks scale, the interpolation matrices
// do not (HSS1D_scalarmult.m:19-33).  The inverse factors no longer apply.
void HSS1D::scalarmult(double c) {
  kernel_op = false;  // c K is no longer the kernel matrix of the points
  HSS_REQUIRE(std::isfinite(c), HSS_ERR_ARG, "scalarmult: c must be finite");
  for (DevBuf<double>* b : {&M_SELF, &M_SIB}) {
    if (b->n == 0) continue;
    k_scale<<<std::max(1, std::min(ceil_div((long long)b->n, 256), 4096)), 256, 0, stream>>>(b->p, (long long)b->n, c);
    check_launch("k_scale");
  }
  inverted = false;
  clear_plans();
  if (dfm()) make_df();
  HSS_CUDA(cudaStreamSynchronize(stream));
}

// The dense matrix the compressed form represents, column block by column block: the
// forward apply of identity columns, the rows of problem p kept.  (The reference builds
// it from the telescoping factors, HSS1D_dense_matrix.m:17-92; both are the same matrix.)
void HSS1D::dense_matrix(int p, double* Kd) {
  HSS_REQUIRE(!cplx, HSS_ERR_ARG, "the dense export of a complex handle is not built (real handles only)");
  HSS_REQUIRE(!rect, HSS_ERR_ARG, "dense_matrix is defined for square handles only");
  HSS_REQUIRE(p >= 0 && p < nprob, HSS_ERR_ARG, "dense_matrix: problem index out of range");
  HSS_REQUIRE(Kd != nullptr, HSS_ERR_ARG, "dense_matrix: NULL output");
  const long long Np = pN[p], base = pbase[p];
  const int blk = 64;
  DevBuf<double> E((size_t)Ntot * blk), Y((size_t)Ntot * blk);
  for (long long j0 = 0; j0 < Np; j0 += blk) {
    const int r = (int)std::min<long long>(blk, Np - j0);
    HSS_CUDA(cudaMemsetAsync(E.p, 0, (size_t)Ntot * r * sizeof(double), stream));
    k_unit_cols<<<1, 64, 0, stream>>>(E.p, Ntot, base + j0, r);
    check_launch("k_unit_cols");
    apply_device(E.p, Y.p, r);
    HSS_CUDA(cudaMemcpy2DAsync(Kd + (size_t)j0 * Np, (size_t)Np * sizeof(double), Y.p + base,
                               (size_t)Ntot * sizeof(double), (size_t)Np * sizeof(double), (size_t)r,
                               cudaMemcpyDeviceToHost, stream));
    HSS_CUDA(cudaStreamSynchronize(stream));
  }
}

// ---------------------------------------------------------------------------
// K_HSS = HSS1D_compress_rectangular_nsym('green', Xin, Xout, TREE, acc, params),
// HSS1D/HSS1D_compress_rectangular_nsym.m:70-266: the M x N matrix K(Xin, Xout).  The
// columns follow the halving tree over Xout; the rows a tree of the same shape over Xin
// whose parents split their rows ceil(m/2) | rest (LOCAL_get_tree_in, :325-356).  Per box
// one circle around its row and column candidates carries one proxy ring (:116-140), and
// A_out = [K(rows inside, cols); K(ring, cols)] and A_in^T = [K(rows, cols inside),
// K(rows, ring)]^T are IDed level-batched with independent ranks (:209-236; no rank
// equalisation).  Point table: Xout at [0, N), Xin at [N, N + M), the rings after.
void HSS1D::compress_rect(long long M, const double* Xin, long long ldin, long long N, const double* Xout,
                          long long ldout, int leaf_, double acc_, const hss_kernel_params& kp_,
                          unsigned long long seed) {
  HSS_REQUIRE(Xin && Xout && M >= 2 && N >= 2 && ldin >= M && ldout >= N && leaf_ >= 1 && acc_ > 0 && acc_ < 1,
              HSS_ERR_ARG, "bad rectangular compress args");
  HSS_REQUIRE(kp_.flag == HSS_SL_L_2D || kp_.flag == HSS_DL_L_2D, HSS_ERR_ARG, "unknown kernel");
  HSS_REQUIRE(M + N < (1LL << 30), HSS_ERR_ARG, "total points too large");
  std::fill(phase_s, phase_s + NPHASE, 0.0);
  rect = true;
  sym = false;
  nprob = 1; leaf = leaf_; acc = acc_; kp = kp_;
  kdev = make_kernel_dev(kp);
  Ntot = N;
  Mtot = M;
  pN = {N}; pbase = {0}; pseed = {seed};
  proot.assign(1, 0);
  const long long NP = N + M;
  X.resize(6 * (size_t)NP);
  for (long long i = 0; i < N; ++i)
    for (int c = 0; c < 6; ++c) X[6 * i + c] = Xout[i + c * ldout];
  for (long long i = 0; i < M; ++i)
    for (int c = 0; c < 6; ++c) X[6 * (N + i) + c] = Xin[i + c * ldin];
  prob.clear(); level.clear(); parent.clear(); c1.clear(); c2.clear(); off.clear(); cnt.clear();
  append_tree(0, 0, (int)N);
  nboxes = (int)level.size();
  maxlev = *std::max_element(level.begin(), level.end());
  // ---- row tree (LOCAL_get_tree_in): parents come before their sons
  off_in.assign(nboxes, 0);
  cnt_in.assign(nboxes, 0);
  cnt_in[0] = (int)M;
  for (int b = 0; b < nboxes; ++b) {
    if (c1[b] < 0 || c2[b] < 0) continue;
    const int half = (cnt_in[b] + 1) / 2;
    off_in[c1[b]] = off_in[b]; cnt_in[c1[b]] = half;
    off_in[c2[b]] = off_in[b] + half; cnt_in[c2[b]] = cnt_in[b] - half;
  }
  for (int b = 0; b < nboxes; ++b)
    HSS_REQUIRE(cnt_in[b] >= 1, HSS_ERR_ARG, "every box of the row tree needs a point (M too small for the tree)");
  auto rows_of = [&](int b) {  // table indices of box b's rows
    std::vector<int> r(cnt_in[b]);
    std::iota(r.begin(), r.end(), (int)N + off_in[b]);
    return r;
  };
  auto cols_of = [&](int b) {
    std::vector<int> r(cnt[b]);
    std::iota(r.begin(), r.end(), off[b]);
    return r;
  };
  // ---- neighbour lists (:397-462): one circle per box around its rows and columns;
  // nei_in keeps the boxes whose columns come inside it, nei_out those whose rows do
  std::vector<std::vector<int>> nei_in(nboxes), nei_out(nboxes);
  nei_in[0] = {0};
  nei_out[0] = {0};
  for (int b = 1; b < nboxes; ++b) {
    std::vector<int> r = rows_of(b);
    const std::vector<int> c = cols_of(b);
    r.insert(r.end(), c.begin(), c.end());
    double xc, yc, R;
    circum_circle(X, r, xc, yc, R);
    const double rr = RADIUS_REL * RADIUS_REL * R * R;
    for (int side = 0; side < 2; ++side) {
      auto& lst = side == 0 ? nei_in : nei_out;
      std::vector<int> pot;
      for (int j : lst[parent[b]]) {
        if (c1[j] >= 0) pot.push_back(c1[j]);
        if (c2[j] >= 0) pot.push_back(c2[j]);
      }
      for (int j : pot) {
        const long long o = side == 0 ? off[j] : N + off_in[j];
        const int n = side == 0 ? cnt[j] : cnt_in[j];
        double mn = INFINITY;
        for (long long i = o; i < o + n; ++i) {
          const double dx = X[6 * (size_t)i] - xc, dy = X[6 * (size_t)i + 1] - yc;
          mn = std::min(mn, dx * dx + dy * dy);
        }
        if (n > 0 && mn < rr) lst[b].push_back(j);
      }
    }
  }
  for (auto* lst : {&nei_in, &nei_out})
    for (int b = 1; b < nboxes; ++b) {
      auto& l = (*lst)[b];
      l.erase(std::remove(l.begin(), l.end(), b), l.end());
      std::sort(l.begin(), l.end());
    }
  // ---- point table with one proxy ring per non-root box, in the order levels run
  std::vector<int> pslot(nboxes, -1);
  int nslot = 0;
  for (int L = maxlev; L >= 1; --L)
    for (int b = 0; b < nboxes; ++b)
      if (level[b] == L) pslot[b] = nslot++;
  const size_t npts = (size_t)NP + (size_t)NPROXY * nslot;
  HSS_REQUIRE(npts < (1ULL << 31), HSS_ERR_ARG, "point table exceeds 2^31 entries");
  std::vector<double> hx(npts, 0.0), hy(npts, 0.0), hnx(npts, 0.0), hny(npts, 0.0), hw(npts, 0.0),
      hk(npts, 0.0);
  for (long long i = 0; i < NP; ++i) {
    hx[i] = X[6 * i]; hy[i] = X[6 * i + 1]; hnx[i] = X[6 * i + 2]; hny[i] = X[6 * i + 3];
    hw[i] = X[6 * i + 4]; hk[i] = X[6 * i + 5];
  }
  pts.reserve(npts);
  pts.upload_range(0, (size_t)NP, hx.data(), hy.data(), hnx.data(), hny.data(), hw.data(), hk.data(), kp, stream);
  nskel.assign(nboxes, 0); kskel.assign(nboxes, 0);
  nskel_in.assign(nboxes, 0); kskel_in.assign(nboxes, 0);
  I_SKUP.assign(nboxes, {}); I_SKDN.assign(nboxes, {});
  J_UP.assign(nboxes, {}); J_DN.assign(nboxes, {});
  census.assign(4 * (size_t)nboxes, 0);
  feat.assign((size_t)NFEAT * nboxes, 0.f);
  qr_steps = qr_steps_full = 0;
  reruns = 0;
  std::vector<DevBuf<double>> Tkeep;
  std::vector<std::array<long long, 2>> Toff(nboxes);
  std::vector<int> Tlev(nboxes, -1);
  for (int L = maxlev; L >= 1; --L) {
    std::vector<int> boxes;
    for (int b = 0; b < nboxes; ++b)
      if (level[b] == L) boxes.push_back(b);
    if (boxes.empty()) continue;
    const int nbL = (int)boxes.size();
    // problem 2q: A_out (rows_out x outs), problem 2q+1: A_in^T (rows_in x inns)
    std::vector<std::vector<int>> outs(nbL), inns(nbL), rows_out(nbL), rows_in(nbL);
    parallel_for(nbL, [&](int q) {
      const int b = boxes[q];
      if (is_leaf(b)) {
        outs[q] = cols_of(b);
        inns[q] = rows_of(b);
      } else {
        HSS_REQUIRE(c1[b] >= 0 && c2[b] >= 0, HSS_ERR_ARG, "one-child boxes are not produced by the halving tree");
        outs[q] = I_SKUP[c1[b]];
        outs[q].insert(outs[q].end(), I_SKUP[c2[b]].begin(), I_SKUP[c2[b]].end());
        inns[q] = I_SKDN[c1[b]];
        inns[q].insert(inns[q].end(), I_SKDN[c2[b]].begin(), I_SKDN[c2[b]].end());
      }
      // circle around [Xin(sort(rows)); Xout(sort(cols))] (:125-126)
      std::vector<int> both = inns[q], so = outs[q];
      std::sort(both.begin(), both.end());
      std::sort(so.begin(), so.end());
      both.insert(both.end(), so.begin(), so.end());
      double xc, yc, R;
      circum_circle(X, both, xc, yc, R);
      const double Rp = RADIUS_REL * R;
      const double stop = 2.0 * M_PI * (1.0 - 1.0 / NPROXY);
      const double step = stop / (double)(NPROXY - 1);
      const size_t pb = (size_t)NP + (size_t)NPROXY * pslot[b];
      for (int t = 0; t < NPROXY; ++t) {
        const double tt = (t == NPROXY - 1) ? stop : (double)t * step;
        const double c = std::cos(tt), s = std::sin(tt);
        hx[pb + t] = xc + Rp * c;
        hy[pb + t] = yc + Rp * s;
        hnx[pb + t] = c;
        hny[pb + t] = s;
        hw[pb + t] = 2.0 * M_PI * Rp / NPROXY;
        hk[pb + t] = 1.0 / Rp;
      }
      std::vector<int> out_maybe, in_maybe;
      for (int j : nei_in[b]) {
        if (is_leaf(j)) {
          const std::vector<int> r = cols_of(j);
          out_maybe.insert(out_maybe.end(), r.begin(), r.end());
        } else {
          for (int s : {c1[j], c2[j]}) out_maybe.insert(out_maybe.end(), I_SKUP[s].begin(), I_SKUP[s].end());
        }
      }
      for (int j : nei_out[b]) {
        if (is_leaf(j)) {
          const std::vector<int> r = rows_of(j);
          in_maybe.insert(in_maybe.end(), r.begin(), r.end());
        } else {
          for (int s : {c1[j], c2[j]}) in_maybe.insert(in_maybe.end(), I_SKDN[s].begin(), I_SKDN[s].end());
        }
      }
      const double rr = Rp * Rp;
      auto inside = [&](int i) {
        const double dx = X[6 * (size_t)i] - xc, dy = X[6 * (size_t)i + 1] - yc;
        return dx * dx + dy * dy < rr;
      };
      for (int i : in_maybe)
        if (inside(i)) rows_out[q].push_back(i);
      for (int i : out_maybe)
        if (inside(i)) rows_in[q].push_back(i);
      for (int t = 0; t < NPROXY; ++t) {
        rows_out[q].push_back((int)(pb + t));
        rows_in[q].push_back((int)(pb + t));
      }
      HSS_REQUIRE(outs[q].size() <= 4096 && inns[q].size() <= 4096, HSS_ERR_RANK,
                  "skeleton set exceeds 4096 points");
      HSS_REQUIRE(!outs[q].empty() && !inns[q].empty(), HSS_ERR_RANK, "empty skeleton set (rank 0 children)");
    }, 16);
    {
      const size_t p0 = (size_t)NP + (size_t)NPROXY * pslot[boxes[0]];
      pts.upload_range(p0, (size_t)NPROXY * nbL, hx.data() + p0, hy.data() + p0, hnx.data() + p0, hny.data() + p0,
                       hw.data() + p0, hk.data() + p0, kp, stream);
    }
    std::vector<int> idx;
    std::vector<long long> o_ro(nbL), o_ri(nbL), o_out(nbL), o_in(nbL);
    for (int q = 0; q < nbL; ++q) {
      o_ro[q] = idx.size(); idx.insert(idx.end(), rows_out[q].begin(), rows_out[q].end());
      o_ri[q] = idx.size(); idx.insert(idx.end(), rows_in[q].begin(), rows_in[q].end());
      o_out[q] = idx.size(); idx.insert(idx.end(), outs[q].begin(), outs[q].end());
      o_in[q] = idx.size(); idx.insert(idx.end(), inns[q].begin(), inns[q].end());
    }
    DevBuf<int> didx;
    upload_vec(didx, idx, stream);
    const int nprob2 = 2 * nbL;
    std::vector<long long> oA(nprob2), oT2(nprob2), oX(nprob2), oY(nprob2), oP(nprob2);
    std::vector<int> pm(nprob2), pn(nprob2);
    long long tA = 0, tT = 0, tX = 0, tY = 0, tP = 0;
    for (int pr = 0; pr < nprob2; ++pr) {
      const int q = pr / 2;
      pm[pr] = (int)(pr % 2 == 0 ? rows_out[q].size() : rows_in[q].size());
      pn[pr] = (int)(pr % 2 == 0 ? outs[q].size() : inns[q].size());
      oA[pr] = tA; tA += (long long)pm[pr] * pn[pr];
      oT2[pr] = tT; tT += (long long)pn[pr] * pn[pr];
      oX[pr] = tX; tX += 2LL * pn[pr];
      oY[pr] = tY; tY += (long long)pm[pr] + pn[pr];
      oP[pr] = tP; tP += pn[pr];
    }
    DevBuf<double> A(tA), W(tA), SW(tT), SV(tT), xw(tX), yw(tY);
    Tkeep.emplace_back(tT);
    DevBuf<double>& Tb = Tkeep.back();
    DevBuf<int> perm(tP), rank(nprob2);
    std::vector<KgenP<double>> kg(nprob2);
    std::vector<IdP> ip(nprob2);
    for (int q = 0; q < nbL; ++q) {
      const int po = 2 * q, pi = po + 1;
      kg[po] = KgenP<double>{didx.p + o_ro[q], didx.p + o_out[q], pm[po], pn[po], A.p + oA[po], pm[po], 0};
      kg[pi] = KgenP<double>{didx.p + o_in[q], didx.p + o_ri[q], pn[pi], pm[pi], A.p + oA[pi], pm[pi], 1};
    }
    for (int pr = 0; pr < nprob2; ++pr)
      ip[pr] = IdP{A.p + oA[pr], W.p + oA[pr], pm[pr], pn[pr], perm.p + oP[pr], rank.p + pr, Tb.p + oT2[pr], -1,
                   SW.p + oT2[pr], SV.p + oT2[pr], xw.p + oX[pr], yw.p + oY[pr], 2 * boxes[pr / 2] + pr % 2, -1,
                   seed, nullptr};
    long long maxe = 0;
    for (auto& g : kg) maxe = std::max(maxe, (long long)g.m * g.n);
    DevBuf<KgenP<double>> dkg;
    upload_vec(dkg, kg, stream);
    for (int o = 0; o < nprob2; o += 65535)
      kgen_batched<double>(dkg.p + o, std::min(65535, nprob2 - o), maxe, view(pts), kdev, stream);
    DevBuf<IdP> dip;
    upload_vec(dip, ip, stream);
    id_adaptive_batched(dip.p, nprob2, acc, stream, id_df);
    std::vector<int> hr, hp;
    download(hr, rank.p, nprob2, stream);
    download(hp, perm.p, tP, stream);
    HSS_CUDA(cudaStreamSynchronize(stream));
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q], po = 2 * q, pi = po + 1;
      const int ko = hr[po], ki = hr[pi];
      nskel[b] = pn[po]; kskel[b] = ko;
      nskel_in[b] = pn[pi]; kskel_in[b] = ki;
      J_UP[b].assign(hp.begin() + oP[po], hp.begin() + oP[po] + pn[po]);
      J_DN[b].assign(hp.begin() + oP[pi], hp.begin() + oP[pi] + pn[pi]);
      I_SKUP[b].resize(ko);
      I_SKDN[b].resize(ki);
      for (int t = 0; t < ko; ++t) I_SKUP[b][t] = outs[q][J_UP[b][t]];
      for (int t = 0; t < ki; ++t) I_SKDN[b][t] = inns[q][J_DN[b][t]];
      Toff[b] = {oT2[po], oT2[pi]};
      Tlev[b] = (int)Tkeep.size() - 1;
      census[4 * b] = pm[po]; census[4 * b + 1] = pm[pi]; census[4 * b + 2] = pn[po]; census[4 * b + 3] = ko;
    }
  }
  // ---- compact T_UP (k_out x (n_out - k_out)), T_DN / T_DN^T (row side) and the J arenas
  oT.assign(nboxes, 0); oTd.assign(nboxes, 0);
  oJ.assign(nboxes, 0); oJd.assign(nboxes, 0);
  long long tu = 0, td = 0, ju = 0, jd = 0;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] < 0) continue;
    oT[b] = tu; tu += (long long)kskel[b] * (nskel[b] - kskel[b]);
    oTd[b] = td; td += (long long)kskel_in[b] * (nskel_in[b] - kskel_in[b]);
    oJ[b] = ju; ju += nskel[b];
    oJd[b] = jd; jd += nskel_in[b];
  }
  T_UP.alloc(std::max(tu, 1LL)); T_DN.alloc(std::max(td, 1LL)); TDNT.alloc(std::max(td, 1LL));
  std::vector<MoveP> mv;
  std::vector<int> hJU(std::max(ju, 1LL)), hJD(std::max(jd, 1LL));
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] < 0) continue;
    std::copy(J_UP[b].begin(), J_UP[b].end(), hJU.begin() + oJ[b]);
    std::copy(J_DN[b].begin(), J_DN[b].end(), hJD.begin() + oJd[b]);
    const double* Tl = Tkeep[Tlev[b]].p;
    const int n = nskel[b], k = kskel[b], ni = nskel_in[b], ki = kskel_in[b];
    if (n - k > 0 && k > 0) mv.push_back(MoveP{Tl + Toff[b][0], T_UP.p + oT[b], nullptr, k, n - k, n, k, 0, 0});
    if (ni - ki > 0 && ki > 0) {
      mv.push_back(MoveP{Tl + Toff[b][1], T_DN.p + oTd[b], nullptr, ki, ni - ki, ni, ki, 0, 0});
      mv.push_back(MoveP{Tl + Toff[b][1], TDNT.p + oTd[b], nullptr, ki, ni - ki, ni, ni - ki, 3, 0});
    }
  }
  run_moves(mv, stream);
  upload_vec(JUPd, hJU, stream);
  upload_vec(JDNd, hJD, stream);
  HSS_CUDA(cudaStreamSynchronize(stream));
  Tkeep.clear();
  // ---- M_SELF = K(Xin(rows), Xout(cols)) on leaves, M_SIB{s1} = K(Xin(I_SKDN{s1}),
  // Xout(I_SKUP{s2})) (:240-266)
  oSelf.assign(nboxes, -1);
  oSib.assign(nboxes, -1);
  long long ts = 0, tb = 0;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] >= 0 && is_leaf(b)) { oSelf[b] = ts; ts += (long long)cnt_in[b] * cnt[b]; }
    if (!is_leaf(b)) {
      const int s1 = c1[b], s2 = c2[b];
      oSib[s1] = tb; tb += (long long)kskel_in[s1] * kskel[s2];
      oSib[s2] = tb; tb += (long long)kskel_in[s2] * kskel[s1];
    }
  }
  M_SELF.alloc(std::max(ts, 1LL));
  M_SIB.alloc(std::max(tb, 1LL));
  std::vector<int> idx;
  std::vector<long long> io;
  auto push = [&](const std::vector<int>& v) { io.push_back(idx.size()); idx.insert(idx.end(), v.begin(), v.end()); };
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] >= 0 && is_leaf(b)) { push(rows_of(b)); push(cols_of(b)); }
    if (!is_leaf(b)) {
      push(I_SKDN[c1[b]]); push(I_SKUP[c2[b]]);
      push(I_SKDN[c2[b]]); push(I_SKUP[c1[b]]);
    }
  }
  DevBuf<int> didx;
  upload_vec(didx, idx, stream);
  std::vector<KgenP<double>> kg;
  size_t q = 0;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] >= 0 && is_leaf(b)) {
      const int* r = didx.p + io[q++];
      const int* c = didx.p + io[q++];
      kg.push_back(KgenP<double>{r, c, cnt_in[b], cnt[b], M_SELF.p + oSelf[b], cnt_in[b], 0});
    }
    if (!is_leaf(b)) {
      const int s1 = c1[b], s2 = c2[b];
      const int* a = didx.p + io[q++];
      const int* bb = didx.p + io[q++];
      const int* c = didx.p + io[q++];
      const int* d = didx.p + io[q++];
      kg.push_back(KgenP<double>{a, bb, kskel_in[s1], kskel[s2], M_SIB.p + oSib[s1], std::max(kskel_in[s1], 1), 0});
      kg.push_back(KgenP<double>{c, d, kskel_in[s2], kskel[s1], M_SIB.p + oSib[s2], std::max(kskel_in[s2], 1), 0});
    }
  }
  long long maxe = 0;
  for (auto& g : kg) maxe = std::max(maxe, (long long)g.m * g.n);
  DevBuf<KgenP<double>> dkg;
  upload_vec(dkg, kg, stream);
  for (size_t o = 0; o < kg.size(); o += 65535) {
    const int c = (int)std::min<size_t>(65535, kg.size() - o);
    kgen_batched<double>(dkg.p + o, c, maxe, view(pts), kdev, stream);
  }
  HSS_CUDA(cudaStreamSynchronize(stream));
  inverted = false;
  clear_plans();
}

// ---------------------------------------------------------------------------
// C_HSS = HSS1D_sum_nsym(A_HSS, B_HSS, acc), HSS1D/HSS1D_sum_nsym.m:30-160: *this = A + B for
// two square handles on one forest.  Level by level (deepest first), every box of every
// problem stacks the operands' outgoing bases RC = [R_A P_A; R_B P_B] and incoming bases
// LC^T (R(:, J) = [I T] from a box's (T, J); P the sons' RHO, the identity on a leaf), IDs
// both in one batched launch with the rank equalised by the fixed-rank ID (:57-66), and keeps
// RHO = RC(:, J_out(1:k)) and LAMBDA^T = LC^T(:, J_in(1:k)).  Sibling blocks become
// LAMBDA_s1 [M_SIB_A 0; 0 M_SIB_B] RHO_s2 (:79-86); self blocks add.
struct RformP {
  const double* T;  // k x (n - k), ld k
  const int* J;     // n, a permutation
  double* R;        // k x n, ld ldr: R(:, J) = [I T]
  int k, n, ldr;
};

__global__ void __launch_bounds__(256) k_rform(const RformP* __restrict__ P) {
  const RformP p = P[blockIdx.x];
  const long long tot = (long long)p.k * p.n;
  for (long long e = threadIdx.x; e < tot; e += 256) {
    const int r = (int)(e % p.k), c = (int)(e / p.k);
    const double v = (c < p.k) ? (r == c ? 1.0 : 0.0) : p.T[r + (size_t)(c - p.k) * p.k];
    p.R[r + (size_t)p.J[c] * p.ldr] = v;
  }
}

void HSS1D::sum(const HSS1D& A, const HSS1D& B, double acc_) {
  HSS_REQUIRE(!A.cplx && !B.cplx, HSS_ERR_ARG, "the sum of complex handles is not built (real handles only)");
  HSS_REQUIRE(!A.rect && !B.rect, HSS_ERR_ARG, "sum is defined for square handles only");
  HSS_REQUIRE(A.nboxes == B.nboxes && A.level == B.level && A.parent == B.parent && A.c1 == B.c1 && A.c2 == B.c2 &&
                  A.off == B.off && A.cnt == B.cnt && A.M_SELF.n == B.M_SELF.n,
              HSS_ERR_ARG, "HSS1D sum needs both operands on one tree");
  HSS_REQUIRE(acc_ > 0 && acc_ < 1, HSS_ERR_ARG, "bad sum tolerance");
  std::fill(phase_s, phase_s + NPHASE, 0.0);
  Ntot = A.Ntot; nprob = A.nprob; nboxes = A.nboxes; leaf = A.leaf; maxlev = A.maxlev; acc = acc_;
  sym = false; rect = false; id_df = false;
  pN = A.pN; pbase = A.pbase; proot = A.proot; pseed = A.pseed;
  prob = A.prob; level = A.level; parent = A.parent; c1 = A.c1; c2 = A.c2; off = A.off; cnt = A.cnt;
  X = A.X; kp = A.kp; kdev = A.kdev;
  precision = HSS_PREC_FP64;
  inverted = false;
  clear_plans();
  nskel.assign(nboxes, 0); kskel.assign(nboxes, 0);
  I_SKUP.assign(nboxes, {}); I_SKDN.assign(nboxes, {});
  J_UP.assign(nboxes, {}); J_DN.assign(nboxes, {});
  census.assign(4 * (size_t)nboxes, 0);
  feat.assign((size_t)NFEAT * nboxes, 0.f);
  qr_steps = qr_steps_full = 0;
  reruns = 0;
  const cudaStream_t st = stream;
  std::vector<DevBuf<double>> keep;  // per level: RHO and LAMBDA^T of its boxes
  std::vector<DevBuf<double>> Tkeep;
  std::vector<std::array<long long, 2>> Toff(nboxes);
  std::vector<int> Tlev(nboxes, -1), mR(nboxes, 0);
  std::vector<const double*> rho(nboxes, nullptr), sig(nboxes, nullptr);
  for (int L = maxlev; L >= 1; --L) {
    std::vector<int> boxes;
    for (int b = 0; b < nboxes; ++b)
      if (level[b] == L) boxes.push_back(b);
    if (boxes.empty()) continue;
    const int nbL = (int)boxes.size(), nprob2 = 2 * nbL;
    // problem 2q: RC (m x n), 2q+1: LC^T (m x n); parents stage R_A, R_B, L_A^T, L_B^T in Y
    std::vector<int> m(nbL), n(nbL);
    std::vector<long long> oZ(nprob2), oY(nbL);
    long long tZ = 0, tY = 0;
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q];
      m[q] = A.kskel[b] + B.kskel[b];
      n[q] = is_leaf(b) ? cnt[b] : kskel[c1[b]] + kskel[c2[b]];
      HSS_REQUIRE(m[q] >= 1 && n[q] >= 1 && n[q] <= 4096, HSS_ERR_RANK, "sum: empty or oversized skeleton basis");
      oZ[2 * q] = tZ; tZ += (long long)m[q] * n[q];
      oZ[2 * q + 1] = tZ; tZ += (long long)m[q] * n[q];
      oY[q] = tY;
      if (!is_leaf(b)) tY += 2LL * ((long long)A.kskel[b] * A.nskel[b] + (long long)B.kskel[b] * B.nskel[b]);
    }
    DevBuf<double> Z(std::max(tZ, 1LL)), Y(std::max(tY, 1LL));
    Z.zero(st);
    std::vector<RformP> rf;
    std::vector<GemmP<double>> gp;
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q], kA = A.kskel[b], kB = B.kskel[b], mm = m[q];
      double* RC = Z.p + oZ[2 * q];
      double* LC = Z.p + oZ[2 * q + 1];
      const double *TUa = A.T_UP.p + A.oT[b], *TDa = A.T_DN.p + A.oT[b];
      const double *TUb = B.T_UP.p + B.oT[b], *TDb = B.T_DN.p + B.oT[b];
      const int *JUa = A.JUPd.p + A.oJ[b], *JDa = A.JDNd.p + A.oJ[b];
      const int *JUb = B.JUPd.p + B.oJ[b], *JDb = B.JDNd.p + B.oJ[b];
      if (is_leaf(b)) {
        const int nn = cnt[b];
        rf.push_back(RformP{TUa, JUa, RC, kA, nn, mm});
        rf.push_back(RformP{TUb, JUb, RC + kA, kB, nn, mm});
        rf.push_back(RformP{TDa, JDa, LC, kA, nn, mm});
        rf.push_back(RformP{TDb, JDb, LC + kA, kB, nn, mm});
        continue;
      }
      const int s1 = c1[b], s2 = c2[b];
      const int nA = A.nskel[b], nB = B.nskel[b];
      const int kA1 = A.kskel[s1], kA2 = A.kskel[s2], kB1 = B.kskel[s1], kB2 = B.kskel[s2];
      const int kC1 = kskel[s1], kC2 = kskel[s2], m1 = mR[s1], m2 = mR[s2];
      HSS_REQUIRE(nA == kA1 + kA2 && nB == kB1 + kB2, HSS_ERR_ARG, "sum: operand skeleton sets do not follow the tree");
      double* RA = Y.p + oY[q];
      double* RB = RA + (size_t)kA * nA;
      double* LA = RB + (size_t)kB * nB;
      double* LB = LA + (size_t)kA * nA;
      rf.push_back(RformP{TUa, JUa, RA, kA, nA, std::max(kA, 1)});
      rf.push_back(RformP{TUb, JUb, RB, kB, nB, std::max(kB, 1)});
      rf.push_back(RformP{TDa, JDa, LA, kA, nA, std::max(kA, 1)});
      rf.push_back(RformP{TDb, JDb, LB, kB, nB, std::max(kB, 1)});
      for (int side = 0; side < 2; ++side) {
        const double* XA = side == 0 ? RA : LA;
        const double* XB = side == 0 ? RB : LB;
        const double* P1 = side == 0 ? rho[s1] : sig[s1];
        const double* P2 = side == 0 ? rho[s2] : sig[s2];
        double* D = side == 0 ? RC : LC;
        const int la = std::max(kA, 1), lb = std::max(kB, 1);
        gp.push_back(GemmP<double>{XA, P1, D, kA, kC1, kA1, la, m1, mm});
        gp.push_back(GemmP<double>{XA + (size_t)kA1 * kA, P2, D + (size_t)kC1 * mm, kA, kC2, kA2, la, m2, mm});
        gp.push_back(GemmP<double>{XB, P1 + kA1, D + kA, kB, kC1, kB1, lb, m1, mm});
        gp.push_back(GemmP<double>{XB + (size_t)kB1 * kB, P2 + kA2, D + kA + (size_t)kC1 * mm, kB, kC2, kB2, lb, m2,
                                   mm});
      }
    }
    if (!rf.empty()) {
      DevBuf<RformP> drf;
      upload_vec(drf, rf, st);
      for (size_t o = 0; o < rf.size(); o += 65535) {
        const int c = (int)std::min<size_t>(65535, rf.size() - o);
        k_rform<<<c, 256, 0, st>>>(drf.p + o);
        check_launch("k_rform");
      }
      HSS_CUDA(cudaStreamSynchronize(st));
    }
    run_gemms(gp, false, false, 1.0, 0.0, st);
    // IDs of RC and LC^T (problems 2 * local box + side of the shared random stream)
    std::vector<long long> oT2(nprob2), oX(nprob2), oYw(nprob2), oP(nprob2);
    long long tT = 0, tX = 0, tYw = 0, tP = 0;
    for (int pr = 0; pr < nprob2; ++pr) {
      const int q = pr / 2;
      oT2[pr] = tT; tT += (long long)n[q] * n[q];
      oX[pr] = tX; tX += 2LL * n[q];
      oYw[pr] = tYw; tYw += (long long)m[q] + n[q];
      oP[pr] = tP; tP += n[q];
    }
    DevBuf<double> W(std::max(tZ, 1LL)), SW(tT), SV(tT), xw(tX), yw(tYw);
    Tkeep.emplace_back(tT);
    DevBuf<double>& Tb = Tkeep.back();
    DevBuf<int> perm(tP), rank(nprob2);
    std::vector<IdP> ip(nprob2);
    for (int pr = 0; pr < nprob2; ++pr) {
      const int q = pr / 2, b = boxes[q];
      const int lb = b - proot[prob[b]];
      ip[pr] = IdP{Z.p + oZ[pr], W.p + oZ[pr], m[q], n[q], perm.p + oP[pr], rank.p + pr, Tb.p + oT2[pr], -1,
                   SW.p + oT2[pr], SV.p + oT2[pr], xw.p + oX[pr], yw.p + oYw[pr], 2 * lb + pr % 2, -1,
                   pseed[prob[b]], nullptr};
    }
    DevBuf<IdP> dip;
    upload_vec(dip, ip, st);
    id_adaptive_batched(dip.p, nprob2, acc, st, false);
    std::vector<int> hr;
    download(hr, rank.p, nprob2, st);
    HSS_CUDA(cudaStreamSynchronize(st));
    bool any = false;
    std::vector<int> kbox(nbL);
    for (int q = 0; q < nbL; ++q) {
      const int ko = hr[2 * q], ki = hr[2 * q + 1], k = std::max(ko, ki);
      kbox[q] = k;
      if (k != ko) { ip[2 * q].force_k = k; any = true; }
      else if (k != ki) { ip[2 * q + 1].force_k = k; any = true; }
      HSS_REQUIRE(k <= std::min(m[q], n[q]), HSS_ERR_RANK, "fixed rank exceeds block size");
    }
    if (any) {
      HSS_CUDA(cudaMemcpyAsync(dip.p, ip.data(), nprob2 * sizeof(IdP), cudaMemcpyHostToDevice, st));
      id_fixed_batched(dip.p, nprob2, st);
    }
    std::vector<int> hp;
    download(hp, perm.p, tP, st);
    HSS_CUDA(cudaStreamSynchronize(st));
    // RHO and LAMBDA^T: the ID's skeleton columns of RC and LC^T
    long long tK = 0;
    std::vector<long long> oK(nbL);
    for (int q = 0; q < nbL; ++q) { oK[q] = tK; tK += 2LL * m[q] * kbox[q]; }
    keep.emplace_back(std::max(tK, 1LL));
    DevBuf<double>& Kb = keep.back();
    std::vector<MoveP> mv;
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q], k = kbox[q], nn = n[q];
      double* r = Kb.p + oK[q];
      double* s = r + (size_t)m[q] * k;
      mv.push_back(MoveP{Z.p + oZ[2 * q], r, perm.p + oP[2 * q], m[q], k, m[q], m[q], 1, 0});
      mv.push_back(MoveP{Z.p + oZ[2 * q + 1], s, perm.p + oP[2 * q + 1], m[q], k, m[q], m[q], 1, 0});
      rho[b] = r;
      sig[b] = s;
      mR[b] = m[q];
      std::vector<int> outs, inns;
      if (is_leaf(b)) {
        outs.resize(cnt[b]);
        std::iota(outs.begin(), outs.end(), off[b]);
        inns = outs;
      } else {
        outs = I_SKUP[c1[b]];
        outs.insert(outs.end(), I_SKUP[c2[b]].begin(), I_SKUP[c2[b]].end());
        inns = I_SKDN[c1[b]];
        inns.insert(inns.end(), I_SKDN[c2[b]].begin(), I_SKDN[c2[b]].end());
      }
      nskel[b] = nn;
      kskel[b] = k;
      J_UP[b].assign(hp.begin() + oP[2 * q], hp.begin() + oP[2 * q] + nn);
      J_DN[b].assign(hp.begin() + oP[2 * q + 1], hp.begin() + oP[2 * q + 1] + nn);
      I_SKUP[b].resize(k);
      I_SKDN[b].resize(k);
      for (int t = 0; t < k; ++t) {
        I_SKUP[b][t] = outs[J_UP[b][t]];
        I_SKDN[b][t] = inns[J_DN[b][t]];
      }
      Toff[b] = {oT2[2 * q], oT2[2 * q + 1]};
      Tlev[b] = (int)Tkeep.size() - 1;
      census[4 * b] = m[q]; census[4 * b + 1] = m[q]; census[4 * b + 2] = nn; census[4 * b + 3] = k;
    }
    run_moves(mv, st);
  }
  pack_T(Tkeep, Toff, Tlev);
  // ---- sibling blocks LAMBDA_s1 [M_SIB_A 0; 0 M_SIB_B] RHO_s2, through P = M_SIB_X RHO_s2(rows of X)
  oSib.assign(nboxes, -1);
  long long tb = 0, tw = 0;
  std::vector<long long> oW(nboxes, 0);
  for (int b = 0; b < nboxes; ++b) {
    if (is_leaf(b)) continue;
    HSS_REQUIRE(c1[b] >= 0 && c2[b] >= 0, HSS_ERR_ARG, "one-child boxes are not produced by the halving tree");
    for (int t = 0; t < 2; ++t) {
      const int s = t == 0 ? c1[b] : c2[b], o = t == 0 ? c2[b] : c1[b];
      oSib[s] = tb; tb += (long long)kskel[s] * kskel[o];
      oW[s] = tw; tw += (long long)(A.kskel[s] + B.kskel[s]) * kskel[o];
    }
  }
  M_SIB.alloc(std::max(tb, 1LL));
  DevBuf<double> Wsib(std::max(tw, 1LL));
  std::vector<GemmP<double>> g1, g2, g3;
  for (int b = 0; b < nboxes; ++b) {
    if (is_leaf(b)) continue;
    for (int t = 0; t < 2; ++t) {
      const int s = t == 0 ? c1[b] : c2[b], o = t == 0 ? c2[b] : c1[b];
      const int kAs = A.kskel[s], kBs = B.kskel[s], kAo = A.kskel[o], kBo = B.kskel[o];
      const int ks = kskel[s], ko = kskel[o];
      double* PA = Wsib.p + oW[s];
      double* PB = PA + (size_t)kAs * ko;
      g1.push_back(GemmP<double>{A.M_SIB.p + A.oSib[s], rho[o], PA, kAs, ko, kAo, std::max(kAs, 1), mR[o],
                                 std::max(kAs, 1)});
      g1.push_back(GemmP<double>{B.M_SIB.p + B.oSib[s], rho[o] + kAo, PB, kBs, ko, kBo, std::max(kBs, 1), mR[o],
                                 std::max(kBs, 1)});
      g2.push_back(GemmP<double>{sig[s], PA, M_SIB.p + oSib[s], ks, ko, kAs, mR[s], std::max(kAs, 1),
                                 std::max(ks, 1)});
      g3.push_back(GemmP<double>{sig[s] + kAs, PB, M_SIB.p + oSib[s], ks, ko, kBs, mR[s], std::max(kBs, 1),
                                 std::max(ks, 1)});
    }
  }
  run_gemms(g1, false, false, 1.0, 0.0, st);
  run_gemms(g2, true, false, 1.0, 0.0, st);
  run_gemms(g3, true, false, 1.0, 1.0, st);
  // ---- self blocks
  oSelf = A.oSelf;
  M_SELF.alloc(std::max<size_t>(A.M_SELF.n, 1));
  if (A.M_SELF.n) {
    HSS_CUDA(cudaMemcpyAsync(M_SELF.p, A.M_SELF.p, A.M_SELF.n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    const long long ne = (long long)A.M_SELF.n;
    k_add_into<<<std::min(ceil_div(ne, 256), 4096), 256, 0, st>>>(ne, B.M_SELF.p, M_SELF.p);
    check_launch("k_add_into");
  }
  HSS_CUDA(cudaStreamSynchronize(st));
}

// T_UP / T_DN / T_DN^T and J arenas from the per-level ID outputs (T of box b: k x (n - k),
// ld n, at Tkeep[Tlev[b]] + Toff[b][side])
void HSS1D::pack_T(const std::vector<DevBuf<double>>& Tkeep, const std::vector<std::array<long long, 2>>& Toff,
                   const std::vector<int>& Tlev) {
  oT.assign(nboxes, 0);
  oJ.assign(nboxes, 0);
  long long tt = 0, tj = 0;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] < 0) continue;
    oT[b] = tt; tt += (long long)kskel[b] * (nskel[b] - kskel[b]);
    oJ[b] = tj; tj += nskel[b];
  }
  T_UP.alloc(std::max(tt, 1LL)); T_DN.alloc(std::max(tt, 1LL)); TDNT.alloc(std::max(tt, 1LL));
  std::vector<MoveP> mv;
  std::vector<int> hJU(std::max(tj, 1LL)), hJD(std::max(tj, 1LL));
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] < 0) continue;
    const int n = nskel[b], k = kskel[b];
    std::copy(J_UP[b].begin(), J_UP[b].end(), hJU.begin() + oJ[b]);
    std::copy(J_DN[b].begin(), J_DN[b].end(), hJD.begin() + oJ[b]);
    if (n - k <= 0 || k == 0) continue;
    const double* Tl = Tkeep[Tlev[b]].p;
    mv.push_back(MoveP{Tl + Toff[b][0], T_UP.p + oT[b], nullptr, k, n - k, n, k, 0, 0});
    mv.push_back(MoveP{Tl + Toff[b][1], T_DN.p + oT[b], nullptr, k, n - k, n, k, 0, 0});
    mv.push_back(MoveP{Tl + Toff[b][1], TDNT.p + oT[b], nullptr, k, n - k, n, n - k, 3, 0});
  }
  run_moves(mv, stream);
  upload_vec(JUPd, hJU, stream);
  upload_vec(JDNd, hJD, stream);
  HSS_CUDA(cudaStreamSynchronize(stream));
}

// ---------------------------------------------------------------------------
// K_HSS = HSS1D_compressLR_nsym(U, V, TREE, acc), HSS1D/HSS1D_compressLR_nsym.m:25-88: the
// N x N matrix U V^T on the halving tree.  Per level (deepest first) every box IDs
// V(out,:).' and U(in,:).' (r x n, gathered and transposed on the device) in one batched
// launch, with the rank equalised by the fixed-rank ID; M_SELF = U(ind,:) V(ind,:).' and
// M_SIB{s1} = U(I_SKDN{s1},:) V(I_SKUP{s2},:).' are batched products.
void HSS1D::compress_lr(long long N, int r, const double* U, long long ldu, const double* V, long long ldv,
                        int leaf_, double acc_, unsigned long long seed) {
  HSS_REQUIRE(U && V && N >= 2 && N < (1LL << 30) && r >= 1 && r <= 4096 && ldu >= N && ldv >= N && leaf_ >= 1 &&
                  acc_ > 0 && acc_ < 1,
              HSS_ERR_ARG, "bad low-rank compress args");
  std::fill(phase_s, phase_s + NPHASE, 0.0);
  rect = false; sym = false; id_df = false;
  nprob = 1; leaf = leaf_; acc = acc_;
  kp = hss_kernel_params{};
  Ntot = N;
  pN = {N}; pbase = {0}; pseed = {seed};
  proot.assign(1, 0);
  X.assign(6 * (size_t)N, 0.0);
  prob.clear(); level.clear(); parent.clear(); c1.clear(); c2.clear(); off.clear(); cnt.clear();
  append_tree(0, 0, (int)N);
  nboxes = (int)level.size();
  maxlev = *std::max_element(level.begin(), level.end());
  precision = HSS_PREC_FP64;
  inverted = false;
  clear_plans();
  const cudaStream_t st = stream;
  DevBuf<double> Ud((size_t)N * r), Vd((size_t)N * r);
  HSS_CUDA(cudaMemcpy2DAsync(Ud.p, N * sizeof(double), U, ldu * sizeof(double), N * sizeof(double), r,
                             cudaMemcpyHostToDevice, st));
  HSS_CUDA(cudaMemcpy2DAsync(Vd.p, N * sizeof(double), V, ldv * sizeof(double), N * sizeof(double), r,
                             cudaMemcpyHostToDevice, st));
  nskel.assign(nboxes, 0); kskel.assign(nboxes, 0);
  I_SKUP.assign(nboxes, {}); I_SKDN.assign(nboxes, {});
  J_UP.assign(nboxes, {}); J_DN.assign(nboxes, {});
  census.assign(4 * (size_t)nboxes, 0);
  feat.assign((size_t)NFEAT * nboxes, 0.f);
  qr_steps = qr_steps_full = 0;
  reruns = 0;
  std::vector<DevBuf<double>> Tkeep;
  std::vector<std::array<long long, 2>> Toff(nboxes);
  std::vector<int> Tlev(nboxes, -1);
  for (int L = maxlev; L >= 1; --L) {
    std::vector<int> boxes;
    for (int b = 0; b < nboxes; ++b)
      if (level[b] == L) boxes.push_back(b);
    if (boxes.empty()) continue;
    const int nbL = (int)boxes.size(), nprob2 = 2 * nbL;
    std::vector<std::vector<int>> outs(nbL), inns(nbL);
    std::vector<int> idx;
    std::vector<long long> oI(nprob2), oA(nprob2), oT2(nprob2), oX(nprob2), oY(nprob2), oP(nprob2);
    long long tA = 0, tT = 0, tX = 0, tY = 0, tP = 0;
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q];
      if (is_leaf(b)) {
        outs[q].resize(cnt[b]);
        std::iota(outs[q].begin(), outs[q].end(), off[b]);
        inns[q] = outs[q];
      } else {
        outs[q] = I_SKUP[c1[b]];
        outs[q].insert(outs[q].end(), I_SKUP[c2[b]].begin(), I_SKUP[c2[b]].end());
        inns[q] = I_SKDN[c1[b]];
        inns[q].insert(inns[q].end(), I_SKDN[c2[b]].begin(), I_SKDN[c2[b]].end());
      }
      const int n = (int)outs[q].size();
      HSS_REQUIRE(n >= 1 && n <= 4096, HSS_ERR_RANK, "empty or oversized skeleton set");
      for (int s = 0; s < 2; ++s) {
        const int pr = 2 * q + s;
        oI[pr] = idx.size();
        const auto& v = s == 0 ? outs[q] : inns[q];
        idx.insert(idx.end(), v.begin(), v.end());
        oA[pr] = tA; tA += (long long)r * n;
        oT2[pr] = tT; tT += (long long)n * n;
        oX[pr] = tX; tX += 2LL * n;
        oY[pr] = tY; tY += (long long)r + n;
        oP[pr] = tP; tP += n;
      }
    }
    DevBuf<int> didx;
    upload_vec(didx, idx, st);
    // A = V(out,:).' / U(in,:).': row gather (n x r) then transpose (r x n)
    DevBuf<double> G(std::max(tA, 1LL)), A(std::max(tA, 1LL)), W(std::max(tA, 1LL)), SW(tT), SV(tT), xw(tX), yw(tY);
    std::vector<MoveP> g, tr;
    for (int pr = 0; pr < nprob2; ++pr) {
      const int n = (int)outs[pr / 2].size();
      g.push_back(MoveP{pr % 2 == 0 ? Vd.p : Ud.p, G.p + oA[pr], didx.p + oI[pr], n, r, (int)N, n, 0, 0});
      tr.push_back(MoveP{G.p + oA[pr], A.p + oA[pr], nullptr, n, r, n, r, 3, 0});
    }
    run_moves(g, st);
    run_moves(tr, st);
    Tkeep.emplace_back(tT);
    DevBuf<double>& Tb = Tkeep.back();
    DevBuf<int> perm(tP), rank(nprob2);
    std::vector<IdP> ip(nprob2);
    for (int pr = 0; pr < nprob2; ++pr) {
      const int n = (int)outs[pr / 2].size();
      ip[pr] = IdP{A.p + oA[pr], W.p + oA[pr], r, n, perm.p + oP[pr], rank.p + pr, Tb.p + oT2[pr], -1,
                   SW.p + oT2[pr], SV.p + oT2[pr], xw.p + oX[pr], yw.p + oY[pr], 2 * boxes[pr / 2] + pr % 2, -1,
                   seed, nullptr};
    }
    DevBuf<IdP> dip;
    upload_vec(dip, ip, st);
    id_adaptive_batched(dip.p, nprob2, acc, st, false);
    std::vector<int> hr;
    download(hr, rank.p, nprob2, st);
    HSS_CUDA(cudaStreamSynchronize(st));
    bool any = false;
    std::vector<int> kbox(nbL);
    for (int q = 0; q < nbL; ++q) {
      const int ko = hr[2 * q], ki = hr[2 * q + 1], k = std::max(ko, ki);
      kbox[q] = k;
      if (k != ko) { ip[2 * q].force_k = k; any = true; }
      else if (k != ki) { ip[2 * q + 1].force_k = k; any = true; }
    }
    if (any) {
      HSS_CUDA(cudaMemcpyAsync(dip.p, ip.data(), nprob2 * sizeof(IdP), cudaMemcpyHostToDevice, st));
      id_fixed_batched(dip.p, nprob2, st);
    }
    std::vector<int> hp;
    download(hp, perm.p, tP, st);
    HSS_CUDA(cudaStreamSynchronize(st));
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q], k = kbox[q], n = (int)outs[q].size();
      nskel[b] = n;
      kskel[b] = k;
      J_UP[b].assign(hp.begin() + oP[2 * q], hp.begin() + oP[2 * q] + n);
      J_DN[b].assign(hp.begin() + oP[2 * q + 1], hp.begin() + oP[2 * q + 1] + n);
      I_SKUP[b].resize(k);
      I_SKDN[b].resize(k);
      for (int t = 0; t < k; ++t) {
        I_SKUP[b][t] = outs[q][J_UP[b][t]];
        I_SKDN[b][t] = inns[q][J_DN[b][t]];
      }
      Toff[b] = {oT2[2 * q], oT2[2 * q + 1]};
      Tlev[b] = (int)Tkeep.size() - 1;
      census[4 * b] = r; census[4 * b + 1] = r; census[4 * b + 2] = n; census[4 * b + 3] = k;
    }
  }
  pack_T(Tkeep, Toff, Tlev);
  Tkeep.clear();
  // ---- M_SELF = U(ind,:) V(ind,:).', M_SIB{s1} = U(I_SKDN{s1},:) V(I_SKUP{s2},:).'
  oSelf.assign(nboxes, -1);
  oSib.assign(nboxes, -1);
  long long ts = 0, tb = 0, tg = 0;
  std::vector<long long> oG(nboxes, 0);
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] >= 0 && is_leaf(b)) { oSelf[b] = ts; ts += (long long)cnt[b] * cnt[b]; }
    if (!is_leaf(b)) {
      const int s1 = c1[b], s2 = c2[b];
      oSib[s1] = tb; tb += (long long)kskel[s1] * kskel[s2];
      oSib[s2] = tb; tb += (long long)kskel[s2] * kskel[s1];
      for (int s : {s1, s2}) { oG[s] = tg; tg += 2LL * kskel[s] * r; }
    }
  }
  M_SELF.alloc(std::max(ts, 1LL));
  M_SIB.alloc(std::max(tb, 1LL));
  // per son s: U(I_SKDN{s},:) and V(I_SKUP{s},:) (k_s x r each)
  std::vector<int> idx;
  std::vector<long long> oIx(nboxes, 0);
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] < 0) continue;
    oIx[b] = idx.size();
    idx.insert(idx.end(), I_SKDN[b].begin(), I_SKDN[b].end());
    idx.insert(idx.end(), I_SKUP[b].begin(), I_SKUP[b].end());
  }
  DevBuf<int> didx;
  upload_vec(didx, idx, st);
  DevBuf<double> Gs(std::max(tg, 1LL));
  std::vector<MoveP> mv;
  std::vector<GemmP<double>> P;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] >= 0 && is_leaf(b))
      P.push_back(GemmP<double>{Ud.p + off[b], Vd.p + off[b], M_SELF.p + oSelf[b], cnt[b], cnt[b], r, (int)N, (int)N,
                                cnt[b]});
    if (parent[b] >= 0 && kskel[b] > 0) {
      const int k = kskel[b];
      mv.push_back(MoveP{Ud.p, Gs.p + oG[b], didx.p + oIx[b], k, r, (int)N, k, 0, 0});
      mv.push_back(MoveP{Vd.p, Gs.p + oG[b] + (size_t)k * r, didx.p + oIx[b] + k, k, r, (int)N, k, 0, 0});
    }
  }
  run_moves(mv, st);
  for (int b = 0; b < nboxes; ++b) {
    if (is_leaf(b)) continue;
    for (int t = 0; t < 2; ++t) {
      const int s = t == 0 ? c1[b] : c2[b], o = t == 0 ? c2[b] : c1[b];
      const int ks = kskel[s], ko = kskel[o];
      if (ks == 0 || ko == 0) continue;
      P.push_back(GemmP<double>{Gs.p + oG[s], Gs.p + oG[o] + (size_t)ko * r, M_SIB.p + oSib[s], ks, ko, r, ks, ko,
                                ks});
    }
  }
  run_gemms(P, false, true, 1.0, 0.0, st);
}

}  // namespace hss

namespace hss {

// ---------------------------------------------------------------------------
// A_NEW = HSS1D_recompress_nsym(A, acc), HSS1D/HSS1D_recompress_nsym.m:26-247: the ranks of
// a compressed matrix reduced to what acc needs (after sums and low-rank updates).
//  (I) top down (:30-146), level by level over every parent: the root's sibling blocks are
//      truncated by their SVDs (singular values above the absolute acc); every other parent
//      stacks its sons' sibling blocks with its far-field factors, Sson = [B, L0 S0] and
//      Tson = [B; T0 R0], and truncates their SVDs, which gives each son a reduced row basis
//      Q^H R and column basis L P, and the parent's reduced sibling blocks;
//  (II) bottom up (:148-246): each box IDs its reduced bases at full rank (pivoted QR of
//      RNEW and LNEW^T, k = min(size)), keeps RHO / LAMBDA, and the sibling blocks become
//      LAMBDA_s1 sib RHO_s2.
// The SVDs are one-sided Jacobi on the GPU (Hestenes; the basis of a cluster of equal
// singular values is the method's own, but every quantity the result keeps is invariant
// under that choice: the skeleton pivots depend on the column norms of projections, T on
// the row space, the sibling blocks on the operator).

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct SvdP {
  double* X;  // m x n, ld m: overwritten by X V = U S (orthogonal columns)
  double* V;  // n x n, ld n: the accumulated rotations
  double* s;  // n: the column norms of X V (the singular values, unsorted)
  int m, n;
};

__global__ void __launch_bounds__(256) k_jacobi_svd(const SvdP* __restrict__ P) {
  const SvdP p = P[blockIdx.x];
  const int m = p.m, n = p.n, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  __shared__ int s_rot;
  for (int e = tid; e < n * n; e += 256) p.V[e] = ((e % n) == (e / n)) ? 1.0 : 0.0;
  __syncthreads();
  const int K2 = (n % 2 == 0) ? n : n + 1;
  for (int sweep = 0; sweep < 60 && n > 1; ++sweep) {
    if (tid == 0) s_rot = 0;
    __syncthreads();
    for (int rnd = 0; rnd < K2 - 1; ++rnd) {
      for (int pi = w; pi < K2 / 2; pi += 8) {
        int a, b;
        if (pi == 0) { a = K2 - 1; b = rnd; }
        else { a = (rnd + pi) % (K2 - 1); b = (rnd - pi + K2 - 1) % (K2 - 1); }
        if (a >= n || b >= n) continue;
        if (a > b) { const int t = a; a = b; b = t; }
        double al = 0.0, be = 0.0, ga = 0.0;
        for (int i = lane; i < m; i += 32) {
          const double u = p.X[i + (size_t)a * m], v = p.X[i + (size_t)b * m];
          al += u * u; be += v * v; ga += u * v;
        }
        al = warp_sum_d(al); be = warp_sum_d(be); ga = warp_sum_d(ga);
        double c = 1.0, s = 0.0;
        int rot = 0;
        if (lane == 0 && ga != 0.0 && fabs(ga) > 1e-15 * sqrt(al * be)) {
          const double zeta = (be - al) / (2.0 * ga);
          const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          c = 1.0 / sqrt(1.0 + t * t);
          s = c * t;
          rot = 1;
        }
        rot = __shfl_sync(0xffffffffu, rot, 0);
        if (rot) {
          c = __shfl_sync(0xffffffffu, c, 0);
          s = __shfl_sync(0xffffffffu, s, 0);
          for (int i = lane; i < m; i += 32) {
            const double u = p.X[i + (size_t)a * m], v = p.X[i + (size_t)b * m];
            p.X[i + (size_t)a * m] = c * u - s * v;
            p.X[i + (size_t)b * m] = s * u + c * v;
          }
          for (int i = lane; i < n; i += 32) {
            const double u = p.V[i + (size_t)a * n], v = p.V[i + (size_t)b * n];
            p.V[i + (size_t)a * n] = c * u - s * v;
            p.V[i + (size_t)b * n] = s * u + c * v;
          }
          if (lane == 0) s_rot = 1;
        }
      }
      __syncthreads();
    }
    const int any = s_rot;
    __syncthreads();
    if (!any) break;
  }
  for (int j = w; j < n; j += 8) {
    double d = 0.0;
    for (int i = lane; i < m; i += 32) { const double v = p.X[i + (size_t)j * m]; d += v * v; }
    d = warp_sum_d(d);
    if (lane == 0) p.s[j] = sqrt(d);
  }
}

// dst (rows x cols, ld ldd) = src columns idx[j] (ld lds), each scaled by scale[j] (or 1)
struct GatherP {
  const double* src;
  double* dst;
  const int* idx;
  const double* scale;
  int rows, cols, lds, ldd;
};

__global__ void __launch_bounds__(256) k_gather_cols(const GatherP* __restrict__ P) {
  const GatherP p = P[blockIdx.x];
  const long long tot = (long long)p.rows * p.cols;
  for (long long e = threadIdx.x; e < tot; e += 256) {
    const int i = (int)(e % p.rows), j = (int)(e / p.rows);
    const double f = p.scale ? p.scale[j] : 1.0;
    p.dst[i + (size_t)j * p.ldd] = f * p.src[i + (size_t)p.idx[j] * p.lds];
  }
}

static void run_gathers(const std::vector<GatherP>& G, cudaStream_t s) {
  if (G.empty()) return;
  DevBuf<GatherP> d;
  upload_vec(d, G, s);
  for (size_t o = 0; o < G.size(); o += 65535) {
    const int c = (int)std::min<size_t>(65535, G.size() - o);
    k_gather_cols<<<c, 256, 0, s>>>(d.p + o);
    check_launch("k_gather_cols");
  }
  HSS_CUDA(cudaStreamSynchronize(s));
}

// a rectangular diagonal matrix (rows x cols, the diagonal d of min(rows, cols) entries)
struct RDiag {
  int rows = 0, cols = 0;
  std::vector<double> d;
};

void HSS1D::recompress(const HSS1D& A, double acc_) {
  HSS_REQUIRE(!A.cplx && !A.rect, HSS_ERR_ARG, "recompress is defined for real square handles");
  HSS_REQUIRE(acc_ > 0 && acc_ < 1, HSS_ERR_ARG, "bad recompress tolerance");
  const cudaStream_t st = stream;
  std::fill(phase_s, phase_s + NPHASE, 0.0);
  Ntot = A.Ntot; nprob = A.nprob; nboxes = A.nboxes; leaf = A.leaf; maxlev = A.maxlev; acc = acc_;
  sym = false; rect = false; id_df = false; cplx = false; kernel_op = false;
  pN = A.pN; pbase = A.pbase; proot = A.proot; pseed = A.pseed;
  prob = A.prob; level = A.level; parent = A.parent; c1 = A.c1; c2 = A.c2; off = A.off; cnt = A.cnt;
  X = A.X; kp = A.kp; kdev = A.kdev;
  precision = HSS_PREC_FP64;
  inverted = false;
  clear_plans();
  for (int b = 0; b < nboxes; ++b)
    HSS_REQUIRE(is_leaf(b) || (c1[b] >= 0 && c2[b] >= 0), HSS_ERR_ARG, "recompress: one-child boxes");
  const int nb = nboxes;
  // the operand's R = [I T_UP](:, J_UP) (k x n) and L^T = [I T_DN](:, J_DN) of every box
  std::vector<DevBuf<double>> Rf(nb), Lt(nb);
  {
    std::vector<RformP> rf;
    for (int b = 0; b < nb; ++b) {
      if (parent[b] < 0) continue;
      const int k = A.kskel[b], n = A.nskel[b];
      Rf[b].alloc(std::max((size_t)k * n, (size_t)1));
      Lt[b].alloc(std::max((size_t)k * n, (size_t)1));
      Rf[b].zero(st);
      Lt[b].zero(st);
      if (k == 0) continue;
      rf.push_back(RformP{A.T_UP.p + A.oT[b], A.JUPd.p + A.oJ[b], Rf[b].p, k, n, k});
      rf.push_back(RformP{A.T_DN.p + A.oT[b], A.JDNd.p + A.oJ[b], Lt[b].p, k, n, k});
    }
    if (!rf.empty()) {
      DevBuf<RformP> drf;
      upload_vec(drf, rf, st);
      for (size_t o = 0; o < rf.size(); o += 65535) {
        const int c = (int)std::min<size_t>(65535, rf.size() - o);
        k_rform<<<c, 256, 0, st>>>(drf.p + o);
        check_launch("k_rform");
      }
    }
  }
  // (I) top down.  Per box: Rp (kn x n_b: rows of the reduced outgoing basis), Lp (n_b x kn),
  // the diagonal factors Tp / Sp, and the reduced sibling block sib (kn_s1 x kn_s2).
  std::vector<DevBuf<double>> Rp(nb), Lp(nb), sib(nb);
  std::vector<int> kn(nb, 0);
  std::vector<RDiag> Tp(nb), Sp(nb);
  const double* Asib = A.M_SIB.p;
  auto gemm = [](std::vector<GemmP<double>>& v, const double* a, int lda, const double* b, int ldb, double* c, int ldc,
                 int M, int N, int K) {
    if (M > 0 && N > 0 && K > 0) v.push_back(GemmP<double>{a, b, c, M, N, K, lda, ldb, ldc});
  };
  for (int L = 0; L < maxlev; ++L) {
    std::vector<int> par;
    for (int b = 0; b < nb; ++b)
      if (level[b] == L && !is_leaf(b)) par.push_back(b);
    if (par.empty()) continue;
    const int np = (int)par.size();
    // the SVD inputs: root [B1 | B2]; other parents T1 = [B2; T0 R0(:, :k1)], T2 = [B1; T0
    // R0(:, k1:)], S1^T = [B1 | L0(:k1, :) S0]^T, S2^T
    struct Job { int m, n; };
    std::vector<std::array<Job, 4>> jobs(np);
    std::vector<std::array<long long, 4>> oX(np), oV(np), oS(np);
    long long tXs = 0, tVs = 0, tSs = 0;
    for (int q = 0; q < np; ++q) {
      const int b = par[q], s1 = c1[b], s2 = c2[b], k1 = A.kskel[s1], k2 = A.kskel[s2];
      if (parent[b] < 0) {
        jobs[q] = {Job{k1, k2}, Job{k2, k1}, Job{0, 0}, Job{0, 0}};
      } else {
        const int rT = Tp[b].rows, cS = Sp[b].cols;
        jobs[q] = {Job{k2 + rT, k1}, Job{k1 + rT, k2}, Job{k2 + cS, k1}, Job{k1 + cS, k2}};
      }
      for (int j = 0; j < 4; ++j) {
        oX[q][j] = tXs; tXs += (long long)jobs[q][j].m * jobs[q][j].n;
        oV[q][j] = tVs; tVs += (long long)jobs[q][j].n * jobs[q][j].n;
        oS[q][j] = tSs; tSs += jobs[q][j].n;
      }
    }
    DevBuf<double> Xs(std::max(tXs, 1LL)), Vs(std::max(tVs, 1LL)), Ss(std::max(tSs, 1LL)), tmp;
    Xs.zero(st);
    std::vector<MoveP> mv;
    std::vector<GemmP<double>> gNN, gTN;  // plain products; A transposed
    // far-field parts of the stacks: T0 R0(:, cols) and L0(rows, :) S0 through diagonal factors
    // (host-built dense diagonal matrices, small)
    std::vector<DevBuf<double>> Dm(2 * np);
    for (int q = 0; q < np; ++q) {
      const int b = par[q], s1 = c1[b], s2 = c2[b], k1 = A.kskel[s1], k2 = A.kskel[s2];
      const double* B1 = Asib + A.oSib[s1];
      const double* B2 = Asib + A.oSib[s2];
      if (parent[b] < 0) {
        mv.push_back(MoveP{B1, Xs.p + oX[q][0], nullptr, k1, k2, k1, k1, 0, 0});
        mv.push_back(MoveP{B2, Xs.p + oX[q][1], nullptr, k2, k1, k2, k2, 0, 0});
        continue;
      }
      const RDiag &T0 = Tp[b], &S0 = Sp[b];
      std::vector<double> hT((size_t)T0.rows * T0.cols, 0.0), hS((size_t)S0.rows * S0.cols, 0.0);
      for (size_t i = 0; i < T0.d.size(); ++i) hT[i + i * T0.rows] = T0.d[i];
      for (size_t i = 0; i < S0.d.size(); ++i) hS[i + i * S0.rows] = S0.d[i];
      upload_vec(Dm[2 * q], hT, st);
      upload_vec(Dm[2 * q + 1], hS, st);
      const int kb = kn[b];  // = T0.cols = S0.rows = rows of R0 = cols of L0
      const double* R0 = Rp[b].p;  // kb x (k1 + k2)
      const double* L0 = Lp[b].p;  // (k1 + k2) x kb
      const int rT = T0.rows, cS = S0.cols;
      // job 0: T1 = [B2; T0 R0(:, :k1)]  ((k2 + rT) x k1)
      mv.push_back(MoveP{B2, Xs.p + oX[q][0], nullptr, k2, k1, k2, k2 + rT, 0, 0});
      gemm(gNN, Dm[2 * q].p, rT, R0, kb, Xs.p + oX[q][0] + k2, k2 + rT, rT, k1, kb);
      // job 1: T2 = [B1; T0 R0(:, k1:)]  ((k1 + rT) x k2)
      mv.push_back(MoveP{B1, Xs.p + oX[q][1], nullptr, k1, k2, k1, k1 + rT, 0, 0});
      gemm(gNN, Dm[2 * q].p, rT, R0 + (size_t)k1 * kb, kb, Xs.p + oX[q][1] + k1, k1 + rT, rT, k2, kb);
      // job 2: S1^T = [B1 | L0(:k1, :) S0]^T = [B1^T; S0^T L0(:k1, :)^T]  ((k2 + cS) x k1)
      mv.push_back(MoveP{B1, Xs.p + oX[q][2], nullptr, k1, k2, k1, k2 + cS, 3, 0});
      // (S0^T L0(:k1,:)^T) = (L0(:k1,:) S0)^T: C (cS x k1) = S0^T (cS x kb) * L0(:k1,:)^T
      gemm(gTN, Dm[2 * q + 1].p, kb, L0, k1 + k2, Xs.p + oX[q][2] + k2, k2 + cS, cS, k1, kb);
      // job 3: S2^T = [B2^T; S0^T L0(k1:, :)^T]  ((k1 + cS) x k2)
      mv.push_back(MoveP{B2, Xs.p + oX[q][3], nullptr, k2, k1, k2, k1 + cS, 3, 0});
      gemm(gTN, Dm[2 * q + 1].p, kb, L0 + k1, k1 + k2, Xs.p + oX[q][3] + k1, k1 + cS, cS, k2, kb);
    }
    run_moves(mv, st);
    // the L0 rows are read transposed: C = S0^T * L0(rows, :)^T needs B transposed too
    if (!gNN.empty()) run_gemms(gNN, false, false, 1.0, 0.0, st);
    if (!gTN.empty()) run_gemms(gTN, true, true, 1.0, 0.0, st);
    std::vector<SvdP> sp;
    for (int q = 0; q < np; ++q)
      for (int j = 0; j < 4; ++j)
        if (jobs[q][j].m > 0 && jobs[q][j].n > 0)
          sp.push_back(SvdP{Xs.p + oX[q][j], Vs.p + oV[q][j], Ss.p + oS[q][j], jobs[q][j].m, jobs[q][j].n});
    {
      DevBuf<SvdP> dsp;
      upload_vec(dsp, sp, st);
      for (size_t o = 0; o < sp.size(); o += 65535) {
        const int c = (int)std::min<size_t>(65535, sp.size() - o);
        k_jacobi_svd<<<c, 256, 0, st>>>(dsp.p + o);
        check_launch("k_jacobi_svd");
      }
    }
    std::vector<double> hs;
    download(hs, Ss.p, std::max(tSs, 1LL), st);
    HSS_CUDA(cudaStreamSynchronize(st));
    // sorted singular values per job, the truncation ranks, and the gathered factors
    std::vector<std::array<std::vector<int>, 4>> ord(np);
    std::vector<std::array<std::vector<double>, 4>> sv(np);
    std::vector<int> hidx;
    std::vector<double> hscale;
    std::vector<std::array<long long, 4>> oI(np);
    for (int q = 0; q < np; ++q)
      for (int j = 0; j < 4; ++j) {
        const int n = jobs[q][j].n;
        std::vector<int> o(n);
        std::iota(o.begin(), o.end(), 0);
        const double* s = hs.data() + oS[q][j];
        std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return s[a] > s[b]; });
        // a thin SVD keeps min(m, n) values
        const int r = std::min(jobs[q][j].m, n);
        ord[q][j] = o;
        sv[q][j].resize(r);
        for (int t = 0; t < r; ++t) sv[q][j][t] = s[o[t]];
        oI[q][j] = (long long)hidx.size();
        for (int t = 0; t < n; ++t) {
          hidx.push_back(o[t]);
          hscale.push_back((t < r && s[o[t]] > 0.0) ? 1.0 / s[o[t]] : 0.0);
        }
      }
    DevBuf<int> didx;
    DevBuf<double> dscale;
    upload_vec(didx, hidx, st);
    upload_vec(dscale, hscale, st);
    auto count = [&](const std::vector<double>& v) {
      int c = 0;
      for (double x : v) c += (x > acc) ? 1 : 0;
      return c;
    };
    // per parent: P1 (k1 x k1n), P2, Q1 (k1 x k1n), Q2 (k2 x k2n), Y1 (rows of T1 x k1n), Y2
    std::vector<std::array<DevBuf<double>, 6>> F(np);
    std::vector<GatherP> gat;
    for (int q = 0; q < np; ++q) {
      const int b = par[q], s1 = c1[b], s2 = c2[b], k1 = A.kskel[s1], k2 = A.kskel[s2];
      int k1n, k2n;
      if (parent[b] < 0) {
        k1n = count(sv[q][0]);  // B1 = P1 D1 Q2^H
        k2n = count(sv[q][1]);  // B2 = P2 D2 Q1^H
        // P1: the normalised columns of X1 V; Q2: V of job 0; P2, Q1 from job 1
        F[q][0].alloc(std::max(1, k1 * k1n));  // P1
        F[q][1].alloc(std::max(1, k2 * k2n));  // P2
        F[q][2].alloc(std::max(1, k1 * k1n));  // Q1
        F[q][3].alloc(std::max(1, k2 * k2n));  // Q2
        gat.push_back(GatherP{Xs.p + oX[q][0], F[q][0].p, didx.p + oI[q][0], dscale.p + oI[q][0], k1, k1n, k1, k1});
        gat.push_back(GatherP{Xs.p + oX[q][1], F[q][1].p, didx.p + oI[q][1], dscale.p + oI[q][1], k2, k2n, k2, k2});
        gat.push_back(GatherP{Vs.p + oV[q][1], F[q][2].p, didx.p + oI[q][1], nullptr, k1, k1n, k1, k1});
        gat.push_back(GatherP{Vs.p + oV[q][0], F[q][3].p, didx.p + oI[q][0], nullptr, k2, k2n, k2, k2});
        // sib{s1} = D1m (k1n x k2n), sib{s2} = D2m; Tp{s1} = D2m, Tp{s2} = D1m; Sp{s1} = D1m,
        // Sp{s2} = D2m (:52-60)
        RDiag D1m, D2m;
        D1m.rows = k1n; D1m.cols = k2n;
        D2m.rows = k2n; D2m.cols = k1n;
        for (int t = 0; t < std::min(k1n, k2n); ++t) { D1m.d.push_back(sv[q][0][t]); D2m.d.push_back(sv[q][1][t]); }
        Tp[s1] = D2m; Tp[s2] = D1m; Sp[s1] = D1m; Sp[s2] = D2m;
        for (int s : {s1, s2}) {
          const RDiag& D = (s == s1) ? D1m : D2m;
          std::vector<double> h((size_t)D.rows * D.cols, 0.0);
          for (size_t i = 0; i < D.d.size(); ++i) h[i + i * D.rows] = D.d[i];
          upload_vec(sib[s], h, st);
          if (h.empty()) sib[s].alloc(1);
        }
      } else {
        const int rT = Tp[b].rows;
        const int kt1 = count(sv[q][0]), kt2 = count(sv[q][1]), ks1 = count(sv[q][2]), ks2 = count(sv[q][3]);
        k1n = std::max(kt1, ks1);
        k2n = std::max(kt2, ks2);
        HSS_REQUIRE(k1n <= (int)sv[q][0].size() && k1n <= (int)sv[q][2].size() && k2n <= (int)sv[q][1].size() &&
                        k2n <= (int)sv[q][3].size(),
                    HSS_ERR_RANK, "recompress: truncation rank above the block size");
        F[q][0].alloc(std::max(1, k1 * k1n));          // P1: V of job 2
        F[q][1].alloc(std::max(1, k2 * k2n));          // P2: V of job 3
        F[q][2].alloc(std::max(1, k1 * k1n));          // Q1: V of job 0
        F[q][3].alloc(std::max(1, k2 * k2n));          // Q2: V of job 1
        F[q][4].alloc(std::max(1, (k2 + rT) * k1n));   // Y1 (normalised)
        F[q][5].alloc(std::max(1, (k1 + rT) * k2n));   // Y2
        gat.push_back(GatherP{Vs.p + oV[q][2], F[q][0].p, didx.p + oI[q][2], nullptr, k1, k1n, k1, k1});
        gat.push_back(GatherP{Vs.p + oV[q][3], F[q][1].p, didx.p + oI[q][3], nullptr, k2, k2n, k2, k2});
        gat.push_back(GatherP{Vs.p + oV[q][0], F[q][2].p, didx.p + oI[q][0], nullptr, k1, k1n, k1, k1});
        gat.push_back(GatherP{Vs.p + oV[q][1], F[q][3].p, didx.p + oI[q][1], nullptr, k2, k2n, k2, k2});
        gat.push_back(GatherP{Xs.p + oX[q][0], F[q][4].p, didx.p + oI[q][0], dscale.p + oI[q][0], k2 + rT, k1n, k2 + rT,
                              k2 + rT});
        gat.push_back(GatherP{Xs.p + oX[q][1], F[q][5].p, didx.p + oI[q][1], dscale.p + oI[q][1], k1 + rT, k2n, k1 + rT,
                              k1 + rT});
        RDiag DT1, DT2, DS1, DS2;
        DT1.rows = DT1.cols = k1n; DS1.rows = DS1.cols = k1n;
        DT2.rows = DT2.cols = k2n; DS2.rows = DS2.cols = k2n;
        DT1.d.assign(sv[q][0].begin(), sv[q][0].begin() + k1n);
        DT2.d.assign(sv[q][1].begin(), sv[q][1].begin() + k2n);
        DS1.d.assign(sv[q][2].begin(), sv[q][2].begin() + k1n);
        DS2.d.assign(sv[q][3].begin(), sv[q][3].begin() + k2n);
        Tp[s1] = DT1; Tp[s2] = DT2; Sp[s1] = DS1; Sp[s2] = DS2;
      }
      kn[s1] = k1n;
      kn[s2] = k2n;
    }
    run_gathers(gat, st);
    // sib, Rp / Lp of the parent (non-root) and of the sons
    std::vector<GemmP<double>> g1, g2, g3, g4;  // NN, TN (A^T B), NT (A B^T), TT
    std::vector<DevBuf<double>> W(np);
    for (int q = 0; q < np; ++q) {
      const int b = par[q], s1 = c1[b], s2 = c2[b], k1 = A.kskel[s1], k2 = A.kskel[s2];
      const int k1n = kn[s1], k2n = kn[s2];
      const double *P1 = F[q][0].p, *P2 = F[q][1].p, *Q1 = F[q][2].p, *Q2 = F[q][3].p;
      if (parent[b] >= 0) {
        const int rT = Tp[b].rows, kb = kn[b];
        // sib{s1} = P1^H Y2(:k1, :) DT2 ; sib{s2} = P2^H Y1(:k2, :) DT1 (Y already divided by
        // the singular values, so Y DT = the unnormalised columns of T V)
        sib[s1].alloc(std::max(1, k1n * k2n));
        sib[s2].alloc(std::max(1, k2n * k1n));
        W[q].alloc(std::max<size_t>(1, (size_t)(k1 + rT) * k2n + (size_t)(k2 + rT) * k1n));
        double* U2 = W[q].p;                              // (k1 + rT) x k2n: T2 V(:, ord)
        double* U1 = W[q].p + (size_t)(k1 + rT) * k2n;    // (k2 + rT) x k1n
        // Y DT: gather the unscaled columns
        std::vector<GatherP> gg;
        gg.push_back(GatherP{Xs.p + oX[q][1], U2, didx.p + oI[q][1], nullptr, k1 + rT, k2n, k1 + rT, k1 + rT});
        gg.push_back(GatherP{Xs.p + oX[q][0], U1, didx.p + oI[q][0], nullptr, k2 + rT, k1n, k2 + rT, k2 + rT});
        run_gathers(gg, st);
        gemm(g2, P1, k1, U2, k1 + rT, sib[s1].p, std::max(k1n, 1), k1n, k2n, k1);
        gemm(g2, P2, k2, U1, k2 + rT, sib[s2].p, std::max(k2n, 1), k2n, k1n, k2);
        // Rp{b} = [R0(:, :k1) Q1, R0(:, k1:) Q2]  (kb x (k1n + k2n)); Lp{b} = [P1^H L0(:k1, :);
        // P2^H L0(k1:, :)]  ((k1n + k2n) x kb)
        DevBuf<double> Rn(std::max(1, kb * (k1n + k2n))), Ln(std::max(1, (k1n + k2n) * kb));
        gemm(g1, Rp[b].p, kb, Q1, k1, Rn.p, kb, kb, k1n, k1);
        gemm(g1, Rp[b].p + (size_t)k1 * kb, kb, Q2, k2, Rn.p + (size_t)k1n * kb, kb, kb, k2n, k2);
        gemm(g2, P1, k1, Lp[b].p, k1 + k2, Ln.p, k1n + k2n, k1n, kb, k1);
        gemm(g2, P2, k2, Lp[b].p + k1, k1 + k2, Ln.p + k1n, k1n + k2n, k2n, kb, k2);
        // run now: Rp{b} / Lp{b} are replaced below
        run_gemms(g1, false, false, 1.0, 0.0, st);
        run_gemms(g2, true, false, 1.0, 0.0, st);
        g1.clear();
        g2.clear();
        Rp[b] = std::move(Rn);
        Lp[b] = std::move(Ln);
      }
      // sons: Rp{s} = Q^H R_s (kn_s x n_s), Lp{s} = L_s P (n_s x kn_s) = (L_s^T)^T P
      for (int side = 0; side < 2; ++side) {
        const int s = side ? s2 : s1, ks = A.kskel[s], ns = A.nskel[s], kns = kn[s];
        const double* Q = side ? Q2 : Q1;
        const double* Pm = side ? P2 : P1;
        Rp[s].alloc(std::max(1, kns * ns));
        Lp[s].alloc(std::max(1, ns * kns));
        gemm(g2, Q, ks, Rf[s].p, ks, Rp[s].p, std::max(kns, 1), kns, ns, ks);
        gemm(g2, Lt[s].p, ks, Pm, ks, Lp[s].p, ns, ns, kns, ks);
      }
    }
    run_gemms(g2, true, false, 1.0, 0.0, st);
  }
  // (II) bottom up
  nskel.assign(nb, 0); kskel.assign(nb, 0);
  I_SKUP.assign(nb, {}); I_SKDN.assign(nb, {});
  J_UP.assign(nb, {}); J_DN.assign(nb, {});
  census.assign(4 * (size_t)nb, 0);
  feat.assign((size_t)NFEAT * nb, 0.f);
  qr_steps = qr_steps_full = 0;
  reruns = 0;
  std::vector<DevBuf<double>> rho(nb), lam(nb);  // rho: kn x k, lam: k x kn
  std::vector<DevBuf<double>> Tkeep;
  std::vector<std::array<long long, 2>> Toff(nb);
  std::vector<int> Tlev(nb, -1);
  // new sibling blocks: offsets over the final ranks, filled level by level
  std::vector<DevBuf<double>> msib(nb);
  for (int L = maxlev; L >= 0; --L) {
    std::vector<int> boxes;
    for (int b = 0; b < nb; ++b)
      if (level[b] == L) boxes.push_back(b);
    if (boxes.empty()) continue;
    // sibling blocks of this level's parents (their sons are final) and RNEW / LNEW^T
    std::vector<GemmP<double>> g1, g2;
    std::vector<DevBuf<double>> tmp(2 * boxes.size());
    for (size_t q = 0; q < boxes.size(); ++q) {
      const int b = boxes[q];
      if (is_leaf(b)) continue;
      const int s1 = c1[b], s2 = c2[b];
      for (int side = 0; side < 2; ++side) {
        const int sa = side ? s2 : s1, sb = side ? s1 : s2;
        const int ka = kskel[sa], kb2 = kskel[sb], kna = kn[sa], knb = kn[sb];
        tmp[2 * q + side].alloc(std::max(1, ka * knb));
        msib[sa].alloc(std::max(1, ka * kb2));
        // lam{sa} sib{sa} (ka x knb), then times rho{sb} (knb x kb2)
        gemm(g1, lam[sa].p, std::max(ka, 1), sib[sa].p, std::max(kna, 1), tmp[2 * q + side].p, std::max(ka, 1), ka,
             knb, kna);
      }
    }
    run_gemms(g1, false, false, 1.0, 0.0, st);
    g1.clear();
    for (size_t q = 0; q < boxes.size(); ++q) {
      const int b = boxes[q];
      if (is_leaf(b)) continue;
      const int s1 = c1[b], s2 = c2[b];
      for (int side = 0; side < 2; ++side) {
        const int sa = side ? s2 : s1, sb = side ? s1 : s2;
        const int ka = kskel[sa], kb2 = kskel[sb], knb = kn[sb];
        gemm(g1, tmp[2 * q + side].p, std::max(ka, 1), rho[sb].p, std::max(knb, 1), msib[sa].p, std::max(ka, 1), ka,
             kb2, knb);
      }
    }
    run_gemms(g1, false, false, 1.0, 0.0, st);
    g1.clear();
    if (L == 0) break;
    // RNEW (kn x n) and LNEW^T (kn x n) of every box of the level
    const int nbL = (int)boxes.size();
    std::vector<int> m(nbL), n(nbL);
    std::vector<long long> oZ(2 * nbL);
    long long tZ = 0;
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q];
      m[q] = kn[b];
      n[q] = is_leaf(b) ? cnt[b] : kskel[c1[b]] + kskel[c2[b]];
      HSS_REQUIRE(m[q] >= 1 && n[q] >= 1 && n[q] <= 4096, HSS_ERR_RANK, "recompress: empty or oversized basis");
      oZ[2 * q] = tZ; tZ += (long long)m[q] * n[q];
      oZ[2 * q + 1] = tZ; tZ += (long long)m[q] * n[q];
    }
    DevBuf<double> Z(std::max(tZ, 1LL));
    Z.zero(st);
    std::vector<MoveP> mv;
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q], kb = m[q];
      double* RN = Z.p + oZ[2 * q];
      double* LNt = Z.p + oZ[2 * q + 1];
      if (is_leaf(b)) {
        mv.push_back(MoveP{Rp[b].p, RN, nullptr, kb, n[q], kb, kb, 0, 0});
        mv.push_back(MoveP{Lp[b].p, LNt, nullptr, n[q], kb, n[q], kb, 3, 0});  // (n x kb)^T
        continue;
      }
      const int s1 = c1[b], s2 = c2[b], ka1 = kn[s1], ka2 = kn[s2];
      // RNEW = [RA(:, :ka1) rho{s1}, RA(:, ka1:) rho{s2}]
      gemm(g1, Rp[b].p, kb, rho[s1].p, std::max(ka1, 1), RN, kb, kb, kskel[s1], ka1);
      gemm(g1, Rp[b].p + (size_t)ka1 * kb, kb, rho[s2].p, std::max(ka2, 1), RN + (size_t)kskel[s1] * kb, kb, kb,
           kskel[s2], ka2);
      // LNEW^T = [LA(:ka1, :)^T lam{s1}^T, LA(ka1:, :)^T lam{s2}^T]: C = A^T B^T
      gemm(g2, Lp[b].p, ka1 + ka2, lam[s1].p, std::max(kskel[s1], 1), LNt, kb, kb, kskel[s1], ka1);
      gemm(g2, Lp[b].p + ka1, ka1 + ka2, lam[s2].p, std::max(kskel[s2], 1), LNt + (size_t)kskel[s1] * kb, kb, kb,
           kskel[s2], ka2);
    }
    run_moves(mv, st);
    run_gemms(g1, false, false, 1.0, 0.0, st);
    run_gemms(g2, true, true, 1.0, 0.0, st);
    // full pivoted QR of both, fixed-rank ID at k = min(kn, n)
    const int nprob2 = 2 * nbL;
    std::vector<long long> oT2(nprob2), oXw(nprob2), oYw(nprob2), oP(nprob2);
    long long tT = 0, tX = 0, tYw = 0, tP = 0;
    for (int pr = 0; pr < nprob2; ++pr) {
      const int q = pr / 2;
      oT2[pr] = tT; tT += (long long)n[q] * n[q];
      oXw[pr] = tX; tX += 2LL * n[q];
      oYw[pr] = tYw; tYw += (long long)m[q] + n[q];
      oP[pr] = tP; tP += n[q];
    }
    DevBuf<double> Wq(std::max(tZ, 1LL)), SW(tT), SV(tT), xw(tX), yw(tYw);
    Tkeep.emplace_back(tT);
    DevBuf<double>& Tb = Tkeep.back();
    DevBuf<int> perm(tP), rank(nprob2);
    std::vector<IdP> ip(nprob2);
    for (int pr = 0; pr < nprob2; ++pr) {
      const int q = pr / 2, b = boxes[q];
      ip[pr] = IdP{Z.p + oZ[pr], Wq.p + oZ[pr], m[q], n[q], perm.p + oP[pr], rank.p + pr, Tb.p + oT2[pr], -1,
                   SW.p + oT2[pr], SV.p + oT2[pr], xw.p + oXw[pr], yw.p + oYw[pr], 2 * (b - proot[prob[b]]) + pr % 2,
                   ID_QR_ONLY, pseed[prob[b]], nullptr};
    }
    DevBuf<IdP> dip;
    upload_vec(dip, ip, st);
    id_adaptive_batched(dip.p, nprob2, acc, st, false);
    for (int pr = 0; pr < nprob2; ++pr) ip[pr].force_k = std::min(m[pr / 2], n[pr / 2]);
    HSS_CUDA(cudaMemcpyAsync(dip.p, ip.data(), nprob2 * sizeof(IdP), cudaMemcpyHostToDevice, st));
    id_fixed_batched(dip.p, nprob2, st);
    std::vector<int> hp;
    download(hp, perm.p, tP, st);
    HSS_CUDA(cudaStreamSynchronize(st));
    std::vector<MoveP> mk;
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q], k = std::min(m[q], n[q]), nn = n[q];
      rho[b].alloc(std::max(1, m[q] * k));
      lam[b].alloc(std::max(1, k * m[q]));
      // rho = RNEW(:, Jout(1:k)) (kn x k); lam = LNEW(Jin(1:k), :) = (LNEW^T(:, Jin(1:k)))^T
      mk.push_back(MoveP{Z.p + oZ[2 * q], rho[b].p, perm.p + oP[2 * q], m[q], k, m[q], m[q], 1, 0});
      std::vector<int> outs, inns;
      if (is_leaf(b)) {
        outs.resize(cnt[b]);
        std::iota(outs.begin(), outs.end(), off[b]);
        inns = outs;
      } else {
        outs = I_SKUP[c1[b]];
        outs.insert(outs.end(), I_SKUP[c2[b]].begin(), I_SKUP[c2[b]].end());
        inns = I_SKDN[c1[b]];
        inns.insert(inns.end(), I_SKDN[c2[b]].begin(), I_SKDN[c2[b]].end());
      }
      nskel[b] = nn;
      kskel[b] = k;
      J_UP[b].assign(hp.begin() + oP[2 * q], hp.begin() + oP[2 * q] + nn);
      J_DN[b].assign(hp.begin() + oP[2 * q + 1], hp.begin() + oP[2 * q + 1] + nn);
      I_SKUP[b].resize(k);
      I_SKDN[b].resize(k);
      for (int t = 0; t < k; ++t) {
        I_SKUP[b][t] = outs[J_UP[b][t]];
        I_SKDN[b][t] = inns[J_DN[b][t]];
      }
      Toff[b] = {oT2[2 * q], oT2[2 * q + 1]};
      Tlev[b] = (int)Tkeep.size() - 1;
      census[4 * b] = m[q]; census[4 * b + 1] = m[q]; census[4 * b + 2] = nn; census[4 * b + 3] = k;
    }
    run_moves(mk, st);
    // lam (k x kn) = transpose of the gathered columns of LNEW^T
    std::vector<DevBuf<double>> lt(nbL);
    std::vector<MoveP> mg, mt;
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q], k = kskel[b];
      lt[q].alloc(std::max(1, m[q] * k));
      mg.push_back(MoveP{Z.p + oZ[2 * q + 1], lt[q].p, perm.p + oP[2 * q + 1], m[q], k, m[q], m[q], 1, 0});
      mt.push_back(MoveP{lt[q].p, lam[b].p, nullptr, m[q], k, m[q], std::max(k, 1), 3, 0});
    }
    run_moves(mg, st);
    run_moves(mt, st);
  }
  pack_T(Tkeep, Toff, Tlev);
  // M_SELF (the operand's) and the new sibling blocks
  oSelf = A.oSelf;
  M_SELF.alloc(std::max<size_t>(A.M_SELF.n, 1));
  if (A.M_SELF.n) HSS_CUDA(cudaMemcpyAsync(M_SELF.p, A.M_SELF.p, A.M_SELF.n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  oSib.assign(nb, -1);
  long long tb = 0;
  for (int b = 0; b < nb; ++b)
    if (!is_leaf(b)) {
      oSib[c1[b]] = tb; tb += (long long)kskel[c1[b]] * kskel[c2[b]];
      oSib[c2[b]] = tb; tb += (long long)kskel[c2[b]] * kskel[c1[b]];
    }
  M_SIB.alloc(std::max(tb, 1LL));
  std::vector<MoveP> mv;
  for (int b = 0; b < nb; ++b)
    if (!is_leaf(b))
      for (int s : {c1[b], c2[b]}) {
        const int o = (s == c1[b]) ? c2[b] : c1[b];
        if (kskel[s] > 0 && kskel[o] > 0)
          mv.push_back(MoveP{msib[s].p, M_SIB.p + oSib[s], nullptr, kskel[s], kskel[o], kskel[s], kskel[s], 0, 0});
      }
  run_moves(mv, st);
  HSS_CUDA(cudaStreamSynchronize(st));
  inverted = false;
  clear_plans();
}

}  // namespace hss
