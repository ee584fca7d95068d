// HSS1D solver for curves (non-symmetric form), FP64.
//
//  compress : HSS1D/HSS1D_compress_nsym.m ('green' trick).  The host walks
//             the tree level by level (deepest first); for every box of a
//             level the GPU generates A_out = K[X_in_inside u X_proxy, X_out]
//             and A_in^T = K[X_in, X_out_inside u X_proxy]^T (:151-156) and runs
//             the pivoted-QR ID with its randomized check (Common/ID.m:40-65),
//             then the fixed-rank re-ID of the side whose rank is raised to
//             k = max(k_out, k_in) (:189-196, ID.m:106-113).  Skeleton index
//             sets go back to the host, which assembles the next level.
//  invert   : HSS1D/HSS1D_invert_nsym.m:44-91, level-batched.
//  apply    : HSS1D/HSS1D_apply_nsym.m:38-130.
//  applyinv : HSS1D/HSS1D_applyinv_nsym.m:43-86.
//  transforminv : HSS1D/HSS1D_transforminv_nsym.m:38-161.
// The HSS1D algebra (transpose, scalar multiple, dense export, rectangular compress, sum,
// low-rank compress) is in hss1d_algebra.cu.
#include "hss1d.h"
#include "hss1d_util.cuh"

#include <chrono>

#include <algorithm>
#include <array>
#include <cmath>
#include <numeric>

namespace hss {


// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_move(const MoveP* __restrict__ P) {
  const MoveP p = P[blockIdx.x];
  const long long tot = (long long)p.nrows * p.ncols;
  for (long long e = threadIdx.x; e < tot; e += 256) {
    const int i = (int)(e % p.nrows), c = (int)(e / p.nrows);
    if (p.mode == 0) {
      const int si = p.idx ? p.idx[i] : i;
      p.dst[i + (size_t)c * p.ldd] = p.src[si + (size_t)c * p.lds];
    } else if (p.mode == 1) {
      const int sc = p.idx ? p.idx[c] : c;
      p.dst[i + (size_t)c * p.ldd] = p.src[i + (size_t)sc * p.lds];
    } else if (p.mode == 2) {
      const int di = p.idx ? p.idx[i] : i;
      double* d = p.dst + di + (size_t)c * p.ldd;
      const double v = p.src[i + (size_t)c * p.lds];
      *d = p.accumulate ? *d + v : v;
    } else if (p.mode == 3) {  // transpose copy dst(c, i) = src(i, c)
      p.dst[c + (size_t)i * p.ldd] = p.src[i + (size_t)c * p.lds];
    } else {
      // real 2 x 2 embeddings (even offsets): 4 conjugate, E(conj X) = S E(X) S; 5 plain
      // transpose, E(X.') = S E(X)^T S; S = diag(1, -1, 1, -1, ...)
      const double v = ((i + c) & 1) ? -p.src[i + (size_t)c * p.lds] : p.src[i + (size_t)c * p.lds];
      if (p.mode == 4) p.dst[i + (size_t)c * p.ldd] = v;
      else p.dst[c + (size_t)i * p.ldd] = v;
    }
  }
}

void move_batched(const MoveP* dP, int batch, cudaStream_t s) {
  if (batch <= 0) return;
  HSS_REQUIRE(batch <= 2147483647, HSS_ERR_ARG, "move batch too large");
  k_move<<<batch, 256, 0, s>>>(dP);
  check_launch("k_move");
}

struct F1P {  // F = [E1 S1; S2 E2] (two children) or F = M (leaf)
  double* F;
  int n, k1;
  const double *E1, *S1, *S2, *E2, *M;
};

__global__ void __launch_bounds__(256) k_assemble1(const F1P* __restrict__ P) {
  const F1P p = P[blockIdx.x];
  const int n = p.n, k1 = p.k1, k2 = n - k1;
  for (long long e = threadIdx.x; e < (long long)n * n; e += 256) {
    const int i = (int)(e % n), j = (int)(e / n);
    double v;
    if (p.M) v = p.M[e];
    else if (i < k1 && j < k1) v = p.E1[i + (size_t)j * k1];
    else if (i < k1) v = p.S1[i + (size_t)(j - k1) * k1];
    else if (j < k1) v = p.S2[(i - k1) + (size_t)j * k2];
    else v = p.E2[(i - k1) + (size_t)(j - k1) * k2];
    p.F[e] = v;
  }
}

// ---------------------------------------------------------------------------
void run_moves(const std::vector<MoveP>& mv, cudaStream_t s) {
  if (mv.empty()) return;
  DevBuf<MoveP> d;
  upload_vec(d, mv, s);
  move_batched(d.p, (int)mv.size(), s);
  HSS_CUDA(cudaStreamSynchronize(s));
}

void run_gemms(const std::vector<GemmP<double>>& P, bool tA, bool tB, double alpha, double beta, cudaStream_t s,
               bool skinny, bool df) {
  if (P.empty()) return;
  int maxM = 0, maxN = 0;
  for (auto& p : P) { maxM = std::max(maxM, p.M); maxN = std::max(maxN, p.N); }
  DevBuf<GemmP<double>> d;
  upload_vec(d, P, s);
  for (size_t off = 0; off < P.size(); off += 65535) {
    const int cnt = (int)std::min<size_t>(65535, P.size() - off);
    if (skinny) gemm_skinny<double>(d.p + off, cnt, maxM, alpha, beta, s);
    else if (df) gemm_batched_df(d.p + off, cnt, maxM, maxN, tA, tB, alpha, beta, s);
    else gemm_batched<double>(d.p + off, cnt, maxM, maxN, tA, tB, alpha, beta, s);
  }
  HSS_CUDA(cudaStreamSynchronize(s));
}

static void invert_many(std::vector<std::pair<double*, int>>& mats, cudaStream_t s, bool df = false) {
  if (mats.empty()) return;
  const int nb = (int)mats.size();
  int maxn = 0;
  long long tot = 0;
  for (auto& m : mats) { maxn = std::max(maxn, m.second); tot += (long long)m.second * m.second; }
  long long totn = 0;
  for (auto& m : mats) totn += m.second;
  DevBuf<int> ipiv(totn), info(nb), aux((size_t)nb * GJ_AUX);
  DevBuf<double> W((size_t)2 * GJ_NB * totn), Wf(tot);
  info.zero(s);
  std::vector<InvP<double>> P(nb);
  long long on = 0, o2 = 0;
  for (int i = 0; i < nb; ++i) {
    const int n = mats[i].second;
    P[i] = InvP<double>{mats[i].first, n, n, ipiv.p + on, W.p + (size_t)2 * GJ_NB * on, Wf.p + o2, info.p + i,
                        aux.p + (size_t)i * GJ_AUX};
    on += n;
    o2 += (long long)n * n;
  }
  DevBuf<InvP<double>> dP;
  upload_vec(dP, P, s);
  for (int o = 0; o < nb; o += 65535) {
    int mx = 0;
    const int cnt = std::min(65535, nb - o);
    for (int i = o; i < o + cnt; ++i) mx = std::max(mx, mats[i].second);
    invert_batched<double>(dP.p + o, cnt, mx, s, df);
  }
  std::vector<int> hi;
  download(hi, info.p, nb, s);
  HSS_CUDA(cudaStreamSynchronize(s));
  for (int v : hi) {
    HSS_REQUIRE(v >= 0, HSS_ERR_NONFINITE, "non-finite pivot in block inversion");
    HSS_REQUIRE(v == 0, HSS_ERR_SINGULAR, "singular diagonal block in inversion");
  }
}

// LOCAL_get_circum_circle (HSS1D_compress_nsym.m:339-356) on X rows idx
void circum_circle(const std::vector<double>& X, const std::vector<int>& idx, double& xc, double& yc, double& R) {
  const int nloc = (int)idx.size();
  auto px = [&](int i) { return X[6 * (size_t)idx[i]]; };
  auto py = [&](int i) { return X[6 * (size_t)idx[i] + 1]; };
  xc = 0.5 * (px(0) + px(nloc - 1));
  yc = 0.5 * (py(0) + py(nloc - 1));
  double mx = -1.0;
  for (int i = 0; i < nloc; ++i) {
    const double dx = px(i) - xc, dy = py(i) - yc;
    mx = std::max(mx, dx * dx + dy * dy);
  }
  R = std::sqrt(mx);
  const double ex = px(0) - px(nloc - 1), ey = py(0) - py(nloc - 1);
  const double e = ex * ex + ey * ey;
  if ((1.2 * R * R) > e) {
    double sx = 0.0, sy = 0.0;
    for (int i = 0; i < nloc; ++i) { sx += px(i); sy += py(i); }
    const double inv = 1.0 / (double)nloc;
    xc = sx * inv;
    yc = sy * inv;
    mx = -1.0;
    for (int i = 0; i < nloc; ++i) {
      const double dx = px(i) - xc, dy = py(i) - yc;
      mx = std::max(mx, dx * dx + dy * dy);
    }
    R = std::sqrt(mx);
  }
}

// LOCAL_get_tree (HSS1D_compress_nsym.m:277-334): problem p's tree over n points from
// point `base`, built breadth first by halving (son1 takes ceil(n/2)) while a box holds
// more than `leaf` points; global box ids continue the forest's numbering.
void HSS1D::append_tree(int p, int base, int n) {
  const int g0 = (int)level.size();
  prob.push_back(p); level.push_back(0); parent.push_back(-1); c1.push_back(-1); c2.push_back(-1);
  off.push_back(base); cnt.push_back(n);
  int last = g0 - 1, created = 1, ilev = 0;
  while (created > 0) {
    const int first = last + 1;
    last = last + created;
    created = 0;
    for (int b = first; b <= last; ++b) {
      const int nbx = cnt[b];
      if (nbx > leaf) {
        const int half = (nbx + 1) / 2;
        const int s1 = last + created + 1;
        c1[b] = s1;
        c2[b] = s1 + 1;
        for (int t = 0; t < 2; ++t) {
          prob.push_back(p);
          level.push_back(ilev + 1);
          parent.push_back(b);
          c1.push_back(-1);
          c2.push_back(-1);
          off.push_back(t == 0 ? off[b] : off[b] + half);
          cnt.push_back(t == 0 ? half : nbx - half);
        }
        created += 2;
      }
    }
    ++ilev;
  }
  HSS_REQUIRE((int)level.size() - g0 >= 3, HSS_ERR_ARG, "each problem must exceed the leaf size (one split)");
}

HSS1D::HSS1D() { HSS_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)); }
HSS1D::~HSS1D() {
  if (stream) cudaStreamDestroy(stream);
}

void HSS1D::compress(int np_, const long long* Np, const double* const* Xp, const long long* ldx, int leaf_,
                     double acc_, const hss_kernel_params& kp_, const unsigned long long* seeds, MLP* mlp,
                     bool sym_) {
  kernel_op = true;
  HSS_REQUIRE(np_ >= 1 && Np && Xp && ldx && leaf_ >= 1 && acc_ > 0 && acc_ < 1, HSS_ERR_ARG, "bad compress args");
  HSS_REQUIRE(kp_.flag == HSS_SL_L_2D || kp_.flag == HSS_DL_L_2D || kp_.flag == HSS_SL_H_2D, HSS_ERR_ARG,
              "unknown kernel");
  // complex (Helmholtz) kernel: the blocks are generated and skeletonized in the real 2 x 2
  // embedding (pair-pivoted ID); the finished handle is the real 2N x 2N embedded matrix
  const bool cx = (kp_.flag == HSS_SL_H_2D);
  HSS_REQUIRE(!cx || (!mlp && !id_df), HSS_ERR_ARG,
              "complex compression: the plain FP64 ID and no rank predictor");
  cplx = cx;
  const int rep = cx ? 2 : 1;
  using clk = std::chrono::steady_clock;
  std::fill(phase_s, phase_s + NPHASE, 0.0);
  auto tick = clk::now();
  auto lap = [&](int ph) {
    const auto t = clk::now();
    phase_s[ph] += std::chrono::duration<double>(t - tick).count();
    tick = t;
  };
  nprob = np_; leaf = leaf_; acc = acc_; kp = kp_; sym = sym_;
  // ID problems per box: outgoing and incoming (nsym), or the outgoing one only (fsym,
  // HSS1D_compress_fsym.m:186-198, whose incoming skeletons equal the outgoing ones)
  const int ps = sym ? 1 : 2;
  kdev = make_kernel_dev(kp);
  pN.assign(Np, Np + nprob);
  pbase.assign(nprob, 0);
  pseed.assign(nprob, 0);
  Ntot = 0;
  for (int p = 0; p < nprob; ++p) {
    HSS_REQUIRE(Xp[p] && pN[p] >= 2 && ldx[p] >= pN[p], HSS_ERR_ARG, "bad problem size");
    pbase[p] = Ntot;
    Ntot += pN[p];
    pseed[p] = seeds ? seeds[p] : 0ULL;
  }
  HSS_REQUIRE(Ntot < (1LL << 30), HSS_ERR_ARG, "total points too large");
  X.resize(6 * (size_t)Ntot);
  for (int p = 0; p < nprob; ++p)
    for (long long i = 0; i < pN[p]; ++i)
      for (int c = 0; c < 6; ++c) X[6 * (pbase[p] + i) + c] = Xp[p][i + c * ldx[p]];
  // ---- trees (LOCAL_get_tree, :277-334), one per problem, global box ids
  prob.clear(); level.clear(); parent.clear(); c1.clear(); c2.clear(); off.clear(); cnt.clear();
  proot.assign(nprob, 0);
  for (int p = 0; p < nprob; ++p) {
    proot[p] = (int)level.size();
    append_tree(p, (int)pbase[p], (int)pN[p]);
  }
  nboxes = (int)level.size();
  maxlev = *std::max_element(level.begin(), level.end());
  // ---- neighbour lists (:376-412), boxes in increasing global id (parents first)
  std::vector<std::vector<int>> nei(nboxes);
  // problems are independent (their boxes are a contiguous id range, parents first)
  auto neighbours = [&](int b) {
    if (parent[b] < 0) { nei[b] = {b}; return; }
    std::vector<int> r(cnt[b]);
    std::iota(r.begin(), r.end(), off[b]);
    double xc, yc, R;
    circum_circle(X, r, xc, yc, R);
    std::vector<int> pot;
    for (int j : nei[parent[b]]) {
      if (c1[j] >= 0) pot.push_back(c1[j]);
      if (c2[j] >= 0) pot.push_back(c2[j]);
    }
    const double rr = RADIUS_REL * RADIUS_REL * R * R;
    for (int j : pot) {
      double mn = INFINITY;
      for (int i = off[j]; i < off[j] + cnt[j]; ++i) {
        const double dx = X[6 * (size_t)i] - xc, dy = X[6 * (size_t)i + 1] - yc;
        mn = std::min(mn, dx * dx + dy * dy);
      }
      if (mn < rr) nei[b].push_back(j);
    }
  };
  parallel_for(nprob, [&](int p) {
    const int b1 = (p + 1 < nprob) ? proot[p + 1] : nboxes;
    for (int b = proot[p]; b < b1; ++b) neighbours(b);
    for (int b = proot[p]; b < b1; ++b) {
      if (parent[b] < 0) continue;
      auto& l = nei[b];
      l.erase(std::remove(l.begin(), l.end(), b), l.end());
      std::sort(l.begin(), l.end());
    }
  }, 1);
  // ---- point table: the Ntot points, then one proxy slot per non-root box in the order the
  // levels are compressed in, so each level uploads one contiguous range.  A slot holds
  // NPROXY points; with the Helmholtz kernel the ring's size grows with the circle
  // (proxy_count), and the slot holds the count for the diagonal of the box's bounding box,
  // which bounds the radius of any circle centred inside it.  A complex handle keeps every
  // entry twice (table entries 2v and 2v + 1 are logical point v: the two real unknowns of
  // a point read the same point).
  std::vector<long long> poff(nboxes, -1);
  std::vector<int> pcap(nboxes, 0);
  long long nprx = 0;
  for (int L = maxlev; L >= 1; --L)
    for (int b = 0; b < nboxes; ++b)
      if (level[b] == L) {
        int cap = NPROXY;
        if (cx) {
          double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
          for (int i = off[b]; i < off[b] + cnt[b]; ++i) {
            x0 = std::min(x0, X[6 * (size_t)i]); x1 = std::max(x1, X[6 * (size_t)i]);
            y0 = std::min(y0, X[6 * (size_t)i + 1]); y1 = std::max(y1, X[6 * (size_t)i + 1]);
          }
          cap = proxy_count(kp, std::hypot(x1 - x0, y1 - y0) * (1.0 + 1e-12), pN[prob[b]]);
        }
        poff[b] = nprx;
        pcap[b] = cap;
        nprx += cap;
      }
  const size_t npts = (size_t)rep * ((size_t)Ntot + (size_t)nprx);
  HSS_REQUIRE(npts < (1ULL << 31), HSS_ERR_ARG, "point table exceeds 2^31 entries");
  std::vector<double> hx(npts, 0.0), hy(npts, 0.0), hnx(npts, 0.0), hny(npts, 0.0), hw(npts, 0.0),
      hk(npts, 0.0);
  auto put = [&](size_t v, double x, double y, double nx, double ny, double w, double kap) {
    for (int r = 0; r < rep; ++r) {
      const size_t e = (size_t)rep * v + r;
      hx[e] = x; hy[e] = y; hnx[e] = nx; hny[e] = ny; hw[e] = w; hk[e] = kap;
    }
  };
  for (long long i = 0; i < Ntot; ++i)
    put((size_t)i, X[6 * i], X[6 * i + 1], X[6 * i + 2], X[6 * i + 3], X[6 * i + 4], X[6 * i + 5]);
  pts.reserve(npts);
  pts.upload_range(0, (size_t)rep * Ntot, hx.data(), hy.data(), hnx.data(), hny.data(), hw.data(), hk.data(), kp,
                   stream);
  nskel.assign(nboxes, 0);
  kskel.assign(nboxes, 0);
  I_SKUP.assign(nboxes, {});
  I_SKDN.assign(nboxes, {});
  J_UP.assign(nboxes, {});
  J_DN.assign(nboxes, {});
  census.assign(4 * (size_t)nboxes, 0);
  feat.assign((size_t)NFEAT * nboxes, 0.f);
  qr_steps = qr_steps_full = 0;
  reruns = 0;
  HSS_REQUIRE(!mlp || mlp->nin == NFEAT, HSS_ERR_ARG, "rank predictor must take 8 features");
  std::vector<DevBuf<double>> Tkeep;  // per level: T of each ID problem (n x n, ld n)
  std::vector<std::vector<long long>> Toff(nboxes);
  std::vector<int> Tlev(nboxes, -1);
  lap(0);
  for (int L = maxlev; L >= 1; --L) {
    std::vector<int> boxes;
    for (int b = 0; b < nboxes; ++b)
      if (level[b] == L) boxes.push_back(b);
    if (boxes.empty()) continue;
    const int nbL = (int)boxes.size();
    std::vector<std::vector<int>> outs(nbL), inns(nbL), rows_out(nbL), rows_in(nbL);
    // every box of the level reads its children's skeletons and writes only its own
    // slots (sets, proxy ring, features): the boxes run in parallel on the host cores
    parallel_for(nbL, [&](int q) {
      const int b = boxes[q];
      auto& out = outs[q];
      auto& inn = inns[q];
      if (is_leaf(b)) {
        out.resize(cnt[b]);
        std::iota(out.begin(), out.end(), off[b]);
        inn = out;
      } else {
        HSS_REQUIRE(c1[b] >= 0 && c2[b] >= 0, HSS_ERR_ARG, "one-child boxes are not produced by the halving tree");
        out = I_SKUP[c1[b]];
        out.insert(out.end(), I_SKUP[c2[b]].begin(), I_SKUP[c2[b]].end());
        inn = I_SKDN[c1[b]];
        inn.insert(inn.end(), I_SKDN[c2[b]].begin(), I_SKDN[c2[b]].end());
      }
      std::vector<int> both = out;
      both.insert(both.end(), inn.begin(), inn.end());
      std::sort(both.begin(), both.end());
      double xc, yc, R;
      circum_circle(X, both, xc, yc, R);
      const double Rp = RADIUS_REL * R;
      const int npx = proxy_count(kp, R, pN[prob[b]]);
      HSS_REQUIRE(npx <= pcap[b], HSS_ERR_ARG, "proxy ring larger than its slot");
      // LOCAL_construct_circle: tt = linspace(0, 2 pi (1 - 1/n), n)
      const double stop = 2.0 * M_PI * (1.0 - 1.0 / npx);
      const double step = (npx > 1) ? stop / (double)(npx - 1) : 0.0;
      const size_t pb = (size_t)Ntot + (size_t)poff[b];
      for (int t = 0; t < npx; ++t) {
        const double tt = (t == npx - 1) ? stop : (double)t * step;
        const double c = std::cos(tt), s = std::sin(tt);
        put(pb + t, xc + Rp * c, yc + Rp * s, c, s, 2.0 * M_PI * Rp / npx, 1.0 / Rp);
      }
    std::vector<int> out_maybe, in_maybe;
      for (int j : nei[b]) {
        if (is_leaf(j)) {
          for (int i = off[j]; i < off[j] + cnt[j]; ++i) { out_maybe.push_back(i); in_maybe.push_back(i); }
        } else if (c1[j] >= 0 && c2[j] >= 0) {
          for (int s : {c1[j], c2[j]}) {
            out_maybe.insert(out_maybe.end(), I_SKUP[s].begin(), I_SKUP[s].end());
          }
          for (int s : {c1[j], c2[j]}) {
            in_maybe.insert(in_maybe.end(), I_SKDN[s].begin(), I_SKDN[s].end());
          }
        } else {
          const int s = std::max(c1[j], c2[j]);
          out_maybe.insert(out_maybe.end(), I_SKUP[s].begin(), I_SKUP[s].end());
          in_maybe.insert(in_maybe.end(), I_SKDN[s].begin(), I_SKDN[s].end());
        }
      }
      const double rr = Rp * Rp;
      std::vector<int> out_inside, in_inside;
      for (int i : out_maybe) {
        const double dx = X[6 * (size_t)i] - xc, dy = X[6 * (size_t)i + 1] - yc;
        if (dx * dx + dy * dy < rr) out_inside.push_back(i);
      }
      for (int i : in_maybe) {
        const double dx = X[6 * (size_t)i] - xc, dy = X[6 * (size_t)i + 1] - yc;
        if (dx * dx + dy * dy < rr) in_inside.push_back(i);
      }
      rows_out[q] = in_inside;
      rows_in[q] = out_inside;
      {  // rank-predictor features of the box (all known before its ID)
        double arc = 0.0, kmax = 0.0;
        for (int i = off[b]; i < off[b] + cnt[b]; ++i) {
          arc += X[6 * (size_t)i + 4];
          kmax = std::max(kmax, std::fabs(X[6 * (size_t)i + 5]));
        }
        float* f = &feat[(size_t)NFEAT * b];
        f[0] = (float)std::log2((double)out.size());
        f[1] = (float)(-std::log10(acc) / 10.0);
        f[2] = (float)std::log2(1.0 + (double)in_inside.size());
        f[3] = (float)std::log2(1.0 + (double)out_inside.size());
        f[4] = (float)((arc > 0.0) ? R / arc : 0.0);
        f[5] = (float)(kmax * R);
        f[6] = (float)L / 16.f;
        f[7] = (float)kp.flag;
      }
      for (int t = 0; t < npx; ++t) {
        rows_out[q].push_back((int)(pb + t));
        rows_in[q].push_back((int)(pb + t));
      }
      HSS_REQUIRE(out.size() <= (size_t)(4096 / rep), HSS_ERR_RANK, "skeleton set exceeds the ID's 4096 columns");
    }, 16);
    lap(1);
    {
      const size_t p0 = (size_t)rep * ((size_t)Ntot + (size_t)poff[boxes[0]]);
      const size_t p1 = (size_t)rep * ((size_t)Ntot + (size_t)poff[boxes.back()] + (size_t)pcap[boxes.back()]);
      pts.upload_range(p0, p1 - p0, hx.data() + p0, hy.data() + p0, hnx.data() + p0, hny.data() + p0,
                       hw.data() + p0, hk.data() + p0, kp, stream);
    }
    // index arrays (table entries: logical point v is entry v, or entries 2v, 2v + 1 of a
    // complex handle) and block storage
    std::vector<int> idx;
    std::vector<long long> o_ro(nbL), o_ri(nbL), o_out(nbL), o_in(nbL);
    auto push_ids = [&](const std::vector<int>& v) {
      for (int a : v)
        for (int r = 0; r < rep; ++r) idx.push_back(rep * a + r);
    };
    for (int q = 0; q < nbL; ++q) {
      o_ro[q] = idx.size(); push_ids(rows_out[q]);
      o_ri[q] = idx.size(); push_ids(rows_in[q]);
      o_out[q] = idx.size(); push_ids(outs[q]);
      o_in[q] = idx.size(); push_ids(inns[q]);
    }
    DevBuf<int> didx;
    upload_vec(didx, idx, stream);
    const int nprob2 = ps * nbL;
    std::vector<long long> oA(nprob2), oT2(nprob2), oX(nprob2), oY(nprob2), oP(nprob2);
    long long tA = 0, tT = 0, tX = 0, tY = 0, tP = 0;
    std::vector<int> pm(nprob2), pn(nprob2);
    for (int q = 0; q < nbL; ++q) {
      for (int s = 0; s < ps; ++s) {
        const int pr = ps * q + s;
        const int m = rep * (int)(s == 0 ? rows_out[q].size() : rows_in[q].size());
        const int n = rep * (int)outs[q].size();
        pm[pr] = m; pn[pr] = n;
        oA[pr] = tA; tA += (long long)m * n;
        oT2[pr] = tT; tT += (long long)n * n;
        oX[pr] = tX; tX += 2LL * n;
        oY[pr] = tY; tY += (long long)m + n;
        oP[pr] = tP; tP += n;
      }
    }
    DevBuf<double> A(tA), W(tA), SW(tT), SV(tT), xw(tX), yw(tY);
    Tkeep.emplace_back(tT);
    DevBuf<double>& Tb = Tkeep.back();
    DevBuf<int> perm(tP), rank(nprob2);
    std::vector<KgenP<double>> kg(nprob2);
    std::vector<IdP> ip(nprob2);
    for (int q = 0; q < nbL; ++q) {
      const int n = rep * (int)outs[q].size(), po = ps * q;
      kg[po] = KgenP<double>{didx.p + o_ro[q], didx.p + o_out[q], pm[po], n, A.p + oA[po], pm[po], 0};
      if (!sym)
        kg[po + 1] = KgenP<double>{didx.p + o_in[q], didx.p + o_ri[q], n, pm[po + 1], A.p + oA[po + 1], pm[po + 1], 1};
    }
    for (int pr = 0; pr < nprob2; ++pr) {
      const int b = boxes[pr / ps], s = pr % ps;
      const int lb = b - proot[prob[b]];  // box id local to its tree: the random stream of the oracle
      ip[pr] = IdP{A.p + oA[pr], W.p + oA[pr], pm[pr], pn[pr], perm.p + oP[pr], rank.p + pr, Tb.p + oT2[pr], -1,
                   SW.p + oT2[pr], SV.p + oT2[pr], xw.p + oX[pr], yw.p + oY[pr], 2 * lb + s, -1,
                   pseed[prob[b]], nullptr};
    }
    long long maxe = 0;
    for (auto& g : kg) maxe = std::max(maxe, (long long)g.m * g.n);
    DevBuf<KgenP<double>> dkg;
    upload_vec(dkg, kg, stream);
    for (int o = 0; o < nprob2; o += 65535)
      kgen_batched<double>(dkg.p + o, std::min(65535, nprob2 - o), maxe, view(pts), kdev, stream);
    lap(2);
    DevBuf<int> stat((size_t)2 * nprob2);
    stat.zero(stream);
    for (int pr = 0; pr < nprob2; ++pr) ip[pr].stat = stat.p + 2 * pr;
    if (mlp) {
      // predicted rank fraction -> QR step budget of both IDs of the box
      std::vector<float> fx((size_t)NFEAT * nbL);
      for (int q = 0; q < nbL; ++q)
        std::copy(&feat[(size_t)NFEAT * boxes[q]], &feat[(size_t)NFEAT * boxes[q]] + NFEAT, &fx[(size_t)NFEAT * q]);
      DevBuf<float> dfx, dy(nbL);
      upload_vec(dfx, fx, stream);
      mlp->forward(dfx.p, dy.p, nbL, stream);
      std::vector<float> yh;
      download(yh, dy.p, nbL, stream);
      HSS_CUDA(cudaStreamSynchronize(stream));
      for (int q = 0; q < nbL; ++q) {
        const int n = (int)outs[q].size();
        const int kh = (int)std::ceil((double)yh[q] * n);
        const int hint = kh + std::max(4, (int)std::ceil(0.15 * kh));
        for (int s = 0; s < ps; ++s) ip[ps * q + s].steps_hint = hint;
      }
    } else if (id_step_test) {
      for (auto& q : ip) q.steps_hint = ID_EVERY_STEP;
    }
    // complex blocks: the pair-pivoted ID of the embedding (the complex ID of Common/ID.m:40-65)
    int maxn = 0;
    for (int v : pn) maxn = std::max(maxn, v);
    auto run_id = [&](const IdP* d, int cnt) {
      if (cx) id_pairs_batched(d, cnt, maxn, acc, stream);
      else id_adaptive_batched(d, cnt, acc, stream, id_df);
    };
    DevBuf<IdP> dip;
    upload_vec(dip, ip, stream);
    run_id(dip.p, nprob2);
    std::vector<int> hr, hs;
    download(hr, rank.p, nprob2, stream);
    download(hs, stat.p, (size_t)2 * nprob2, stream);
    HSS_CUDA(cudaStreamSynchronize(stream));
    {
      // boxes whose truncated factorization could not settle the rank are redone in full
      std::vector<IdP> redo;
      std::vector<int> redo_ix;
      for (int pr = 0; pr < nprob2; ++pr)
        if (hs[2 * pr] == 2) { IdP r = ip[pr]; r.steps_hint = -1; redo.push_back(r); redo_ix.push_back(pr); }
      if (!redo.empty()) {
        DevBuf<IdP> dr;
        upload_vec(dr, redo, stream);
        run_id(dr.p, (int)redo.size());
        download(hr, rank.p, nprob2, stream);
        download(hs, stat.p, (size_t)2 * nprob2, stream);
        HSS_CUDA(cudaStreamSynchronize(stream));
        reruns += (int)redo.size();
        for (int pr : redo_ix) ip[pr].steps_hint = -1;
      }
    }
    for (int pr = 0; pr < nprob2; ++pr) {
      qr_steps += hs[2 * pr + 1];
      qr_steps_full += std::min(pm[pr], pn[pr]);
    }
    bool any = false;
    std::vector<int> kbox(nbL);
    for (int q = 0; q < nbL; ++q) {
      const int ko = hr[ps * q] / rep, ki = hr[ps * q + ps - 1] / rep;  // ranks in points
      const int k = std::max(ko, ki);
      kbox[q] = k;
      const int po = ps * q, pi = ps * q + ps - 1, kr = rep * k;
      if (k != ko) { ip[po].force_k = kr; any = true; HSS_REQUIRE(kr <= std::min(pm[po], pn[po]), HSS_ERR_RANK, "fixed rank exceeds block size"); }
      else if (k != ki) { ip[pi].force_k = kr; any = true; HSS_REQUIRE(kr <= std::min(pm[pi], pn[pi]), HSS_ERR_RANK, "fixed rank exceeds block size"); }
    }
    if (any) {
      // a fixed-rank re-ID needs R(0:k, :) of the full factorization up to k
      std::vector<IdP> redo;
      for (int pr = 0; pr < nprob2; ++pr)
        if (ip[pr].force_k >= 0 && hs[2 * pr + 1] < ip[pr].force_k) {
          IdP r = ip[pr];
          r.force_k = -1;
          r.steps_hint = -1;
          redo.push_back(r);
        }
      if (!redo.empty()) {
        DevBuf<IdP> dr;
        upload_vec(dr, redo, stream);
        run_id(dr.p, (int)redo.size());
        HSS_CUDA(cudaStreamSynchronize(stream));
        reruns += (int)redo.size();
      }
      HSS_CUDA(cudaMemcpyAsync(dip.p, ip.data(), nprob2 * sizeof(IdP), cudaMemcpyHostToDevice, stream));
      id_fixed_batched(dip.p, nprob2, stream);
    }
    std::vector<int> hp;
    download(hp, perm.p, tP, stream);
    HSS_CUDA(cudaStreamSynchronize(stream));
    lap(3);
    for (int q = 0; q < nbL; ++q) {
      const int b = boxes[q];
      const int n = (int)outs[q].size(), k = kbox[q], po = ps * q, pi = ps * q + ps - 1;
      nskel[b] = n;
      kskel[b] = k;
      J_UP[b].resize(n);
      J_DN[b].resize(n);
      for (int t = 0; t < n; ++t) {  // a pair-pivoted ID moves the two columns of a point together
        J_UP[b][t] = hp[oP[po] + rep * t] / rep;
        J_DN[b][t] = hp[oP[pi] + rep * t] / rep;
      }
      I_SKUP[b].resize(k);
      I_SKDN[b].resize(k);
      for (int t = 0; t < k; ++t) {
        I_SKUP[b][t] = outs[q][J_UP[b][t]];
        I_SKDN[b][t] = inns[q][J_DN[b][t]];
      }
      Toff[b] = {oT2[po], oT2[pi]};
      Tlev[b] = (int)Tkeep.size() - 1;
      census[4 * b] = pm[po] / rep; census[4 * b + 1] = pm[pi] / rep; census[4 * b + 2] = n; census[4 * b + 3] = k;
    }
    lap(4);
  }
  if (cx) {
    // from here on the handle is the real 2N x 2N embedding: point i is unknowns 2i, 2i + 1
    // (interleaved real and imaginary parts), and every size and index set counts unknowns
    auto twice = [](std::vector<int>& v) {
      std::vector<int> w(2 * v.size());
      for (size_t i = 0; i < v.size(); ++i) { w[2 * i] = 2 * v[i]; w[2 * i + 1] = 2 * v[i] + 1; }
      v.swap(w);
    };
    for (int b = 0; b < nboxes; ++b) {
      off[b] *= 2; cnt[b] *= 2; nskel[b] *= 2; kskel[b] *= 2;
      twice(I_SKUP[b]); twice(I_SKDN[b]); twice(J_UP[b]); twice(J_DN[b]);
    }
    for (int p = 0; p < nprob; ++p) { pN[p] *= 2; pbase[p] *= 2; }
    Ntot *= 2;
  }
  // ---- compact T_UP / T_DN / T_DN^T and J arenas
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
    // complex fsym: T_DN = T_UP is kept as conj(T_UP) (the handle's T_DN convention)
    const bool cj = cplx && sym;
    mv.push_back(MoveP{Tl + Toff[b][1], T_DN.p + oT[b], nullptr, k, n - k, n, k, cj ? 4 : 0, 0});
    mv.push_back(MoveP{Tl + Toff[b][1], TDNT.p + oT[b], nullptr, k, n - k, n, n - k, cj ? 5 : 3, 0});
  }
  run_moves(mv, stream);
  upload_vec(JUPd, hJU, stream);
  upload_vec(JDNd, hJD, stream);
  Tkeep.clear();
  // ---- M_SELF (leaves) and M_SIB (:220-271)
  oSelf.assign(nboxes, -1);
  oSib.assign(nboxes, -1);
  long long ts = 0, tb = 0;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] >= 0 && is_leaf(b)) { oSelf[b] = ts; ts += (long long)cnt[b] * cnt[b]; }
    if (!is_leaf(b)) {
      const int s1 = c1[b], s2 = c2[b];
      oSib[s1] = tb; tb += (long long)kskel[s1] * kskel[s2];
      oSib[s2] = tb; tb += (long long)kskel[s2] * kskel[s1];
    }
  }
  M_SELF.alloc(std::max(ts, 1LL));
  M_SIB.alloc(std::max(tb, 1LL));
  std::vector<int> idx;
  std::vector<KgenP<double>> kg;
  std::vector<long long> io;
  auto push = [&](const std::vector<int>& v) { io.push_back(idx.size()); idx.insert(idx.end(), v.begin(), v.end()); };
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] >= 0 && is_leaf(b)) {
      std::vector<int> r(cnt[b]);
      std::iota(r.begin(), r.end(), off[b]);
      push(r);
    }
    if (!is_leaf(b)) {
      push(I_SKDN[c1[b]]); push(I_SKUP[c2[b]]);
      if (!sym) { push(I_SKDN[c2[b]]); push(I_SKUP[c1[b]]); }
    }
  }
  DevBuf<int> didx;
  upload_vec(didx, idx, stream);
  size_t q = 0;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] >= 0 && is_leaf(b)) {
      const int* r = didx.p + io[q++];
      kg.push_back(KgenP<double>{r, r, cnt[b], cnt[b], M_SELF.p + oSelf[b], cnt[b], 0});
    }
    if (!is_leaf(b)) {
      const int s1 = c1[b], s2 = c2[b];
      const int* a = didx.p + io[q++];
      const int* bb = didx.p + io[q++];
      kg.push_back(KgenP<double>{a, bb, kskel[s1], kskel[s2], M_SIB.p + oSib[s1], kskel[s1], 0});
      if (!sym) {
        const int* c = didx.p + io[q++];
        const int* d = didx.p + io[q++];
        kg.push_back(KgenP<double>{c, d, kskel[s2], kskel[s1], M_SIB.p + oSib[s2], kskel[s2], 0});
      }
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
  if (sym) {  // M_SIB{c2} = M_SIB{c1}.' (HSS1D_compress_fsym.m:245; plain transpose when complex)
    std::vector<MoveP> mv;
    for (int b = 0; b < nboxes; ++b)
      if (!is_leaf(b) && kskel[c1[b]] > 0 && kskel[c2[b]] > 0)
        mv.push_back(MoveP{M_SIB.p + oSib[c1[b]], M_SIB.p + oSib[c2[b]], nullptr, kskel[c1[b]], kskel[c2[b]],
                           kskel[c1[b]], kskel[c2[b]], cplx ? 5 : 3, 0});
    run_moves(mv, stream);
  }
  HSS_CUDA(cudaStreamSynchronize(stream));
  lap(5);
  inverted = false;
}

// ---------------------------------------------------------------------------
// Kinv_HSS = HSS1D_transforminv_nsym(K_HSS, HSSinv, FTinv), HSS1D/HSS1D_transforminv_nsym.m:38-161.
// Rewrites the inverse factors as an HSS1D matrix in the compressed format, so that the
// forward apply of K applies the inverse.  Three tree sweeps, each level batched over every
// box of every problem: (1) top-down, the diagonal blocks of each parent's Dinv (FTinv at
// the top) move into its sons' Dinv as L * block * R (:38-77); (2) bottom-up, each box's
// Linv/Rinv become [I; T] form through P = Linv(J_UP(1:k),:) and Q = Rinv(:,J_DN(1:k)), whose
// factors move into the parent's rows and columns (:83-125); (3) the parents' off-diagonal
// blocks become sibling matrices and the leaves' Dinv the self blocks (:128-161).
void HSS1D::transforminv(HSS1D& K) {
  HSS_REQUIRE(!rect, HSS_ERR_ARG, "transforminv is defined for square handles only");
  HSS_REQUIRE(inverted, HSS_ERR_STATE, "transforminv needs the inverse factors (call invert first)");
  K.Ntot = Ntot; K.nprob = nprob; K.nboxes = nboxes; K.leaf = leaf; K.maxlev = maxlev; K.acc = acc; K.sym = sym;
  K.pN = pN; K.pbase = pbase; K.proot = proot; K.pseed = pseed;
  K.prob = prob; K.level = level; K.parent = parent; K.c1 = c1; K.c2 = c2; K.off = off; K.cnt = cnt;
  K.nskel = nskel; K.kskel = kskel; K.I_SKUP = I_SKUP; K.I_SKDN = I_SKDN;
  K.J_UP = J_DN;  // Kinv's up projection comes from Rinv, whose skeleton order is J_DN (:151-154)
  K.J_DN = J_UP;
  K.X = X; K.kp = kp; K.kdev = kdev; K.census = census;
  K.oT = oT; K.oSelf = oSelf; K.oSib = oSib; K.oJ = oJ;
  K.cplx = cplx;
  K.inverted = false;
  const cudaStream_t st = stream;
  auto d2d = [&](DevBuf<double>& dst, const DevBuf<double>& src) {
    dst.alloc(std::max<size_t>(src.n, 1));
    if (src.n) HSS_CUDA(cudaMemcpyAsync(dst.p, src.p, src.n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  };
  K.JUPd.alloc(std::max<size_t>(JDNd.n, 1));
  K.JDNd.alloc(std::max<size_t>(JUPd.n, 1));
  if (JDNd.n) HSS_CUDA(cudaMemcpyAsync(K.JUPd.p, JDNd.p, JDNd.n * sizeof(int), cudaMemcpyDeviceToDevice, st));
  if (JUPd.n) HSS_CUDA(cudaMemcpyAsync(K.JDNd.p, JUPd.p, JUPd.n * sizeof(int), cudaMemcpyDeviceToDevice, st));
  K.T_UP.alloc(std::max<size_t>(T_UP.n, 1));
  K.T_DN.alloc(std::max<size_t>(T_DN.n, 1));
  K.TDNT.alloc(std::max<size_t>(TDNT.n, 1));
  K.M_SELF.alloc(std::max<size_t>(M_SELF.n, 1));
  K.M_SIB.alloc(std::max<size_t>(M_SIB.n, 1));
  DevBuf<double> Lw, Rw, Dw, FTw;
  d2d(Lw, Linv);
  d2d(Rw, Rinv);
  d2d(Dw, Dinv);
  d2d(FTw, FTinv);
  int maxk = 1;
  for (int b = 0; b < nboxes; ++b) maxk = std::max(maxk, kskel[b]);
  DevBuf<double> zero((size_t)maxk * maxk), Wt(std::max<size_t>(Linv.n, 1));
  zero.zero(st);
  // the block of box s's parent that belongs to s: (matrix, leading dim, offset of s)
  auto parent_block = [&](int s, double*& B, int& ld, int& o) {
    const int f = parent[s];
    if (parent[f] < 0) { B = FTw.p + oFT[prob[f]]; ld = ktop[prob[f]]; }
    else { B = Dw.p + oD[f]; ld = nskel[f]; }
    o = (s == c2[f] && c1[f] >= 0) ? kskel[c1[f]] : 0;
  };
  // (1) top-down: D_s += L_s * D_f(ind_s, ind_s) * R_s, then clear that block
  for (int Lv = 1; Lv <= maxlev; ++Lv) {
    std::vector<GemmP<double>> G1, G2;
    std::vector<MoveP> Z;
    for (int s = 0; s < nboxes; ++s) {
      if (level[s] != Lv) continue;
      const int n = nskel[s], k = kskel[s];
      if (k == 0) continue;
      double* B;
      int ld, o;
      parent_block(s, B, ld, o);
      double* blk = B + o + (size_t)o * ld;
      G1.push_back(GemmP<double>{Lw.p + oL[s], blk, Wt.p + oL[s], n, k, k, n, ld, n});
      G2.push_back(GemmP<double>{Wt.p + oL[s], Rw.p + oR[s], Dw.p + oD[s], n, n, k, n, k, n});
      Z.push_back(MoveP{zero.p, blk, nullptr, k, k, k, ld, 0, 0});
    }
    run_gemms(G1, false, false, 1.0, 0.0, st);
    run_gemms(G2, false, false, 1.0, 1.0, st);
    run_moves(Z, st);
  }
  // (2) bottom-up: [I T] forms and the parents' row / column factors
  for (int Lv = maxlev; Lv >= 1; --Lv) {
    std::vector<int> boxes;
    for (int b = 0; b < nboxes; ++b)
      if (level[b] == Lv && kskel[b] > 0) boxes.push_back(b);
    if (boxes.empty()) continue;
    std::vector<long long> oq(boxes.size()), orr(boxes.size()), ocol(boxes.size());
    long long tq = 0, tr = 0, tc = 0;
    for (size_t i = 0; i < boxes.size(); ++i) {
      const int b = boxes[i], k = kskel[b], f = parent[b];
      const int nf = (parent[f] < 0) ? ktop[prob[f]] : nskel[f];
      oq[i] = tq; tq += (long long)k * k;
      orr[i] = tr; tr += (long long)k * (2 * nf);   // P * Lw_f(ind,:) and P * D_f(ind,:)
      ocol[i] = tc; tc += (long long)(2 * nf) * k;  // Rw_f(:,ind) * Q and D_f(:,ind) * Q
    }
    DevBuf<double> Pm(tq), Qm(tq), Pi(tq), Qi(tq), Lr(std::max<size_t>(Linv.n, 1)), Rr(std::max<size_t>(Linv.n, 1)),
        Tr(std::max(tr, 1LL)), Tc(std::max(tc, 1LL));
    std::vector<MoveP> mv;
    for (size_t i = 0; i < boxes.size(); ++i) {
      const int b = boxes[i], n = nskel[b], k = kskel[b], nr = n - k;
      mv.push_back(MoveP{Lw.p + oL[b], Pm.p + oq[i], JUPd.p + oJ[b], k, k, n, k, 0, 0});  // P = L(JC(1:k),:)
      mv.push_back(MoveP{Rw.p + oR[b], Qm.p + oq[i], JDNd.p + oJ[b], k, k, k, k, 1, 0});  // Q = R(:,JR(1:k))
      if (nr > 0) {
        mv.push_back(MoveP{Lw.p + oL[b], Lr.p + oL[b], JUPd.p + oJ[b] + k, nr, k, n, nr, 0, 0});  // L(JC(k+1:n),:)
        mv.push_back(MoveP{Rw.p + oR[b], Rr.p + oL[b], JDNd.p + oJ[b] + k, k, nr, k, k, 1, 0});  // R(:,JR(k+1:n))
      }
    }
    run_moves(mv, st);
    mv.clear();
    for (size_t i = 0; i < boxes.size(); ++i) {  // copies to invert, after the gathers above
      const int k = kskel[boxes[i]];
      mv.push_back(MoveP{Pm.p + oq[i], Pi.p + oq[i], nullptr, k, k, k, k, 0, 0});
      mv.push_back(MoveP{Qm.p + oq[i], Qi.p + oq[i], nullptr, k, k, k, k, 0, 0});
    }
    run_moves(mv, st);
    std::vector<std::pair<double*, int>> mats;
    for (size_t i = 0; i < boxes.size(); ++i) {
      const int k = kskel[boxes[i]];
      mats.push_back({Pi.p + oq[i], k});
      mats.push_back({Qi.p + oq[i], k});
    }
    invert_many(mats, st);
    // Kinv T_DN^T = L(JC(k+1:n),:) / P ; Kinv T_UP = Q \ R(:,JR(k+1:n))
    std::vector<GemmP<double>> GL, GR;
    mv.clear();
    for (size_t i = 0; i < boxes.size(); ++i) {
      const int b = boxes[i], n = nskel[b], k = kskel[b], nr = n - k;
      if (nr <= 0) continue;
      GL.push_back(GemmP<double>{Lr.p + oL[b], Pi.p + oq[i], K.TDNT.p + oT[b], nr, k, k, nr, k, nr});
      GR.push_back(GemmP<double>{Qi.p + oq[i], Rr.p + oL[b], K.T_UP.p + oT[b], k, nr, k, k, k, k});
      mv.push_back(MoveP{K.TDNT.p + oT[b], K.T_DN.p + oT[b], nullptr, nr, k, nr, k, 3, 0});
    }
    run_gemms(GL, false, false, 1.0, 0.0, st);
    run_gemms(GR, false, false, 1.0, 0.0, st);
    run_moves(mv, st);
    // parents: rows ind *= P (Linv_f and D_f), then columns ind *= Q (Rinv_f and D_f); the
    // sons of one parent own disjoint rows and columns, so the level is one batch each
    std::vector<GemmP<double>> GP, GQ;
    std::vector<MoveP> backP, backQ;
    for (size_t i = 0; i < boxes.size(); ++i) {
      const int b = boxes[i], k = kskel[b], f = parent[b];
      double* B;
      int ld, o;
      parent_block(b, B, ld, o);
      const int nf = ld;
      double* tr0 = Tr.p + orr[i];
      double* tc0 = Tc.p + ocol[i];
      if (parent[f] >= 0) {
        const int kf = kskel[f];
        GP.push_back(GemmP<double>{Pm.p + oq[i], Lw.p + oL[f] + o, tr0, k, kf, k, k, nf, k});
        backP.push_back(MoveP{tr0, Lw.p + oL[f] + o, nullptr, k, kf, k, nf, 0, 0});
        GQ.push_back(GemmP<double>{Rw.p + oR[f] + (size_t)o * kf, Qm.p + oq[i], tc0, kf, k, k, kf, k, kf});
        backQ.push_back(MoveP{tc0, Rw.p + oR[f] + (size_t)o * kf, nullptr, kf, k, kf, kf, 0, 0});
        tr0 += (size_t)k * nf;
        tc0 += (size_t)nf * k;
      }
      GP.push_back(GemmP<double>{Pm.p + oq[i], B + o, tr0, k, nf, k, k, ld, k});
      backP.push_back(MoveP{tr0, B + o, nullptr, k, nf, k, ld, 0, 0});
      GQ.push_back(GemmP<double>{B + (size_t)o * ld, Qm.p + oq[i], tc0, nf, k, k, ld, k, nf});
      backQ.push_back(MoveP{tc0, B + (size_t)o * ld, nullptr, nf, k, nf, ld, 0, 0});
    }
    run_gemms(GP, false, false, 1.0, 0.0, st);
    run_moves(backP, st);
    run_gemms(GQ, false, false, 1.0, 0.0, st);
    run_moves(backQ, st);
  }
  // (3) sibling blocks from each parent's off-diagonal blocks; self blocks from leaf Dinv
  std::vector<MoveP> mv;
  for (int f = 0; f < nboxes; ++f) {
    if (c1[f] < 0 || c2[f] < 0) continue;
    const int a = c1[f], b = c2[f], ka = kskel[a], kb = kskel[b];
    const double* B;
    int ld;
    if (parent[f] < 0) { B = FTw.p + oFT[prob[f]]; ld = ktop[prob[f]]; }
    else { B = Dw.p + oD[f]; ld = nskel[f]; }
    if (ka > 0 && kb > 0) {
      mv.push_back(MoveP{B + (size_t)ka * ld, K.M_SIB.p + oSib[a], nullptr, ka, kb, ld, ka, 0, 0});
      mv.push_back(MoveP{B + ka, K.M_SIB.p + oSib[b], nullptr, kb, ka, ld, kb, 0, 0});
    }
  }
  for (int b = 0; b < nboxes; ++b)
    if (parent[b] >= 0 && is_leaf(b))
      mv.push_back(MoveP{Dw.p + oD[b], K.M_SELF.p + oSelf[b], nullptr, nskel[b], nskel[b], nskel[b], cnt[b], 0, 0});
  run_moves(mv, st);
  HSS_CUDA(cudaStreamSynchronize(st));
}

// ---------------------------------------------------------------------------
void HSS1D::invert() {
  HSS_REQUIRE(!rect, HSS_ERR_ARG, "invert is defined for square handles only");
  clear_plans();
  oL.assign(nboxes, 0); oR.assign(nboxes, 0); oD.assign(nboxes, 0); oE.assign(nboxes, 0);
  long long tl = 0, td = 0, te = 0;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] < 0) continue;
    const long long n = nskel[b], k = kskel[b];
    oL[b] = tl; oR[b] = tl; tl += n * k;
    oD[b] = td; td += n * n;
    oE[b] = te; te += k * k;
  }
  Linv.alloc(std::max(tl, 1LL)); Rinv.alloc(std::max(tl, 1LL)); Dinv.alloc(std::max(td, 1LL));
  Einv.alloc(std::max(te, 1LL));
  DevBuf<double> Fw(std::max(td, 1LL)), W1(std::max(td, 1LL)), W2(std::max(td, 1LL)), W3(std::max(tl, 1LL));
  for (int Lv = maxlev; Lv >= 1; --Lv) {
    std::vector<int> boxes;
    for (int b = 0; b < nboxes; ++b)
      if (level[b] == Lv) boxes.push_back(b);
    if (boxes.empty()) continue;
    std::vector<F1P> fa;
    std::vector<std::pair<double*, int>> mats;
    for (int b : boxes) {
      const int n = nskel[b];
      if (is_leaf(b)) {
        fa.push_back(F1P{Fw.p + oD[b], n, 0, nullptr, nullptr, nullptr, nullptr, M_SELF.p + oSelf[b]});
      } else {
        const int s1 = c1[b], s2 = c2[b];
        fa.push_back(F1P{Fw.p + oD[b], n, kskel[s1], Einv.p + oE[s1], M_SIB.p + oSib[s1], M_SIB.p + oSib[s2],
                         Einv.p + oE[s2], nullptr});
      }
      mats.push_back({Fw.p + oD[b], n});
    }
    {
      DevBuf<F1P> d;
      upload_vec(d, fa, stream);
      k_assemble1<<<(int)fa.size(), 256, 0, stream>>>(d.p);
      check_launch("k_assemble1");
      HSS_CUDA(cudaStreamSynchronize(stream));
    }
    invert_many(mats, stream, dfinv());
    std::vector<MoveP> mv;
    for (int b : boxes) {
      const int n = nskel[b];
      mv.push_back(MoveP{Fw.p + oD[b], W1.p + oD[b], JUPd.p + oJ[b], n, n, n, n, 0, 0});   // Finv[J_UP, :]
      mv.push_back(MoveP{Fw.p + oD[b], W2.p + oD[b], JDNd.p + oJ[b], n, n, n, n, 1, 0});   // Finv[:, J_DN]
    }
    run_moves(mv, stream);
    std::vector<GemmP<double>> P1, P2;
    for (int b : boxes) {
      const int n = nskel[b], k = kskel[b], nr = n - k;
      if (nr <= 0 || k == 0) continue;
      // RF = W1[0:k,:] + T_UP W1[k:n,:]   ;  FL = W2[:,0:k] + W2[:,k:n] T_DN^T
      P1.push_back(GemmP<double>{T_UP.p + oT[b], W1.p + oD[b] + k, W1.p + oD[b], k, n, nr, k, n, n});
      P2.push_back(GemmP<double>{W2.p + oD[b] + (size_t)k * n, T_DN.p + oT[b], W2.p + oD[b], n, k, nr, n, k, n});
    }
    run_gemms(P1, false, false, 1.0, 1.0, stream, false, dfinv());
    run_gemms(P2, false, true, 1.0, 1.0, stream, false, dfinv());
    mv.clear();
    for (int b : boxes) {
      const int n = nskel[b], k = kskel[b];
      mv.push_back(MoveP{W1.p + oD[b], W3.p + oL[b], JDNd.p + oJ[b], k, n, n, k, 1, 0});  // RF[:, J_DN]
    }
    run_moves(mv, stream);
    P1.clear();
    for (int b : boxes) {
      const int n = nskel[b], k = kskel[b], nr = n - k;
      if (nr <= 0 || k == 0) continue;
      P1.push_back(GemmP<double>{W3.p + oL[b] + (size_t)k * k, T_DN.p + oT[b], W3.p + oL[b], k, k, nr, k, k, k});
    }
    run_gemms(P1, false, true, 1.0, 1.0, stream, false, dfinv());
    mv.clear();
    mats.clear();
    for (int b : boxes) {
      const int k = kskel[b];
      mv.push_back(MoveP{W3.p + oL[b], Einv.p + oE[b], nullptr, k, k, k, k, 0, 0});
      mats.push_back({Einv.p + oE[b], k});
    }
    run_moves(mv, stream);
    invert_many(mats, stream, dfinv());
    // Linv = FL E ; Rinv = E RF ; Dinv = Finv - Linv RF
    std::vector<GemmP<double>> PL, PR, PD;
    mv.clear();
    for (int b : boxes) {
      const int n = nskel[b], k = kskel[b];
      PL.push_back(GemmP<double>{W2.p + oD[b], Einv.p + oE[b], Linv.p + oL[b], n, k, k, n, k, n});
      PR.push_back(GemmP<double>{Einv.p + oE[b], W1.p + oD[b], Rinv.p + oR[b], k, n, k, k, n, k});
      mv.push_back(MoveP{Fw.p + oD[b], Dinv.p + oD[b], nullptr, n, n, n, n, 0, 0});
    }
    run_gemms(PL, false, false, 1.0, 0.0, stream, false, dfinv());
    run_gemms(PR, false, false, 1.0, 0.0, stream, false, dfinv());
    run_moves(mv, stream);
    for (int b : boxes) {
      const int n = nskel[b], k = kskel[b];
      PD.push_back(GemmP<double>{Linv.p + oL[b], W1.p + oD[b], Dinv.p + oD[b], n, n, k, n, n, n});
    }
    run_gemms(PD, false, false, -1.0, 1.0, stream, false, dfinv());
  }
  // top of every tree: FT = [E2 M_SIB2; M_SIB3 E3] (the root's children, reference boxes 2 and 3)
  ktop.assign(nprob, 0);
  oFT.assign(nprob, 0);
  long long tft = 0;
  for (int p = 0; p < nprob; ++p) {
    const int r = proot[p];
    ktop[p] = kskel[c1[r]] + kskel[c2[r]];
    oFT[p] = tft;
    tft += (long long)ktop[p] * ktop[p];
  }
  FTinv.alloc(std::max(tft, 1LL));
  std::vector<F1P> fa;
  std::vector<std::pair<double*, int>> mats;
  for (int p = 0; p < nprob; ++p) {
    const int r = proot[p], a = c1[r], b = c2[r];
    fa.push_back(F1P{FTinv.p + oFT[p], ktop[p], kskel[a], Einv.p + oE[a], M_SIB.p + oSib[a], M_SIB.p + oSib[b],
                     Einv.p + oE[b], nullptr});
    mats.push_back({FTinv.p + oFT[p], ktop[p]});
  }
  DevBuf<F1P> d;
  upload_vec(d, fa, stream);
  k_assemble1<<<(int)fa.size(), 256, 0, stream>>>(d.p);
  check_launch("k_assemble1 top");
  HSS_CUDA(cudaStreamSynchronize(stream));
  invert_many(mats, stream, dfinv());
  inverted = true;
  if (dfm()) make_df();
}

// ---------------------------------------------------------------------------
// per-level stacked vectors: rows of level L are its boxes in id order
struct Stack1 {
  std::vector<long long> base;  // per level: element offset of the level block
  std::vector<int> ld;          // per level: total rows
  std::vector<long long> row;   // per box: row offset within its level
};

// k: skeleton size of each box (the column side's kskel, or the row side's on a
// rectangular handle)
static Stack1 make_stack(const HSS1D& H, int width, const std::vector<int>& k) {
  Stack1 s;
  s.base.assign(H.maxlev + 2, 0);
  s.ld.assign(H.maxlev + 2, 0);
  s.row.assign(H.nboxes, 0);
  for (int b = 0; b < H.nboxes; ++b) {
    if (H.parent[b] < 0) continue;
    s.row[b] = s.ld[H.level[b]];
    s.ld[H.level[b]] += k[b];
  }
  long long acc = 0;
  for (int L = 0; L <= H.maxlev + 1; ++L) { s.base[L] = acc; acc += (long long)s.ld[L] * width; }
  s.base.push_back(acc);
  return s;
}

void Plan1::gemm(const std::vector<GemmP<double>>& P, double alpha, double beta, cudaStream_t s) {
  if (P.empty()) return;
  Step st;
  st.batch = (int)P.size();
  int maxK = 0;
  for (auto& p : P) { st.maxM = std::max(st.maxM, p.M); st.maxN = std::max(st.maxN, p.N); maxK = std::max(maxK, p.K); }
  st.alpha = alpha;
  st.beta = beta;
  st.ksplit = df ? skinny_ksplit_df(st.batch, st.maxM, maxK) : skinny_ksplit<double>(st.batch, st.maxM, maxK);
  if (st.ksplit > 1) st.part.alloc((size_t)st.batch * st.ksplit * st.maxM * 8);
  st.g.upload(P, s);
  steps.push_back(std::move(st));
}

void Plan1::moves(const std::vector<MoveP>& mv, cudaStream_t s) {
  if (mv.empty()) return;
  Step st;
  st.move = true;
  st.batch = (int)mv.size();
  st.m.upload(mv, s);
  steps.push_back(std::move(st));
}

void Plan1::run(cudaStream_t s) const {
  for (auto& st : steps) {
    for (int o = 0; o < st.batch; o += 65535) {
      const int cnt = std::min(65535, st.batch - o);
      double* part = st.part.p ? st.part.p + (size_t)o * st.ksplit * st.maxM * 8 : nullptr;
      if (st.move) move_batched(st.m.p + o, cnt, s);
      else if (df) gemm_skinny_split_df(st.g.p + o, cnt, st.maxM, st.maxN, st.alpha, st.beta, st.ksplit, part, s);
      else gemm_skinny_split<double>(st.g.p + o, cnt, st.maxM, st.maxN, st.alpha, st.beta, st.ksplit, part, s);
    }
  }
}

int Plan1::launches() const {
  int n = 0;
  for (auto& st : steps) n += ((st.batch + 65534) / 65535) * ((!st.move && st.ksplit > 1) ? 2 : 1);
  return n;
}

void HSS1D::ensure_work() {
  const Stack1 S = make_stack(*this, 8, kskel), Sd = make_stack(*this, 8, rk());
  v1.ensure(std::max(S.base.back(), 1LL));
  v2.ensure(std::max(Sd.base.back(), 1LL));
  long long ts = 0;
  for (int b = 0; b < nboxes; ++b)
    if (parent[b] >= 0) ts += (long long)std::max({nskel[b] - kskel[b], rn()[b] - rk()[b], 1}) * 8;
  v3.ensure(std::max(ts, 1LL));
  Xs.ensure((size_t)Ntot * 8);
  Ys.ensure((size_t)rows() * 8);
}

// inverse apply of r columns Xs -> Ys (HSS1D_applyinv_nsym.m:43-86): up Rinv, top FTinv,
// down Linv (+ Dinv on the box input)
Plan1& HSS1D::inv_plan(int r) {
  auto it = inv_plans.find(r);
  if (it != inv_plans.end()) return it->second;
  ensure_work();
  Plan1& pl = inv_plans[r];
  pl.df = dfm();
  const double* RI = dfm() ? Rinv_df.p : Rinv.p;
  const double* LI = dfm() ? Linv_df.p : Linv.p;
  const double* DI = dfm() ? Dinv_df.p : Dinv.p;
  const double* FT = dfm() ? FTinv_df.p : FTinv.p;
  const Stack1 S = make_stack(*this, 8, kskel);
  const double* ff = Xs.p;
  double* xx = Ys.p;
  auto vin = [&](int b, const double*& p, int& ld) {
    if (is_leaf(b)) { p = ff + off[b]; ld = (int)Ntot; }
    else { const int L = level[b] + 1; p = v1.p + S.base[L] + S.row[c1[b]]; ld = S.ld[L]; }
  };
  std::vector<std::vector<int>> bylev(maxlev + 1);
  for (int b = 0; b < nboxes; ++b)
    if (parent[b] >= 0) bylev[level[b]].push_back(b);
  for (int L = maxlev; L >= 1; --L) {
    std::vector<GemmP<double>> P;
    for (int b : bylev[L]) {
      const double* in;
      int ldi;
      vin(b, in, ldi);
      P.push_back(GemmP<double>{RI + oR[b], in, v1.p + S.base[L] + S.row[b], kskel[b], r, nskel[b], kskel[b],
                                ldi, S.ld[L]});
    }
    pl.gemm(P, 1.0, 0.0, stream);
  }
  {
    std::vector<GemmP<double>> P;
    for (int p = 0; p < nprob; ++p) {
      const int a = c1[proot[p]];
      P.push_back(GemmP<double>{FT + oFT[p], v1.p + S.base[1] + S.row[a], v2.p + S.base[1] + S.row[a],
                                ktop[p], r, ktop[p], ktop[p], S.ld[1], S.ld[1]});
    }
    pl.gemm(P, 1.0, 0.0, stream);
  }
  for (int L = 1; L <= maxlev; ++L) {
    std::vector<GemmP<double>> P1, P2;
    for (int b : bylev[L]) {
      double* out;
      int ldo;
      if (is_leaf(b)) { out = xx + off[b]; ldo = (int)Ntot; }
      else { out = v2.p + S.base[L + 1] + S.row[c1[b]]; ldo = S.ld[L + 1]; }
      const double* in;
      int ldi;
      vin(b, in, ldi);
      P1.push_back(GemmP<double>{LI + oL[b], v2.p + S.base[L] + S.row[b], out, nskel[b], r, kskel[b], nskel[b],
                                 S.ld[L], ldo});
      P2.push_back(GemmP<double>{DI + oD[b], in, out, nskel[b], r, nskel[b], nskel[b], ldi, ldo});
    }
    pl.gemm(P1, 1.0, 0.0, stream);
    pl.gemm(P2, 1.0, 1.0, stream);
  }
  HSS_CUDA(cudaStreamSynchronize(stream));
  return pl;
}

static void split_into(const DevBuf<double>& src, DevBuf<double>& dst, cudaStream_t s) {
  dst.alloc(std::max<size_t>((src.n + 1) & ~(size_t)1, 2));  // whole (hi, hi, lo, lo) blocks
  split_df(src.p, dst.p, (long long)src.n, s);
}

// float-pair copies of the operators the solve products read
void HSS1D::make_df() {
  split_into(T_UP, T_UP_df, stream);
  split_into(TDNT, TDNT_df, stream);
  split_into(M_SELF, M_SELF_df, stream);
  split_into(M_SIB, M_SIB_df, stream);
  if (inverted) {
    split_into(Linv, Linv_df, stream);
    split_into(Rinv, Rinv_df, stream);
    split_into(Dinv, Dinv_df, stream);
    split_into(FTinv, FTinv_df, stream);
  }
  HSS_CUDA(cudaStreamSynchronize(stream));
}

void HSS1D::set_precision(int prec) {
  HSS_REQUIRE(prec == HSS_PREC_FP64 || prec == HSS_PREC_DFLOAT || prec == HSS_PREC_DFLOAT_INV, HSS_ERR_ARG,
              "HSS1D runs in HSS_PREC_FP64, HSS_PREC_DFLOAT or HSS_PREC_DFLOAT_INV");
  precision = prec;
  clear_plans();
  if (dfm()) make_df();
}

void HSS1D::applyinv_device(const double* dX, double* dY, int nrhs) {
  HSS_REQUIRE(!rect, HSS_ERR_ARG, "applyinv is defined for square handles only");
  HSS_REQUIRE(inverted, HSS_ERR_STATE, "hss1d_applyinv before hss1d_invert");
  for (int c0 = 0; c0 < nrhs; c0 += 8) {
    const int r = std::min(8, nrhs - c0);
    Plan1& pl = inv_plan(r);
    HSS_CUDA(cudaMemcpyAsync(Xs.p, dX + (size_t)c0 * Ntot, (size_t)Ntot * r * sizeof(double),
                             cudaMemcpyDeviceToDevice, stream));
    run_graph(g_inv, r, stream, use_graphs, [&] { pl.run(stream); });
    HSS_CUDA(cudaMemcpyAsync(dY + (size_t)c0 * Ntot, Ys.p, (size_t)Ntot * r * sizeof(double),
                             cudaMemcpyDeviceToDevice, stream));
  }
}

// forward apply of r columns Xs -> Ys (HSS1D_apply_nsym.m:38-100): up projections
// q(J(1:k)) + T_UP q(J(k+1:n)), top siblings, down evaluations with M_SIB / M_SELF.  On a
// rectangular handle (HSS1D_apply_rect_nsym.m:30-106) the down pass runs on the row tree:
// its stack, T_DN, J_DN and the leaves' rows come from the row side (rk(), roff() ...).
Plan1& HSS1D::fwd_plan(int r) {
  auto it = fwd_plans.find(r);
  if (it != fwd_plans.end()) return it->second;
  ensure_work();
  Plan1& pl = fwd_plans[r];
  pl.df = dfm();
  const double* TU = dfm() ? T_UP_df.p : T_UP.p;
  const double* TD = dfm() ? TDNT_df.p : TDNT.p;
  const double* MS = dfm() ? M_SELF_df.p : M_SELF.p;
  const double* MB = dfm() ? M_SIB_df.p : M_SIB.p;
  const std::vector<int>&kd = rk(), &nd = rn(), &od = roff(), &cd = rcnt();
  const std::vector<long long>&oTdn = roT(), &oJdn = roJ();
  const int ldu = (int)rows();
  const Stack1 S = make_stack(*this, 8, kskel), Sd = make_stack(*this, 8, kd);
  std::vector<long long> oS(nboxes, 0);
  long long ts = 0;
  for (int b = 0; b < nboxes; ++b) {
    if (parent[b] < 0) continue;
    oS[b] = ts;
    ts += (long long)std::max({nskel[b] - kskel[b], nd[b] - kd[b], 1}) * 8;
  }
  const double* qq = Xs.p;
  double* uu = Ys.p;
  auto vin = [&](int b, const double*& p, int& ld) {
    if (is_leaf(b)) { p = qq + off[b]; ld = (int)Ntot; }
    else { const int L = level[b] + 1; p = v1.p + S.base[L] + S.row[c1[b]]; ld = S.ld[L]; }
  };
  std::vector<std::vector<int>> bylev(maxlev + 1);
  for (int b = 0; b < nboxes; ++b)
    if (parent[b] >= 0) bylev[level[b]].push_back(b);
  for (int L = maxlev; L >= 1; --L) {
    std::vector<MoveP> mv;
    std::vector<GemmP<double>> P;
    for (int b : bylev[L]) {
      const int n = nskel[b], k = kskel[b], nr = n - k;
      const double* in;
      int ldi;
      vin(b, in, ldi);
      mv.push_back(MoveP{in, v1.p + S.base[L] + S.row[b], JUPd.p + oJ[b], k, r, ldi, S.ld[L], 0, 0});
      if (nr > 0) {
        mv.push_back(MoveP{in, v3.p + oS[b], JUPd.p + oJ[b] + k, nr, r, ldi, nr, 0, 0});
        P.push_back(GemmP<double>{TU + oT[b], v3.p + oS[b], v1.p + S.base[L] + S.row[b], k, r, nr, k, nr,
                                  S.ld[L]});
      }
    }
    pl.moves(mv, stream);
    pl.gemm(P, 1.0, 1.0, stream);
  }
  {
    std::vector<GemmP<double>> P;
    for (int p = 0; p < nprob; ++p) {
      const int a = c1[proot[p]], b = c2[proot[p]];
      P.push_back(GemmP<double>{MB + oSib[a], v1.p + S.base[1] + S.row[b], v2.p + Sd.base[1] + Sd.row[a],
                                kd[a], r, kskel[b], std::max(kd[a], 1), S.ld[1], Sd.ld[1]});
      P.push_back(GemmP<double>{MB + oSib[b], v1.p + S.base[1] + S.row[a], v2.p + Sd.base[1] + Sd.row[b],
                                kd[b], r, kskel[a], std::max(kd[b], 1), S.ld[1], Sd.ld[1]});
    }
    pl.gemm(P, 1.0, 0.0, stream);
  }
  for (int L = 1; L <= maxlev; ++L) {
    std::vector<GemmP<double>> PT, PS;
    std::vector<MoveP> mv;
    for (int b : bylev[L]) {
      const int n = nd[b], k = kd[b], nr = n - k;
      const double* dn = v2.p + Sd.base[L] + Sd.row[b];
      double* out;
      int ldo;
      if (is_leaf(b)) { out = uu + od[b]; ldo = ldu; }
      else { out = v2.p + Sd.base[L + 1] + Sd.row[c1[b]]; ldo = Sd.ld[L + 1]; }
      if (nr > 0) PT.push_back(GemmP<double>{TD + oTdn[b], dn, v3.p + oS[b], nr, r, k, nr, Sd.ld[L], nr});
      mv.push_back(MoveP{dn, out, JDNd.p + oJdn[b], k, r, Sd.ld[L], ldo, 2, 0});
      if (nr > 0) mv.push_back(MoveP{v3.p + oS[b], out, JDNd.p + oJdn[b] + k, nr, r, nr, ldo, 2, 0});
      if (is_leaf(b)) {
        PS.push_back(GemmP<double>{MS + oSelf[b], qq + off[b], out, cd[b], r, cnt[b], cd[b], (int)Ntot, ldo});
      } else {
        const int s1 = c1[b], s2 = c2[b];
        const double* up1 = v1.p + S.base[L + 1] + S.row[s1];
        const double* up2 = v1.p + S.base[L + 1] + S.row[s2];
        PS.push_back(GemmP<double>{MB + oSib[s1], up2, out, kd[s1], r, kskel[s2], std::max(kd[s1], 1),
                                   S.ld[L + 1], ldo});
        PS.push_back(GemmP<double>{MB + oSib[s2], up1, out + kd[s1], kd[s2], r, kskel[s1], std::max(kd[s2], 1),
                                   S.ld[L + 1], ldo});
      }
    }
    pl.gemm(PT, 1.0, 0.0, stream);
    pl.moves(mv, stream);
    pl.gemm(PS, 1.0, 1.0, stream);
  }
  HSS_CUDA(cudaStreamSynchronize(stream));
  return pl;
}

void HSS1D::apply_device(const double* dX, double* dY, int nrhs) {
  for (int c0 = 0; c0 < nrhs; c0 += 8) {
    const int r = std::min(8, nrhs - c0);
    Plan1& pl = fwd_plan(r);
    HSS_CUDA(cudaMemcpyAsync(Xs.p, dX + (size_t)c0 * Ntot, (size_t)Ntot * r * sizeof(double),
                             cudaMemcpyDeviceToDevice, stream));
    run_graph(g_fwd, r, stream, use_graphs, [&] { pl.run(stream); });
    HSS_CUDA(cudaMemcpyAsync(dY + (size_t)c0 * rows(), Ys.p, (size_t)rows() * r * sizeof(double),
                             cudaMemcpyDeviceToDevice, stream));
  }
}

// ---------------------------------------------------------------------------
// Refinement (Common/Iterative_Refinement.m:20-35) against the FP64 forward operator.
__global__ void k_res1(long long N, int r, const double* __restrict__ f, const double* __restrict__ y,
                       double* __restrict__ res, double* __restrict__ part) {
  __shared__ double sa[8], sb[8];
  for (int c = 0; c < r; ++c) {
    double a = 0.0, b = 0.0;
    for (long long i = blockIdx.x * 256LL + threadIdx.x; i < N; i += (long long)gridDim.x * 256) {
      const double fv = f[i + c * N];
      const double rv = fv - y[i + c * N];
      res[i + c * N] = rv;
      a += rv * rv;
      b += fv * fv;
    }
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) { sa[threadIdx.x >> 5] = a; sb[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double ta = 0.0, tb = 0.0;
      for (int w = 0; w < 8; ++w) { ta += sa[w]; tb += sb[w]; }
      part[((long long)blockIdx.x * r + c) * 2] = ta;
      part[((long long)blockIdx.x * r + c) * 2 + 1] = tb;
    }
    __syncthreads();
  }
}

__global__ void k_axpy1(long long n, const double* __restrict__ d, double* __restrict__ x) {
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < n; e += (long long)gridDim.x * 256) x[e] += d[e];
}

void HSS1D::solve_device(const double* df, double* dx, int nrhs, double tol, int maxit, double* relres,
                         int* iters) {
  HSS_REQUIRE(!rect, HSS_ERR_ARG, "solve is defined for square handles only");
  HSS_REQUIRE(inverted, HSS_ERR_STATE, "hss1d_solve before hss1d_invert");
  HSS_REQUIRE(nrhs >= 1 && maxit >= 1, HSS_ERR_ARG, "nrhs and maxit must be >= 1");
  const long long cnt = Ntot * nrhs;
  ir_y.ensure(cnt);
  ir_res.ensure(cnt);
  ir_dd.ensure(cnt);
  DevBuf<double>& y = ir_y;
  DevBuf<double>& res = ir_res;
  DevBuf<double>& dd = ir_dd;
  const int gx = 256;
  ir_part.ensure((size_t)gx * nrhs * 2);
  ir_host.ensure((size_t)gx * nrhs * 2);
  const double* hp = ir_host.p;
  applyinv_device(df, dx, nrhs);
  int used = 1;
  double worst = 0.0;
  while (true) {
    apply_device(dx, y.p, nrhs);
    k_res1<<<gx, 256, 0, stream>>>(Ntot, nrhs, df, y.p, res.p, ir_part.p);
    check_launch("k_res1");
    HSS_CUDA(cudaMemcpyAsync(ir_host.p, ir_part.p, (size_t)gx * nrhs * 2 * sizeof(double), cudaMemcpyDeviceToHost,
                             stream));
    HSS_CUDA(cudaStreamSynchronize(stream));
    worst = 0.0;
    for (int c = 0; c < nrhs; ++c) {
      double a = 0.0, b = 0.0;
      for (int q = 0; q < gx; ++q) { a += hp[((size_t)q * nrhs + c) * 2]; b += hp[((size_t)q * nrhs + c) * 2 + 1]; }
      const double rel = (b > 0.0) ? std::sqrt(a / b) : std::sqrt(a);
      HSS_REQUIRE(std::isfinite(rel), HSS_ERR_NONFINITE, "non-finite residual in refinement");
      worst = std::max(worst, rel);
    }
    if (worst <= tol || used >= maxit) break;
    applyinv_device(res.p, dd.p, nrhs);
    k_axpy1<<<std::max(1, std::min(ceil_div(cnt, 256), 4096)), 256, 0, stream>>>(cnt, dd.p, dx);
    check_launch("k_axpy1");
    ++used;
  }
  HSS_CUDA(cudaStreamSynchronize(stream));
  if (relres) *relres = worst;
  if (iters) *iters = used;
}

}  // namespace hss
