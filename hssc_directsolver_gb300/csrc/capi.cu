// extern "C" boundary of libhssgpu.so (declared in include/hssgpu.h).
//
// Every entry point converts exceptions into status codes; the message of the
// last failure on the calling thread is kept for hss_last_error().
#include <cstring>
#include <string>

#include "dense.cuh"
#include "hss1d.h"
#include "hss2d.h"
#include "mlp.h"

#include <complex>
#include <numeric>

#include "kgen.cuh"

namespace hss {
void batched_inverse_noalloc(double* d_A, int n, int batch, int* d_info, cudaStream_t s);
void dr_corrections(double h, std::complex<double> k, std::complex<double>& corr0, std::complex<double>& corr1);
void dr_stencil(double h, std::complex<double> k, long long n, int order, std::vector<long long>& J,
                std::vector<std::complex<double>>& w, std::vector<int>& stencil);
static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace hss

using namespace hss;

#define HSS_TRY try {
#define HSS_CATCH                                                      \
  }                                                                    \
  catch (const hss::Error& e) {                                        \
    hss::set_last_error(e.what());                                     \
    return e.code;                                                     \
  }                                                                    \
  catch (const std::bad_alloc&) {                                      \
    hss::set_last_error("host allocation failed");                    \
    return HSS_ERR_NOMEM;                                              \
  }                                                                    \
  catch (const std::exception& e) {                                    \
    hss::set_last_error(e.what());                                     \
    return HSS_ERR_ARG;                                                \
  }                                                                    \
  return HSS_OK;

static cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

static void require_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    throw Error(HSS_ERR_CUDA, "no CUDA device available");
  }
}

template <typename R>
static void batched_inverse(R* d_A, int n, int batch, int* d_info, cudaStream_t s) {
  HSS_REQUIRE(d_A && d_info && n > 0 && batch > 0, HSS_ERR_ARG, "bad arguments");
  DevBuf<int> ipiv((size_t)batch * n), aux((size_t)batch * GJ_AUX);
  DevBuf<R> W((size_t)batch * 2 * GJ_NB * n), Wf((size_t)batch * n * n);
  HSS_CUDA(cudaMemsetAsync(d_info, 0, batch * sizeof(int), s));
  std::vector<InvP<R>> P(batch);
  for (int b = 0; b < batch; ++b)
    P[b] = InvP<R>{d_A + (size_t)b * n * n, n, n, ipiv.p + (size_t)b * n, W.p + (size_t)b * 2 * GJ_NB * n,
                   Wf.p + (size_t)b * n * n, d_info + b, aux.p + (size_t)b * GJ_AUX};
  DevBuf<InvP<R>> dP(batch);
  HSS_CUDA(cudaMemcpyAsync(dP.p, P.data(), batch * sizeof(InvP<R>), cudaMemcpyHostToDevice, s));
  invert_batched<R>(dP.p, batch, n, s);
  HSS_CUDA(cudaStreamSynchronize(s));
}

extern "C" {

const char* hss_last_error(void) { return hss::g_last_error.c_str(); }

int hss_version(void) { return 100; }

// Kernel_Eval on device buffers: points (x column, y column) already on the device.
static void kernel_eval_device(const hss_kernel_params* kp, const double* dX1, int64_t m, const double* dX2,
                               int64_t n, double* dA, cudaStream_t s) {
  HSS_REQUIRE(kp && dX1 && dX2 && dA && m > 0 && n > 0, HSS_ERR_ARG, "kernel_eval: bad arguments");
  HSS_REQUIRE(m + n <= (int64_t)INT32_MAX, HSS_ERR_ARG, "kernel_eval: too many points");
  const bool cplx = kp->flag == HSS_SL_H_2D;
  HSS_REQUIRE(kp->flag == HSS_SL_L_2D || cplx, HSS_ERR_ARG,
              "kernel_eval: HSS_SL_L_2D or HSS_SL_H_2D (the double layer needs normals and weights)");
  HSS_REQUIRE(std::isfinite(kp->h) && kp->h > 0, HSS_ERR_ARG, "kernel_eval: h must be positive");
  if (cplx)
    HSS_REQUIRE(std::isfinite(kp->kh) && kp->kh > 0 && std::isfinite(kp->dr_re) && std::isfinite(kp->dr_im),
                HSS_ERR_ARG, "kernel_eval: kh must be positive and the DR weight finite");
  require_device();
  const size_t np = (size_t)(m + n);
  std::vector<double> hx(np), hy(np), zero(np, 0.0);
  HSS_CUDA(cudaMemcpyAsync(hx.data(), dX1, m * sizeof(double), cudaMemcpyDeviceToHost, s));
  HSS_CUDA(cudaMemcpyAsync(hy.data(), dX1 + m, m * sizeof(double), cudaMemcpyDeviceToHost, s));
  HSS_CUDA(cudaMemcpyAsync(hx.data() + m, dX2, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  HSS_CUDA(cudaMemcpyAsync(hy.data() + m, dX2 + n, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  HSS_CUDA(cudaStreamSynchronize(s));
  // the point table carries the modulations b(x), c(y), evaluated on the host
  PointTable T;
  T.upload(hx, hy, zero, zero, zero, zero, *kp, s);
  std::vector<int> ids(np);
  std::iota(ids.begin(), ids.end(), 0);
  DevBuf<int> dids(np);
  dids.upload(ids, s);
  if (cplx) {
    KgenCP P{dids.p, dids.p + m, (int)m, (int)n, dA, (long long)m};
    DevBuf<KgenCP> dP(1);
    HSS_CUDA(cudaMemcpyAsync(dP.p, &P, sizeof(P), cudaMemcpyHostToDevice, s));
    kgen_complex_batched(dP.p, 1, m * n, view(T), make_helm_dev(*kp), s);
  } else {
    KgenP<double> P{dids.p, dids.p + m, (int)m, (int)n, dA, (int)m, 0};
    DevBuf<KgenP<double>> dP(1);
    HSS_CUDA(cudaMemcpyAsync(dP.p, &P, sizeof(P), cudaMemcpyHostToDevice, s));
    kgen_batched<double>(dP.p, 1, m * n, view(T), make_kernel_dev(*kp), s);
  }
  HSS_CUDA(cudaStreamSynchronize(s));
}

int hss_kernel_eval(const hss_kernel_params* kp, const double* X1, int64_t m, const double* X2, int64_t n,
                    double* A) {
  HSS_TRY
  HSS_REQUIRE(kp && X1 && X2 && A && m > 0 && n > 0, HSS_ERR_ARG, "kernel_eval: bad arguments");
  HSS_REQUIRE(kp->flag == HSS_SL_L_2D || kp->flag == HSS_SL_H_2D, HSS_ERR_ARG,
              "kernel_eval: HSS_SL_L_2D or HSS_SL_H_2D (the double layer needs normals and weights)");
  require_device();
  struct Stream {
    cudaStream_t s = nullptr;
    Stream() { HSS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
    ~Stream() { cudaStreamDestroy(s); }
  } st;
  const size_t cnt = (size_t)m * (size_t)n * (kp->flag == HSS_SL_H_2D ? 2 : 1);
  DevBuf<double> dX1(2 * (size_t)m), dX2(2 * (size_t)n), out(cnt);
  HSS_CUDA(cudaMemcpyAsync(dX1.p, X1, 2 * m * sizeof(double), cudaMemcpyHostToDevice, st.s));
  HSS_CUDA(cudaMemcpyAsync(dX2.p, X2, 2 * n * sizeof(double), cudaMemcpyHostToDevice, st.s));
  kernel_eval_device(kp, dX1.p, m, dX2.p, n, out.p, st.s);
  HSS_CUDA(cudaMemcpyAsync(A, out.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, st.s));
  HSS_CUDA(cudaStreamSynchronize(st.s));
  HSS_CATCH
}

int hss_kernel_eval_device(const hss_kernel_params* kp, const double* d_X1, int64_t m, const double* d_X2, int64_t n,
                           double* d_A, void* stream) {
  HSS_TRY
  kernel_eval_device(kp, d_X1, m, d_X2, n, d_A, as_stream(stream));
  HSS_CATCH
}

// max over columns of ||f - u|| / ||f|| (host vectors, N x nrhs column-major)
static double host_relres(const double* f, const double* u, long long N, int nrhs) {
  double worst = 0.0;
  for (int c = 0; c < nrhs; ++c) {
    long double a = 0.0L, b = 0.0L;
    for (long long i = 0; i < N; ++i) {
      const long double fv = f[i + c * N], rv = fv - (long double)u[i + c * N];
      a += rv * rv;
      b += fv * fv;
    }
    const double rel = (b > 0.0L) ? (double)std::sqrt(a / b) : (double)std::sqrt(a);
    HSS_REQUIRE(std::isfinite(rel), HSS_ERR_NONFINITE, "non-finite kernel residual");
    worst = std::max(worst, rel);
  }
  return worst;
}

// u = K x on the device for the problems of a point table (one KmvP per problem), host x and u
static void kernel_matvec_host(const PointTable& pts, const KernelDev& kd, const std::vector<KmvP>& probs0,
                               long long Nrows, const double* x, double* u, int nrhs, cudaStream_t s) {
  DevBuf<double> dx((size_t)Nrows * nrhs), du((size_t)Nrows * nrhs), part;
  HSS_CUDA(cudaMemcpyAsync(dx.p, x, (size_t)Nrows * nrhs * sizeof(double), cudaMemcpyHostToDevice, s));
  int maxM = 0, maxN = 0;
  for (auto& p : probs0) { maxM = std::max(maxM, p.m); maxN = std::max(maxN, p.n); }
  DevBuf<KmvP> dP(probs0.size());
  for (int c0 = 0; c0 < nrhs; c0 += 8) {
    const int r = std::min(8, nrhs - c0);
    std::vector<KmvP> P = probs0;
    for (auto& p : P) {
      p.q = dx.p + (size_t)c0 * Nrows + p.s0;
      p.ldq = (int)Nrows;
      p.u = du.p + (size_t)c0 * Nrows + p.t0;
      p.ldu = (int)Nrows;
    }
    HSS_CUDA(cudaMemcpyAsync(dP.p, P.data(), P.size() * sizeof(KmvP), cudaMemcpyHostToDevice, s));
    kernel_matvec(dP.p, (int)P.size(), maxM, maxN, r, view(pts), kd, part, s);
    HSS_CUDA(cudaStreamSynchronize(s));
  }
  HSS_CUDA(cudaMemcpyAsync(u, du.p, (size_t)Nrows * nrhs * sizeof(double), cudaMemcpyDeviceToHost, s));
  HSS_CUDA(cudaStreamSynchronize(s));
}

int hss_dr_corrections(double h, double k_re, double k_im, double* corr) {
  HSS_TRY
  HSS_REQUIRE(corr != nullptr, HSS_ERR_ARG, "corr is NULL");
  std::complex<double> c0, c1;
  dr_corrections(h, std::complex<double>(k_re, k_im), c0, c1);
  corr[0] = c0.real(); corr[1] = c0.imag(); corr[2] = c1.real(); corr[3] = c1.imag();
  HSS_CATCH
}

int hss_dr_stencil(double h, double k_re, double k_im, int64_t n, int32_t order, int32_t* count, int64_t* J,
                   double* w, int32_t* stencil) {
  HSS_TRY
  HSS_REQUIRE(count && J && w && stencil && n > 0, HSS_ERR_ARG, "DR_stencil: bad arguments");
  std::vector<long long> j;
  std::vector<std::complex<double>> wv;
  std::vector<int> st;
  dr_stencil(h, std::complex<double>(k_re, k_im), n, order, j, wv, st);
  *count = (int32_t)j.size();
  for (size_t e = 0; e < j.size(); ++e) {
    J[e] = j[e];
    w[2 * e] = wv[e].real();
    w[2 * e + 1] = wv[e].imag();
    for (int r = 0; r < 3; ++r) stencil[3 * e + r] = st[3 * e + r];
  }
  HSS_CATCH
}

int hss_device_count(int* count) {
  HSS_TRY
  HSS_REQUIRE(count != nullptr, HSS_ERR_ARG, "count is NULL");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) { cudaGetLastError(); n = 0; }
  *count = n;
  HSS_CATCH
}

// ---------------------------------------------------------------- HSS1D --
static void hss1d_make(hss1d_matrix** out, int nprob, const long long* N, const double* const* X,
                       const long long* ldx, int leaf, double acc, const hss_kernel_params* kp,
                       const unsigned long long* seeds, MLP* mlp = nullptr, bool sym = false,
                       int id_prec = HSS_PREC_FP64) {
  HSS_REQUIRE(out && X && kp && N && ldx, HSS_ERR_ARG, "NULL argument");
  const bool step_test = (id_prec & HSS_ID_STEP_TEST) != 0;
  id_prec &= ~HSS_ID_STEP_TEST;
  HSS_REQUIRE(id_prec == HSS_PREC_FP64 || id_prec == HSS_PREC_DFLOAT, HSS_ERR_ARG,
              "ID precision: HSS_PREC_FP64 or HSS_PREC_DFLOAT");
  HSS_REQUIRE(!(step_test && mlp), HSS_ERR_ARG, "HSS_ID_STEP_TEST replaces the rank predictor: pass no model");
  require_device();
  *out = nullptr;
  auto* h = new hss1d_matrix{nullptr};
  try {
    h->impl = new HSS1D();
    h->impl->id_df = (id_prec == HSS_PREC_DFLOAT);
    h->impl->id_step_test = step_test;
    h->impl->compress(nprob, N, X, ldx, leaf, acc, *kp, seeds, mlp, sym);
  } catch (...) {
    delete h->impl;
    delete h;
    throw;
  }
  *out = h;
}

int hss1d_compress(hss1d_matrix** out, const double* X, int64_t N, int64_t ldx, int32_t leaf, double acc,
                   const hss_kernel_params* kp, uint64_t seed) {
  HSS_TRY
  const long long n = N, l = ldx;
  const unsigned long long sd = seed;
  hss1d_make(out, 1, &n, &X, &l, leaf, acc, kp, &sd);
  HSS_CATCH
}

int hss1d_compress_fsym(hss1d_matrix** out, const double* X, int64_t N, int64_t ldx, int32_t leaf, double acc,
                        const hss_kernel_params* kp, uint64_t seed) {
  HSS_TRY
  const long long n = N, l = ldx;
  const unsigned long long sd = seed;
  hss1d_make(out, 1, &n, &X, &l, leaf, acc, kp, &sd, nullptr, true);
  HSS_CATCH
}

int hss1d_compress_batch(hss1d_matrix** out, int32_t nprob, const int64_t* N, const double* const* X,
                         const int64_t* ldx, int32_t leaf, double acc, const hss_kernel_params* kp,
                         const uint64_t* seeds) {
  HSS_TRY
  HSS_REQUIRE(nprob >= 1 && N && ldx, HSS_ERR_ARG, "bad batch arguments");
  std::vector<long long> n(N, N + nprob), l(ldx, ldx + nprob);
  std::vector<unsigned long long> sd(nprob, 0ULL);
  if (seeds)
    for (int p = 0; p < nprob; ++p) sd[p] = seeds[p];
  hss1d_make(out, nprob, n.data(), X, l.data(), leaf, acc, kp, sd.data());
  HSS_CATCH
}

int hss1d_compress_batch_learned(hss1d_matrix** out, int32_t nprob, const int64_t* N, const double* const* X,
                                 const int64_t* ldx, int32_t leaf, double acc, const hss_kernel_params* kp,
                                 const uint64_t* seeds, hss_mlp* M) {
  HSS_TRY
  HSS_REQUIRE(nprob >= 1 && N && ldx && M && M->impl, HSS_ERR_ARG, "bad batch arguments");
  std::vector<long long> n(N, N + nprob), l(ldx, ldx + nprob);
  std::vector<unsigned long long> sd(nprob, 0ULL);
  if (seeds)
    for (int p = 0; p < nprob; ++p) sd[p] = seeds[p];
  hss1d_make(out, nprob, n.data(), X, l.data(), leaf, acc, kp, sd.data(), M->impl);
  HSS_CATCH
}

int hss1d_compress_batch_ex(hss1d_matrix** out, int32_t nprob, const int64_t* N, const double* const* X,
                            const int64_t* ldx, int32_t leaf, double acc, const hss_kernel_params* kp,
                            const uint64_t* seeds, hss_mlp* M, int32_t id_precision) {
  HSS_TRY
  HSS_REQUIRE(nprob >= 1 && N && ldx && (!M || M->impl), HSS_ERR_ARG, "bad batch arguments");
  std::vector<long long> n(N, N + nprob), l(ldx, ldx + nprob);
  std::vector<unsigned long long> sd(nprob, 0ULL);
  if (seeds)
    for (int p = 0; p < nprob; ++p) sd[p] = seeds[p];
  hss1d_make(out, nprob, n.data(), X, l.data(), leaf, acc, kp, sd.data(), M ? M->impl : nullptr, false,
             id_precision);
  HSS_CATCH
}

int hss1d_features(const hss1d_matrix* H, float* feat, float* rank_frac) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  const HSS1D* h = H->impl;
  if (feat) std::copy(h->feat.begin(), h->feat.end(), feat);
  if (rank_frac)
    for (int b = 0; b < h->nboxes; ++b) {
      const int n = h->census[4 * b + 2];
      rank_frac[b] = (n > 0) ? (float)h->census[4 * b + 3] / (float)n : 0.f;
    }
  HSS_CATCH
}

int hss1d_phase_times(const hss1d_matrix* H, double* seconds) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && seconds, HSS_ERR_ARG, "NULL argument");
  std::copy(H->impl->phase_s, H->impl->phase_s + HSS1D::NPHASE, seconds);
  HSS_CATCH
}

int hss1d_id_stats(const hss1d_matrix* H, int64_t* qr_steps, int64_t* qr_steps_full, int32_t* reruns) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  if (qr_steps) *qr_steps = H->impl->qr_steps;
  if (qr_steps_full) *qr_steps_full = H->impl->qr_steps_full;
  if (reruns) *reruns = H->impl->reruns;
  HSS_CATCH
}

// --------------------------------------------------------------- MLP --
int hss_mlp_create(hss_mlp** out, int32_t nin, int32_t hidden, uint64_t seed) {
  HSS_TRY
  HSS_REQUIRE(out, HSS_ERR_ARG, "NULL argument");
  require_device();
  *out = nullptr;
  auto* m = new hss_mlp{nullptr};
  try {
    m->impl = new MLP(nin, hidden, seed);
  } catch (...) {
    delete m;
    throw;
  }
  *out = m;
  HSS_CATCH
}

int hss_mlp_nparams(const hss_mlp* M, int32_t* np) {
  HSS_TRY
  HSS_REQUIRE(M && M->impl && np, HSS_ERR_ARG, "NULL argument");
  *np = mlp_nparams(M->impl->nin, M->impl->H);
  HSS_CATCH
}

int hss_mlp_get_params(const hss_mlp* M, float* params) {
  HSS_TRY
  HSS_REQUIRE(M && M->impl && params, HSS_ERR_ARG, "NULL argument");
  MLP* m = M->impl;
  const int np = mlp_nparams(m->nin, m->H);
  HSS_CUDA(cudaMemcpyAsync(params, m->p.p, np * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  HSS_CUDA(cudaStreamSynchronize(m->stream));
  HSS_CATCH
}

int hss_mlp_set_params(hss_mlp* M, const float* params) {
  HSS_TRY
  HSS_REQUIRE(M && M->impl && params, HSS_ERR_ARG, "NULL argument");
  MLP* m = M->impl;
  const int np = mlp_nparams(m->nin, m->H);
  HSS_CUDA(cudaMemcpyAsync(m->p.p, params, np * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  m->m.zero(m->stream);
  m->v.zero(m->stream);
  m->step = 0;
  HSS_CUDA(cudaStreamSynchronize(m->stream));
  HSS_CATCH
}

int hss_mlp_grad(hss_mlp* M, const float* X, const float* t, int32_t B, float* grad, float* loss) {
  HSS_TRY
  HSS_REQUIRE(M && M->impl && X && t && B >= 1, HSS_ERR_ARG, "bad arguments");
  MLP* m = M->impl;
  const int np = mlp_nparams(m->nin, m->H);
  DevBuf<float> dX, dt;
  dX.upload(std::vector<float>(X, X + (size_t)B * m->nin), m->stream);
  dt.upload(std::vector<float>(t, t + B), m->stream);
  const float l = m->grad(dX.p, dt.p, B, 1.f / (float)B, m->stream, true);
  if (grad) {
    HSS_CUDA(cudaMemcpyAsync(grad, m->g.p, np * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    HSS_CUDA(cudaStreamSynchronize(m->stream));
  }
  if (loss) *loss = l;
  HSS_CATCH
}

int hss_mlp_train(hss_mlp* M, const float* X, const float* t, int32_t B, int32_t epochs, int32_t batch, float lr,
                  float* loss) {
  HSS_TRY
  HSS_REQUIRE(M && M->impl && X && t && B >= 1, HSS_ERR_ARG, "bad arguments");
  MLP* m = M->impl;
  DevBuf<float> dX, dt;
  dX.upload(std::vector<float>(X, X + (size_t)B * m->nin), m->stream);
  dt.upload(std::vector<float>(t, t + B), m->stream);
  const float l = m->train(dX.p, dt.p, B, epochs, batch, lr);
  if (loss) *loss = l;
  HSS_CATCH
}

int hss_mlp_predict(hss_mlp* M, const float* X, int32_t B, float* y) {
  HSS_TRY
  HSS_REQUIRE(M && M->impl && X && y && B >= 0, HSS_ERR_ARG, "bad arguments");
  if (B == 0) return HSS_OK;
  MLP* m = M->impl;
  DevBuf<float> dX, dy(B);
  dX.upload(std::vector<float>(X, X + (size_t)B * m->nin), m->stream);
  m->forward(dX.p, dy.p, B, m->stream);
  HSS_CUDA(cudaMemcpyAsync(y, dy.p, B * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  HSS_CUDA(cudaStreamSynchronize(m->stream));
  HSS_CATCH
}

int hss_mlp_destroy(hss_mlp* M) {
  HSS_TRY
  if (M) {
    delete M->impl;
    delete M;
  }
  HSS_CATCH
}

// a complex handle counts unknowns internally (two per point); the interface counts points
static long long pts1(const HSS1D* h, long long v) { return h->cplx ? v / 2 : v; }

int hss1d_forest_info(const hss1d_matrix* H, int32_t* nprob, int64_t* Ntot, int32_t* root, int64_t* pbase) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  const HSS1D* h = H->impl;
  if (nprob) *nprob = h->nprob;
  if (Ntot) *Ntot = pts1(h, h->Ntot);
  for (int p = 0; p < h->nprob; ++p) {
    if (root) root[p] = h->proot[p];
    if (pbase) pbase[p] = pts1(h, h->pbase[p]);
  }
  HSS_CATCH
}

int hss1d_is_complex(const hss1d_matrix* H, int32_t* is_complex) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && is_complex, HSS_ERR_ARG, "NULL argument");
  *is_complex = H->impl->cplx ? 1 : 0;
  HSS_CATCH
}

int hss1d_info(const hss1d_matrix* H, int32_t* nboxes, int32_t* level, int32_t* parent, int32_t* c1, int32_t* c2,
               int32_t* off, int32_t* cnt, int32_t* nskel, int32_t* kskel) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  const HSS1D* h = H->impl;
  if (nboxes) *nboxes = h->nboxes;
  for (int b = 0; b < h->nboxes; ++b) {
    if (level) level[b] = h->level[b];
    if (parent) parent[b] = h->parent[b];
    if (c1) c1[b] = h->c1[b];
    if (c2) c2[b] = h->c2[b];
    if (off) off[b] = (int32_t)pts1(h, h->off[b]);
    if (cnt) cnt[b] = (int32_t)pts1(h, h->cnt[b]);
    if (nskel) nskel[b] = (int32_t)pts1(h, h->nskel[b]);
    if (kskel) kskel[b] = (int32_t)pts1(h, h->kskel[b]);
  }
  HSS_CATCH
}

int hss1d_export_box(const hss1d_matrix* H, int32_t box, int32_t* I_skup, int32_t* I_skdn, int32_t* J_up,
                     int32_t* J_dn, double* T_up, double* T_dn) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  const HSS1D* h = H->impl;
  HSS_REQUIRE(box >= 0 && box < h->nboxes && h->parent[box] >= 0, HSS_ERR_ARG,
              "box out of range (a root has no skeleton)");
  if (h->cplx) {
    // points and complex T (interleaved), de-embedded: T = E(0::2, 0::2) + i E(1::2, 0::2);
    // T_DN is kept conjugated
    const int n = h->nskel[box] / 2, k = h->kskel[box] / 2, k2 = 2 * k;
    for (int t = 0; t < k; ++t) {
      if (I_skup) I_skup[t] = h->I_SKUP[box][2 * t] / 2;
      if (I_skdn) I_skdn[t] = h->I_SKDN[box][2 * t] / 2;
    }
    for (int t = 0; t < n; ++t) {
      if (J_up) J_up[t] = h->J_UP[box][2 * t] / 2;
      if (J_dn) J_dn[t] = h->J_DN[box][2 * t] / 2;
    }
    const size_t tc = (size_t)k2 * (2 * (n - k));
    std::vector<double> E(tc);
    for (int side = 0; side < 2; ++side) {
      double* dst = side ? T_dn : T_up;
      if (!dst || tc == 0) continue;
      const double* src = side ? h->T_DN.p + h->oT[box] : h->T_UP.p + h->oT[box];
      HSS_CUDA(cudaMemcpy(E.data(), src, tc * sizeof(double), cudaMemcpyDeviceToHost));
      for (int c = 0; c < n - k; ++c)
        for (int r = 0; r < k; ++r) {
          const size_t e = 2 * r + (size_t)(2 * c) * k2;
          dst[2 * (r + (size_t)c * k)] = E[e];
          dst[2 * (r + (size_t)c * k) + 1] = side ? -E[e + 1] : E[e + 1];
        }
    }
    return HSS_OK;
  }
  const int n = h->nskel[box], k = h->kskel[box];
  const int nd = h->rn()[box], kd = h->rk()[box];
  if (I_skup) std::memcpy(I_skup, h->I_SKUP[box].data(), k * sizeof(int32_t));
  if (I_skdn)  // rectangular handles: row indices into Xin
    for (int t = 0; t < kd; ++t) I_skdn[t] = h->I_SKDN[box][t] - (h->rect ? (int)h->Ntot : 0);
  if (J_up) std::memcpy(J_up, h->J_UP[box].data(), n * sizeof(int32_t));
  if (J_dn) std::memcpy(J_dn, h->J_DN[box].data(), nd * sizeof(int32_t));
  const size_t tc = (size_t)k * (n - k), tcd = (size_t)kd * (nd - kd);
  if (tc > 0 && T_up)
    HSS_CUDA(cudaMemcpy(T_up, h->T_UP.p + h->oT[box], tc * sizeof(double), cudaMemcpyDeviceToHost));
  if (tcd > 0 && T_dn)
    HSS_CUDA(cudaMemcpy(T_dn, h->T_DN.p + h->roT()[box], tcd * sizeof(double), cudaMemcpyDeviceToHost));
  HSS_CATCH
}

int hss1d_compress_rect(hss1d_matrix** out, const double* Xin, int64_t M, int64_t ldin, const double* Xout,
                        int64_t N, int64_t ldout, int32_t leaf, double acc, const hss_kernel_params* kp,
                        uint64_t seed) {
  HSS_TRY
  HSS_REQUIRE(out && kp, HSS_ERR_ARG, "NULL argument");
  require_device();
  *out = nullptr;
  auto* h = new hss1d_matrix{nullptr};
  try {
    h->impl = new HSS1D();
    h->impl->compress_rect(M, Xin, ldin, N, Xout, ldout, leaf, acc, *kp, seed);
  } catch (...) {
    delete h->impl;
    delete h;
    throw;
  }
  *out = h;
  HSS_CATCH
}

int hss1d_rect_info(const hss1d_matrix* H, int64_t* M, int32_t* off_in, int32_t* cnt_in, int32_t* nskel_in,
                    int32_t* kskel_in) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  const HSS1D* h = H->impl;
  if (M) *M = pts1(h, h->rows());
  for (int b = 0; b < h->nboxes; ++b) {
    if (off_in) off_in[b] = (int32_t)pts1(h, h->roff()[b]);
    if (cnt_in) cnt_in[b] = (int32_t)pts1(h, h->rcnt()[b]);
    if (nskel_in) nskel_in[b] = (int32_t)pts1(h, h->rn()[b]);
    if (kskel_in) kskel_in[b] = (int32_t)pts1(h, h->rk()[b]);
  }
  HSS_CATCH
}

int hss1d_sum(const hss1d_matrix* A, const hss1d_matrix* B, double acc, hss1d_matrix** C) {
  HSS_TRY
  HSS_REQUIRE(A && A->impl && B && B->impl && C, HSS_ERR_ARG, "NULL argument");
  require_device();
  *C = nullptr;
  auto* h = new hss1d_matrix{nullptr};
  try {
    h->impl = new HSS1D();
    h->impl->sum(*A->impl, *B->impl, acc);
  } catch (...) {
    delete h->impl;
    delete h;
    throw;
  }
  *C = h;
  HSS_CATCH
}

int hss1d_recompress(const hss1d_matrix* A, double acc, hss1d_matrix** out) {
  HSS_TRY
  HSS_REQUIRE(A && A->impl && out, HSS_ERR_ARG, "NULL argument");
  require_device();
  *out = nullptr;
  auto* h = new hss1d_matrix{nullptr};
  try {
    h->impl = new HSS1D();
    h->impl->recompress(*A->impl, acc);
  } catch (...) {
    delete h->impl;
    delete h;
    throw;
  }
  *out = h;
  HSS_CATCH
}

int hss1d_compress_lr(hss1d_matrix** out, const double* U, const double* V, int64_t N, int32_t r, int64_t ldu,
                      int64_t ldv, int32_t leaf, double acc, uint64_t seed) {
  HSS_TRY
  HSS_REQUIRE(out, HSS_ERR_ARG, "NULL argument");
  require_device();
  *out = nullptr;
  auto* h = new hss1d_matrix{nullptr};
  try {
    h->impl = new HSS1D();
    h->impl->compress_lr(N, r, U, ldu, V, ldv, leaf, acc, seed);
  } catch (...) {
    delete h->impl;
    delete h;
    throw;
  }
  *out = h;
  HSS_CATCH
}

int hss1d_invert(hss1d_matrix* H) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  H->impl->invert();
  HSS_CATCH
}

static void host_roundtrip1(HSS1D* h, const double* X, double* Y, int nrhs, bool inv) {
  HSS_REQUIRE(X && Y && nrhs >= 1, HSS_ERR_ARG, "bad vector arguments");
  const size_t cnt = (size_t)h->Ntot * nrhs, cnt_out = (size_t)h->rows() * nrhs;
  h->io_in.ensure(cnt);
  h->io_out.ensure(cnt_out);
  HSS_CUDA(cudaMemcpyAsync(h->io_in.p, X, cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  if (inv) h->applyinv_device(h->io_in.p, h->io_out.p, nrhs);
  else h->apply_device(h->io_in.p, h->io_out.p, nrhs);
  HSS_CUDA(cudaMemcpyAsync(Y, h->io_out.p, cnt_out * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  HSS_CUDA(cudaStreamSynchronize(h->stream));
}

int hss1d_apply(hss1d_matrix* H, const double* qq, double* uu, int32_t nrhs) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  host_roundtrip1(H->impl, qq, uu, nrhs, false);
  HSS_CATCH
}

int hss1d_applyinv(hss1d_matrix* H, const double* ff, double* xx, int32_t nrhs) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  HSS_REQUIRE(H->impl->inverted, HSS_ERR_STATE, "hss1d_applyinv before hss1d_invert");
  host_roundtrip1(H->impl, ff, xx, nrhs, true);
  HSS_CATCH
}

int hss1d_applyinv_device(hss1d_matrix* H, const double* d_ff, double* d_xx, int32_t nrhs, void* stream) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && d_ff && d_xx && nrhs >= 1, HSS_ERR_ARG, "bad arguments");
  HSS1D* h = H->impl;
  cudaStream_t s = as_stream(stream);
  cudaEvent_t ev;
  HSS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  if (s) { HSS_CUDA(cudaEventRecord(ev, s)); HSS_CUDA(cudaStreamWaitEvent(h->stream, ev, 0)); }
  h->applyinv_device(d_ff, d_xx, nrhs);
  HSS_CUDA(cudaEventRecord(ev, h->stream));
  if (s) HSS_CUDA(cudaStreamWaitEvent(s, ev, 0));
  else HSS_CUDA(cudaStreamSynchronize(h->stream));
  cudaEventDestroy(ev);
  HSS_CATCH
}

int hss1d_solve(hss1d_matrix* H, const double* f, double* x, int32_t nrhs, double tol, int32_t maxit,
                double* relres, int32_t* iters) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && f && x && nrhs >= 1, HSS_ERR_ARG, "bad arguments");
  HSS1D* h = H->impl;
  const size_t cnt = (size_t)h->Ntot * nrhs;
  h->io_in.ensure(cnt);
  h->io_out.ensure(cnt);
  HSS_CUDA(cudaMemcpyAsync(h->io_in.p, f, cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int it = 0;
  h->solve_device(h->io_in.p, h->io_out.p, nrhs, tol, maxit, relres, &it);
  HSS_CUDA(cudaMemcpyAsync(x, h->io_out.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  HSS_CUDA(cudaStreamSynchronize(h->stream));
  if (iters) *iters = it;
  HSS_CATCH
}

int hss1d_solve_device(hss1d_matrix* H, const double* d_f, double* d_x, int32_t nrhs, double tol, int32_t maxit,
                       double* relres, int32_t* iters, void* stream) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && d_f && d_x && nrhs >= 1, HSS_ERR_ARG, "bad arguments");
  HSS1D* h = H->impl;
  cudaStream_t s = as_stream(stream);
  cudaEvent_t ev;
  HSS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  if (s) { HSS_CUDA(cudaEventRecord(ev, s)); HSS_CUDA(cudaStreamWaitEvent(h->stream, ev, 0)); }
  int it = 0;
  h->solve_device(d_f, d_x, nrhs, tol, maxit, relres, &it);
  HSS_CUDA(cudaEventRecord(ev, h->stream));
  if (s) HSS_CUDA(cudaStreamWaitEvent(s, ev, 0));
  cudaEventDestroy(ev);
  if (iters) *iters = it;
  HSS_CATCH
}

int hss1d_transforminv(hss1d_matrix* H, hss1d_matrix** out) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && out, HSS_ERR_ARG, "NULL argument");
  *out = nullptr;
  auto* k = new hss1d_matrix{nullptr};
  try {
    k->impl = new HSS1D();
    H->impl->transforminv(*k->impl);
  } catch (...) {
    delete k->impl;
    delete k;
    throw;
  }
  *out = k;
  HSS_CATCH
}

int hss1d_transpose(const hss1d_matrix* H, hss1d_matrix** out) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && out, HSS_ERR_ARG, "NULL argument");
  *out = nullptr;
  auto* k = new hss1d_matrix{nullptr};
  try {
    k->impl = new HSS1D();
    H->impl->transpose(*k->impl);
  } catch (...) {
    delete k->impl;
    delete k;
    throw;
  }
  *out = k;
  HSS_CATCH
}

int hss1d_scalarmult(hss1d_matrix* H, double c) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  H->impl->scalarmult(c);
  HSS_CATCH
}

int hss1d_dense_matrix(hss1d_matrix* H, int32_t prob, double* Kd) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  H->impl->dense_matrix(prob, Kd);
  HSS_CATCH
}

int hss1d_apply_submatrix(hss1d_matrix* H, const uint8_t* I_dn, const uint8_t* I_up, const double* qq, int32_t nrhs,
                          double* uu) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && I_dn && I_up && qq && uu && nrhs >= 1, HSS_ERR_ARG, "bad arguments");
  HSS1D* h = H->impl;
  HSS_REQUIRE(!h->rect, HSS_ERR_ARG, "apply_submatrix is defined for square handles only");
  HSS_REQUIRE(!h->cplx, HSS_ERR_ARG, "apply_submatrix of a complex handle is not built (real handles only)");
  const size_t N = (size_t)h->Ntot;
  // K(I_dn, I_up) qq(I_up) = rows I_dn of K (qq with the columns outside I_up zeroed)
  std::vector<double> q(N * nrhs), y(N * nrhs);
  for (int c = 0; c < nrhs; ++c)
    for (size_t i = 0; i < N; ++i) q[i + c * N] = I_up[i] ? qq[i + c * N] : 0.0;
  host_roundtrip1(h, q.data(), y.data(), nrhs, false);
  size_t m = 0;
  for (size_t i = 0; i < N; ++i) m += I_dn[i] ? 1 : 0;
  for (int c = 0; c < nrhs; ++c) {
    size_t r = 0;
    for (size_t i = 0; i < N; ++i)
      if (I_dn[i]) uu[r++ + c * m] = y[i + c * N];
  }
  HSS_CATCH
}

int hss1d_apply_submatrix_boxes(const hss1d_matrix* H, const uint8_t* I_dn, const uint8_t* I_up, uint8_t* Box_dn,
                                uint8_t* Box_up) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && !H->impl->rect, HSS_ERR_ARG, "square handle required");
  HSS_REQUIRE(!H->impl->cplx, HSS_ERR_ARG, "point masks of a complex handle are not built (real handles only)");
  HSS_REQUIRE(H && H->impl && I_dn && I_up && Box_dn && Box_up, HSS_ERR_ARG, "NULL argument");
  const HSS1D* h = H->impl;
  // children have larger ids than their parents: one pass from the leaves up
  for (int b = h->nboxes - 1; b >= 0; --b) {
    bool dn = false, up = false;
    if (h->is_leaf(b)) {
      for (int i = 0; i < h->cnt[b]; ++i) {
        dn = dn || I_dn[h->off[b] + i];
        up = up || I_up[h->off[b] + i];
      }
    } else {
      for (int s : {h->c1[b], h->c2[b]})
        if (s >= 0) { dn = dn || Box_dn[s]; up = up || Box_up[s]; }
    }
    Box_dn[b] = dn ? 1 : 0;
    Box_up[b] = up ? 1 : 0;
  }
  HSS_CATCH
}

int hss1d_set_precision(hss1d_matrix* H, int32_t precision) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  H->impl->set_precision(precision);
  HSS_CATCH
}

int hss1d_destroy(hss1d_matrix* H) {
  HSS_TRY
  if (H) {
    delete H->impl;
    delete H;
  }
  HSS_CATCH
}

// ---------------------------------------------------------------- HSS2D --
int hss2d_build_tree(hss2d_matrix** out, const hss2d_params* p) {
  HSS_TRY
  HSS_REQUIRE(out != nullptr && p != nullptr, HSS_ERR_ARG, "NULL argument");
  HSS_REQUIRE(p->interform == HSS_INTER_DENSE || p->interform == HSS_INTER_LOWRANK, HSS_ERR_ARG,
              "INTERform must be 'dense' or 'lowrank'");
  HSS_REQUIRE(p->k_cut >= 0, HSS_ERR_ARG, "k_cut must be >= 0");
  HSS_REQUIRE(p->transinv == 0 || p->transinv == 1, HSS_ERR_ARG, "transinv must be 0 or 1");
  HSS_REQUIRE(p->transinv == 0 || (p->kp.b_alpha == 0.0 && p->kp.c_alpha == 0.0), HSS_ERR_ARG,
              "translation-invariant mode needs an unmodulated kernel (b = c = 1)");
  HSS_REQUIRE(p->precision == HSS_PREC_FP64 || p->precision == HSS_PREC_MIXED || p->precision == HSS_PREC_DFLOAT ||
                  p->precision == HSS_PREC_DFLOAT_INV || p->precision == HSS_PREC_TC,
              HSS_ERR_ARG, "bad precision");
  require_device();
  *out = nullptr;
  auto* h = new hss2d_matrix{nullptr};
  try {
    h->impl = new HSS2D(*p);
    h->impl->build_tree();
  } catch (...) {
    delete h->impl;
    delete h;
    throw;
  }
  *out = h;
  HSS_CATCH
}

int hss2d_compress(hss2d_matrix* H) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  H->impl->compress();
  HSS_CATCH
}

int hss2d_invert(hss2d_matrix* H) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  H->impl->invert();
  HSS_CATCH
}

static void host_roundtrip(HSS2D* h, const double* X, double* Y, int nrhs, int which, double tol, int maxit,
                           double* relres, int* iters) {
  HSS_REQUIRE(X && Y && nrhs >= 1, HSS_ERR_ARG, "bad vector arguments");
  const size_t cnt = (size_t)h->geo.N * nrhs;
  h->io_in.ensure(cnt);
  h->io_out.ensure(cnt);
  HSS_CUDA(cudaMemcpyAsync(h->io_in.p, X, cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  if (which == 0) h->apply_device(h->io_in.p, h->io_out.p, nrhs, h->stream);
  else if (which == 1) h->applyinv_device(h->io_in.p, h->io_out.p, nrhs, h->stream);
  else h->solve_device(h->io_in.p, h->io_out.p, nrhs, tol, maxit, relres, iters, h->stream);
  HSS_CUDA(cudaMemcpyAsync(Y, h->io_out.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  HSS_CUDA(cudaStreamSynchronize(h->stream));
}

int hss2d_apply(hss2d_matrix* H, const double* X, double* Y, int32_t nrhs) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  host_roundtrip(H->impl, X, Y, nrhs, 0, 0.0, 1, nullptr, nullptr);
  HSS_CATCH
}

int hss2d_apply_device(hss2d_matrix* H, const double* d_X, double* d_Y, int32_t nrhs, void* stream) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && d_X && d_Y, HSS_ERR_ARG, "NULL argument");
  H->impl->apply_device(d_X, d_Y, nrhs, as_stream(stream));
  HSS_CATCH
}

int hss2d_applyinv(hss2d_matrix* H, const double* X, double* Y, int32_t nrhs) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  host_roundtrip(H->impl, X, Y, nrhs, 1, 0.0, 1, nullptr, nullptr);
  HSS_CATCH
}

int hss2d_applyinv_device(hss2d_matrix* H, const double* d_X, double* d_Y, int32_t nrhs, void* stream) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && d_X && d_Y, HSS_ERR_ARG, "NULL argument");
  H->impl->applyinv_device(d_X, d_Y, nrhs, as_stream(stream));
  HSS_CATCH
}

int hss2d_solve(hss2d_matrix* H, const double* f, double* x, int32_t nrhs, double tol, int32_t maxit,
                double* relres, int32_t* iters) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  int it = 0;
  host_roundtrip(H->impl, f, x, nrhs, 2, tol, maxit, relres, &it);
  if (iters) *iters = it;
  HSS_CATCH
}

int hss2d_solve_device(hss2d_matrix* H, const double* d_f, double* d_x, int32_t nrhs, double tol, int32_t maxit,
                       double* relres, int32_t* iters, void* stream) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && d_f && d_x, HSS_ERR_ARG, "NULL argument");
  int it = 0;
  H->impl->solve_device(d_f, d_x, nrhs, tol, maxit, relres, &it, as_stream(stream));
  if (iters) *iters = it;
  HSS_CATCH
}

int hss2d_set_autotune(hss2d_matrix* H, int32_t on) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  H->impl->set_autotune(on != 0);
  HSS_CATCH
}

int hss2d_is_complex(const hss2d_matrix* H, int32_t* is_complex) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && is_complex, HSS_ERR_ARG, "NULL argument");
  *is_complex = H->impl->cplx ? 1 : 0;
  HSS_CATCH
}

int hss2d_info(const hss2d_matrix* H, int32_t* depth, int32_t* nboxes, int64_t* N) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  if (depth) *depth = H->impl->geo.depth;
  if (nboxes) *nboxes = H->impl->geo.nboxes;
  if (N) *N = H->impl->cplx ? H->impl->geo.N / 2 : H->impl->geo.N;
  HSS_CATCH
}

int hss2d_box_sizes(const hss2d_matrix* H, int32_t* n, int32_t* k, int32_t* nproxy) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  const auto& g = H->impl->geo;
  const int u = H->impl->cplx ? 2 : 1;  // complex trees report points, not embedded entries
  for (int lev = 0; lev <= g.depth; ++lev) {
    const auto& L = g.levels[lev];
    for (int i = 0; i < L.nb; ++i) {
      const int b = (1 << lev) - 1 + i;
      if (n) n[b] = L.n / u;
      if (k) k[b] = L.k / u;
      if (nproxy) nproxy[b] = (L.poff[i + 1] - L.poff[i]) / u;
    }
  }
  HSS_CATCH
}

int hss2d_export_box(const hss2d_matrix* H, int32_t box, int32_t* I_src, int32_t* J, double* T_up, double* T_dn) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  HSS2D* h = H->impl;
  HSS_REQUIRE(box >= 0 && box < h->geo.nboxes, HSS_ERR_ARG, "box out of range");
  int lev = 0;
  while (((1 << (lev + 1)) - 1) <= box) ++lev;
  const auto& g = h->geo.levels[lev];
  const int i = box - ((1 << lev) - 1);
  const size_t tcnt = (size_t)g.k * (g.n - g.k);
  if (h->cplx) {
    // points (every other embedded entry) and T as interleaved complex (k x (n - k) points)
    const int nc = g.n / 2, kc = g.k / 2;
    for (int q = 0; q < nc; ++q) {
      if (I_src) I_src[q] = g.Isrc[(size_t)i * g.n + 2 * q] / 2;
      if (J) J[q] = g.J[(size_t)i * g.n + 2 * q] / 2;
    }
    if (lev > 0 && tcnt > 0) {
      auto& d = h->L[lev];
      const size_t fi = h->fo(i);
      std::vector<double> t(tcnt);
      double* outs[2] = {T_up, T_dn};
      const double* srcs[2] = {d.Tup.p, d.Tdn.p};
      for (int w = 0; w < 2; ++w) {
        if (!outs[w]) continue;
        HSS_CUDA(cudaMemcpy(t.data(), srcs[w] + fi * tcnt, tcnt * sizeof(double), cudaMemcpyDeviceToHost));
        // T_dn is held conjugated (its real transpose is then the embedded plain transpose)
        const double sg = (w == 1) ? -1.0 : 1.0;
        for (int c = 0; c < (g.n - g.k) / 2; ++c)
          for (int r = 0; r < kc; ++r) {
            outs[w][2 * (r + (size_t)c * kc)] = t[2 * r + (size_t)(2 * c) * g.k];
            outs[w][2 * (r + (size_t)c * kc) + 1] = sg * t[2 * r + 1 + (size_t)(2 * c) * g.k];
          }
      }
    }
    return HSS_OK;
  }
  if (I_src) std::memcpy(I_src, g.Isrc.data() + (size_t)i * g.n, g.n * sizeof(int32_t));
  if (J) std::memcpy(J, g.J.data() + (size_t)i * g.n, g.n * sizeof(int32_t));
  if (lev > 0 && tcnt > 0) {
    auto& d = h->L[lev];
    const size_t fi = h->fo(i);
    if (T_up) HSS_CUDA(cudaMemcpy(T_up, d.Tup.p + fi * tcnt, tcnt * sizeof(double), cudaMemcpyDeviceToHost));
    if (T_dn) HSS_CUDA(cudaMemcpy(T_dn, d.Tdn.p + fi * tcnt, tcnt * sizeof(double), cudaMemcpyDeviceToHost));
  }
  HSS_CATCH
}

int hss2d_export_inverse(const hss2d_matrix* H, int32_t box, double* FI, double* E) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  HSS2D* h = H->impl;
  HSS_REQUIRE(h->inverted, HSS_ERR_STATE, "export_inverse before invert");
  HSS_REQUIRE(box >= 0 && box < h->geo.nboxes, HSS_ERR_ARG, "box out of range");
  int lev = 0;
  while (((1 << (lev + 1)) - 1) <= box) ++lev;
  const auto& g = h->geo.levels[lev];
  const int i = box - ((1 << lev) - 1);
  auto& d = h->L[lev];
  const size_t fi = h->fo(i);
  auto fetch = [&](int which, size_t cnt, double* dst) {
    if (!dst) return;
    if (h->prm.precision == HSS_PREC_MIXED) {
      std::vector<float> t(cnt);
      HSS_CUDA(cudaMemcpy(t.data(), d.ff[which].p + fi * cnt, cnt * sizeof(float), cudaMemcpyDeviceToHost));
      for (size_t q = 0; q < cnt; ++q) dst[q] = t[q];
    } else {
      HSS_CUDA(cudaMemcpy(dst, d.fd[which].p + fi * cnt, cnt * sizeof(double), cudaMemcpyDeviceToHost));
    }
  };
  if (h->cplx) {
    // the complex blocks (interleaved) out of their real embeddings
    auto fetch_c = [&](int which, int nn, double* dst) {
      if (!dst) return;
      std::vector<double> t((size_t)nn * nn);
      fetch(which, t.size(), t.data());
      for (int c = 0; c < nn / 2; ++c)
        for (int r = 0; r < nn / 2; ++r) {
          dst[2 * (r + (size_t)c * (nn / 2))] = t[2 * r + (size_t)(2 * c) * nn];
          dst[2 * (r + (size_t)c * (nn / 2)) + 1] = t[2 * r + 1 + (size_t)(2 * c) * nn];
        }
    };
    fetch_c(0, g.n, FI);
    if (lev > 0) fetch_c(1, g.k, E);
    return HSS_OK;
  }
  fetch(0, (size_t)g.n * g.n, FI);
  if (lev > 0) fetch(1, (size_t)g.k * g.k, E);
  HSS_CATCH
}

int hss2d_bicgstab(hss2d_matrix* A, hss2d_matrix* M, const double* f, double* x, int32_t nrhs, double tol,
                   int32_t maxit, double* relres, int32_t* iters) {
  HSS_TRY
  HSS_REQUIRE(A && A->impl && f && x, HSS_ERR_ARG, "NULL argument");
  HSS_REQUIRE(nrhs >= 1, HSS_ERR_ARG, "nrhs must be >= 1");
  HSS2D* h = A->impl;
  const size_t cnt = (size_t)h->geo.N * nrhs;
  DevBuf<double> df(cnt), dx(cnt);
  HSS_CUDA(cudaMemcpyAsync(df.p, f, cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int it = 0;
  bicgstab_device(*h, M ? M->impl : nullptr, df.p, dx.p, nrhs, tol, maxit, relres, &it);
  HSS_CUDA(cudaMemcpyAsync(x, dx.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  HSS_CUDA(cudaStreamSynchronize(h->stream));
  if (iters) *iters = it;
  HSS_CATCH
}

int hss2d_gmres(hss2d_matrix* A, hss2d_matrix* M, const double* f, double* x, int32_t nrhs, double tol,
                int32_t restart, int32_t maxit, double* relres, int32_t* iters) {
  HSS_TRY
  HSS_REQUIRE(A && A->impl && f && x, HSS_ERR_ARG, "NULL argument");
  HSS_REQUIRE(nrhs >= 1, HSS_ERR_ARG, "nrhs must be >= 1");
  HSS2D* h = A->impl;
  const size_t cnt = (size_t)h->geo.N * nrhs;
  DevBuf<double> df(cnt), dx(cnt);
  HSS_CUDA(cudaMemcpyAsync(df.p, f, cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int it = 0;
  gmres_device(*h, M ? M->impl : nullptr, df.p, dx.p, nrhs, tol, restart, maxit, relres, &it);
  HSS_CUDA(cudaMemcpyAsync(x, dx.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  HSS_CUDA(cudaStreamSynchronize(h->stream));
  if (iters) *iters = it;
  HSS_CATCH
}

int hss2d_proxy_points(const hss2d_params* p, int32_t box, int32_t n_src, double* xy, int32_t cap, int32_t* count) {
  HSS_TRY
  HSS_REQUIRE(p && xy && count && cap >= 0 && n_src >= 0, HSS_ERR_ARG, "proxy points: bad arguments");
  HSS_REQUIRE(p->Ng > 0 && p->npan > 1 && (p->npan & (p->npan - 1)) == 0, HSS_ERR_ARG,
              "npan must be a power of two >= 2 and Ng > 0");
  const int depth = (int)std::lround(2.0 * (std::log((double)p->npan) / std::log(2.0) - 1.0) + 3.0) - 1;
  HSS_REQUIRE(box >= 0 && box < (1 << (depth + 1)) - 1, HSS_ERR_ARG, "box out of range");
  int lev = 0;
  while (((1 << (lev + 1)) - 1) <= box) ++lev;
  // the box centre by the alternating bisection (x split on even levels, y on odd)
  double cx = 0.0, cy = 0.0;
  int path[32], np = 0;
  for (int b = box; b > 0; b = (b - 1) / 2) path[np++] = b;
  for (int l = 0, q = np - 1; q >= 0; ++l, --q) {
    const double d = 0.5 * std::ldexp(1.0, -(l / 2));
    const bool first = (path[q] % 2) == 1;  // child 2b + 1
    if (l % 2 == 0) cx += first ? -d : d;
    else cy += first ? d : -d;
  }
  std::vector<double> px, py;
  level_proxy(*p, lev, cx, cy, n_src, px, py);
  *count = (int32_t)px.size();
  HSS_REQUIRE((int)px.size() <= cap, HSS_ERR_ARG, "proxy points: more points than cap");
  for (size_t q = 0; q < px.size(); ++q) {
    xy[q] = px[q];
    xy[cap + q] = py[q];
  }
  HSS_CATCH
}

int hss2d_kernel_residual_rows(hss2d_matrix* H, int64_t row0, int64_t nrows, const double* f, const double* x,
                               int32_t nrhs, double* relres) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && f && x && relres && nrhs >= 1, HSS_ERR_ARG, "kernel residual: bad arguments");
  auto* h = H->impl;
  HSS_REQUIRE(h->tree_built, HSS_ERR_STATE, "kernel residual before the tree is built");
  const int u = h->cplx ? 2 : 1;
  const long long N = h->geo.N;
  HSS_REQUIRE(row0 >= 0 && nrows >= 1 && (row0 + nrows) * u <= N, HSS_ERR_ARG, "kernel residual: rows out of range");
  std::vector<double> ufull((size_t)N * nrhs, 0.0);
  kernel_matvec_host(h->pts, h->kdev, {KmvP{(int)(u * row0), (int)(u * nrows), 0, (int)N, nullptr, 0, nullptr, 0}}, N,
                     x, ufull.data(), nrhs, h->stream);
  const long long m = u * nrows;
  std::vector<double> ur((size_t)m * nrhs);
  for (int c = 0; c < nrhs; ++c)
    std::memcpy(ur.data() + (size_t)c * m, ufull.data() + (size_t)c * N + u * row0, m * sizeof(double));
  *relres = host_relres(f, ur.data(), m, nrhs);
  HSS_CATCH
}

int hss2d_phase_times(const hss2d_matrix* H, double* seconds) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && seconds, HSS_ERR_ARG, "NULL argument");
  std::copy(H->impl->phase_s, H->impl->phase_s + 5, seconds);
  HSS_CATCH
}

int hss2d_interp_ranks(const hss2d_matrix* H, int32_t* q_up, int32_t* q_dn) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl, HSS_ERR_ARG, "NULL handle");
  const HSS2D* h = H->impl;
  HSS_REQUIRE(h->tree_built, HSS_ERR_STATE, "tree not built");
  for (int lev = 0; lev <= h->geo.depth; ++lev) {
    const int nb = h->geo.levels[lev].nb, b0 = (1 << lev) - 1;
    const bool lr = lev < (int)h->qrank_up.size() && !h->qrank_up[lev].empty();
    for (int i = 0; i < nb; ++i) {
      const size_t f = h->fo(i);
      if (q_up) q_up[b0 + i] = lr ? h->qrank_up[lev][f] : -1;
      if (q_dn) q_dn[b0 + i] = lr ? h->qrank_dn[lev][f] : -1;
    }
  }
  HSS_CATCH
}

int hss2d_solve_bytes(const hss2d_matrix* H, int64_t* bytes) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && bytes, HSS_ERR_ARG, "NULL argument");
  *bytes = H->impl->solve_bytes();
  HSS_CATCH
}

int hss2d_solve_launches(const hss2d_matrix* H, int32_t nrhs, int32_t* launches) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && launches, HSS_ERR_ARG, "NULL argument");
  *launches = H->impl->solve_launches(nrhs);
  HSS_CATCH
}

int hss2d_destroy(hss2d_matrix* H) {
  HSS_TRY
  if (H) {
    delete H->impl;
    delete H;
  }
  HSS_CATCH
}

// ---------------------------------------------------------------- primitives --
int hss_batched_inverse_device(double* d_A, int32_t n, int32_t batch, int32_t* d_info, void* stream) {
  HSS_TRY
  batched_inverse<double>(d_A, n, batch, d_info, as_stream(stream));
  HSS_CATCH
}

int hss_batched_inverse_noalloc_device(double* d_A, int32_t n, int32_t batch, int32_t* d_info, void* stream) {
  HSS_TRY
  batched_inverse_noalloc(d_A, n, batch, d_info, as_stream(stream));
  HSS_CATCH
}

int hss_batched_inverse_device_f32(float* d_A, int32_t n, int32_t batch, int32_t* d_info, void* stream) {
  HSS_TRY
  batched_inverse<float>(d_A, n, batch, d_info, as_stream(stream));
  HSS_CATCH
}

static void batched_lstsq(double* d_A, int32_t m, int32_t n, int32_t kf, int32_t batch, bool df, void* stream) {
  HSS_REQUIRE(d_A && m > 0 && n > kf && kf > 0 && kf <= m && batch > 0, HSS_ERR_ARG, "bad arguments");
  cudaStream_t s = as_stream(stream);
  const int nr = n - kf;
  DevBuf<double> V((size_t)batch * m * QR_NB), Tf((size_t)batch * QR_NB * QR_NB), diag((size_t)batch * kf);
  DevBuf<double> X((size_t)batch * kf * nr);
  std::vector<QrP<double>> P(batch);
  for (int b = 0; b < batch; ++b)
    P[b] = QrP<double>{d_A + (size_t)b * m * n, m, n, kf, m, V.p + (size_t)b * m * QR_NB,
                       Tf.p + (size_t)b * QR_NB * QR_NB, diag.p + (size_t)b * kf, X.p + (size_t)b * kf * nr, kf};
  DevBuf<QrP<double>> dP(batch);
  HSS_CUDA(cudaMemcpyAsync(dP.p, P.data(), batch * sizeof(QrP<double>), cudaMemcpyHostToDevice, s));
  lstsq_batched<double>(dP.p, batch, m, n, kf, s, df);
  // the solution goes to A(0:kf, kf:n) (leading dimension m)
  for (int b = 0; b < batch; ++b)
    HSS_CUDA(cudaMemcpy2DAsync(d_A + (size_t)b * m * n + (size_t)kf * m, (size_t)m * sizeof(double),
                               X.p + (size_t)b * kf * nr, (size_t)kf * sizeof(double), (size_t)kf * sizeof(double),
                               nr, cudaMemcpyDeviceToDevice, s));
  HSS_CUDA(cudaStreamSynchronize(s));
}

int hss_batched_lstsq_device(double* d_A, int32_t m, int32_t n, int32_t kf, int32_t batch, void* stream) {
  HSS_TRY
  batched_lstsq(d_A, m, n, kf, batch, false, stream);
  HSS_CATCH
}

int hss_batched_lstsq_device_ex(double* d_A, int32_t m, int32_t n, int32_t kf, int32_t batch, int32_t precision,
                                void* stream) {
  HSS_TRY
  HSS_REQUIRE(precision == HSS_PREC_FP64 || precision == HSS_PREC_DFLOAT, HSS_ERR_ARG,
              "least-squares precision must be HSS_PREC_FP64 or HSS_PREC_DFLOAT");
  batched_lstsq(d_A, m, n, kf, batch, precision == HSS_PREC_DFLOAT, stream);
  HSS_CATCH
}

int hss_batched_id_device(const double* d_A, int32_t m, int32_t n, int32_t batch, double acc, uint64_t seed,
                          int32_t force_k, int32_t* d_rank, int32_t* d_perm, double* d_T, void* stream) {
  HSS_TRY
  HSS_REQUIRE(d_A && d_rank && d_perm && d_T && m > 0 && n > 0 && n <= 4096 && batch > 0, HSS_ERR_ARG,
              "bad arguments");
  HSS_REQUIRE(force_k < 0 || force_k <= std::min(m, n), HSS_ERR_RANK, "fixed rank exceeds min(m, n)");
  cudaStream_t s = as_stream(stream);
  DevBuf<double> W((size_t)batch * m * n), SW((size_t)batch * n * n), SV((size_t)batch * n * n);
  DevBuf<double> x((size_t)batch * 2 * n), y((size_t)batch * (m + n));
  std::vector<IdP> P(batch);
  for (int b = 0; b < batch; ++b)
    P[b] = IdP{d_A + (size_t)b * m * n, W.p + (size_t)b * m * n, m, n, d_perm + (size_t)b * n, d_rank + b,
               d_T + (size_t)b * n * n, -1, SW.p + (size_t)b * n * n, SV.p + (size_t)b * n * n,
               x.p + (size_t)b * 2 * n, y.p + (size_t)b * (m + n), b, -1, (unsigned long long)seed, nullptr};
  DevBuf<IdP> dP(batch);
  HSS_CUDA(cudaMemcpyAsync(dP.p, P.data(), batch * sizeof(IdP), cudaMemcpyHostToDevice, s));
  id_adaptive_batched(dP.p, batch, acc, s);
  if (force_k >= 0) {
    for (auto& q : P) q.force_k = force_k;
    HSS_CUDA(cudaMemcpyAsync(dP.p, P.data(), batch * sizeof(IdP), cudaMemcpyHostToDevice, s));
    id_fixed_batched(dP.p, batch, s);
  }
  HSS_CUDA(cudaStreamSynchronize(s));
  HSS_CATCH
}

int hss_batched_gemm_device(const double* d_A, const double* d_B, double* d_C, int32_t M, int32_t N, int32_t K,
                            int32_t batch, void* stream) {
  HSS_TRY
  HSS_REQUIRE(d_A && d_B && d_C && M > 0 && N > 0 && K > 0 && batch > 0, HSS_ERR_ARG, "bad arguments");
  cudaStream_t s = as_stream(stream);
  std::vector<GemmP<double>> P(batch);
  for (int b = 0; b < batch; ++b)
    P[b] = GemmP<double>{d_A + (size_t)b * M * K, d_B + (size_t)b * K * N, d_C + (size_t)b * M * N, M, N, K, M, K, M};
  DevBuf<GemmP<double>> dP(batch);
  HSS_CUDA(cudaMemcpyAsync(dP.p, P.data(), batch * sizeof(GemmP<double>), cudaMemcpyHostToDevice, s));
  if (N <= 8) gemm_skinny<double>(dP.p, batch, M, 1.0, 0.0, s);
  else gemm_batched<double>(dP.p, batch, M, N, false, false, 1.0, 0.0, s);
  HSS_CUDA(cudaStreamSynchronize(s));
  HSS_CATCH
}

int hss_batched_gemv_tc_device(const double* d_A, const double* d_B, double* d_C, int32_t M, int32_t N, int32_t K,
                               int32_t batch, void* stream) {
  HSS_TRY
  HSS_REQUIRE(d_A && d_B && d_C && M > 0 && N >= 1 && N <= TC_NR && K > 0 && batch > 0 && batch <= 65535,
              HSS_ERR_ARG, "tensor-core product: 1..4 columns and a positive size");
  cudaStream_t s = as_stream(stream);
  const size_t pb = tc_packed_bytes(M, K);
  DevBuf<unsigned char> packed(pb * batch);
  DevBuf<int> rexp((size_t)M * batch), err(1);
  err.zero(s);
  std::vector<TcPackP> P(batch);
  std::vector<TcProd> Q(batch);
  for (int b = 0; b < batch; ++b) {
    TcPackP q{};
    q.A[0] = d_A + (size_t)b * M * K;
    q.K[0] = K;
    q.lda[0] = M;
    q.sign[0] = 1.0;
    q.M = M;
    q.out = packed.p + pb * b;
    q.rexp = rexp.p + (size_t)b * M;
    P[b] = q;
    TcProd t{};
    t.A = q.out;
    t.rexp = q.rexp;
    t.B[0] = d_B + (size_t)b * K * N;
    t.K[0] = K;
    t.ldb[0] = K;
    t.C = d_C + (size_t)b * M * N;
    t.ldc = M;
    t.M = M;
    t.r = N;
    Q[b] = t;
  }
  DevBuf<TcPackP> dP(batch);
  HSS_CUDA(cudaMemcpyAsync(dP.p, P.data(), batch * sizeof(TcPackP), cudaMemcpyHostToDevice, s));
  tc_pack(dP.p, batch, M, K, s);
  TcStep st;
  st.build(Q, 1.0, 0.0, err.p, s);
  st.run(s);
  int herr = 0;
  HSS_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  HSS_CUDA(cudaStreamSynchronize(s));
  HSS_REQUIRE(herr == 0, HSS_ERR_CUDA, "tensor-core product: a pipeline wait timed out");
  HSS_CATCH
}

int hss2d_kernel_residual(hss2d_matrix* H, const double* f, const double* x, int32_t nrhs, double* relres) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && f && x && relres && nrhs >= 1, HSS_ERR_ARG, "kernel residual: bad arguments");
  auto* h = H->impl;
  HSS_REQUIRE(h->tree_built, HSS_ERR_STATE, "kernel residual before the tree is built");
  const long long N = h->geo.N;
  std::vector<double> u((size_t)N * nrhs);
  kernel_matvec_host(h->pts, h->kdev, {KmvP{0, (int)N, 0, (int)N, nullptr, 0, nullptr, 0}}, N, x, u.data(), nrhs,
                     h->stream);
  *relres = host_relres(f, u.data(), N, nrhs);
  HSS_CATCH
}

int hss1d_kernel_residual(hss1d_matrix* H, const double* f, const double* x, int32_t nrhs, double* relres) {
  HSS_TRY
  HSS_REQUIRE(H && H->impl && f && x && relres && nrhs >= 1, HSS_ERR_ARG, "kernel residual: bad arguments");
  auto* h = H->impl;
  HSS_REQUIRE(!h->rect, HSS_ERR_ARG, "kernel residual: square handles only");
  HSS_REQUIRE(h->kernel_op, HSS_ERR_ARG,
              "kernel residual: the handle holds no kernel matrix of its points (a low-rank or algebra result)");
  std::vector<KmvP> P;
  for (size_t p = 0; p < h->pN.size(); ++p)
    P.push_back(KmvP{(int)h->pbase[p], (int)h->pN[p], (int)h->pbase[p], (int)h->pN[p], nullptr, 0, nullptr, 0});
  std::vector<double> u((size_t)h->Ntot * nrhs);
  kernel_matvec_host(h->pts, h->kdev, P, h->Ntot, x, u.data(), nrhs, h->stream);
  *relres = host_relres(f, u.data(), h->Ntot, nrhs);
  HSS_CATCH
}

}  // extern "C"
