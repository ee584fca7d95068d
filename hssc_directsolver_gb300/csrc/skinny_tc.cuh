// Skinny products on the tensor cores (tcgen05) for the HSS solves.
//
// The solve reads every inverse factor once per right-hand-side batch (4 columns), so it
// is a stream of matrix-times-skinny-block products.  GB300's FP64 pipe is far too slow
// for them and its double-float CUDA-core form is FP32-pipe bound.  Here each static FP64
// factor is cut once, when it is formed, into S bf16 "digit" slices of a fixed-point
// number per row:
//     a = 2^e_r * sum_{i=1..S} alpha_i 256^-i,   alpha_i integers in [-128, 127],
// (the Ozaki splitting of Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59 (2012), with
// fixed-point digits), and the right-hand sides are cut the same way per column inside the
// kernel.  Every digit product is exact in bf16 x bf16 -> fp32, and a sum of at most 240
// of them (|alpha beta| <= 2^14) stays below 2^22, so the tensor-core accumulation in
// FP32 is exact.  The kernel keeps the digit pairs of weight 256^-t, t <= S + 1, adds
// them in 64-bit integers and converts once to FP64: the product carries ~2^-48 of the
// row and column maxima, as the double-float product does, at 2 S bytes per entry.
//
// Packed layout of one product A (M x K, rows padded to 8, K padded to 16): 128-row tiles,
// each split into K steps of 16; block (tile t, step q) holds the S slices one after the
// other, each as (rows_t / 8) groups of two 8 x 8 core matrices (256 bytes): the canonical
// no-swizzle K-major layout of the tensor core's shared-memory operand, so one bulk copy
// moves a block into shared memory unchanged.
#pragma once

#include "common.cuh"

namespace hss {

constexpr int TC_S = 6;          // digit slices per entry (8 bits each)
constexpr int TC_ROWS = 128;     // rows per tile (the MMA's M)
constexpr int TC_KS = 16;        // K per pipeline stage (one bf16 MMA step)
constexpr int TC_KITEM = 240;    // K per work item: |sum of digit products| < 240 * 2^14 < 2^22
constexpr int TC_NR = 4;         // right-hand sides per product
constexpr int TC_STAGES = 7;     // shared-memory pipeline depth (24 KB stages)

// bytes of the packed digit slices of an M x K product
size_t tc_packed_bytes(int M, int K);

// A = [sign_0 A_0, sign_1 A_1, sign_2 A_2] (column-major segments side by side)
struct TcPackP {
  const double* A[3];
  int K[3], lda[3];
  double sign[3];
  int M;
  unsigned char* out;  // tc_packed_bytes(M, K_0 + K_1 + K_2) bytes, 256-byte aligned
  int* rexp;           // M row exponents
};
// pack a batch of products (device descriptors); every entry of `out` is written
void tc_pack(const TcPackP* dP, int batch, int maxM, int maxK, cudaStream_t s);

// C (M x r) = alpha * [A_0 A_1 A_2] [B_0; B_1; B_2] + beta * C with A packed by tc_pack
struct TcProd {
  const unsigned char* A;
  const int* rexp;
  const double* B[3];
  int K[3], ldb[3];
  double* C;
  int ldc, M, r;
  int ksplit;           // K chunks of TC_KITEM columns
  int nparts;           // parts per row tile: runs of consecutive chunks, each summed by one CTA (<= 8)
  long long part_off;   // first entry of this product's part sums (nparts * M * 4 (value, exponent) pairs)
  int* cnt;             // per row tile: parts finished (the last one adds the part sums; reset to 0)
};

// One launch over a list of products: work items (product, tile, K chunk), grouped into
// parts (runs of consecutive chunks of one tile) that the host balances over persistent
// CTAs.  A CTA adds the chunks of a part in 64-bit integers; when a tile has several parts,
// the CTA finishing its last part adds the part sums in a fixed order (no second launch).
struct TcStep {
  DevBuf<TcProd> prods;
  DevBuf<int4> items;     // (product, tile, K chunk, part << 5 | headroom << 2 | last << 1 | first)
  DevBuf<int> cta_off;    // item range of each CTA
  DevBuf<long long> part; // split-K partials: (integer sum, exponent) per row and column
  DevBuf<int> cnt;        // tile counters of the split products
  DevBuf<int> pdone;      // per phase: CTAs finished with it (and a final count that resets them)
  int* err = nullptr;     // device word set by a wait that gave up (owned by the caller)
  int grid = 0, maxM = 0, nprod = 0, nphase = 1;
  double alpha = 1.0, beta = 0.0;
  void build(const std::vector<TcProd>& P, double alpha, double beta, int* d_err, cudaStream_t s);
  // a chain: phase ph + 1 reads what phase ph writes; one cooperative launch runs them all,
  // every CTA waiting (bounded) for the previous phase before it reads its right-hand sides
  void build(const std::vector<std::vector<TcProd>>& phases, double alpha, double beta, int* d_err,
             cudaStream_t s);
  void run(cudaStream_t s) const;
  int launches() const { return grid > 0 ? 1 : 0; }
};

}  // namespace hss
