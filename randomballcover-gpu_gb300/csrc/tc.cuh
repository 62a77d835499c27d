// tc.cuh -- interface of the tensor-core (precision form) list search.
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace rbc {

// Rows kept per query by the tensor pass: 4k, at least 40 and at most 56 (the
// warp merge holds 64 pairs: the list plus one lane's 8 candidates).
constexpr uint32_t kShortlistMin = 40, kShortlistMax = 56;
// Largest k the tensor pass answers; wider queries take the FP32 search.
constexpr uint32_t kTcMaxK = 32;
inline uint32_t tc_shortlist(uint32_t k) {
  const uint32_t s = 4 * k;
  return s < kShortlistMin ? kShortlistMin : (s > kShortlistMax ? kShortlistMax : s);
}

// Operand format of the tensor form, chosen at build from the data:
//   kTcExact  every centered database value is exact in BF16 (e.g. integer
//             features): one BF16 x BF16 product per pair;
//   kTcSplit  otherwise: FP16 hi + lo halves of power-of-two scaled values,
//             three products per pair, hi.hi into one accumulator and the
//             corrections hi.lo + lo.hi into another; queries are centered on
//             mu (the mean of the representatives) before splitting.
enum TcFormat : uint32_t { kTcExact = 0, kTcSplit = 1 };

// Tensor-core search of list-major work items (the planner's SearchItems):
// item = rows [p0, p0 + np) of one list x up to 128 * mt queries qidx[q0 ..).
struct TcArgs {
  const SearchItem *items;
  const uint32_t *nitems;   // device count written by the planner
  const uint32_t *qidx;     // item query slots -> query index (batch-local)
  const float *Dqr;         // m x nr query-representative distances (exact FP32)
  uint32_t nr;
  uint32_t kb;              // 64-wide K blocks of one operand half (kp / 64)
  uint32_t zero_row;        // an all-zero row of the query operand (gathered for empty slots)
  uint32_t d;
  const float *w;           // per database row: ||x'||^2 + 2 c.x' (x' = x - c, c its representative)
  const uint4 *wh;          // BF16 format: per row the w pieces, 32 bytes (TcBuild::Wh)
  const float *lscale;      // per list: power-of-two scale of the stored halves
  const float *lxmax;       // per list: bound on ||x'||
  const float *lcnorm;      // per list: ||c - mu||
  const float *qscale;      // per query: power-of-two scale of its halves
  const float *qnorm;       // per query: ||q - mu||
  const uint8_t *q_inexact; // per query: some value not exact in the operand format
  uint32_t x_inexact;
  uint32_t format;          // TcFormat
  uint32_t sl;              // shortlist length SL
  float *sl_a;              // [2][m][SL] approx distances, ascending
  uint32_t *sl_row;         // [2][m][SL] database rows (list-major index)
  uint32_t *sl_sel;         // per query: current buffer
  uint32_t *sl_theta;       // per query: largest approx kept once SL rows are held, at most the
                            // cap (float bits)
  const uint32_t *sl_cap;   // per query: cap on sl_theta (float bits; nullptr: none)
  uint32_t *sl_lock;
  uint32_t *emax;           // per query: max error bound over the lists searched (float bits)
  uint64_t m;
  const uint64_t *offsets;  // list starts (for the work counters)
  unsigned long long *stats;  // [0] (query, row) pairs, [1] (query, list) pairs; may be null
  uint32_t *err;
  uint32_t a_stages, b_stages;  // set by launch_tc_search from the shared-memory budget
  uint32_t stage_words;         // set by launch_tc_search: words of one merge staging area (0: none)
  uint32_t stage_lanes;         // set by launch_tc_search: lanes of an epilogue warp with a staging
                                // area (32, or 16: the warp merges in two rounds)
  // keep_k != 0 (launches with one query tile, k <= the per-thread buffer):
  // each thread keeps its query's best buffer-full of candidates of an item
  // and merges them once at the item's end; every row it leaves out has
  // approx at least the buffer's last value then, recorded in drop[q]
  // (float bits, atomic min; 0x7F7F7F7F when nothing was left out)
  uint32_t keep_k;
  uint32_t *drop;
  // profiling (RBC_TC_TRACE set): per CTA kTcTraceWords clock64 counters of
  // where each role's cycles went; null otherwise
  unsigned long long *trace;
};
constexpr uint32_t kTcTraceWords = 16;
// CTA 0 also logs a window of kTcTraceEvents accumulator blocks from block
// kTcTraceFirst on: per block the clocks of [0] its MMAs' issue start, [1]
// their commit, [2] the epilogue seeing it full, [3] its release, and per B
// tile [4] the start and [5] the end of the MMA warp's wait for it (after
// the grid's counters)
constexpr uint32_t kTcTraceEvents = 128, kTcTraceFirst = 2000;

struct RerankArgs {
  const float *X;        // FP32 database rows (list-major), stride ld
  const uint32_t *pid;   // row -> original id
  const float *Q;        // FP32 query rows, stride ld
  uint32_t ld, dp, k, sl;
  uint64_t m;
  const float *sl_a;
  const uint32_t *sl_row;
  const uint32_t *sl_sel;
  const uint32_t *emax;
  const uint32_t *sl_cap; // per query: the cap on the shortlist threshold (nullptr: none)
  const uint32_t *drop;   // per query: bound on the approx of rows the search left out of
                          // candidate buffers (float bits; nullptr: none)
  const uint32_t *tplan;  // per query: the threshold the plan pruned with when it was a
                          // prediction (the k-th exact distance must not exceed it)
  uint32_t *tau;         // if set: the k-th exact distance (float bits) -> pruning threshold
  uint32_t *cap_out;     // with tau (or nullptr): the shortlist cap tau (1 + 2^-7) written here
  uint32_t *theta;       //   and the shortlist threshold lowered to it
  uint32_t *ids;         // if set (with dists): results and certificate
  float *dists;
  uint32_t ldo;
  uint32_t *nfail;
  uint32_t *fail;
};

// Upper bound on |approx(q, x) - exact(q, x)| for every row x of list r, where
//   approx = fl(Dqr + fl(alpha D + w)),  alpha D ~ -2 (q - mu).x'  (tensor cores),
//   Dqr ~ ||q - c||^2, w ~ ||x'||^2 + 2 (c - mu).x', x' = x - c,
// (mu = 0 in the exact format) and exact is the reference's sequential FP32
// difference-form distance.  Inputs: Dqr (computed), qn = ||q - mu||,
// X = bound on ||x'||, C = ||c - mu||.  Terms, with u = 2^-24, g = gamma_{d+3}:
//   operand representation   eps_rep |q-mu| |x'|       (BF16 rounding of
//                            inexact operands, or the hi/lo residuals)
//   accumulation             nacc 2^-22 |q-mu| |x'|    (twice the bound of
//                            truncating FP32 accumulation of nacc products;
//                            the split format's correction accumulator holds
//                            terms 2^-10 smaller)
//   centering                2u |q-mu| |x'|            (x', q - mu rounded)
//   ||q-c||^2 and w          g (||q-c||^2 + ||x'||^2 + 2 C |x'|)
//   three final roundings    u (||q-c||^2 + 3 (2|q-mu||x'| + ||x'||^2 + 2C|x'|))
//   the exact distance       g (||q-c|| + |x'|)^2
//   BF16 format only, where w is folded into the product (D = q.x' - w/2,
//   the three BF16 pieces of w added by a last MMA step of 16 terms):
//     the pieces' residual   2^-24 W,  W = ||x'||^2 + 2C|x'| >= |w|
//     that step's rounding   2 * 16 2^-22 (|q-mu||x'| + 0.51 W)
//     pieces underflowing    2^-120 (absolute)
// doubled as a margin.
__host__ __device__ inline float tc_error_bound(float Dqr, float qn, float X, float C, uint32_t q_inexact,
                                                uint32_t x_inexact, uint32_t format, uint32_t d) {
  const float u = 5.9604644775390625e-08f;
  const float g = (d + 3) * u / (1.f - (d + 3) * u);
  float eps, nacc;
  if (format == kTcSplit) {
    // hi = fl16(v), lo = fl16(v - hi): |v - hi - lo| <= 2^-22 |v|; lo.lo omitted <= 2^-22
    eps = 3.f * 2.384185791015625e-07f + d * 5.9604644775390625e-08f;  // + FP16 underflow margin
    nacc = d * 1.01f;
  } else {
    const float b = 1.f / 256.f;
    const float bq = q_inexact ? b : 0.f, bx = x_inexact ? b : 0.f;
    eps = bq + bx + bq * bx;
    nacc = d * (1.f + bq) * (1.f + bx);
  }
  const float qc2 = Dqr * (1.f + g), Q = qn * (1.f + g), Cb = C * (1.f + g);
  const float qx = Q * X;
  const float A = 2.f * (eps + nacc * 2.384185791015625e-07f + 2.f * u) * qx;
  const float B = g * (qc2 + X * X + 2.f * Cb * X);
  const float R = u * (qc2 + 3.f * (2.f * qx + X * X + 2.f * Cb * X));
  const float F = g * (sqrtf(qc2) + X) * (sqrtf(qc2) + X);
  float Wf = 0.f;
  if (format != kTcSplit) {
    const float W = X * X + 2.f * Cb * X;
    Wf = 5.9604644775390625e-08f * W + 32.f * 2.384185791015625e-07f * (qx + 0.51f * W) + 7.52316384526264e-37f;
  }
  // the float evaluation of this bound errs by far less than the final factor 2 covers
  return 2.f * (A + B + R + F + Wf) * (1.f + 1e-5f);
}

bool tc_supported(uint32_t dp);
uint32_t tc_kp(uint32_t d);
int tc_grid();
uint32_t tc_query_tile(uint32_t format);  // queries per work item (128 x tiles per CTA)
cudaError_t tc_make_map(CUtensorMap *map, const void *ptr, uint64_t rows, uint32_t cols, uint32_t box_rows);

// Build: centered rows of each list (x' = x - c_r), the format check, per-list
// scales and bounds, the half-precision operand rows and w.
struct TcBuild {
  void *Xh;          // n_pad x cols halves (cols = kp, or 2 kp for the split format)
  void *Wh;          // BF16 format: (n_pad + 128) x 16 halves, the w operand of the folded product
  float *w;          // n_pad + 128
  float *lscale, *lxmax, *lcnorm;  // nr each
  float *mu;         // kp: the query centering vector (zero in the exact format)
  uint32_t *iperm;   // n: original id -> list-major row (shortlist rows are list-major)
  uint32_t *rep_rows;  // nr: list-major row of each representative; w = +inf there, so the
                       // tensor search never meets these rows (each query's shortlist
                       // starts with its nearest representatives instead)
  uint32_t format, x_inexact, cols;
};
int tc_build(const float *Xp, const uint32_t *perm, const uint64_t *offsets, const float *R, const float *radius,
             const uint32_t *rep_ids, uint64_t n, uint64_t n_pad, uint32_t nr, uint32_t d, uint32_t ld, uint32_t kp,
             TcBuild *out, uint64_t *bytes, cudaStream_t s);

// Queries: half-precision operand rows (m rows + one zero row), scales, norms, flags.
cudaError_t launch_tc_queries(const float *Q, uint32_t ld, uint64_t m, uint32_t d, uint32_t kp, uint32_t format,
                              const float *mu, void *Qh, float *qscale, float *qnorm, uint8_t *q_inexact,
                              cudaStream_t s);
// Per query: tau = min(tau, predicted) when `predicted` is given, the cap
// tau (1 + 2^-10) on the shortlist threshold, and the threshold lowered to it.
cudaError_t launch_cap(uint32_t *tau, const float *predicted, uint64_t m, uint32_t *cap, uint32_t *theta,
                       cudaStream_t s);
cudaError_t launch_sl_init(float *sl_a, uint32_t *sl_row, uint32_t *sel, uint32_t *theta, uint32_t *lock,
                           uint32_t *emax, uint64_t m, uint32_t sl, cudaStream_t s);
// Each query's sl (<= 64) nearest representatives under (Dqr, representative
// index), as (exact distance, list-major row) pairs sorted by distance: the
// rows the tensor search leaves out (w = +inf), which start every shortlist.
// The first P (<= 32) of them, as (representative, distance), go to
// probe / probed, as the plain form's probe table would hold them.
cudaError_t launch_rep_seed(const float *Dqr, uint64_t m, uint32_t nr, const uint32_t *rep_rows, uint32_t sl,
                            float *seed_a, uint32_t *seed_row, uint32_t P, uint32_t *probe, float *probed,
                            cudaStream_t s);
// Seed the shortlists (after launch_sl_init) with each query's exact top-sl
// over its probed lists (res_d / res_i: kw-wide lists of original ids, from
// the FP32 search; rows become list-major through iperm) merged with its
// nearest representatives (seed_a / seed_row, sl per query), each row once;
// the shortlist threshold becomes the sl-th distance and tau the k-th (float
// bits).
// With cap non-null, also the shortlist cap tau (1 + 2^-7) (float bits) and
// the threshold lowered to it.
cudaError_t launch_sl_seed(const float *res_d, const uint32_t *res_i, uint32_t kw, const uint32_t *iperm,
                           const float *seed_a, const uint32_t *seed_row, uint64_t m, uint32_t sl, uint32_t k,
                           float *sl_a, uint32_t *sl_row, uint32_t *theta, uint32_t *tau, uint32_t *cap,
                           cudaStream_t s);
// narrow: one 128-query tile per B tile in the BF16 format as well (items
// planned with query tiles of 128), for item sets whose tiles run sparse --
// the probe rounds; in the split format it selects the probe round's variant
// (16 candidate-buffer entries per lane, which its keep-best mode needs).
cudaError_t launch_tc_search(const CUtensorMap &tmA, const CUtensorMap &tmB, const TcArgs &a, int grid,
                             cudaStream_t s, bool narrow = false);
cudaError_t launch_rerank(int metric, const RerankArgs &a, cudaStream_t s);

// ---------------------------------------------------------------- batched tensor queries (rbc_batch)
// One instance of a batched tensor search: its tensor maps, its arguments
// (stage fields from tc_stage_plan) and its CTA range in the batched grid.
// (CUtensorMap's own alignment keeps every map of a table on the boundary
// TMA needs.)
struct TcBatchEntry {
  CUtensorMap tmA, tmB;
  TcArgs a;
  uint32_t cta0, ctas;
};
// The shared-memory stage plan launch_tc_search takes for a's kb, sl and
// format (narrow: one query tile per B tile): fills a's stage fields and
// returns the dynamic shared-memory bytes (0 when nothing fits).
size_t tc_stage_plan(TcArgs &a, bool narrow);
// Every instance of the table (ascending cta0, one format and width) in one
// launch of total_ctas CTAs, each with smem bytes of dynamic shared memory
// (the largest of the instances' plans).
cudaError_t launch_tc_search_batch(const TcBatchEntry *tab, uint32_t ninst, uint32_t total_ctas, uint32_t format,
                                   bool narrow, size_t smem, cudaStream_t s);
// Everything a tensor query sets up before its probe round, per instance:
// the nearest representatives and the probe table (as launch_rep_seed), the
// operand rows (launch_tc_queries), empty shortlists (launch_sl_init), empty
// kw-wide FP32 lists with open thresholds (launch_init_results), candidate
// drop bounds at 0x7F7F7F7F, and zeroed control words and counters.
struct TcPrepArgs {
  const float *Dqr;
  uint64_t m;
  uint32_t nr, sl, P;
  const uint32_t *rep_rows;
  float *seed_a;
  uint32_t *seed_row, *probe;
  float *probed;
  const float *Qp;
  uint32_t ld, d, kp, format;
  const float *mu;
  uint16_t *Qh;
  float *qscale, *qnorm;
  uint8_t *qinex;
  float *sl_a;
  uint32_t *sl_row, *sl_sel, *sl_theta, *sl_lock, *emax, *drop;
  float *res_d;
  uint32_t *res_i, *tau, *lock;
  uint32_t kw;
  uint32_t *ctl[4];  // 16 words each (nullptr: none)
  unsigned long long *stats;  // 4 counters
};
cudaError_t launch_tc_prep_batch(const TcPrepArgs *tab, uint32_t ninst, uint64_t m_max, cudaStream_t s);
// The arguments of launch_sl_seed, one instance.
struct SlSeedArgs {
  const float *res_d;
  const uint32_t *res_i;
  uint32_t kw;
  const uint32_t *iperm;
  const float *seed_a;
  const uint32_t *seed_row;
  uint64_t m;
  uint32_t sl, k;
  float *sl_a;
  uint32_t *sl_row, *theta, *tau, *cap;
};
cudaError_t launch_sl_seed_batch(const SlSeedArgs *tab, uint32_t ninst, uint64_t m_max, cudaStream_t s);
// launch_rerank over every instance of the table (instances with m = 0 do nothing).
cudaError_t launch_rerank_batch(int metric, const RerankArgs *tab, uint32_t ninst, uint64_t m_max, cudaStream_t s);

}  // namespace rbc
