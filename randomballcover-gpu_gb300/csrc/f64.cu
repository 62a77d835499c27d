// f64.cu -- the double-precision variant: the reference built with
// real = double (defs.h:27-31, readme.txt:134-152), where every distance is
// the sequential double sum of (q-x)^2 or |q-x| terms, each operation rounded
// to double, ties broken by the lower id.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the variant does
// not search in double.  Database and queries are rounded to float, the FP32
// engine (exact RBC, its tensor form, or brute force) returns each query's kq
// nearest rows under the float distance, and those kq rows are reranked with
// the double arithmetic.  A per-query certificate proves that no row outside
// the shortlist can enter the double top k; a query it cannot certify is
// searched in double over the whole database (f64_scan_kernel).
//
// The certificate.  u = 2^-24, tau = 2^-150 (largest rounding error of a
// subnormal float).  For a row x outside the shortlist the float distance f
// is at least f_kq, the shortlist's last float distance.  With t = q - x and
// t~ the engine's float difference of the rounded values,
//   |t~_i - t_i| <= u |t_i| + c_i,   c_i = u (1+u)(|q_i| + |x_i|) + 2 tau (1+u)
// (two conversions and one subtraction; float subtraction and addition are
// exact when the result is subnormal).  The float sum of d non-negative
// rounded terms is at most (1 + g32) times their exact sum, g32 = d u 1.001,
// and a rounded square is at most (1+u) t~^2 + tau.  Hence, squared L2:
//   ||t~|| >= sqrt((f / (1+g32) - d tau) / (1+u)),
//   ||t||  >= (||t~|| - C) / (1+u),  C = u (1+u)(||q|| + max ||x||) + 2 tau (1+u) sqrt(d),
// and for L1 (no squares): sum |t_i| >= (f / (1+g32) - C1) / (1+u) with the
// L1 norms and 2 tau (1+u) d in C1.  The double distance is at least
// S (1 - g64) - d 2^-1074, g64 = (d+3) 2^-53 1.01, for the exact sum S.  If
// that lower bound, taken at f = f_kq and evaluated with every operation
// rounded towards the safe side, is strictly above the k-th reranked double
// distance, every row outside the shortlist ranks after the k-th, ties
// included.  A shortlist that holds every row (n < kq) is certified as is.
//
// Values must be finite and within +-2^56, so that no float distance of
// d <= 512 terms can overflow; rbc_build_f64 rejects other data and the
// brute-force calls search such data in double directly.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "engine.cuh"
#include "rbc_common.cuh"

namespace rbc {

namespace {

#define FCK(expr)                                       \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #expr); \
  } while (0)
#define FTRY(expr)                  \
  do {                              \
    int rc_ = (expr);               \
    if (rc_ != RBC_OK) return rc_;  \
  } while (0)

constexpr double kRangeLimit = 72057594037927936.0;  // 2^56
constexpr uint32_t kMaxSlots = 65535;                // grid.y limit of the scan kernels

// The double build's distVec (utils.cu:183-191 with real = double): the
// __d*_rn intrinsics are never contracted into FMA.
template <int METRIC>
__device__ __forceinline__ double dist64(const double *__restrict__ q, const double *__restrict__ x, uint32_t d) {
  double acc = 0.0;
  for (uint32_t i = 0; i < d; i++) {
    const double t = __dsub_rn(q[i], x[i]);
    acc = __dadd_rn(acc, METRIC == RBC_L1 ? fabs(t) : __dmul_rn(t, t));
  }
  return acc;
}

template <int W>
__device__ __forceinline__ double entry64(const double (&ld)[W], uint32_t kth) {
  double v = ld[0];
#pragma unroll
  for (int w = 1; w < W; w++) v = kth >= 32u * w ? ld[w] : v;
  return __shfl_sync(0xffffffffu, v, kth & 31);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One warp per row: the float copy (zero padded to ld32), optionally the
// double copy (zero padded to ld64), the largest row L2 and L1 norms
// (norm_max[0], [1], as double bits), and bit 1 of *flag for a value that is
// not finite or beyond 2^56.
__global__ void f64_prep_kernel(const double *__restrict__ src, uint64_t lds, uint64_t rows, uint32_t d,
                                float *__restrict__ dst32, uint32_t ld32, double *__restrict__ dst64, uint32_t ld64,
                                unsigned long long *norm_max, uint32_t *flag) {
  const uint64_t r = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (r >= rows) return;
  const double *row = src + r * lds;
  double s2 = 0.0, s1 = 0.0;
  bool bad = false;
  const uint32_t w = ld32 > ld64 ? ld32 : ld64;
  for (uint32_t c = lane; c < w; c += 32) {
    const double v = c < d ? row[c] : 0.0;
    if (!(fabs(v) <= kRangeLimit)) bad = true;  // NaN fails the comparison too
    s2 += v * v;
    s1 += fabs(v);
    if (dst32 && c < ld32) dst32[r * ld32 + c] = __double2float_rn(v);
    if (dst64 && c < ld64) dst64[r * ld64 + c] = v;
  }
  s2 = warp_sum(s2);
  s1 = warp_sum(s1);
  bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) {
    if (bad) {
      atomicOr(flag, 1u);
    } else if (norm_max) {
      atomicMax(norm_max, (unsigned long long)__double_as_longlong(sqrt(s2)));
      atomicMax(norm_max + 1, (unsigned long long)__double_as_longlong(s1));
    }
  }
}

// Is the lower bound on the double distance of any row whose float distance
// is at least f strictly above ek (see the file comment)?  qn, xn: upper
// bounds of the query's and the database's largest norms.  Every step is
// rounded towards the safe side, so the bound holds as computed.
template <int METRIC>
__device__ __forceinline__ bool certified(double f, double ek, double qn, double xn, uint32_t d) {
  const double u = 0x1p-24, tau = 0x1p-150, opu = 1 + 0x1p-24;  // all exact in double
  const double dd = (double)d;
  const double opg32 = __dadd_ru(1.0, __dmul_ru(__dmul_ru(dd, u), 1.001));
  const double omg64 = __dsub_rd(1.0, __dmul_ru(__dmul_ru(dd + 3, 0x1p-53), 1.01));
  const double nrm = __dmul_ru(__dmul_ru(u, opu), __dadd_ru(qn, xn));
  double S;
  if (METRIC == RBC_L1) {
    const double C1 = __dadd_ru(nrm, __dmul_ru(2 * tau * opu, dd));
    S = __ddiv_rd(__dsub_rd(__ddiv_rd(f, opg32), C1), opu);
  } else {
    const double C = __dadd_ru(nrm, __dmul_ru(2 * tau * opu, __dsqrt_ru(dd)));
    const double rt2 = __ddiv_rd(__dsub_rd(__ddiv_rd(f, opg32), __dmul_ru(dd, tau)), opu);
    const double r = __ddiv_rd(__dsub_rd(rt2 > 0 ? __dsqrt_rd(rt2) : 0.0, C), opu);
    S = r > 0 ? __dmul_rd(r, r) : 0.0;
  }
  const double lb = __dsub_rd(__dmul_rd(S > 0 ? S : 0.0, omg64), dd * 0x1p-1074);
  return lb > ek;
}

struct RerankArgs64 {
  const double *X;        // double rows by original id, stride ldx
  const double *Q;        // double queries, stride ldq
  const uint32_t *cand_i; // m x kq float shortlist (ids, ascending float distance)
  const float *cand_d;    // its float distances
  const unsigned long long *norm_max;  // database's largest L2 / L1 row norms
  uint64_t ldx, ldq, m;
  uint32_t d, dp, k, kq, ldo;
  uint32_t *ids;          // m x k outputs (stride ldo)
  double *dists;
  uint32_t *nfail, *fail; // queries the certificate leaves open
};

// One warp per query: double distances of the shortlist, sorted under
// (dist, id), the first k written, then the certificate.
template <int METRIC, int W>
__global__ void __launch_bounds__(128) f64_rerank_kernel(const RerankArgs64 a) {
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= a.m) return;
  const double *qr = a.Q + q * a.ldq;
  double s2 = 0.0, s1 = 0.0;
  for (uint32_t c = lane; c < a.d; c += 32) {
    const double v = qr[c];
    s2 += v * v;
    s1 += fabs(v);
  }
  s2 = warp_sum(s2);
  s1 = warp_sum(s1);
  double ld[W];
  uint32_t li[W];
#pragma unroll
  for (int w = 0; w < W; w++) {
    ld[w] = DBL_MAX;
    li[w] = RBC_DUMMY;
  }
  const uint32_t *ci = a.cand_i + q * a.kq;
#pragma unroll
  for (int w = 0; w < W; w++) {
    const uint32_t j = 32 * w + lane;
    uint32_t id = j < a.kq ? ci[j] : RBC_DUMMY;
    double e = DBL_MAX;
    if (id != RBC_DUMMY) e = dist64<METRIC>(qr, a.X + (uint64_t)id * a.ldx, a.d);
    warp_merge_into_w<W>(ld, li, e, id);
  }
#pragma unroll
  for (int w = 0; w < W; w++) {
    const uint32_t j = 32 * w + lane;
    if (j < a.k) {
      if (a.ids) a.ids[q * a.ldo + j] = li[w];
      if (a.dists) a.dists[q * a.ldo + j] = ld[w];
    }
  }
  bool ok = true;
  if (ci[a.kq - 1] != RBC_DUMMY) {
    const double ek = entry64<W>(ld, a.k - 1);
    const double f = (double)a.cand_d[q * a.kq + a.kq - 1];
    // the norms' own sums carry at most (d+1) 2^-53 relative error: inflate
    const double inflate = 1 + 0x1p-36;
    const double qn = __dmul_ru(METRIC == RBC_L1 ? s1 : __dsqrt_ru(s2), inflate);
    const double xn = __dmul_ru(__longlong_as_double((long long)a.norm_max[METRIC == RBC_L1 ? 1 : 0]), inflate);
    ok = certified<METRIC>(f, ek, qn, xn, a.dp);
  }
  if (!ok && lane == 0) a.fail[atomicAdd(a.nfail, 1u)] = (uint32_t)q;
}

struct ScanArgs64 {
  const double *X;
  const double *Q;
  uint64_t ldx, ldq, n, chunk;
  uint32_t d, nchunk, slot0;
  const uint32_t *qrows;  // query of each slot (nullptr: the slot itself)
  double *part_d;         // [slot][chunk][KW] partial lists
  uint32_t *part_i;
  const double *ranges;   // range-count form: counts[q] += #{x : dist < ranges[q]}
  uint32_t *counts;
};

// Double brute force over a chunk of rows for one query: each lane computes
// whole distances; each warp keeps a KW-entry list in registers; the block's
// eight lists are merged into one partial list per (query, chunk).
template <int METRIC, int W>
__global__ void __launch_bounds__(256) f64_scan_kernel(const ScanArgs64 a) {
  constexpr int KW = 32 * W;
  __shared__ double qs[kMaxDim];
  __shared__ double sd[8][KW];
  __shared__ uint32_t si[8][KW];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t slot = a.slot0 + blockIdx.y;
  const uint64_t q = a.qrows ? a.qrows[slot] : slot;
  for (uint32_t c = tid; c < a.d; c += blockDim.x) qs[c] = a.Q[q * a.ldq + c];
  __syncthreads();
  const uint64_t r0 = (uint64_t)blockIdx.x * a.chunk, r1 = r0 + a.chunk < a.n ? r0 + a.chunk : a.n;
  double ld[W];
  uint32_t li[W];
#pragma unroll
  for (int w = 0; w < W; w++) {
    ld[w] = DBL_MAX;
    li[w] = RBC_DUMMY;
  }
  double kd = DBL_MAX;
  uint32_t ki = RBC_DUMMY;
  for (uint64_t base = r0 + 32 * warp; base < r1; base += 256) {
    const uint64_t row = base + lane;
    double e = DBL_MAX;
    uint32_t id = RBC_DUMMY;
    if (row < r1) {
      e = dist64<METRIC>(qs, a.X + row * a.ldx, a.d);
      id = (uint32_t)row;
    }
    if (__any_sync(0xffffffffu, pair_less(e, id, kd, ki))) {
      warp_merge_into_w<W>(ld, li, e, id);
      kd = __shfl_sync(0xffffffffu, ld[W - 1], 31);
      ki = __shfl_sync(0xffffffffu, li[W - 1], 31);
    }
  }
#pragma unroll
  for (int w = 0; w < W; w++) {
    sd[warp][32 * w + lane] = ld[w];
    si[warp][32 * w + lane] = li[w];
  }
  __syncthreads();
  if (warp == 0) {
    for (int o = 1; o < 8; o++) {
      double od[W];
      uint32_t oi[W];
#pragma unroll
      for (int w = 0; w < W; w++) {
        od[w] = sd[o][32 * w + lane];
        oi[w] = si[o][32 * w + lane];
      }
      warp_merge_lists_w<W>(ld, li, od, oi);
    }
    const uint64_t p = ((uint64_t)blockIdx.y * a.nchunk + blockIdx.x) * KW;
#pragma unroll
    for (int w = 0; w < W; w++) {
      a.part_d[p + 32 * w + lane] = ld[w];
      a.part_i[p + 32 * w + lane] = li[w];
    }
  }
}

// One warp per slot: merge the slot's partial lists and write its first k
// pairs to output row qrows[slot] (or slot).
template <int W>
__global__ void f64_final_kernel(const double *__restrict__ part_d, const uint32_t *__restrict__ part_i,
                                 uint32_t nslots, uint32_t slot0, uint32_t nchunk, uint32_t k,
                                 const uint32_t *qrows, uint32_t *ids, double *dists, uint32_t ldo) {
  constexpr int KW = 32 * W;
  const uint64_t s = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= nslots) return;
  double ld[W];
  uint32_t li[W];
  const uint64_t p0 = s * nchunk * KW;
#pragma unroll
  for (int w = 0; w < W; w++) {
    ld[w] = part_d[p0 + 32 * w + lane];
    li[w] = part_i[p0 + 32 * w + lane];
  }
  for (uint32_t c = 1; c < nchunk; c++) {
    double od[W];
    uint32_t oi[W];
#pragma unroll
    for (int w = 0; w < W; w++) {
      od[w] = part_d[p0 + (uint64_t)c * KW + 32 * w + lane];
      oi[w] = part_i[p0 + (uint64_t)c * KW + 32 * w + lane];
    }
    warp_merge_lists_w<W>(ld, li, od, oi);
  }
  const uint64_t row = qrows ? qrows[slot0 + s] : slot0 + s;
#pragma unroll
  for (int w = 0; w < W; w++) {
    const uint32_t j = 32 * w + lane;
    if (j < k) {
      if (ids) ids[row * ldo + j] = li[w];
      if (dists) dists[row * ldo + j] = ld[w];
    }
  }
}

// Range counts in double: counts[q] += #{rows of the chunk with dist < ranges[q]}.
template <int METRIC>
__global__ void __launch_bounds__(256) f64_range_kernel(const ScanArgs64 a) {
  __shared__ double qs[kMaxDim];
  __shared__ uint32_t wsum[8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t q = a.slot0 + blockIdx.y;
  for (uint32_t c = tid; c < a.d; c += blockDim.x) qs[c] = a.Q[q * a.ldq + c];
  __syncthreads();
  const double range = a.ranges[q];
  const uint64_t r0 = (uint64_t)blockIdx.x * a.chunk, r1 = r0 + a.chunk < a.n ? r0 + a.chunk : a.n;
  uint32_t cnt = 0;
  for (uint64_t row = r0 + tid; row < r1; row += blockDim.x) cnt += dist64<METRIC>(qs, a.X + row * a.ldx, a.d) < range;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) wsum[warp] = cnt;
  __syncthreads();
  if (tid == 0) {
    uint32_t t = 0;
    for (int w = 0; w < 8; w++) t += wsum[w];
    if (t) atomicAdd(a.counts + q, t);
  }
}

// D[i][j] = double distance of row i of A and row j of B (16 x 16 threads
// per block, one pair each).
template <int METRIC>
__global__ void f64_dense_kernel(const double *__restrict__ A, uint64_t na, const double *__restrict__ B, uint64_t nb,
                                 uint32_t lda, uint32_t ldb, uint32_t d, double *__restrict__ D, uint64_t ldD) {
  const uint64_t i = blockIdx.y * 16ull + threadIdx.y, j = blockIdx.x * 16ull + threadIdx.x;
  if (i < na && j < nb) D[i * ldD + j] = dist64<METRIC>(A + i * lda, B + j * ldb, d);
}

uint32_t scan_chunks(uint64_t n, uint32_t nslots) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t want = (4ull * sms + nslots - 1) / nslots;
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, (n + 2047) / 2048));
}

template <int METRIC, int W>
cudaError_t launch_scan_w(const ScanArgs64 &a, uint32_t nslots, cudaStream_t s) {
  f64_scan_kernel<METRIC, W><<<dim3(a.nchunk, nslots), 256, 0, s>>>(a);
  return launched();
}

// Double k-NN by brute force for nq queries (rows qrows[i], or 0..nq-1),
// written to ids / dists rows of the same index.
int scan_knn(const double *X, uint64_t ldx, uint64_t n, const double *Q, uint64_t ldq, uint32_t d, uint32_t k,
             int metric, const uint32_t *qrows, uint64_t nq, uint32_t *ids, double *dists, uint32_t ldo,
             cudaStream_t s) {
  if (nq == 0) return RBC_OK;
  const uint32_t kw = list_width_for(k), W = kw / 32;
  const uint32_t group = (uint32_t)std::min<uint64_t>(nq, kMaxSlots);
  const uint32_t nchunk = scan_chunks(n, group);
  DevBuf pd, pi;
  FCK(pd.alloc((uint64_t)group * nchunk * kw * 8, s));
  FCK(pi.alloc((uint64_t)group * nchunk * kw * 4, s));
  ScanArgs64 a{};
  a.X = X;
  a.Q = Q;
  a.ldx = ldx;
  a.ldq = ldq;
  a.n = n;
  a.d = d;
  a.nchunk = nchunk;
  a.chunk = (n + nchunk - 1) / nchunk;
  a.qrows = qrows;
  a.part_d = pd.as<double>();
  a.part_i = pi.as<uint32_t>();
  for (uint64_t s0 = 0; s0 < nq; s0 += group) {
    const uint32_t ns = (uint32_t)std::min<uint64_t>(group, nq - s0);
    a.slot0 = (uint32_t)s0;
    cudaError_t e;
    if (metric == RBC_L1)
      e = W == 1 ? launch_scan_w<RBC_L1, 1>(a, ns, s) : W == 2 ? launch_scan_w<RBC_L1, 2>(a, ns, s)
                                                               : launch_scan_w<RBC_L1, 4>(a, ns, s);
    else
      e = W == 1 ? launch_scan_w<RBC_L2, 1>(a, ns, s) : W == 2 ? launch_scan_w<RBC_L2, 2>(a, ns, s)
                                                               : launch_scan_w<RBC_L2, 4>(a, ns, s);
    FCK(e);
    const unsigned blocks = (unsigned)(((uint64_t)ns * 32 + 127) / 128);
    if (W == 1)
      f64_final_kernel<1><<<blocks, 128, 0, s>>>(a.part_d, a.part_i, ns, a.slot0, nchunk, k, qrows, ids, dists, ldo);
    else if (W == 2)
      f64_final_kernel<2><<<blocks, 128, 0, s>>>(a.part_d, a.part_i, ns, a.slot0, nchunk, k, qrows, ids, dists, ldo);
    else
      f64_final_kernel<4><<<blocks, 128, 0, s>>>(a.part_d, a.part_i, ns, a.slot0, nchunk, k, qrows, ids, dists, ldo);
    FCK(launched());
  }
  return RBC_OK;
}

template <int METRIC, int W>
cudaError_t launch_rerank_w(const RerankArgs64 &a, cudaStream_t s) {
  f64_rerank_kernel<METRIC, W><<<(unsigned)((a.m * 32 + 127) / 128), 128, 0, s>>>(a);
  return launched();
}

cudaError_t launch_rerank64(int metric, const RerankArgs64 &a, cudaStream_t s) {
  const uint32_t W = list_width_for(a.kq) / 32;
  if (metric == RBC_L1)
    return W == 1 ? launch_rerank_w<RBC_L1, 1>(a, s) : W == 2 ? launch_rerank_w<RBC_L1, 2>(a, s)
                                                              : launch_rerank_w<RBC_L1, 4>(a, s);
  return W == 1 ? launch_rerank_w<RBC_L2, 1>(a, s) : W == 2 ? launch_rerank_w<RBC_L2, 2>(a, s)
                                                            : launch_rerank_w<RBC_L2, 4>(a, s);
}

cudaError_t launch_prep(const double *src, uint64_t lds, uint64_t rows, uint32_t d, float *dst32, uint32_t ld32,
                        double *dst64, uint32_t ld64, unsigned long long *norm_max, uint32_t *flag, cudaStream_t s) {
  if (rows == 0) return cudaSuccess;
  f64_prep_kernel<<<(unsigned)((rows * 32 + 255) / 256), 256, 0, s>>>(src, lds, rows, d, dst32, ld32, dst64, ld64,
                                                                      norm_max, flag);
  return launched();
}

// Rerank the float shortlists of m queries in double, then search the
// queries the certificate leaves open in double over the whole database.
// X is the double database by original id (stride ldx); fl_i / fl_d are the
// float engine's kq-wide results.  Returns the number of open queries.
int rerank_and_settle(const double *X, uint64_t ldx, uint64_t n, const double *Q, uint64_t ldq, uint32_t d,
                      uint32_t dp, uint32_t k, uint32_t kq, int metric, const uint32_t *fl_i, const float *fl_d,
                      const unsigned long long *norm_max, uint64_t m, uint32_t *ids, double *dists, uint32_t ldo,
                      uint64_t *nopen, cudaStream_t s) {
  DevBuf ctl, failq;
  FCK(ctl.alloc(16, s));
  FCK(failq.alloc(m * 4, s));
  FCK(cudaMemsetAsync(ctl.p, 0, 16, s));
  RerankArgs64 a{};
  a.X = X;
  a.Q = Q;
  a.cand_i = fl_i;
  a.cand_d = fl_d;
  a.norm_max = norm_max;
  a.ldx = ldx;
  a.ldq = ldq;
  a.m = m;
  a.d = d;
  a.dp = dp;
  a.k = k;
  a.kq = kq;
  a.ldo = ldo;
  a.ids = ids;
  a.dists = dists;
  a.nfail = ctl.as<uint32_t>();
  a.fail = failq.as<uint32_t>();
  FCK(launch_rerank64(metric, a, s));
  uint32_t nf = 0;
  FCK(cudaMemcpyAsync(&nf, ctl.p, 4, cudaMemcpyDeviceToHost, s));
  FCK(cudaStreamSynchronize(s));
  *nopen = nf;
  return scan_knn(X, ldx, n, Q, ldq, d, k, metric, failq.as<uint32_t>(), nf, ids, dists, ldo, s);
}

uint32_t f64_shortlist(uint32_t k) { return std::min<uint32_t>(kMaxListWidth, std::max(2 * k, k + 16)); }

int check_f64_args(uint32_t d, uint32_t ldx, uint32_t ldq, uint32_t k, uint32_t ldo, int metric, const char *what) {
  const std::string w(what);
  if (d == 0) return fail(RBC_ERR_INVALID, w + ": d must be >= 1");
  if (ldx < d || ldq < d) return fail(RBC_ERR_INVALID, w + ": leading dimension smaller than d");
  if (pad4(d) > kMaxDim) return fail(RBC_ERR_UNSUPPORTED, w + ": d larger than " + std::to_string(kMaxDim));
  if (k < 1 || k > (uint32_t)kMaxListWidth) return fail(RBC_ERR_INVALID, w + ": k must be in [1, 128]");
  if (ldo < k) return fail(RBC_ERR_INVALID, w + ": ldo < k");
  if (metric != RBC_L2 && metric != RBC_L1) return fail(RBC_ERR_INVALID, w + ": unknown metric");
  return RBC_OK;
}

}  // namespace

cudaError_t launch_dense_dist64(int metric, const double *A, uint64_t na, const double *B, uint64_t nb, uint32_t ld,
                                uint32_t d, double *D, uint64_t ldD, cudaStream_t s) {
  if (na == 0 || nb == 0) return cudaSuccess;
  for (uint64_t i0 = 0; i0 < na; i0 += 16ull * 65535) {
    const uint64_t rows = std::min<uint64_t>(na - i0, 16ull * 65535);
    const dim3 grid((unsigned)((nb + 15) / 16), (unsigned)((rows + 15) / 16));
    if (metric == RBC_L1)
      f64_dense_kernel<RBC_L1><<<grid, dim3(16, 16), 0, s>>>(A + i0 * ld, rows, B, nb, ld, ld, d, D + i0 * ldD, ldD);
    else
      f64_dense_kernel<RBC_L2><<<grid, dim3(16, 16), 0, s>>>(A + i0 * ld, rows, B, nb, ld, ld, d, D + i0 * ldD, ldD);
    cudaError_t e = launched();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Build from double rows: the FP32 index over the float-rounded rows, plus
// the double rows (original order) and their largest norms for the rerank.
int build_index_f64(const double *dX, uint64_t n, uint32_t d, uint32_t ldx, const rbc_build_params *p,
                    cudaStream_t s, rbc_index **out) {
  if (!out) return fail(RBC_ERR_INVALID, "rbc_build_f64: out is NULL");
  *out = nullptr;
  if (!p) return fail(RBC_ERR_INVALID, "rbc_build_f64: params is NULL");
  if (!dX) return fail(RBC_ERR_INVALID, "rbc_build_f64: X is NULL");
  if (d == 0 || ldx < d) return fail(RBC_ERR_INVALID, "rbc_build_f64: bad d or ldx");
  if (pad4(d) > kMaxDim) return fail(RBC_ERR_UNSUPPORTED, "rbc_build_f64: d larger than 512");
  if (n == 0 || n >= 0xFFFFFFFFull) return fail(RBC_ERR_INVALID, "rbc_build_f64: n must be in [1, 2^32-1)");
  if (p->flags & RBC_BUILD_ONESHOT)
    return fail(RBC_ERR_UNSUPPORTED, "rbc_build_f64: one-shot lists are built from float distances only");
  // the legacy API's layout (kBuildKeepInput): rows of pad16(d) doubles and
  // pad16(n) rows, the padding zero, exposed as its rbcStruct.dx
  const bool legacy = (p->flags & kBuildKeepInput) != 0;
  rbc_build_params pf = *p;
  pf.flags &= ~kBuildKeepInput;
  const uint32_t ld32 = pad16(d), ld64 = legacy ? pad16(d) : (d + 1) / 2 * 2;
  const uint64_t rows64 = legacy ? (n + 15) / 16 * 16 : n;
  DevBuf Xf, ctl;
  double *X64 = nullptr;
  unsigned long long *nm = nullptr;
  FCK(Xf.alloc(n * ld32 * 4, s));
  FCK(ctl.alloc(16, s));
  FCK(cudaMemsetAsync(ctl.p, 0, 16, s));
  FCK(cudaMalloc((void **)&X64, rows64 * ld64 * 8));
  cudaError_t e = rows64 > n ? cudaMemsetAsync(X64 + n * ld64, 0, (rows64 - n) * ld64 * 8, s) : cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc((void **)&nm, 16);
  if (e == cudaSuccess) e = cudaMemsetAsync(nm, 0, 16, s);
  if (e == cudaSuccess) e = launch_prep(dX, ldx, n, d, Xf.as<float>(), ld32, X64, ld64, nm, ctl.as<uint32_t>(), s);
  uint32_t flag = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, ctl.p, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  int rc = e == cudaSuccess ? RBC_OK : cuda_fail(e, "rbc_build_f64: conversion");
  if (rc == RBC_OK && flag)
    rc = fail(RBC_ERR_UNSUPPORTED, "rbc_build_f64: values must be finite and within +-2^56");
  rbc_index *idx = nullptr;
  if (rc == RBC_OK) rc = build_index(Xf.as<float>(), n, d, ld32, &pf, s, &idx);
  if (rc != RBC_OK) {
    cudaFree(X64);
    if (nm) cudaFree(nm);
    return rc;
  }
  idx->X64 = X64;
  idx->ld64 = ld64;
  idx->norm64 = nm;
  idx->flags |= RBC_BUILD_F64;
  idx->device_bytes += rows64 * ld64 * 8 + 16;
  *out = idx;
  return RBC_OK;
}

int query_index_f64(rbc_index *idx, const double *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
                    uint32_t *dIds, double *dDists, uint32_t ldo, cudaStream_t s) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_query_f64: index is NULL");
  if (!(idx->flags & RBC_BUILD_F64)) return fail(RBC_ERR_INVALID, "rbc_query_f64: index was not built by rbc_build_f64");
  FTRY(check_f64_args(idx->d, idx->d, ldq, k, ldo, idx->metric, "rbc_query_f64"));
  if (m == 0) return RBC_OK;
  if (!dQ || (!dIds && !dDists)) return fail(RBC_ERR_INVALID, "rbc_query_f64: NULL buffer");
  if (m >= 0xFFFFFFFFull) return fail(RBC_ERR_INVALID, "rbc_query_f64: m must be below 2^32-1");
  const uint32_t base = mode & 0xFFu;
  if (base != RBC_QUERY_EXACT && base != RBC_QUERY_EXACT_TC)
    return fail(RBC_ERR_UNSUPPORTED, "rbc_query_f64: exact modes only (RBC_QUERY_EXACT, RBC_QUERY_EXACT_TC)");
  const uint32_t kq = f64_shortlist(k);
  const uint32_t ld32 = idx->ld;
  const uint64_t mb = std::min<uint64_t>(m, 1ull << 20);
  DevBuf Qf, fi, fd, ctl;
  FCK(Qf.alloc(mb * ld32 * 4, s));
  FCK(fi.alloc(mb * kq * 4, s));
  FCK(fd.alloc(mb * kq * 4, s));
  FCK(ctl.alloc(16, s));
  uint64_t open_total = 0;
  rbc_query_stats agg{};
  for (uint64_t b0 = 0; b0 < m; b0 += mb) {
    const uint64_t mq = std::min(mb, m - b0);
    const double *Qb = dQ + b0 * ldq;
    uint32_t *ib = dIds ? dIds + b0 * ldo : nullptr;
    double *db = dDists ? dDists + b0 * ldo : nullptr;
    FCK(cudaMemsetAsync(ctl.p, 0, 16, s));
    FCK(launch_prep(Qb, ldq, mq, idx->d, Qf.as<float>(), ld32, nullptr, 0, nullptr, ctl.as<uint32_t>(), s));
    uint32_t flag = 0;
    FCK(cudaMemcpyAsync(&flag, ctl.p, 4, cudaMemcpyDeviceToHost, s));
    FCK(cudaStreamSynchronize(s));
    uint64_t nopen = mq;
    if (flag) {
      // queries outside the float range: searched in double throughout
      FTRY(scan_knn(idx->X64, idx->ld64, idx->n, Qb, ldq, idx->d, k, idx->metric, nullptr, mq, ib, db, ldo, s));
    } else {
      FTRY(query_index(idx, Qf.as<float>(), mq, ld32, kq, mode, fi.as<uint32_t>(), fd.as<float>(), kq, s));
      agg.rep_pairs += idx->stats.rep_pairs;
      agg.lists_probed += idx->stats.lists_probed;
      agg.point_pairs += idx->stats.point_pairs;
      FTRY(rerank_and_settle(idx->X64, idx->ld64, idx->n, Qb, ldq, idx->d, idx->dp, k, kq, idx->metric,
                             fi.as<uint32_t>(), fd.as<float>(), idx->norm64, mq, ib, db, ldo, &nopen, s));
    }
    open_total += nopen;
  }
  FCK(cudaStreamSynchronize(s));
  FCK(cudaGetLastError());
  idx->stats = agg;
  idx->stats.queries = m;
  idx->stats.fallback_queries = open_total;
  return RBC_OK;
}

int brute_knn_f64(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m, uint32_t ldq, uint32_t d,
                  uint32_t k, int metric, uint32_t *dIds, double *dDists, uint32_t ldo, uint64_t *nopen,
                  cudaStream_t s) {
  FTRY(check_f64_args(d, ldx, ldq, k, ldo, metric, "rbc_brute_knn_f64"));
  if (m == 0) return RBC_OK;
  if (!dQ || (!dIds && !dDists) || (n && !dX)) return fail(RBC_ERR_INVALID, "rbc_brute_knn_f64: NULL buffer");
  if (n >= 0xFFFFFFFFull || m >= 0xFFFFFFFFull)
    return fail(RBC_ERR_INVALID, "rbc_brute_knn_f64: n, m must be below 2^32-1");
  *nopen = 0;
  if (n == 0) {  // every neighbour missing
    return scan_knn(dX, ldx, 0, dQ, ldq, d, k, metric, nullptr, m, dIds, dDists, ldo, s);
  }
  const uint32_t ld32 = pad16(d), kq = f64_shortlist(k);
  DevBuf Xf, Qf, fi, fd, ctl;
  FCK(ctl.alloc(32, s));
  FCK(cudaMemsetAsync(ctl.p, 0, 32, s));
  FCK(Xf.alloc(n * ld32 * 4, s));
  FCK(Qf.alloc(m * ld32 * 4, s));
  unsigned long long *nm = reinterpret_cast<unsigned long long *>(ctl.as<unsigned char>() + 16);
  FCK(launch_prep(dX, ldx, n, d, Xf.as<float>(), ld32, nullptr, 0, nm, ctl.as<uint32_t>(), s));
  FCK(launch_prep(dQ, ldq, m, d, Qf.as<float>(), ld32, nullptr, 0, nullptr, ctl.as<uint32_t>(), s));
  uint32_t flag = 0;
  FCK(cudaMemcpyAsync(&flag, ctl.p, 4, cudaMemcpyDeviceToHost, s));
  FCK(cudaStreamSynchronize(s));
  if (flag) {  // data outside the float range: double throughout
    *nopen = m;
    FTRY(scan_knn(dX, ldx, n, dQ, ldq, d, k, metric, nullptr, m, dIds, dDists, ldo, s));
    FCK(cudaStreamSynchronize(s));
    return RBC_OK;
  }
  FCK(fi.alloc(m * kq * 4, s));
  FCK(fd.alloc(m * kq * 4, s));
  FTRY(brute_knn(Xf.as<float>(), n, ld32, Qf.as<float>(), m, ld32, d, kq, metric, fi.as<uint32_t>(), fd.as<float>(),
                 kq, s));
  FTRY(rerank_and_settle(dX, ldx, n, dQ, ldq, d, pad4(d), k, kq, metric, fi.as<uint32_t>(), fd.as<float>(), nm, m,
                         dIds, dDists, ldo, nopen, s));
  FCK(cudaStreamSynchronize(s));
  FCK(cudaGetLastError());
  return RBC_OK;
}

int brute_range_count_f64(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m, uint32_t ldq,
                          uint32_t d, int metric, const double *dRanges, uint32_t *dCounts, cudaStream_t s) {
  FTRY(check_f64_args(d, ldx, ldq, 1, 1, metric, "rbc_brute_range_count_f64"));
  if (m == 0) return RBC_OK;
  if (!dQ || !dRanges || !dCounts || (n && !dX)) return fail(RBC_ERR_INVALID, "rbc_brute_range_count_f64: NULL buffer");
  if (n >= 0xFFFFFFFFull || m >= 0xFFFFFFFFull)
    return fail(RBC_ERR_INVALID, "rbc_brute_range_count_f64: n, m must be below 2^32-1");
  FCK(cudaMemsetAsync(dCounts, 0, m * 4, s));
  if (n) {
    ScanArgs64 a{};
    a.X = dX;
    a.Q = dQ;
    a.ldx = ldx;
    a.ldq = ldq;
    a.n = n;
    a.d = d;
    a.ranges = dRanges;
    a.counts = dCounts;
    for (uint64_t s0 = 0; s0 < m; s0 += kMaxSlots) {
      const uint32_t ns = (uint32_t)std::min<uint64_t>(kMaxSlots, m - s0);
      a.nchunk = scan_chunks(n, ns);
      a.chunk = (n + a.nchunk - 1) / a.nchunk;
      a.slot0 = (uint32_t)s0;
      if (metric == RBC_L1)
        f64_range_kernel<RBC_L1><<<dim3(a.nchunk, ns), 256, 0, s>>>(a);
      else
        f64_range_kernel<RBC_L2><<<dim3(a.nchunk, ns), 256, 0, s>>>(a);
      FCK(launched());
    }
  }
  FCK(cudaStreamSynchronize(s));
  return RBC_OK;
}

}  // namespace rbc

extern "C" {

int rbc_build_f64(const double *dX, uint64_t n, uint32_t d, uint32_t ldx, const rbc_build_params *params,
                  void *stream, rbc_index **out) {
  return rbc::build_index_f64(dX, n, d, ldx, params, (cudaStream_t)stream, out);
}

int rbc_query_f64(rbc_index *index, const double *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
                  uint32_t *dIds, double *dDists, uint32_t ldo, void *stream) {
  return rbc::query_index_f64(index, dQ, m, ldq, k, mode, dIds, dDists, ldo, (cudaStream_t)stream);
}

int rbc_brute_knn_f64(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m, uint32_t ldq,
                      uint32_t d, uint32_t k, int metric, uint32_t *dIds, double *dDists, uint32_t ldo,
                      uint64_t *open_queries, void *stream) {
  uint64_t nopen = 0;
  int rc = rbc::brute_knn_f64(dX, n, ldx, dQ, m, ldq, d, k, metric, dIds, dDists, ldo, &nopen, (cudaStream_t)stream);
  if (open_queries) *open_queries = nopen;
  return rc;
}

int rbc_brute_range_count_f64(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m, uint32_t ldq,
                              uint32_t d, int metric, const double *dRanges, uint32_t *dCounts, void *stream) {
  return rbc::brute_range_count_f64(dX, n, ldx, dQ, m, ldq, d, metric, dRanges, dCounts, (cudaStream_t)stream);
}

}  // extern "C"
