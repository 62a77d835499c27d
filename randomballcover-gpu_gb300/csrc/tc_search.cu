// tc_search.cu -- the precision form: list search on the 5th-generation
// tensor cores (tcgen05), BF16 operands, FP32 accumulation in tensor memory,
// followed by an exact FP32 rerank with a certified error bound.
//
// For a query q and database row x the engine's exact distance (L2) is the
// reference's sequential float sum of (q_i - x_i)^2 (utils.cu:183-191).  The
// tensor form computes instead
//     approx(q, x) = ||q||^2 + ||x||^2 - 2 q.x
// with q.x from a BF16 x BF16 -> FP32 tcgen05.mma, and keeps for every query
// the SL = 40 rows of smallest approx (a shortlist of 4k for k = 10).  The
// rerank computes the exact distance of each shortlisted row and sorts them by
// (distance, id).  |approx - exact| <= E(q) holds for every row, with E from
// the norms, the dimension and whether the inputs are exact in BF16 (see
// tc_error_bound).  If the shortlist's largest approx minus E is still above
// the k-th exact distance, no row outside the shortlist can be in the top k,
// so the result equals the FP32 oracle's; otherwise the query is recomputed
// by the plain FP32 path.  Either way the ids are bit-exact.
//
// Kernel structure (one persistent CTA per SM, 384 threads):
//   warp 0      TMA producer: the 128-query A tile of each work unit, then
//               128-row B tiles of the unit's row range into a 3-stage ring
//               (128-byte swizzled, K-major), and each B tile's row norms
//               (one 512-byte bulk copy) into a 4-slot ring;
//   warp 1      tcgen05.mma issuer: 128x128xK per B tile into one of four
//               128-column TMEM accumulators; tcgen05.commit frees the smem
//               stage and hands the accumulator to the epilogue;
//   warps 4-11  epilogue, two warpgroups taking alternate tiles: tcgen05.ld
//               of the accumulator row of its query (one TMEM lane per
//               thread), approx via one FMA with the row norm, a running
//               minimum per 32 columns against the query's threshold (one
//               branch per 32 values), sorted insertion into a per-thread
//               shortlist in shared memory; at the end of a unit the
//               shortlist is merged into the query's global shortlist
//               (double-buffered) under a bounded per-query lock.
// All mbarrier waits are bounded (sm100.cuh); a timeout sets the error word.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "kernels.cuh"
#include "sm100.cuh"
#include "tc.cuh"

namespace rbc {

namespace {

using namespace sm100;

constexpr int kBM = 128, kBN = 128, kStages = 3, kBufs = 4, kEpiGroups = 2;
constexpr int kThreads = 128 + 128 * kEpiGroups;
constexpr int kSL = kShortlist, kLST = kShortlist + 1;  // odd stride: no bank conflicts across threads
constexpr uint32_t kTile16K = 16384;                    // 128 rows x 128 bytes (one 64-wide K block)
constexpr uint32_t kLockSpin = 1u << 22;

struct TileSeq {
  const TcUnit *units;
  uint32_t u, nunits, stride;
  uint64_t p, p0, p1;
  __device__ void start(const TcUnit *us, uint32_t first, uint32_t n, uint32_t st) {
    units = us;
    u = first;
    nunits = n;
    stride = st;
    if (u < nunits) load();
  }
  __device__ void load() {
    p0 = units[u].p0;
    p1 = units[u].p1;
    p = p0;
  }
  __device__ bool valid() const { return u < nunits; }
  __device__ void advance() {
    p += kBN;
    if (p >= p1) {
      u += stride;
      if (u < nunits) load();
    }
  }
  __device__ bool first() const { return p == p0; }
  __device__ bool last() const { return p + kBN >= p1; }
};

__device__ __forceinline__ bool row_less(float a, uint32_t ra, float b, uint32_t rb) {
  return a < b || (a == b && ra < rb);
}

// Merge a thread's sorted local shortlist into the query's global one (the
// current buffer is read, the merged list goes to the other buffer, then the
// buffers swap), under the query's lock.
__device__ void publish(const TcArgs &a, uint32_t q, const float *myla, const uint32_t *myli, uint32_t nl) {
  uint32_t spins = 0;
  while (atomicCAS(a.sl_lock + q, 0u, 1u) != 0u) {
    if (++spins > kLockSpin) {
      raise_error(a.err, RBC_ERR_ITER_LIMIT);
      return;
    }
    __nanosleep(64);
  }
  __threadfence();
  const uint32_t sel = __ldcg(a.sl_sel + q);
  const float *ga = a.sl_a + ((uint64_t)sel * a.m_pad + q) * kSL;
  const uint32_t *gi = a.sl_row + ((uint64_t)sel * a.m_pad + q) * kSL;
  float *oa = a.sl_a + ((uint64_t)(sel ^ 1u) * a.m_pad + q) * kSL;
  uint32_t *oi = a.sl_row + ((uint64_t)(sel ^ 1u) * a.m_pad + q) * kSL;
  float cur_a[kSL];
  uint32_t cur_i[kSL];
  uint32_t ng = 0;
#pragma unroll
  for (int t = 0; t < kSL; t++) {
    cur_a[t] = __ldcg(ga + t);
    cur_i[t] = __ldcg(gi + t);
  }
  for (int t = 0; t < kSL; t++) ng += cur_i[t] != RBC_DUMMY;
  uint32_t i = 0, j = 0, t = 0;
  float last = FLT_MAX;
  for (; t < kSL && (i < nl || j < ng); t++) {
    const bool take_local = j >= ng || (i < nl && row_less(myla[i], myli[i], cur_a[j], cur_i[j]));
    if (take_local) {
      oa[t] = last = myla[i];
      oi[t] = myli[i];
      i++;
    } else {
      oa[t] = last = cur_a[j];
      oi[t] = cur_i[j];
      j++;
    }
  }
  // FLT_MAX, not +inf, while the list is short: padded rows (norm +inf)
  // must never pass the filter.
  const float newtheta = t == kSL ? last : FLT_MAX;
  for (; t < kSL; t++) {
    oa[t] = INFINITY;
    oi[t] = RBC_DUMMY;
  }
  a.sl_theta[q] = __float_as_uint(newtheta);
  a.sl_sel[q] = sel ^ 1u;
  __threadfence();
  atomicExch(a.sl_lock + q, 0u);
}

__global__ void __launch_bounds__(kThreads, 1)
    tc_search_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_a_full, bar_a_empty, bar_b_full[kStages], bar_b_empty[kStages],
      bar_t_full[kBufs], bar_t_empty[kBufs], bar_x_full[kBufs];
  __shared__ uint32_t tmem_slot;

  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t kb = a.kblocks;
  unsigned char *sA = base;
  unsigned char *sB = sA + kb * kTile16K;
  float *xs = reinterpret_cast<float *>(sB + kStages * kb * kTile16K);  // kBufs x 128 row norms
  float *la = xs + kBufs * kBN;                                          // per epilogue thread: kLST approx
  uint32_t *li = reinterpret_cast<uint32_t *>(la + kEpiGroups * kBM * kLST);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 1) {
    tmem_alloc(&tmem_slot, 512);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(&bar_a_full, 1);
    mbar_init(&bar_a_empty, 1);
    for (int s = 0; s < kStages; s++) {
      mbar_init(&bar_b_full[s], 1);
      mbar_init(&bar_b_empty[s], 1);
    }
    for (int b = 0; b < kBufs; b++) {
      mbar_init(&bar_t_full[b], 1);
      mbar_init(&bar_t_empty[b], 4);
      mbar_init(&bar_x_full[b], 1);
    }
    fence_barrier_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t bytes_a = kb * kTile16K, bytes_b = kb * kTile16K;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      prefetch_tensormap(&tmA);
      prefetch_tensormap(&tmB);
      uint32_t it = 0, uc = 0;
      bool ok = true;
      for (uint32_t u = blockIdx.x; u < a.nunits && ok; u += gridDim.x, uc++) {
        const TcUnit un = a.units[u];
        if (uc > 0 && !(ok = mbar_wait(&bar_a_empty, (uc - 1) & 1, a.err))) break;
        mbar_expect_tx(&bar_a_full, bytes_a);
        for (uint32_t k = 0; k < kb; k++)
          tma_load_2d(sA + k * kTile16K, &tmA, (int32_t)(k * 64), (int32_t)(un.tile * kBM), &bar_a_full);
        for (uint64_t p = un.p0; p < un.p1; p += kBN, it++) {
          const uint32_t s = it % kStages, use = it / kStages, b = it % kBufs;
          if (use > 0 && !(ok = mbar_wait(&bar_b_empty[s], (use - 1) & 1, a.err))) break;
          mbar_expect_tx(&bar_b_full[s], bytes_b);
          for (uint32_t k = 0; k < kb; k++)
            tma_load_2d(sB + (s * kb + k) * kTile16K, &tmB, (int32_t)(k * 64), (int32_t)p, &bar_b_full[s]);
          // the norm slot b is free once the epilogue released tile it - kBufs
          if (it >= kBufs && !(ok = mbar_wait(&bar_t_empty[b], ((it / kBufs) - 1) & 1, a.err))) break;
          mbar_expect_tx(&bar_x_full[b], kBN * 4);
          bulk_load(xs + b * kBN, a.xn + p, kBN * 4, &bar_x_full[b]);
        }
      }
      // drain: wait (bounded) for the copies still in flight before leaving
      for (uint32_t j = 0; j < kBufs && j < it; j++) {
        const uint32_t t = it - 1 - j;
        if (j < kStages) mbar_wait(&bar_b_full[t % kStages], (t / kStages) & 1, nullptr);
        mbar_wait(&bar_x_full[t % kBufs], (t / kBufs) & 1, nullptr);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(kBM, kBN);
      uint32_t it = 0, uc = 0;
      bool ok = true;
      for (uint32_t u = blockIdx.x; u < a.nunits && ok; u += gridDim.x, uc++) {
        const TcUnit un = a.units[u];
        if (!(ok = mbar_wait(&bar_a_full, uc & 1, a.err))) break;
        for (uint64_t p = un.p0; p < un.p1; p += kBN, it++) {
          const uint32_t s = it % kStages, b = it % kBufs;
          if (!(ok = mbar_wait(&bar_b_full[s], (it / kStages) & 1, a.err))) break;
          if (it >= kBufs && !(ok = mbar_wait(&bar_t_empty[b], ((it / kBufs) - 1) & 1, a.err))) break;
          tc_fence_after();
          const uint32_t d = tmem + b * kBN;
          for (uint32_t k = 0; k < kb; k++) {
            const uint32_t a0 = smem_u32(sA + k * kTile16K);
            const uint32_t b0 = smem_u32(sB + (s * kb + k) * kTile16K);
#pragma unroll
            for (uint32_t kk = 0; kk < 4; kk++)
              mma_bf16(d, sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), idesc, (k | kk) != 0);
          }
          mma_commit(&bar_b_empty[s]);
          mma_commit(&bar_t_full[b]);
        }
        if (ok) mma_commit(&bar_a_empty);
      }
    }
  } else if (warp >= 4) {
    // ------------------------------------------------ epilogue (two warpgroups)
    const uint32_t grp = (warp - 4) >> 2, ew = warp & 3, et = ew * 32 + lane;
    float *myla = la + (grp * kBM + et) * kLST;
    uint32_t *myli = li + (grp * kBM + et) * kLST;
    TileSeq cur;
    cur.start(a.units, blockIdx.x, a.nunits, gridDim.x);
    uint32_t it = 0, nl = 0, q = 0;
    float theta = 0.f;
    bool ok = true;
    for (; cur.valid() && ok; cur.advance(), it++) {
      if (cur.first()) {
        q = a.units[cur.u].tile * kBM + et;
        nl = 0;
        theta = __uint_as_float(__ldcg(a.sl_theta + q));
      }
      if ((it & 1u) == grp) {
        const uint32_t b = it % kBufs;
        if (!(ok = mbar_wait(&bar_t_full[b], (it / kBufs) & 1, a.err))) break;
        if (!(ok = mbar_wait(&bar_x_full[b], (it / kBufs) & 1, a.err))) break;
        tc_fence_after();
        const float *xr = xs + b * kBN;
        const uint32_t taddr = tmem + ((32u * ew) << 16) + b * kBN;
#pragma unroll 1
        for (uint32_t c = 0; c < kBN / 32; c++) {
          uint32_t r[32];
          tmem_ld32(taddr + c * 32, r);
          tmem_wait_ld();
          float v[32];
          float mn = INFINITY;
#pragma unroll
          for (int j4 = 0; j4 < 8; j4++) {
            const float4 x4 = *reinterpret_cast<const float4 *>(xr + c * 32 + 4 * j4);
            v[4 * j4 + 0] = fmaf(-2.f, __uint_as_float(r[4 * j4 + 0]), x4.x);
            v[4 * j4 + 1] = fmaf(-2.f, __uint_as_float(r[4 * j4 + 1]), x4.y);
            v[4 * j4 + 2] = fmaf(-2.f, __uint_as_float(r[4 * j4 + 2]), x4.z);
            v[4 * j4 + 3] = fmaf(-2.f, __uint_as_float(r[4 * j4 + 3]), x4.w);
            mn = fminf(mn, fminf(fminf(v[4 * j4], v[4 * j4 + 1]), fminf(v[4 * j4 + 2], v[4 * j4 + 3])));
          }
          if (mn <= theta) {
#pragma unroll
            for (int e = 0; e < 32; e++) {
              if (!(v[e] <= theta)) continue;
              const uint32_t row = (uint32_t)(cur.p + c * 32 + e);
              // sorted insertion by (approx, row) into the thread's shortlist
              if (nl == kSL && !row_less(v[e], row, myla[kSL - 1], myli[kSL - 1])) continue;
              int pos = nl < kSL ? (int)nl++ : kSL - 1;
              while (pos > 0 && row_less(v[e], row, myla[pos - 1], myli[pos - 1])) {
                myla[pos] = myla[pos - 1];
                myli[pos] = myli[pos - 1];
                pos--;
              }
              myla[pos] = v[e];
              myli[pos] = row;
              if (nl == kSL) theta = fminf(theta, myla[kSL - 1]);
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bar_t_empty[b]);
      }
      if (cur.last() && nl > 0) publish(a, q, myla, myli, nl);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ------------------------------------------------------------------ support kernels
// BF16 rows (K padded to a multiple of 64 with zeros), FP32 squared norms and
// a flag raised if any value is not exactly representable in BF16.  One warp
// per row; rows past `rows` (up to rows_pad) get zero data and norm `pad_norm`.
__global__ void to_bf16_kernel(const float *__restrict__ src, uint32_t ld, uint64_t rows, uint64_t rows_pad,
                               uint32_t d, uint32_t kp, __nv_bfloat16 *__restrict__ dst, float *__restrict__ norm,
                               float pad_norm, uint32_t *__restrict__ inexact, uint32_t *__restrict__ maxnorm_bits) {
  const uint64_t r = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (r >= rows_pad) return;
  float ss = 0.f;
  uint32_t bad = 0;
  for (uint32_t c = lane; c < kp; c += 32) {
    float v = (r < rows && c < d) ? src[r * ld + c] : 0.f;
    __nv_bfloat16 h = __float2bfloat16_rn(v);
    bad |= __bfloat162float(h) != v;
    dst[r * kp + c] = h;
    ss = fmaf(v, v, ss);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if (lane == 0) {
    norm[r] = r < rows ? ss : pad_norm;
    if (r < rows) {
      if (bad && inexact) atomicOr(inexact, 1u);
      if (maxnorm_bits) atomicMax(maxnorm_bits, __float_as_uint(sqrtf(ss)));
    }
  }
}

// Per-query flag for the error bound: 1 if the row is not exact in BF16.
__global__ void row_inexact_kernel(const float *__restrict__ src, uint32_t ld, uint64_t rows, uint32_t d,
                                   uint8_t *__restrict__ flag) {
  const uint64_t r = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (r >= rows) return;
  uint32_t bad = 0;
  for (uint32_t c = lane; c < d; c += 32) {
    float v = src[r * ld + c];
    bad |= __bfloat162float(__float2bfloat16_rn(v)) != v;
  }
  bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) flag[r] = (uint8_t)bad;
}

// Both shortlist buffers empty, buffer 0 current, thresholds open, locks free.
__global__ void sl_init_kernel(float *sl_a, uint32_t *sl_row, uint32_t *sel, uint32_t *theta, uint32_t *lock,
                               uint64_t m) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < 2 * m * kSL) {
    sl_a[i] = INFINITY;
    sl_row[i] = RBC_DUMMY;
  }
  if (i < m) {
    sel[i] = 0;
    theta[i] = __float_as_uint(FLT_MAX);
    lock[i] = 0;
  }
}

// Exact rerank of each query slot's shortlist and the certificate (one warp
// per slot); results and failures are reported under the slot's query index.
template <int METRIC>
__global__ void rerank_kernel(RerankArgs a) {
  const uint64_t sq = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sq >= a.m) return;
  const uint64_t q = a.order ? a.order[sq] : sq;
  const float *qrow = a.Q + sq * a.ld;
  const uint64_t slot = ((uint64_t)a.sl_sel[sq] * a.m_pad + sq) * kSL;
  const float *sa_q = a.sl_a + slot;
  const uint32_t *sr_q = a.sl_row + slot;
  float ld = FLT_MAX, cd = FLT_MAX;
  uint32_t li = RBC_DUMMY, ci = RBC_DUMMY;
  uint32_t valid = 0;
  for (int round = 0; round < 2; round++) {
    const int t = round * 32 + lane;
    float dv = FLT_MAX;
    uint32_t id = RBC_DUMMY;
    if (t < kSL) {
      const uint32_t row = sr_q[t];
      if (row != RBC_DUMMY) {
        const float *xr = a.X + (uint64_t)row * a.ld;
        float acc = 0.f;
        for (uint32_t c = 0; c < a.dp; c += 4) {
          const float4 qv = *reinterpret_cast<const float4 *>(qrow + c);
          const float4 xv = *reinterpret_cast<const float4 *>(xr + c);
          acc = accum<METRIC>(acc, qv.x, xv.x);
          acc = accum<METRIC>(acc, qv.y, xv.y);
          acc = accum<METRIC>(acc, qv.z, xv.z);
          acc = accum<METRIC>(acc, qv.w, xv.w);
        }
        dv = acc;
        id = a.pid[row];
      }
    }
    valid += __popc(__ballot_sync(0xffffffffu, id != RBC_DUMMY));
    if (round == 0) {
      ld = dv;
      li = id;
      warp_sort32(ld, li);
    } else {
      cd = dv;
      ci = id;
      warp_merge_into(ld, li, cd, ci);
    }
  }
  // certificate: every row outside the shortlist has approx >= a_last, so its
  // exact distance is >= a_last + ||q||^2 - E(q) > tau_k when certified.
  const float tau = __shfl_sync(0xffffffffu, ld, a.k - 1);
  bool certified = true;
  if (valid == kSL) {
    const double a_last = (double)sa_q[kSL - 1] + (double)a.qn[sq];
    const double E = tc_error_bound(a.qn[sq], a.maxnorm, a.q_inexact ? a.q_inexact[sq] : 1, a.x_inexact, a.dp);
    certified = a_last - E > (double)tau;
  }
  if (lane < (int)a.k) {
    if (a.ids) a.ids[q * a.ldo + lane] = li;
    if (a.dists) a.dists[q * a.ldo + lane] = ld;
  }
  if (lane == 0 && !certified) {
    uint32_t s = atomicAdd(a.nfail, 1u);
    a.fail[s] = (uint32_t)q;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

}  // namespace

// ------------------------------------------------------------------ host side
bool tc_supported(uint32_t dp) { return dp <= 128; }

uint32_t tc_kp(uint32_t d) { return (d + 63) / 64 * 64; }

size_t tc_smem_bytes(uint32_t kp) {
  const uint32_t kb = kp / 64;
  return 1024 + (size_t)(1 + kStages) * kb * kTile16K + (size_t)kBufs * kBN * 4 +
         (size_t)kEpiGroups * kBM * kLST * 8;
}

cudaError_t tc_make_map(CUtensorMap *map, const void *ptr, uint64_t rows, uint32_t kp, uint32_t box_rows) {
  if (!g_encode) {
    cudaDriverEntryPointQueryResult qr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void **)&g_encode, 12000,
                                                     cudaEnableDefault, &qr);
    if (e != cudaSuccess) return e;
    if (qr != cudaDriverEntryPointSuccess || !g_encode) return cudaErrorNotSupported;
  }
  cuuint64_t dims[2] = {kp, rows};
  cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_to_bf16(const float *src, uint32_t ld, uint64_t rows, uint64_t rows_pad, uint32_t d, uint32_t kp,
                           void *dst, float *norm, float pad_norm, uint32_t *inexact, uint32_t *maxnorm_bits,
                           cudaStream_t s) {
  const uint64_t threads = rows_pad * 32;
  to_bf16_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
      src, ld, rows, rows_pad, d, kp, reinterpret_cast<__nv_bfloat16 *>(dst), norm, pad_norm, inexact, maxnorm_bits);
  return launched();
}

cudaError_t launch_row_inexact(const float *src, uint32_t ld, uint64_t rows, uint32_t d, uint8_t *flag,
                               cudaStream_t s) {
  if (rows == 0) return cudaSuccess;
  const uint64_t threads = rows * 32;
  row_inexact_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(src, ld, rows, d, flag);
  return launched();
}

cudaError_t launch_sl_init(float *sl_a, uint32_t *sl_row, uint32_t *sel, uint32_t *theta, uint32_t *lock,
                           uint64_t m, cudaStream_t s) {
  const uint64_t total = std::max<uint64_t>(2 * m * kSL, 1);
  sl_init_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(sl_a, sl_row, sel, theta, lock, m);
  return launched();
}

int tc_grid() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

cudaError_t launch_tc_search(const CUtensorMap &tmA, const CUtensorMap &tmB, const TcArgs &a, int grid,
                             cudaStream_t s) {
  const size_t smem = tc_smem_bytes(a.kblocks * 64);
  cudaError_t e = cudaFuncSetAttribute(tc_search_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (a.nunits == 0) return cudaSuccess;
  tc_search_kernel<<<grid, kThreads, smem, s>>>(tmA, tmB, a);
  return launched();
}

cudaError_t launch_rerank(int metric, const RerankArgs &a, cudaStream_t s) {
  if (a.m == 0) return cudaSuccess;
  const uint64_t threads = a.m * 32;
  const unsigned grid = (unsigned)((threads + 255) / 256);
  if (metric == RBC_L1)
    rerank_kernel<RBC_L1><<<grid, 256, 0, s>>>(a);
  else
    rerank_kernel<RBC_L2><<<grid, 256, 0, s>>>(a);
  return launched();
}

}  // namespace rbc
