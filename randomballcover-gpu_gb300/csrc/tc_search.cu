// tc_search.cu -- the precision form: list search on the 5th-generation
// tensor cores (tcgen05), half-precision operands, FP32 accumulation in tensor
// memory, followed by an exact FP32 rerank with a certified error bound.
//
// For a query q and a database row x of list r (representative c) the
// engine's exact distance (L2) is the reference's sequential float sum of
// (q_i - x_i)^2 (utils.cu:183-191).  With x' = x - c the identity
//     ||q - x||^2 = ||q - c||^2 + (||x'||^2 + 2 c.x') - 2 q.x'
// splits it into the exact query-representative distance Dqr (already computed
// for the pruning), a per-row constant w = ||x'||^2 + 2 c.x' (build time) and
// one dot product q.x' on the tensor cores.  Centering the database rows on
// their representative keeps |x'| at the scale of the list, so the product's
// error -- proportional to |q| |x'| -- stays far below the gaps between
// neighbour distances.  Operand formats (chosen at build from the data):
//   exact  every x' value is exact in BF16 (e.g. integer features): one
//          BF16 x BF16 product; q in BF16 (exact for integer queries);
//   split  FP16 hi + lo halves of power-of-two scaled values (per list for x',
//          per query for q), three products hi.hi + hi.lo + lo.hi.
// Each query keeps the SL = 40 rows of smallest approx (a shortlist of 4k for
// k = 10).  The rerank computes their exact distances and sorts by
// (distance, id).  |approx - exact| <= E(q) over every row searched, with E
// from tc_error_bound; if the shortlist's largest approx minus E is above the
// k-th exact distance, no other row can be in the top k, so the result equals
// the FP32 oracle's; otherwise the query is recomputed by the plain FP32 path.
//
// Work items are the planner's list-major items: rows [p0, p0 + np) of one
// list against up to 128 MT queries (MT = 2 in the exact format, 1 in split).
// Kernel structure (one persistent CTA per SM, 384 threads):
//   warp 0      TMA producer: the item's query rows gathered from the half-
//               precision query matrix with tile::gather4 (128-byte swizzled,
//               K-major), then 128-row B tiles of the item into a ring;
//   warp 1      tcgen05.mma issuer: per B tile MT accumulators of 128 x 128
//               in tensor memory (four 128-column slots), commits free the
//               B stage and hand the slot to the epilogue;
//   warp 2      stages each B tile's row constants w into shared memory
//               (cp.async; +inf past the item's rows, which masks them);
//   warps 4-11  epilogue, two warpgroups (MT = 2: one per query tile; MT = 1:
//               alternate B tiles): tcgen05.ld of its query row, one FMA per
//               value, a running minimum per 32 columns against the query's
//               threshold, candidates into a small per-thread buffer that is
//               merged into the query's global shortlist (double-buffered,
//               bounded per-query lock) when full and at the end of the item.
// All mbarrier waits are bounded (sm100.cuh); a timeout sets the error word.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

#include "engine.cuh"
#include "sm100.cuh"
#include "tc.cuh"

namespace rbc {

namespace {

using namespace sm100;

constexpr int kBM = 128, kBN = 128, kEpiGroups = 2;
constexpr int kThreads = 128 + 128 * kEpiGroups;
constexpr int kSL = kShortlist;
constexpr int kLocal = 12, kLST = kLocal + 1;  // per-thread candidate buffer (odd stride: no bank conflicts)
constexpr uint32_t kTile16K = 16384;           // 128 rows x 128 bytes (one 64-wide K block of halves)
constexpr uint32_t kLockSpin = 1u << 22;
constexpr uint32_t kMaxA = 2, kMaxB = 4;
constexpr size_t kSmemLimit = 232448;

__device__ __forceinline__ bool row_less(float a, uint32_t ra, float b, uint32_t rb) {
  return a < b || (a == b && ra < rb);
}

// Filter threshold on v = alpha D + w for a query whose shortlist threshold is
// theta: any v above it gives approx = fl(Dqr + v) > theta.
__device__ __forceinline__ float v_threshold(float theta, float dq) {
  const float t = (theta - dq) + 2.4e-7f * (fabsf(theta) + fabsf(dq));
  return fminf(t, FLT_MAX);  // never +inf: masked columns carry v = +inf
}

// Merge a thread's sorted candidates into the query's global shortlist (the
// current buffer is read, the merged list goes to the other buffer, then the
// buffers swap), under the query's lock.  Returns the query's threshold.
__device__ float publish(const TcArgs &a, uint32_t q, const float *myla, const uint32_t *myli, uint32_t nl) {
  uint32_t spins = 0;
  while (atomicCAS(a.sl_lock + q, 0u, 1u) != 0u) {
    if (++spins > kLockSpin) {
      raise_error(a.err, RBC_ERR_ITER_LIMIT);
      return __uint_as_float(__ldcg(a.sl_theta + q));
    }
    __nanosleep(64);
  }
  __threadfence();
  const uint32_t sel = __ldcg(a.sl_sel + q);
  const float *ga = a.sl_a + ((uint64_t)sel * a.m + q) * kSL;
  const uint32_t *gi = a.sl_row + ((uint64_t)sel * a.m + q) * kSL;
  float *oa = a.sl_a + ((uint64_t)(sel ^ 1u) * a.m + q) * kSL;
  uint32_t *oi = a.sl_row + ((uint64_t)(sel ^ 1u) * a.m + q) * kSL;
  uint32_t i = 0, j = 0, t = 0;
  float last = FLT_MAX;
  float ca = __ldcg(ga);
  uint32_t ci = __ldcg(gi);
  for (; t < kSL; t++) {
    const bool have_g = j < kSL && ci != RBC_DUMMY;
    if (i >= nl && !have_g) break;
    const bool take_local = !have_g || (i < nl && row_less(myla[i], myli[i], ca, ci));
    if (take_local) {
      oa[t] = last = myla[i];
      oi[t] = myli[i];
      i++;
    } else {
      oa[t] = last = ca;
      oi[t] = ci;
      j++;
      if (j < kSL) {
        ca = __ldcg(ga + j);
        ci = __ldcg(gi + j);
      }
    }
  }
  // FLT_MAX, not +inf, while the list is short
  const float theta = t == kSL ? last : FLT_MAX;
  for (; t < kSL; t++) {
    oa[t] = INFINITY;
    oi[t] = RBC_DUMMY;
  }
  a.sl_theta[q] = __float_as_uint(theta);
  a.sl_sel[q] = sel ^ 1u;
  __threadfence();
  atomicExch(a.sl_lock + q, 0u);
  return theta;
}

struct Cand {
  uint32_t nl;
  float thv;
};

// Sorted insertion of (dq + v, row) into a thread's candidate buffer; a full
// buffer is first merged into the global shortlist, which tightens the filter.
__device__ __noinline__ Cand insert_candidate(const TcArgs &a, uint32_t q, float *myla, uint32_t *myli, uint32_t nl,
                                              float thv, float dq, float v, uint32_t row) {
  if (nl == kLocal) {
    thv = v_threshold(publish(a, q, myla, myli, nl), dq);
    nl = 0;
    if (!(v <= thv)) return Cand{nl, thv};
  }
  const float av = dq + v;
  int pos = (int)nl++;
  while (pos > 0 && row_less(av, row, myla[pos - 1], myli[pos - 1])) {
    myla[pos] = myla[pos - 1];
    myli[pos] = myli[pos - 1];
    pos--;
  }
  myla[pos] = av;
  myli[pos] = row;
  return Cand{nl, thv};
}

__device__ const float g_inf = INFINITY;

__device__ __forceinline__ void cp_async4(float *smem, const float *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_mbar_arrive(uint64_t *bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int MT, bool SPLIT>
__global__ void __launch_bounds__(kThreads, 1)
    tc_search_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const __grid_constant__ TcArgs a) {
  constexpr uint32_t NSLOT = 4 / MT;  // tensor-memory slots of MT x 128 columns
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_a_full[kMaxA], bar_a_empty[kMaxA], bar_b_full[kMaxB], bar_b_empty[kMaxB],
      bar_t_full[4], bar_t_empty[4], bar_x_full[4];
  __shared__ uint32_t tmem_slot;

  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t kb = a.kb, kbh = SPLIT ? 2 * kb : kb;  // K blocks of a stored row (hi [+ lo])
  const uint32_t AS = a.a_stages, BS = a.b_stages;
  const uint32_t a_tile = kbh * kTile16K, a_stage = MT * a_tile, b_stage = kbh * kTile16K;
  unsigned char *sA = base;
  unsigned char *sB = sA + AS * a_stage;
  float *xs = reinterpret_cast<float *>(sB + BS * b_stage);  // NSLOT x 128 row constants
  float *la = xs + NSLOT * kBN;                                // per epilogue thread: kLST approx
  uint32_t *li = reinterpret_cast<uint32_t *>(la + kEpiGroups * kBM * kLST);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 1) {
    tmem_alloc(&tmem_slot, 512);
    tmem_relinquish();
  }
  if (tid == 0) {
    for (uint32_t s = 0; s < kMaxA; s++) {
      mbar_init(&bar_a_full[s], 1);
      mbar_init(&bar_a_empty[s], 1);
    }
    for (uint32_t s = 0; s < kMaxB; s++) {
      mbar_init(&bar_b_full[s], 1);
      mbar_init(&bar_b_empty[s], 1);
    }
    for (uint32_t b = 0; b < 4; b++) {
      mbar_init(&bar_t_full[b], 1);
      mbar_init(&bar_t_empty[b], MT == 2 ? 8 : 4);
      mbar_init(&bar_x_full[b], 32);
    }
    fence_barrier_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t nitems = *a.nitems;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      prefetch_tensormap(&tmA);
      prefetch_tensormap(&tmB);
    }
    uint32_t ai = 0, bi = 0;
    unsigned long long pairs = 0, lists = 0;
    bool ok = true;
    for (uint32_t it = blockIdx.x; it < nitems && ok; it += gridDim.x, ai++) {
      const SearchItem item = a.items[it];
      const uint32_t sa = ai % AS;
      if (ai >= AS) ok = mbar_wait(&bar_a_empty[sa], ((ai / AS) - 1) & 1, a.err);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      if (lane == 0) mbar_expect_tx(&bar_a_full[sa], a_stage);
      __syncwarp();
      unsigned char *dA = sA + sa * a_stage;
#pragma unroll
      for (int g = 0; g < MT; g++) {
        int32_t rr[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const uint32_t slot = g * kBM + 4 * lane + j;
          rr[j] = (int32_t)(slot < item.nq ? a.qidx[item.q0 + slot] : a.zero_row);
        }
        for (uint32_t k = 0; k < kbh; k++)
          tma_gather4(dA + g * a_tile + k * kTile16K + lane * 512, &tmA, (int32_t)(k * 64), rr[0], rr[1], rr[2],
                      rr[3], &bar_a_full[sa]);
      }
      const uint32_t ntiles = (item.np + kBN - 1) / kBN;
      if (lane == 0) {
        pairs += (unsigned long long)item.nq * item.np;
        if (a.offsets && item.p0 == a.offsets[item.list]) lists += item.nq;
        for (uint32_t t = 0; t < ntiles; t++) {
          const uint32_t b = bi + t, sb = b % BS, use = b / BS;
          if (use > 0 && !(ok = mbar_wait(&bar_b_empty[sb], (use - 1) & 1, a.err))) break;
          mbar_expect_tx(&bar_b_full[sb], b_stage);
          const int32_t row = (int32_t)(item.p0 + (uint64_t)t * kBN);
          for (uint32_t k = 0; k < kbh; k++)
            tma_load_2d(sB + sb * b_stage + k * kTile16K, &tmB, (int32_t)(k * 64), row, &bar_b_full[sb]);
        }
      }
      bi += ntiles;
      ok = __shfl_sync(0xffffffffu, ok, 0);
    }
    if (lane == 0) {
      // drain: wait (bounded) for the copies still in flight before leaving
      for (uint32_t j = 0; j < BS && j < bi; j++) {
        const uint32_t b = bi - 1 - j;
        mbar_wait(&bar_b_full[b % BS], (b / BS) & 1, nullptr);
      }
      for (uint32_t j = 0; j < AS && j < ai; j++) {
        const uint32_t i = ai - 1 - j;
        mbar_wait(&bar_a_full[i % AS], (i / AS) & 1, nullptr);
      }
      if (a.stats && pairs) {
        atomicAdd(a.stats, pairs);
        atomicAdd(a.stats + 1, lists);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc = SPLIT ? idesc_f16_f32(kBM, kBN) : idesc_bf16_f32(kBM, kBN);
      uint32_t ai = 0, bi = 0;
      bool ok = true;
      for (uint32_t it = blockIdx.x; it < nitems && ok; it += gridDim.x, ai++) {
        const SearchItem item = a.items[it];
        const uint32_t sa = ai % AS;
        if (!(ok = mbar_wait(&bar_a_full[sa], (ai / AS) & 1, a.err))) break;
        const uint32_t ntiles = (item.np + kBN - 1) / kBN;
        for (uint32_t t = 0; t < ntiles; t++, bi++) {
          const uint32_t sb = bi % BS, slot = bi % NSLOT;
          if (!(ok = mbar_wait(&bar_b_full[sb], (bi / BS) & 1, a.err))) break;
          if (bi >= NSLOT && !(ok = mbar_wait(&bar_t_empty[slot], ((bi / NSLOT) - 1) & 1, a.err))) break;
          tc_fence_after();
          const uint32_t b0 = smem_u32(sB + sb * b_stage);
#pragma unroll
          for (int g = 0; g < MT; g++) {
            const uint32_t d = tmem + (slot * MT + g) * kBN;
            const uint32_t a0 = smem_u32(sA + sa * a_stage + g * a_tile);
            for (uint32_t k = 0; k < kb; k++) {
#pragma unroll
              for (uint32_t kk = 0; kk < 4; kk++) {
                const uint32_t off = k * kTile16K + kk * 32;
                mma_bf16(d, sw128_desc(a0 + off), sw128_desc(b0 + off), idesc, (k | kk) != 0);
                if (SPLIT) {
                  const uint32_t lo = kb * kTile16K;
                  mma_bf16(d, sw128_desc(a0 + off), sw128_desc(b0 + lo + off), idesc, 1);
                  mma_bf16(d, sw128_desc(a0 + lo + off), sw128_desc(b0 + off), idesc, 1);
                }
              }
            }
          }
          mma_commit(&bar_b_empty[sb]);
          mma_commit(&bar_t_full[slot]);
        }
        if (ok) mma_commit(&bar_a_empty[sa]);
      }
    }
  } else if (warp == 2) {
    // ------------------------------------------------ row constants of each B tile
    uint32_t bi = 0;
    bool ok = true;
    for (uint32_t it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
      const SearchItem item = a.items[it];
      const uint32_t ntiles = (item.np + kBN - 1) / kBN;
      for (uint32_t t = 0; t < ntiles; t++, bi++) {
        const uint32_t slot = bi % NSLOT;
        if (bi >= NSLOT) ok = mbar_wait(&bar_t_empty[slot], ((bi / NSLOT) - 1) & 1, a.err);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
        const uint32_t valid = min((uint32_t)kBN, item.np - t * kBN);
        float *dst = xs + slot * kBN;
        const float *src = a.w + item.p0 + (uint64_t)t * kBN;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const uint32_t c = lane + 32 * j;
          cp_async4(dst + c, c < valid ? src + c : &g_inf);  // +inf masks rows past the item
        }
        cp_async_mbar_arrive(&bar_x_full[slot]);
      }
    }
    cp_async_wait_all();
  } else if (warp >= 4) {
    // ------------------------------------------------ epilogue (two warpgroups)
    const uint32_t grp = (warp - 4) >> 2, ew = warp & 3, et = ew * 32 + lane;
    float *myla = la + (grp * kBM + et) * kLST;
    uint32_t *myli = li + (grp * kBM + et) * kLST;
    const uint32_t arow = (MT == 2 ? grp * kBM : 0) + et;  // this thread's row of the item's query tiles
    uint32_t bi = 0;
    bool ok = true;
    for (uint32_t it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
      const SearchItem item = a.items[it];
      const uint32_t ntiles = (item.np + kBN - 1) / kBN;
      const bool valid = arow < item.nq;
      bool have = false;
      uint32_t q = 0, nl = 0;
      // rows past the item's queries keep a threshold no value passes
      float dq = 0.f, alpha = -2.f, thv = -FLT_MAX;
      for (uint32_t t = 0; t < ntiles; t++, bi++) {
        if (MT == 1 && (bi & 1u) != grp) continue;
        const uint32_t slot = bi % NSLOT;
        if (!have && valid) {
          q = a.qidx[item.q0 + arow];
          dq = a.Dqr[(uint64_t)q * a.nr + item.list];
          thv = v_threshold(__uint_as_float(__ldcg(a.sl_theta + q)), dq);
          if (SPLIT) alpha = -2.f / (a.qscale[q] * a.lscale[item.list]);
          const float E = tc_error_bound(dq, a.qnorm[q], a.lxmax[item.list], a.lcnorm[item.list],
                                         a.q_inexact ? a.q_inexact[q] : 1u, a.x_inexact, a.format, a.d);
          atomicMax(a.emax + q, __float_as_uint(E));
        }
        have = true;
        if (!(ok = mbar_wait(&bar_t_full[slot], (bi / NSLOT) & 1, a.err))) break;
        if (!(ok = mbar_wait(&bar_x_full[slot], (bi / NSLOT) & 1, a.err))) break;
        tc_fence_after();
        const float *xr = xs + slot * kBN;
        const uint32_t taddr = tmem + ((32u * ew) << 16) + (slot * MT + (MT == 2 ? grp : 0)) * kBN;
        const uint64_t p = item.p0 + (uint64_t)t * kBN;
#pragma unroll 1
        for (uint32_t c = 0; c < kBN / 32; c++) {
          uint32_t r[32];
          __syncwarp();
          tmem_ld32(taddr + c * 32, r);
          tmem_wait_ld();
          float v[32];
          float mn = INFINITY;
#pragma unroll
          for (int j4 = 0; j4 < 8; j4++) {
            const float4 x4 = *reinterpret_cast<const float4 *>(xr + c * 32 + 4 * j4);
            v[4 * j4 + 0] = fmaf(alpha, __uint_as_float(r[4 * j4 + 0]), x4.x);
            v[4 * j4 + 1] = fmaf(alpha, __uint_as_float(r[4 * j4 + 1]), x4.y);
            v[4 * j4 + 2] = fmaf(alpha, __uint_as_float(r[4 * j4 + 2]), x4.z);
            v[4 * j4 + 3] = fmaf(alpha, __uint_as_float(r[4 * j4 + 3]), x4.w);
            mn = fminf(mn, fminf(fminf(v[4 * j4], v[4 * j4 + 1]), fminf(v[4 * j4 + 2], v[4 * j4 + 3])));
          }
          if (mn <= thv) {
#pragma unroll
            for (int e = 0; e < 32; e++) {
              if (v[e] <= thv) {
                const Cand cs = insert_candidate(a, q, myla, myli, nl, thv, dq, v[e], (uint32_t)(p + c * 32 + e));
                nl = cs.nl;
                thv = cs.thv;
              }
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bar_t_empty[slot]);
      }
      if (valid && nl > 0) publish(a, q, myla, myli, nl);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ------------------------------------------------------------------ build kernels
// The list of list-major row p: offsets[r] <= p < offsets[r + 1].
__device__ __forceinline__ uint32_t list_of(const uint64_t *off, uint32_t nr, uint64_t p) {
  uint32_t lo = 0, hi = nr;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (off[mid] <= p)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Power of two s with s * maxabs in [2^13, 2^14) (1 for an all-zero row or list).
__device__ __forceinline__ float half_scale(float maxabs) {
  if (!(maxabs > 0.f)) return 1.f;
  const int e = max(-120, min(120, 13 - ilogbf(maxabs)));
  return ldexpf(1.f, e);
}

// One warp per row: x' = x - c (FP32), w = ||x'||^2 + 2 c.x', the BF16
// exactness flag and the largest |x'_i| of the list.
__global__ void tc_center_kernel(const float *__restrict__ Xp, uint32_t ld, const uint64_t *__restrict__ off,
                                 uint32_t nr, const float *__restrict__ R, uint64_t n, uint32_t d,
                                 float *__restrict__ w, uint32_t *__restrict__ inexact,
                                 uint32_t *__restrict__ lmax_bits) {
  const uint64_t p = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (p >= n) return;
  const uint32_t r = list_of(off, nr, p);
  const float *x = Xp + p * ld, *c = R + (uint64_t)r * ld;
  float sxx = 0.f, scx = 0.f, mx = 0.f;
  uint32_t bad = 0;
  for (uint32_t i = lane; i < d; i += 32) {
    const float v = __fsub_rn(x[i], c[i]);
    bad |= __bfloat162float(__float2bfloat16_rn(v)) != v;
    sxx = fmaf(v, v, sxx);
    scx = fmaf(c[i], v, scx);
    mx = fmaxf(mx, fabsf(v));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sxx += __shfl_xor_sync(0xffffffffu, sxx, o);
    scx += __shfl_xor_sync(0xffffffffu, scx, o);
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if (lane == 0) {
    w[p] = sxx + 2.f * scx;
    if (bad) atomicOr(inexact, 1u);
    atomicMax(lmax_bits + r, __float_as_uint(mx));
  }
}

// Per list: the operand scale, a bound on ||x'|| from the list radius (the
// largest member distance, relative error <= gamma_{d+1}) and ||c||.
__global__ void tc_list_params_kernel(const float *__restrict__ R, uint32_t ld, uint32_t nr, uint32_t d,
                                      const float *__restrict__ radius, const uint32_t *__restrict__ lmax_bits,
                                      uint32_t format, float *__restrict__ lscale, float *__restrict__ lxmax,
                                      float *__restrict__ lcnorm) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nr) return;
  const double u = 5.9604644775390625e-08, g = (d + 3) * u / (1.0 - (d + 3) * u);
  lscale[r] = format == kTcSplit ? half_scale(__uint_as_float(lmax_bits[r])) : 1.f;
  lxmax[r] = __double2float_ru(sqrt((double)radius[r] / (1.0 - g)) * (1.0 + g));
  double cc = 0.0;
  for (uint32_t i = 0; i < d; i++) cc += (double)R[(uint64_t)r * ld + i] * R[(uint64_t)r * ld + i];
  lcnorm[r] = __double2float_ru(sqrt(cc));
}

// One warp per row of the padded operand: BF16 x' (exact format) or FP16
// hi | lo of s_r x' (split format); rows past n are zero.
__global__ void tc_convert_kernel(const float *__restrict__ Xp, uint32_t ld, const uint64_t *__restrict__ off,
                                  uint32_t nr, const float *__restrict__ R, uint64_t n, uint64_t n_pad, uint32_t d,
                                  uint32_t kp, uint32_t format, const float *__restrict__ lscale,
                                  uint16_t *__restrict__ Xh) {
  const uint64_t p = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (p >= n_pad) return;
  const uint32_t cols = format == kTcSplit ? 2 * kp : kp;
  uint16_t *dst = Xh + p * cols;
  if (p >= n) {
    for (uint32_t i = lane; i < cols; i += 32) dst[i] = 0;
    return;
  }
  const uint32_t r = list_of(off, nr, p);
  const float *x = Xp + p * ld, *c = R + (uint64_t)r * ld;
  const float s = lscale[r];
  for (uint32_t i = lane; i < kp; i += 32) {
    const float v = i < d ? __fsub_rn(x[i], c[i]) : 0.f;
    if (format == kTcSplit) {
      const float sv = v * s;
      const __half hi = __float2half_rn(sv);
      const __half lo = __float2half_rn(sv - __half2float(hi));
      dst[i] = __half_as_ushort(hi);
      dst[kp + i] = __half_as_ushort(lo);
    } else {
      dst[i] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
    }
  }
}

// One warp per query row (row m is the zero row): the operand row, its scale,
// ||q|| and whether some value is not exact in BF16.
__global__ void tc_query_kernel(const float *__restrict__ Q, uint32_t ld, uint64_t m, uint32_t d, uint32_t kp,
                                uint32_t format, uint16_t *__restrict__ Qh, float *__restrict__ qscale,
                                float *__restrict__ qnorm, uint8_t *__restrict__ qinex) {
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (q > m) return;
  const uint32_t cols = format == kTcSplit ? 2 * kp : kp;
  uint16_t *dst = Qh + q * cols;
  if (q == m) {
    for (uint32_t i = lane; i < cols; i += 32) dst[i] = 0;
    return;
  }
  const float *x = Q + q * ld;
  float ss = 0.f, mx = 0.f;
  uint32_t bad = 0;
  for (uint32_t i = lane; i < d; i += 32) {
    const float v = x[i];
    ss = fmaf(v, v, ss);
    mx = fmaxf(mx, fabsf(v));
    bad |= __bfloat162float(__float2bfloat16_rn(v)) != v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  const float t = format == kTcSplit ? half_scale(mx) : 1.f;
  for (uint32_t i = lane; i < kp; i += 32) {
    const float v = i < d ? x[i] : 0.f;
    if (format == kTcSplit) {
      const float sv = v * t;
      const __half hi = __float2half_rn(sv);
      const __half lo = __float2half_rn(sv - __half2float(hi));
      dst[i] = __half_as_ushort(hi);
      dst[kp + i] = __half_as_ushort(lo);
    } else {
      dst[i] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
    }
  }
  if (lane == 0) {
    qscale[q] = t;
    qnorm[q] = sqrtf(ss) * (1.f + 1e-6f);
    qinex[q] = (uint8_t)(format == kTcSplit ? 0 : bad);
  }
}

// Both shortlist buffers empty, buffer 0 current, thresholds open, locks free,
// error bounds zero.
__global__ void sl_init_kernel(float *sl_a, uint32_t *sl_row, uint32_t *sel, uint32_t *theta, uint32_t *lock,
                               uint32_t *emax, uint64_t m) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < 2 * m * kSL) {
    sl_a[i] = INFINITY;
    sl_row[i] = RBC_DUMMY;
  }
  if (i < m) {
    sel[i] = 0;
    theta[i] = __float_as_uint(FLT_MAX);
    lock[i] = 0;
    emax[i] = 0;
  }
}

// Exact rerank of each query's shortlist (one warp per query): the k-th exact
// distance as a pruning threshold, or the results and the certificate.
template <int METRIC>
__global__ void rerank_kernel(RerankArgs a) {
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= a.m) return;
  const float *qrow = a.Q + q * a.ld;
  const uint64_t slot = ((uint64_t)a.sl_sel[q] * a.m + q) * kSL;
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
  const float kth = __shfl_sync(0xffffffffu, ld, a.k - 1);
  if (a.tau && lane == 0) atomicMin(a.tau + q, fbits(kth));
  if (!a.ids && !a.dists) return;
  // certificate: every row searched but not in the shortlist has approx >=
  // a_last, so its exact distance is >= a_last - E > kth when certified
  bool certified = true;
  if (valid == kSL) {
    const double a_last = (double)sa_q[kSL - 1];
    const double E = (double)__uint_as_float(a.emax[q]);
    certified = a_last - E > (double)kth;
  }
  if (lane < (int)a.k) {
    if (a.ids) a.ids[q * a.ldo + lane] = li;
    if (a.dists) a.dists[q * a.ldo + lane] = ld;
  }
  if (lane == 0 && !certified) {
    const uint32_t s = atomicAdd(a.nfail, 1u);
    a.fail[s] = (uint32_t)q;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

template <int MT, bool SPLIT>
size_t smem_bytes(uint32_t kb, uint32_t as, uint32_t bs) {
  const size_t kbh = SPLIT ? 2 * kb : kb;
  return 1024 + (size_t)as * MT * kbh * kTile16K + (size_t)bs * kbh * kTile16K + (size_t)(4 / MT) * kBN * 4 +
         (size_t)kEpiGroups * kBM * kLST * 8;
}

template <int MT, bool SPLIT>
cudaError_t launch_tc(const CUtensorMap &tmA, const CUtensorMap &tmB, TcArgs a, int grid, cudaStream_t s) {
  uint32_t as = kMaxA, bs = kMaxB;
  while (smem_bytes<MT, SPLIT>(a.kb, as, bs) > kSmemLimit) {
    if (bs > 2)
      bs--;
    else if (as > 1)
      as--;
    else
      return cudaErrorInvalidConfiguration;
  }
  a.a_stages = as;
  a.b_stages = bs;
  const size_t smem = smem_bytes<MT, SPLIT>(a.kb, as, bs);
  cudaError_t e =
      cudaFuncSetAttribute(tc_search_kernel<MT, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  tc_search_kernel<MT, SPLIT><<<grid, kThreads, smem, s>>>(tmA, tmB, a);
  return launched();
}

}  // namespace

// ------------------------------------------------------------------ host side
bool tc_supported(uint32_t dp) { return dp <= 128; }

uint32_t tc_kp(uint32_t d) { return (d + 63) / 64 * 64; }

uint32_t tc_query_tile(uint32_t format) { return format == kTcSplit ? kBM : 2 * kBM; }

cudaError_t tc_make_map(CUtensorMap *map, const void *ptr, uint64_t rows, uint32_t cols, uint32_t box_rows) {
  if (!g_encode) {
    cudaDriverEntryPointQueryResult qr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void **)&g_encode, 12000,
                                                     cudaEnableDefault, &qr);
    if (e != cudaSuccess) return e;
    if (qr != cudaDriverEntryPointSuccess || !g_encode) return cudaErrorNotSupported;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void *>(ptr), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

int tc_build(const float *Xp, const uint64_t *offsets, const float *R, const float *radius, uint64_t n,
             uint64_t n_pad, uint32_t nr, uint32_t d, uint32_t ld, uint32_t kp, TcBuild *out, uint64_t *bytes,
             cudaStream_t s) {
  TcBuild &t = *out;
  DevBuf fl, lmax;
  cudaError_t e = fl.alloc(4, s);
  if (e == cudaSuccess) e = lmax.alloc(nr * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(fl.p, 0, 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(lmax.p, 0, nr * 4, s);
  if (e == cudaSuccess) e = cudaMalloc(&t.w, (n_pad + kBN) * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(t.w, 0, (n_pad + kBN) * 4, s);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_build: tensor-form buffers");
  const unsigned grid_n = (unsigned)((n * 32 + 255) / 256);
  tc_center_kernel<<<grid_n, 256, 0, s>>>(Xp, ld, offsets, nr, R, n, d, t.w, fl.as<uint32_t>(), lmax.as<uint32_t>());
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_build: centering");
  uint32_t inexact = 0;
  if ((e = cudaMemcpyAsync(&inexact, fl.p, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_fail(e, "rbc_build: format check");
  t.format = inexact ? kTcSplit : kTcExact;
  t.x_inexact = 0;  // the split format's residuals are in the bound; the exact format has none
  t.cols = t.format == kTcSplit ? 2 * kp : kp;
  const size_t xh_bytes = (size_t)n_pad * t.cols * 2;
  e = cudaMalloc(&t.Xh, xh_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&t.lscale, nr * 4);
  if (e == cudaSuccess) e = cudaMalloc(&t.lxmax, nr * 4);
  if (e == cudaSuccess) e = cudaMalloc(&t.lcnorm, nr * 4);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_build: tensor-form operands");
  *bytes += xh_bytes + (n_pad + kBN) * 4 + 3ull * nr * 4;
  tc_list_params_kernel<<<(nr + 127) / 128, 128, 0, s>>>(R, ld, nr, d, radius, lmax.as<uint32_t>(), t.format,
                                                        t.lscale, t.lxmax, t.lcnorm);
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_build: list parameters");
  tc_convert_kernel<<<(unsigned)((n_pad * 32 + 255) / 256), 256, 0, s>>>(
      Xp, ld, offsets, nr, R, n, n_pad, d, kp, t.format, t.lscale, static_cast<uint16_t *>(t.Xh));
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_build: operand rows");
  return RBC_OK;
}

cudaError_t launch_tc_queries(const float *Q, uint32_t ld, uint64_t m, uint32_t d, uint32_t kp, uint32_t format,
                              void *Qh, float *qscale, float *qnorm, uint8_t *q_inexact, cudaStream_t s) {
  const uint64_t threads = (m + 1) * 32;
  tc_query_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(Q, ld, m, d, kp, format,
                                                                    static_cast<uint16_t *>(Qh), qscale, qnorm,
                                                                    q_inexact);
  return launched();
}

cudaError_t launch_sl_init(float *sl_a, uint32_t *sl_row, uint32_t *sel, uint32_t *theta, uint32_t *lock,
                           uint32_t *emax, uint64_t m, cudaStream_t s) {
  const uint64_t total = std::max<uint64_t>(2 * m * kSL, 1);
  sl_init_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(sl_a, sl_row, sel, theta, lock, emax, m);
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
  if (a.kb < 1 || a.kb > 2) return cudaErrorInvalidValue;
  return a.format == kTcSplit ? launch_tc<1, true>(tmA, tmB, a, grid, s) : launch_tc<2, false>(tmA, tmB, a, grid, s);
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
