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
//          per query for q - mu, mu the mean of the representatives; the
//          identity then carries w = ||x'||^2 + 2 (c - mu).x'), three products:
//          hi.hi into one tensor-memory accumulator, hi.lo + lo.hi into a
//          second one, so the large accumulation runs over d terms only.
// In the exact format w is folded into the product: three BF16 pieces of w
// per row ride with each B tile and one more MMA step against a constant
// -1/4 tile leaves D = q.x' - w/2 in tensor memory, so v = -2 D needs no
// per-value arithmetic.
//
// Each query keeps the SL = 4k rows (40 to 56) of smallest approx.  Every
// shortlist starts with the query's SL nearest representatives (database rows
// whose exact distances Dqr the pruning already has), merged with the exact
// probe results of the FP32 path; the representatives' rows carry w = +inf,
// so the tensor search never meets them again.  A representative outside the
// seed is no nearer than the seed's largest distance, which bounds the
// shortlist's from above, so the certificate below covers it like any other
// row left out.  The rerank computes the shortlist's exact distances and sorts
// by (distance, id).  |approx - exact| <= E(q) over every row searched, with E
// from tc_error_bound; if the shortlist's largest approx minus E is above the
// k-th exact distance, no other row can be in the top k, so the result equals
// the FP32 oracle's; otherwise the query is recomputed by the plain FP32 path.
//
// Work items are the planner's list-major items: rows [p0, p0 + np) of one
// list against up to 128 MT queries (MT = 2 in the exact format's pruned
// round; 1 in its probe round and in the split format).
// Kernel structure (one persistent CTA per SM, 384 threads):
//   warp 0      TMA producer: 128-row B tiles of each item into a ring (with
//               the tile's w pieces, one bulk copy, in the exact format);
//   warps 1-2   tcgen05.mma issuers.  BF16 format: per item, tcgen05.cp moves
//               the gathered query tiles from their shared-memory stage into
//               tensor memory (the stage then takes the next item's gather,
//               and the MMAs read A from tensor memory, so shared memory
//               serves only the B operand); the accumulator of each (B tile,
//               query tile) pair is one of three 128 x 128 blocks taken in
//               turn, the query tiles fill the other 128 columns.  With two
//               query tiles warp 1 issues tile 0's MMAs and warp 2 tile 1's
//               (each a whole warp with one elected lane issuing, so one
//               warp's waits and commits do not hold up the other's).
//               Split format: warp 1, per B tile MT x 2 accumulators of
//               128 x 128 (512 columns hold 4 / (2 MT) slots), A from shared
//               memory.  Commits free the B stage and hand the accumulator to
//               the epilogue;
//   warp 2      split format: stages each B tile's row constants w into
//               shared memory (cp.async; +inf past the item's rows);
//   warp 3      per item: gathers the query rows with tile::gather4 (128-byte
//               swizzled, K-major) and stages each row's query, Dqr and error
//               bound;
//   warps 4-11  epilogue, two warpgroups (MT = 2: one per query tile; MT = 1:
//               alternate B tiles): tcgen05.ld of its query row, a 3-input max
//               per pair of columns against the query's threshold (the split
//               format forms approx with FMAs), candidates into a small
//               per-thread buffer that is merged into the query's global
//               shortlist (double-buffered, bounded per-query lock) when full
//               and at the end of the item.
// All mbarrier waits are bounded (sm100.cuh); a timeout sets the error word.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "engine.cuh"
#include "sm100.cuh"
#include "tc.cuh"

namespace rbc {

namespace {

using namespace sm100;

constexpr int kBM = 128, kBN = 128, kEpiGroups = 2;
constexpr int kThreads = 128 + 128 * kEpiGroups;
constexpr int kLocal = 8;  // per-thread candidate buffer, in registers (16 in the probe round's
                           // BF16 instance, whose lists meet many more candidates)
constexpr uint32_t kTile16K = 16384;           // 128 rows x 128 bytes (one 64-wide K block of halves)
// BF16 format: the accumulator of one (B tile, query tile) pair is one of
// kBlocks blocks of 128 columns in tensor memory columns [0, 384), taken in
// turn; the item's query tiles sit at [kTmemA, kTmemA + MT x 64).  The
// epilogue reads a block kChunk columns at a time.
constexpr uint32_t kBlocks = 3, kTmemA = 384, kChunk = 64;
constexpr uint32_t kWTile = 4096;              // 128 rows x 32 bytes: the folded w operand of one B tile
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

// The query's cap on its shortlist threshold (FLT_MAX without one).
__device__ __forceinline__ float query_cap(const TcArgs &a, uint32_t q) {
  return a.sl_cap ? __uint_as_float(__ldg(a.sl_cap + q)) : FLT_MAX;
}

// The cap an exact bound t on the final k-th distance puts on a shortlist
// threshold: t (1 + 2^-7), rounded up (FLT_MAX while t is open).  A row whose
// approx exceeds it cannot reach the top k while the error bound stays below
// 2^-7 t; the certificate checks that bound, and the margin keeps it far
// from failing (at 2^-10, a few c3 queries a call failed it).
__device__ __forceinline__ float tau_cap(float t) {
  return t < FLT_MAX ? fminf(__fmul_ru(t, 1.0078125f), FLT_MAX) : FLT_MAX;
}

// Merge one lane's sorted candidates (nl <= kLocal entries in the owner
// lane's registers la/li) into query q's global shortlist, with the whole
// warp: the current
// buffer (40 sorted entries) and the candidates form 64 (approx, row) pairs,
// two per lane, which a bitonic network sorts; the 40 smallest go to the
// other buffer, then the buffers swap, under the query's lock.  Called by all
// 32 lanes with the same arguments; returns the query's new threshold.
__device__ __forceinline__ float warp_publish(const TcArgs &a, uint32_t q, const float (&la)[kLocal],
                                              const uint32_t (&li)[kLocal], uint32_t nl, uint32_t owner) {
  const uint32_t lane = threadIdx.x & 31;
  uint32_t got = 1;
  if (lane == owner) {
    uint32_t spins = 0;
    while (atomicCAS(a.sl_lock + q, 0u, 1u) != 0u) {
      if (++spins > kLockSpin) {
        raise_error(a.err, RBC_ERR_ITER_LIMIT);
        got = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
  }
  got = __shfl_sync(0xffffffffu, got, owner);
  __syncwarp();
  if (!got) return __uint_as_float(__ldcg(a.sl_theta + q));
  const uint32_t sel = __ldcg(a.sl_sel + q);
  const uint32_t SL = a.sl, tail = SL - 32;  // entries past the first 32
  const uint64_t cur = ((uint64_t)sel * a.m + q) * SL, nxt = ((uint64_t)(sel ^ 1u) * a.m + q) * SL;
  float a0 = __ldcg(a.sl_a + cur + lane);
  uint32_t i0 = __ldcg(a.sl_row + cur + lane);
  float a1 = INFINITY;
  uint32_t i1 = RBC_DUMMY;
  if (lane < tail) {
    a1 = __ldcg(a.sl_a + cur + 32 + lane);
    i1 = __ldcg(a.sl_row + cur + 32 + lane);
  }
#pragma unroll
  for (uint32_t j = 0; j < (uint32_t)kLocal; j++) {  // the owner's candidates to lanes tail ..
    const float ca = __shfl_sync(0xffffffffu, la[j], owner);
    const uint32_t ci = __shfl_sync(0xffffffffu, li[j], owner);
    if (lane == tail + j && j < nl) {
      a1 = ca;
      i1 = ci;
    }
  }
  warp_sort32(a1, i1);  // the list's tail and the candidates, ascending
  // bitonic merge of two ascending 32-lists: lower half = ranks 0..31
  const float ra = __shfl_sync(0xffffffffu, a1, 31 - lane);
  const uint32_t ri = __shfl_sync(0xffffffffu, i1, 31 - lane);
  if (pair_less(ra, ri, a0, i0)) {
    a1 = a0;
    i1 = i0;
    a0 = ra;
    i0 = ri;
  } else {
    a1 = ra;
    i1 = ri;
  }
  warp_bitonic_merge32(a0, i0);
  warp_bitonic_merge32(a1, i1);
  a.sl_a[nxt + lane] = a0;
  a.sl_row[nxt + lane] = i0;
  if (lane < tail) {
    a.sl_a[nxt + 32 + lane] = a1;
    a.sl_row[nxt + 32 + lane] = i1;
  }
  const float alast = __shfl_sync(0xffffffffu, a1, tail - 1);
  const uint32_t ilast = __shfl_sync(0xffffffffu, i1, tail - 1);
  // FLT_MAX, not +inf, while the list is short; never above the query's cap
  const float theta = fminf(ilast != RBC_DUMMY ? alast : FLT_MAX, query_cap(a, q));
  __threadfence();
  __syncwarp();
  if (lane == owner) {
    a.sl_theta[q] = __float_as_uint(theta);
    a.sl_sel[q] = sel ^ 1u;
    __threadfence();
    atomicExch(a.sl_lock + q, 0u);
  }
  return theta;
}

// Sorted insertion of (av, row) into a lane's register buffer (ascending,
// empty slots +inf); with the buffer full the last entry falls off (and an
// entry not below it is not inserted).
template <int LOC>
__device__ __forceinline__ void insert_local(float (&la)[LOC], uint32_t (&li)[LOC], float av, uint32_t row) {
#pragma unroll
  for (int j = LOC - 1; j > 0; j--) {
    const bool shift = row_less(av, row, la[j - 1], li[j - 1]);
    const bool here = !shift && row_less(av, row, la[j], li[j]);
    la[j] = shift ? la[j - 1] : (here ? av : la[j]);
    li[j] = shift ? li[j - 1] : (here ? row : li[j]);
  }
  if (row_less(av, row, la[0], li[0])) {
    la[0] = av;
    li[0] = row;
  }
}

// Merge one lane's candidates into its own query's shortlist, every lane of
// the warp at once (each on its own query): the current buffer is copied into
// the lane's shared-memory staging area with 16-byte loads (one round trip),
// the candidates are inserted there, the result goes to the other buffer and
// the buffers swap, under the query's lock.  Returns the new threshold.
// The lock is a plain mutex held by one thread: taking it with an acquire CAS
// and releasing it with a release store orders the critical section's loads
// and stores against every other holder's without separate fences.
__device__ __forceinline__ uint32_t lock_cas_acquire(uint32_t *p) {
  uint32_t old;
  asm volatile("atom.acquire.gpu.global.cas.b32 %0, [%1], 0, 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}
__device__ __forceinline__ void unlock_release(uint32_t *p) {
  asm volatile("st.release.gpu.global.b32 [%0], 0;" ::"l"(p) : "memory");
}

template <int LOC>
__device__ __forceinline__ float lane_merge(const TcArgs &a, uint32_t q, const float (&la)[LOC],
                                            const uint32_t (&li)[LOC], uint32_t nl, float *stage) {
  uint32_t spins = 0;
  while (lock_cas_acquire(a.sl_lock + q) != 0u) {
    if (++spins > kLockSpin) {
      raise_error(a.err, RBC_ERR_ITER_LIMIT);
      return __uint_as_float(__ldcg(a.sl_theta + q));
    }
    __nanosleep(64);
  }
  const uint32_t SL = a.sl, sel = __ldcg(a.sl_sel + q);
  const uint64_t cur = ((uint64_t)sel * a.m + q) * SL, nxt = ((uint64_t)(sel ^ 1u) * a.m + q) * SL;
  float *sa = stage;
  uint32_t *sr = reinterpret_cast<uint32_t *>(stage + SL);
  // SL is a multiple of 4, so every list starts on a 16-byte boundary
  for (uint32_t j = 0; j < SL / 4; j++) {
    const float4 va = __ldcg(reinterpret_cast<const float4 *>(a.sl_a + cur) + j);
    const uint4 vr = __ldcg(reinterpret_cast<const uint4 *>(a.sl_row + cur) + j);
    sa[4 * j] = va.x; sa[4 * j + 1] = va.y; sa[4 * j + 2] = va.z; sa[4 * j + 3] = va.w;
    sr[4 * j] = vr.x; sr[4 * j + 1] = vr.y; sr[4 * j + 2] = vr.z; sr[4 * j + 3] = vr.w;
  }
#pragma unroll
  for (uint32_t e = 0; e < (uint32_t)LOC; e++) {
    if (e >= nl) break;
    const float av = la[e];
    const uint32_t ar = li[e];
    if (!row_less(av, ar, sa[SL - 1], sr[SL - 1])) break;  // candidates ascend: the rest do not fit either
    int pos = (int)SL - 1;
    while (pos > 0 && row_less(av, ar, sa[pos - 1], sr[pos - 1])) {
      sa[pos] = sa[pos - 1];
      sr[pos] = sr[pos - 1];
      pos--;
    }
    sa[pos] = av;
    sr[pos] = ar;
  }
  for (uint32_t j = 0; j < SL / 4; j++) {
    reinterpret_cast<float4 *>(a.sl_a + nxt)[j] = make_float4(sa[4 * j], sa[4 * j + 1], sa[4 * j + 2], sa[4 * j + 3]);
    reinterpret_cast<uint4 *>(a.sl_row + nxt)[j] = make_uint4(sr[4 * j], sr[4 * j + 1], sr[4 * j + 2], sr[4 * j + 3]);
  }
  // FLT_MAX, not +inf, while the list is short; never above the query's cap
  const float theta = fminf(sr[SL - 1] != RBC_DUMMY ? sa[SL - 1] : FLT_MAX, query_cap(a, q));
  a.sl_theta[q] = __float_as_uint(theta);
  a.sl_sel[q] = sel ^ 1u;
  unlock_release(a.sl_lock + q);  // after every store above
  return theta;
}

// Per-item state of one query row, staged by warp 3 for the epilogue (split
// format; the BF16 format needs only the query and Dqr).
struct RowState {
  uint32_t q;
  float dq, thv, alpha;
};
struct RowStateF {
  uint32_t q;
  float dq;
};

__device__ const float g_inf = INFINITY;

// r[base + e] for a run-time e in [0, 32), with static register indices only:
// five levels of selects on the bits of e.
template <int N>
__device__ __forceinline__ float select32(const uint32_t (&r)[N], int base, int e) {
  float s[16];
#pragma unroll
  for (int i = 0; i < 16; i++) s[i] = __uint_as_float((e & 16) ? r[base + 16 + i] : r[base + i]);
#pragma unroll
  for (int i = 0; i < 8; i++) s[i] = (e & 8) ? s[i + 8] : s[i];
#pragma unroll
  for (int i = 0; i < 4; i++) s[i] = (e & 4) ? s[i + 4] : s[i];
#pragma unroll
  for (int i = 0; i < 2; i++) s[i] = (e & 2) ? s[i + 2] : s[i];
  return (e & 1) ? s[1] : s[0];
}

// max(a, b, c) in one instruction (sm_100 and later)
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

__device__ __forceinline__ void cp_async4(float *smem, const float *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_mbar_arrive(uint64_t *bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }


template <int MT, bool SPLIT, bool PROBE>
__device__ __forceinline__ void tc_search_body(const CUtensorMap *pA, const CUtensorMap *pB, const TcArgs &a,
                                               const uint32_t cta, const uint32_t ncta) {
  constexpr uint32_t ACC = SPLIT ? 2 : 1;     // accumulators per query tile: hi.hi (+ corrections)
  constexpr uint32_t NSLOT = 4 / (MT * ACC);  // split format: tensor-memory slots of MT x ACC x 128 columns
  // BF16 format: w is folded into the product.  Each B stage carries the
  // tile's w operand (three BF16 pieces per row: the tile's 128 rows of a.wh
  // are one contiguous 4 KB block, brought by one bulk copy) and one
  // more MMA per accumulator multiplies it by a constant -1/4 tile, so the
  // accumulator holds D = q.x' - w / 2 and v = -2 D needs no per-value work
  // in the epilogue.  The split format adds w in the epilogue instead.
  constexpr bool FOLD = !SPLIT;
  constexpr uint32_t kIssuers = (FOLD && MT == 2) ? 2 : 1;  // warps issuing MMAs
  // candidate buffer entries per lane: 16 in the probe round (its lists meet
  // many more candidates; in the BF16 format MT = 1 is the probe round's),
  // kLocal otherwise
  constexpr int LOC = (MT == 1 && (!SPLIT || PROBE)) ? 2 * kLocal : kLocal;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_a_full[kMaxA], bar_a_empty[kMaxA], bar_b_full[kMaxB], bar_b_empty[kMaxB],
      bar_t_full[4], bar_t_empty[4], bar_x_full[4], bar_r_full[2], bar_r_empty[2], bar_q_free[2];
  // BF16 format: per accumulator block and issuer, "full" (the issuer's
  // commit, waited by the epilogue group of the same query tile) and "empty"
  // (arrivals of the other group, waited by this issuer); with two issuers a
  // block's uses alternate between them, and one barrier per block would let
  // a waiter run two phases ahead, where the parity test aliases
  __shared__ __align__(8) uint64_t bar_bf[kBlocks][2], bar_be[kBlocks][2];
  __shared__ uint32_t tmem_slot;

  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t kb = a.kb, kbh = SPLIT ? 2 * kb : kb;  // K blocks of a stored row (hi [+ lo])
  const uint32_t AS = a.a_stages, BS = a.b_stages;
  const uint32_t a_tile = kbh * kTile16K, a_stage = MT * a_tile, b_bytes = kbh * kTile16K;
  const uint32_t b_stage = b_bytes + (FOLD ? kWTile : 0u);  // B tile [+ its w operand]
  unsigned char *sA = base;
  unsigned char *sB = sA + AS * a_stage;
  unsigned char *sC = sB + BS * b_stage;
  // split: NSLOT x 128 row constants; BF16: the constant tile of the w product
  float *xs = reinterpret_cast<float *>(sC);
  unsigned char *sK = sC;
  unsigned char *sR = sC + (FOLD ? kWTile : NSLOT * kBN * 4);
  RowState *rs = reinterpret_cast<RowState *>(sR);    // 2 x 256 staged row states
  RowStateF *rsf = reinterpret_cast<RowStateF *>(sR);
  float *mstage = reinterpret_cast<float *>(sR + 2 * 2 * kBM * (FOLD ? sizeof(RowStateF) : sizeof(RowState)));
  // per epilogue thread: a.stage_words of merge staging (or none)

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 1) {
    tmem_alloc(&tmem_slot, 512);
    tmem_relinquish();
  }
  if (tid == 0) {
    for (uint32_t s = 0; s < kMaxA; s++) {
      mbar_init(&bar_a_full[s], 1);
      mbar_init(&bar_a_empty[s], kIssuers);
    }
    for (uint32_t s = 0; s < kMaxB; s++) {
      mbar_init(&bar_b_full[s], 1);
      mbar_init(&bar_b_empty[s], kIssuers);
    }
    for (uint32_t b = 0; b < 4; b++) {
      mbar_init(&bar_t_full[b], 1);
      mbar_init(&bar_t_empty[b], 4);  // one epilogue warpgroup reads each accumulator
      mbar_init(&bar_x_full[b], 32);
    }
    for (uint32_t b = 0; b < 2; b++) {
      mbar_init(&bar_r_full[b], 1);
      mbar_init(&bar_r_empty[b], 8);
    }
    mbar_init(&bar_q_free[0], 1);
    mbar_init(&bar_q_free[1], 1);
    for (uint32_t b = 0; b < kBlocks; b++)
      for (uint32_t i = 0; i < 2; i++) {
        mbar_init(&bar_bf[b][i], 1);
        mbar_init(&bar_be[b][i], 4);  // one epilogue warpgroup
      }
    fence_barrier_init();
  }
  if (FOLD && tid < (int)(kWTile / 16)) {
    // every row of the constant tile is -1/4 at halves 0-2 and 8-10, zero
    // elsewhere (the w operand rows hold w1 w2 w3 at the same places), so the
    // layout of the 16-half rows does not matter
    const uint32_t m4 = 0xBE80BE80u, m1 = 0x0000BE80u;  // BF16 -0.25
    reinterpret_cast<uint4 *>(sK)[tid] = make_uint4(m4, m1, 0u, 0u);
    fence_proxy_async();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t nitems = *a.nitems;
  // profiling clock (RBC_TC_TRACE): read only when tracing
  auto tclk = [&]() -> long long { return a.trace ? clock64() : 0ll; };

  if (warp == 0) {
    // ------------------------------------------------ TMA producer of the B tiles
    if (lane == 0) {
      prefetch_tensormap(pB);
      uint32_t bi = 0;
      unsigned long long pairs = 0, lists = 0, t_wait = 0;
      const long long t_all = tclk();
      bool ok = true;
      for (uint32_t it = cta; it < nitems && ok; it += ncta) {
        const SearchItem item = a.items[it];
        const uint32_t ntiles = (item.np + kBN - 1) / kBN;
        pairs += (unsigned long long)item.nq * item.np;
        if (a.offsets && item.p0 == a.offsets[item.list]) lists += item.nq;
        for (uint32_t t = 0; t < ntiles; t++, bi++) {
          const uint32_t sb = bi % BS, use = bi / BS;
          const long long t0 = tclk();
          if (use > 0 && !(ok = mbar_wait(&bar_b_empty[sb], (use - 1) & 1, a.err))) break;
          t_wait += tclk() - t0;
          mbar_expect_tx(&bar_b_full[sb], b_stage);
          const int32_t row = (int32_t)(item.p0 + (uint64_t)t * kBN);
          for (uint32_t k = 0; k < kbh; k++)
            tma_load_2d(sB + sb * b_stage + k * kTile16K, pB, (int32_t)(k * 64), row, &bar_b_full[sb]);
          if (FOLD) bulk_load(sB + sb * b_stage + b_bytes, a.wh + 2 * (uint64_t)row, kWTile, &bar_b_full[sb]);
        }
      }
      // drain: wait (bounded) for the copies still in flight before leaving
      for (uint32_t j = 0; j < BS && j < bi; j++) {
        const uint32_t b = bi - 1 - j;
        mbar_wait(&bar_b_full[b % BS], (b / BS) & 1, nullptr);
      }
      if (a.stats && pairs) {
        atomicAdd(a.stats, pairs);
        atomicAdd(a.stats + 1, lists);
      }
      if (a.trace) {
        a.trace[cta * kTcTraceWords + 6] = t_wait;
        a.trace[cta * kTcTraceWords + 7] = tclk() - t_all;
        a.trace[cta * kTcTraceWords + 15] = bi;
      }
    }
  } else if (warp == 1 || (FOLD && MT == 2 && warp == 2)) {
    // ------------------------------------------------ MMA issuers
    if constexpr (FOLD) {
      // BF16 format: the item's query tiles are copied from their shared-
      // memory stage into tensor memory (the stage then takes the next item's
      // gather while this item runs) and read from there; the accumulator of
      // each (B tile, query tile) pair u = MT t + g takes block u mod kBlocks.
      // MT = 2: warp 1 issues query tile 0's MMAs and warp 2 query tile 1's,
      // each copying its own tile into tensor memory behind its own
      // query-free barrier, both committing to a B stage's empty barrier
      // (count two) and to the query stage's (count two): the per-tile waits,
      // fences and commits of an issuing warp are halved.  MT = 1: warp 1.
      // The whole warp runs the loop (every lane polls, a vote makes the
      // outcome uniform), so the operands are warp-uniform and one elected
      // lane issues each instruction; the descriptors of a B stage are built
      // once and offset by constants (the start address field is in 16-byte
      // units and no offset carries out of it).
      const uint32_t g = MT == 2 ? (uint32_t)warp - 1 : 0u;
      const uint32_t idesc = idesc_bf16_f32(kBM, kBN);
      const uint32_t tAg = tmem + kTmemA + g * kb * 4 * 8;
      const uint64_t kd = sw32_desc(smem_u32(sK));
      const uint32_t n_items = __shfl_sync(0xffffffffu, nitems, 0);
      uint32_t ai = 0, bi = 0;
      uint32_t site = 0;  // diagnostics: the wait that gave up
      auto wait = [&](uint64_t *bar, uint32_t parity) {
        const bool r = __all_sync(0xffffffffu, mbar_wait(bar, parity, a.err)) != 0;
        if (!r && a.trace && lane == 0)
          a.trace[(size_t)ncta * kTcTraceWords + 6 * kTcTraceEvents + cta * 4 + g] =
              (1ull << 63) | ((unsigned long long)site << 56) | ((unsigned long long)ai << 32) | (bi << 1) | parity;
        return r;
      };
      // ring positions and phase parities kept as counters (no runtime divisions in the loop)
      uint32_t sa = 0, aph = 0, sb = 0, bph = 0;
      bool ok = true;
      long long *ev = (a.trace && cta == 0)
                          ? reinterpret_cast<long long *>(a.trace + (size_t)ncta * kTcTraceWords)
                          : nullptr;
      // cycles (warp 1): [0] all, [1] waiting for the query tile, [2] for the
      // previous item's MMAs, [3] for B tiles, [4] for accumulator blocks; [5] MMAs
      unsigned long long tr[6] = {0, 0, 0, 0, 0, 0};
      const bool tracing = a.trace != nullptr;  // clock reads only when tracing
      auto clk = [&]() -> long long { return tracing ? clock64() : 0ll; };
      const long long t_all = clk();
      long long t0;
      for (uint32_t it = cta; it < n_items && ok; it += ncta, ai++) {
        const uint32_t ntiles = __shfl_sync(0xffffffffu, (a.items[it].np + kBN - 1) / kBN, 0);
        t0 = clk();
        site = 1;
        if (!(ok = wait(&bar_a_full[sa], aph))) break;
        tr[1] += clk() - t0;
        // this issuer's previous MMAs read its query tile in tensor memory until they complete
        t0 = clk();
        site = 2;
        if (ai > 0 && !(ok = wait(&bar_q_free[g], (ai - 1) & 1))) break;
        tr[2] += clk() - t0;
        tc_fence_after();
        const uint64_t ad0 = sw128_desc(smem_u32(sA + sa * a_stage + g * a_tile));
#pragma unroll
        for (uint32_t k = 0; k < 2; k++)
          if (k < kb) {
#pragma unroll
            for (uint32_t kk = 0; kk < 4; kk++)
              tmem_cp_128x256b_warp(tAg + (k * 4 + kk) * 8, ad0 + ((k * kTile16K + kk * 32) >> 4));
          }
        mma_commit_warp(&bar_a_empty[sa]);  // the stage is free once the copies are done
        if (++sa == AS) {
          sa = 0;
          aph ^= 1u;
        }
        for (uint32_t t = 0; t < ntiles && ok; t++, bi++) {
          t0 = clk();
          site = 3;
          if (!(ok = wait(&bar_b_full[sb], bph))) break;
          const long long t1 = clk();
          tr[3] += t1 - t0;
          if (ev && g == 0 && lane == 0 && MT * bi >= kTcTraceFirst && MT * bi < kTcTraceFirst + kTcTraceEvents) {
            ev[4 * kTcTraceEvents + MT * bi - kTcTraceFirst] = t0;
            ev[5 * kTcTraceEvents + MT * bi - kTcTraceFirst] = t1;
          }
          const uint32_t b0 = smem_u32(sB + sb * b_stage);
          const uint64_t bd0 = sw128_desc(b0), wd0 = sw32_desc(b0 + b_bytes);
          // use j = u / kBlocks of block blk: with two issuers this issuer's
          // uses of the block are every other one, so its barriers count
          // phases j / 2; with one, j
          const uint32_t u = MT * bi + g, blk = u % kBlocks, j = u / kBlocks;
          t0 = clk();
          site = 4;
          if (j > 0 && !(ok = wait(&bar_be[blk][g], (kIssuers == 2 ? (j - 1) >> 1 : j - 1) & 1))) break;
          const long long t2 = clk();
          tr[4] += t2 - t0;
          tc_fence_after();
          const uint32_t d = tmem + blk * kBN;
#pragma unroll
          for (uint32_t k = 0; k < 2; k++)
            if (k < kb) mma_bf16_ts_kblock_warp(d, tAg + k * 4 * 8, bd0 + ((k * kTile16K) >> 4), idesc, k);
          // -w / 2 last: the products' partial sums stay at the scale of |q| |x'|
          mma_bf16_warp(d, kd, wd0, idesc, 1);
          tr[5] += kb * 4 + 1;
          mma_commit_warp(&bar_bf[blk][g]);
          mma_commit_warp(&bar_b_empty[sb]);
          if (ev && lane == 0 && u >= kTcTraceFirst && u < kTcTraceFirst + kTcTraceEvents) {
            ev[u - kTcTraceFirst] = t2;
            ev[kTcTraceEvents + u - kTcTraceFirst] = clk();
          }
          if (++sb == BS) {
            sb = 0;
            bph ^= 1u;
          }
        }
        if (ok) mma_commit_warp(&bar_q_free[g]);
      }
      tr[0] = clk() - t_all;
      if (a.trace && g == 0 && lane == 0)
        for (int j = 0; j < 6; j++) a.trace[cta * kTcTraceWords + j] = tr[j];
    } else {
      // split format: one query tile, A from shared memory; per B tile three
      // MMAs per K step (hi.hi into the first accumulator, hi.lo + lo.hi
      // into the second).  Issued like the BF16 path: the whole warp runs the
      // loop, one elected lane issues, descriptors offset by constants.
      static_assert(MT == 1, "the split format runs one query tile per B tile");
      const uint32_t idesc = idesc_f16_f32(kBM, kBN);
      const uint32_t n_items = __shfl_sync(0xffffffffu, nitems, 0);
      auto wait = [&](uint64_t *bar, uint32_t parity) {
        return __all_sync(0xffffffffu, mbar_wait(bar, parity, a.err)) != 0;
      };
      uint32_t bi = 0, sa = 0, aph = 0, sb = 0, bph = 0, slot = 0, sph = 0;
      const uint32_t lo = (kb * kTile16K) >> 4;  // the lo halves, in descriptor units
      bool ok = true;
      for (uint32_t it = cta; it < n_items && ok; it += ncta) {
        const uint32_t ntiles = __shfl_sync(0xffffffffu, (a.items[it].np + kBN - 1) / kBN, 0);
        if (!(ok = wait(&bar_a_full[sa], aph))) break;
        const uint64_t ad0 = sw128_desc(smem_u32(sA + sa * a_stage));
        for (uint32_t t = 0; t < ntiles; t++, bi++) {
          if (!(ok = wait(&bar_b_full[sb], bph))) break;
          if (bi >= NSLOT && !(ok = wait(&bar_t_empty[slot], sph ^ 1u))) break;
          tc_fence_after();
          const uint64_t bd0 = sw128_desc(smem_u32(sB + sb * b_stage));
          const uint32_t d = tmem + slot * ACC * kBN;
#pragma unroll
          for (uint32_t k = 0; k < 2; k++)
            if (k < kb) {
#pragma unroll
              for (uint32_t kk = 0; kk < 4; kk++) {
                const uint32_t off = (k * kTile16K + kk * 32) >> 4;
                const uint32_t acc = (k | kk) != 0;
                mma_bf16_warp(d, ad0 + off, bd0 + off, idesc, acc);
                mma_bf16_warp(d + kBN, ad0 + off, bd0 + lo + off, idesc, acc);
                mma_bf16_warp(d + kBN, ad0 + lo + off, bd0 + off, idesc, 1);
              }
            }
          mma_commit_warp(&bar_b_empty[sb]);
          mma_commit_warp(&bar_t_full[slot]);
          if (++sb == BS) {
            sb = 0;
            bph ^= 1u;
          }
          if (++slot == NSLOT) {
            slot = 0;
            sph ^= 1u;
          }
        }
        if (ok) mma_commit_warp(&bar_a_empty[sa]);
        if (++sa == AS) {
          sa = 0;
          aph ^= 1u;
        }
      }
    }
  } else if (warp == 2 && !FOLD) {
    // ------------------------------------------------ row constants of each B tile (split format)
    uint32_t bi = 0;
    bool ok = true;
    for (uint32_t it = cta; it < nitems && ok; it += ncta) {
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
  } else if (warp == 3) {
    // ------------------------------------------------ per item: row states and the query tile gather
    if (lane == 0) prefetch_tensormap(pA);
    uint32_t ai = 0;
    bool ok = true;
    unsigned long long w3[2] = {0, 0};  // cycles waiting for a row-state slot, for the query stage
    const long long t_all = tclk();
    for (uint32_t it = cta; it < nitems && ok; it += ncta, ai++) {
      const SearchItem item = a.items[it];
      const uint32_t slot = ai & 1, sa = ai % AS;
      // The query tiles' gather goes out first: it needs only the query rows
      // and a free query stage, not the row-state slot, which frees only when
      // the epilogue finishes the item before last.  Then the item's row
      // states are read from global memory (their latency hides behind the
      // slot's wait) and written.
      // lane l owns rows 4l..4l+3 of each query tile (one gather4 per tile and K block)
      int32_t rr[MT][4];
      float dqv[MT][4], qnv[MT][4];
      uint32_t qin[MT][4];
#pragma unroll
      for (int g = 0; g < MT; g++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const uint32_t row = g * kBM + 4 * lane + j;
          rr[g][j] = row < item.nq ? (int32_t)a.qidx[item.q0 + row] : (int32_t)a.zero_row;
        }
      long long t0 = tclk();
      if (ai >= AS) ok = mbar_wait(&bar_a_empty[sa], ((ai / AS) - 1) & 1, a.err);
      w3[1] += tclk() - t0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      {
        unsigned char *dA = sA + sa * a_stage;
        if (lane == 0) mbar_expect_tx(&bar_a_full[sa], a_stage);
        __syncwarp();
#pragma unroll
        for (int g = 0; g < MT; g++)
          for (uint32_t k = 0; k < kbh; k++)
            tma_gather4(dA + g * a_tile + k * kTile16K + lane * 512, pA, (int32_t)(k * 64), rr[g][0], rr[g][1],
                        rr[g][2], rr[g][3], &bar_a_full[sa]);
      }
#pragma unroll
      for (int g = 0; g < MT; g++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const uint32_t row = g * kBM + 4 * lane + j, q = (uint32_t)rr[g][j];
          const bool v = row < item.nq;
          dqv[g][j] = v ? a.Dqr[(uint64_t)q * a.nr + item.list] : 0.f;
          qnv[g][j] = v ? a.qnorm[q] : 0.f;
          qin[g][j] = v ? (a.q_inexact ? a.q_inexact[q] : 1u) : 0u;
        }
      const float X = a.lxmax[item.list], C = a.lcnorm[item.list];
      t0 = tclk();
      if (ai >= 2) ok = mbar_wait(&bar_r_empty[slot], ((ai >> 1) - 1) & 1, a.err);
      w3[0] += tclk() - t0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      RowState *dst = rs + slot * 2 * kBM;
      RowStateF *dstf = rsf + slot * 2 * kBM;
      const float ls = SPLIT ? a.lscale[item.list] : 1.f;
#pragma unroll
      for (int g = 0; g < MT; g++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const uint32_t row = g * kBM + 4 * lane + j;
          RowState st{0u, 0.f, -FLT_MAX, -2.f};  // rows past the item's queries: no value passes
          if (row < item.nq) {
            const uint32_t q = (uint32_t)rr[g][j];
            const float dq = dqv[g][j];
            st.q = q;
            st.dq = dq;
            if (!FOLD) st.thv = v_threshold(__uint_as_float(__ldcg(a.sl_theta + q)), dq);
            if (SPLIT) st.alpha = -2.f / (a.qscale[q] * ls);
            const float E = tc_error_bound(dq, qnv[g][j], X, C, qin[g][j], a.x_inexact, a.format, a.d);
            atomicMax(a.emax + q, __float_as_uint(E));
          }
          if (FOLD)
            dstf[row] = RowStateF{st.q, st.dq};
          else
            dst[row] = st;
        }
      __syncwarp();
      if (lane == 0) mbar_arrive(&bar_r_full[slot]);
    }
    if (lane == 0 && a.trace) {
      a.trace[cta * kTcTraceWords + 8] = w3[0];
      a.trace[cta * kTcTraceWords + 9] = w3[1];
      a.trace[cta * kTcTraceWords + 10] = tclk() - t_all;
    }
    if (lane == 0) {
      // drain: wait (bounded) for the gathers still in flight before leaving
      for (uint32_t j = 0; j < AS && j < ai; j++) {
        const uint32_t i = ai - 1 - j;
        mbar_wait(&bar_a_full[i % AS], (i / AS) & 1, nullptr);
      }
    }
  } else if (warp >= 4) {
    // ------------------------------------------------ epilogue (two warpgroups)
    const uint32_t grp = (warp - 4) >> 2, ew = warp & 3, et = ew * 32 + lane;
    float myla[LOC];  // this lane's candidates, ascending (approx, row)
    uint32_t myli[LOC];
#pragma unroll
    for (int j = 0; j < LOC; j++) {
      myla[j] = INFINITY;
      myli[j] = RBC_DUMMY;
    }
    const uint32_t arow = (MT == 2 ? grp * kBM : 0) + et;  // this thread's row of the item's query tiles
    // keep-best mode when the buffer holds k and four more (the margin keeps
    // the rows left out clear of the k-th distance for the certificate)
    const bool keep = a.keep_k != 0 && a.keep_k + 4 <= (uint32_t)LOC && a.drop != nullptr;
    uint32_t ai = 0, bi = 0;
    bool ok = true;
    const uint32_t sl_lanes = a.stage_lanes ? a.stage_lanes : 32u;
    float *mystage = mstage + ((warp - 4) * sl_lanes + lane % sl_lanes) * a.stage_words;
    // merge the buffers of the lanes in `need` into their queries' shortlists:
    // every lane with a staging area at once, each on its own query (a warp
    // with 16 areas takes its lanes in two rounds), or one lane at a time with
    // the whole warp (when shared memory holds no staging areas)
    // cycles (reported by one thread): waiting for row states, for
    // accumulators, merging shortlists
    unsigned long long ep[3] = {0, 0, 0};
    const long long t_all = tclk();
    auto flush = [&](uint32_t need, uint32_t q, uint32_t &nl, float &thv, float dq) {
      const long long tf = tclk();
      if (a.stage_words) {
        for (uint32_t r0 = 0; r0 < 32; r0 += sl_lanes) {
          if (((need >> lane) & 1u) && lane - r0 < sl_lanes) {
            thv = v_threshold(lane_merge<LOC>(a, q, myla, myli, nl, mystage), dq);
            nl = 0;
#pragma unroll
            for (int j = 0; j < LOC; j++) {
              myla[j] = INFINITY;
              myli[j] = RBC_DUMMY;
            }
          }
          __syncwarp();
        }
        ep[2] += tclk() - tf;
        return;
      }
      while (need) {
        const uint32_t l = __ffs(need) - 1;
        need &= need - 1;
        const uint32_t ql = __shfl_sync(0xffffffffu, q, l), nll = __shfl_sync(0xffffffffu, nl, l);
        float th = 0.f;
        // the warp network takes kLocal candidates at a time
#pragma unroll
        for (int h = 0; h < (LOC + kLocal - 1) / kLocal; h++) {
          float ha[kLocal];
          uint32_t hi[kLocal];
#pragma unroll
          for (int j = 0; j < kLocal; j++) {
            ha[j] = h * kLocal + j < LOC ? myla[h * kLocal + j < LOC ? h * kLocal + j : 0] : INFINITY;
            hi[j] = h * kLocal + j < LOC ? myli[h * kLocal + j < LOC ? h * kLocal + j : 0] : RBC_DUMMY;
          }
          const uint32_t nh = min(max((int)nll - h * kLocal, 0), kLocal);
          if (h == 0 || nh > 0) th = warp_publish(a, ql, ha, hi, nh, l);
        }
        if (lane == l) {
          nl = 0;
          thv = v_threshold(th, dq);
#pragma unroll
          for (int j = 0; j < LOC; j++) {
            myla[j] = INFINITY;
            myli[j] = RBC_DUMMY;
          }
        }
      }
      ep[2] += tclk() - tf;
    };
    for (uint32_t it = cta; it < nitems && ok; it += ncta, ai++) {
      const SearchItem item = a.items[it];
      const uint32_t ntiles = (item.np + kBN - 1) / kBN;
      const uint32_t rslot = ai & 1;
      long long tw = tclk();
      if (!(ok = mbar_wait(&bar_r_full[rslot], (ai >> 1) & 1, a.err))) break;
      ep[0] += tclk() - tw;
      uint32_t q;
      float dq, alpha = -2.f, thv;
      if (FOLD) {
        const RowStateF st = rsf[rslot * 2 * kBM + arow];
        q = st.q;
        dq = st.dq;
        thv = arow < item.nq ? FLT_MAX : -FLT_MAX;  // the first tile's refresh sets it
      } else {
        const RowState st = rs[rslot * 2 * kBM + arow];
        q = st.q;
        dq = st.dq;
        alpha = st.alpha;
        thv = st.thv;
      }
      uint32_t nl = 0;
      bool dropped = false;  // keep-best mode: some row of the item was left out
      // other CTAs tighten the query's shortlist all the time: each tile
      // refreshes the filter with the threshold read one tile earlier (a
      // larger, older value only lets more candidates through), so the read's
      // latency hides behind a tile of work
      float th_next = arow < item.nq ? __uint_as_float(__ldcg(a.sl_theta + q)) : FLT_MAX;
      // candidates among CW values v (32 columns at a time, the row of
      // column e being rbase + e): the values go to a per-thread copy
      // (indexed by the candidate bits), then into the lane's buffer; full
      // buffers are merged by the warp, which tightens the filter, until none
      // are left
      // Keep-best mode: a full buffer keeps the best LOC candidates, its last
      // value tightens the filter, and the merge waits for the item's end.
      auto candidates = [&](auto &r, uint32_t rbase0) {
        constexpr uint32_t CWN = sizeof(r) / sizeof(r[0]);
#pragma unroll
        for (uint32_t h = 0; h < CWN / 32; h++) {
          uint32_t pend = 0;
#pragma unroll
          for (int e = 0; e < 32; e++) pend |= (uint32_t)(__uint_as_float(r[32 * h + e]) <= thv) << e;
          const uint32_t rbase = rbase0 + 32 * h;
          while (__any_sync(0xffffffffu, pend != 0)) {
            while (pend && (keep || nl < (uint32_t)LOC)) {
              const int e = __ffs(pend) - 1;
              pend &= pend - 1;
              // the column's value by a select tree over the registers (an
              // indexed array would live in local memory, whose traffic
              // competes with the MMAs' shared-memory operand reads)
              const float v = select32(r, 32 * h, e);
              if (v <= thv) {
                insert_local<LOC>(myla, myli, dq + v, rbase + e);
                if (nl < (uint32_t)LOC) nl++;
                if (keep && nl == (uint32_t)LOC) {
                  dropped = true;
                  thv = fminf(thv, v_threshold(myla[LOC - 1], dq));
                }
              }
            }
            if (!keep) flush(__ballot_sync(0xffffffffu, pend != 0), q, nl, thv, dq);
          }
        }
      };
      for (uint32_t t = 0; t < ntiles && ok; t++, bi++) {
        if (MT == 1 && (bi & 1u) != grp) continue;
        const float th_now = th_next;
        th_next = arow < item.nq ? __uint_as_float(__ldcg(a.sl_theta + q)) : FLT_MAX;
        const uint32_t p = (uint32_t)(item.p0 + (uint64_t)t * kBN);
        const uint32_t valid = min((uint32_t)kBN, item.np - t * kBN);
        if constexpr (FOLD) {
          if (arow < item.nq) thv = fminf(thv, v_threshold(th_now, dq));
          // v = -2 D <= thv  <=>  D >= -thv / 2 (rounded down: never misses a value)
          const float tD = __fmul_rd(-0.5f, thv);
          // this group's accumulator block of the tile (MT = 2: its query
          // tile; MT = 1: every other tile), kChunk columns at a time
          const uint32_t gq = MT == 2 ? grp : 0u;  // the issuer of this group's blocks
          const uint32_t u = MT * bi + gq, blk = u % kBlocks, j = u / kBlocks;
          tw = tclk();
          if (!(ok = mbar_wait(&bar_bf[blk][gq], (kIssuers == 2 ? j >> 1 : j) & 1, a.err))) {
            if (a.trace && lane == 0)
              a.trace[(size_t)ncta * kTcTraceWords + 6 * kTcTraceEvents + cta * 4 + 2 + grp] =
                  (1ull << 63) | (5ull << 56) | ((unsigned long long)ai << 32) | (bi << 1) | (j & 1);
            break;
          }
          const long long tfull = tclk();
          ep[1] += tfull - tw;
          const bool logu = a.trace && cta == 0 && ew == 0 && lane == 0 && u >= kTcTraceFirst &&
                            u < kTcTraceFirst + kTcTraceEvents;
          long long *evu = logu ? reinterpret_cast<long long *>(a.trace + (size_t)ncta * kTcTraceWords) +
                                      (u - kTcTraceFirst)
                                : nullptr;
          if (evu) evu[2 * kTcTraceEvents] = tfull;
          tc_fence_after();
#pragma unroll 1
          for (uint32_t c = 0; c < kBN / kChunk; c++) {
            uint32_t r[kChunk];
            __syncwarp();
            tmem_ld64(tmem + ((32u * ew) << 16) + blk * kBN + c * kChunk, r);
            tmem_wait_ld();
            // the block goes back to the MMA warp once its last values are in
            // registers, before this chunk's candidates are handled
            if (c == kBN / kChunk - 1) {
              tc_fence_before();
              __syncwarp();
              // the next use of the block is the other issuer's (two issuers)
              if (lane == 0) mbar_arrive(&bar_be[blk][kIssuers == 2 ? 1u - gq : 0u]);
              if (evu) evu[3 * kTcTraceEvents] = clock64();
            }
            // columns past the item's rows hold other rows' values
            const uint32_t c0 = c * kChunk;
            if (valid < c0 + kChunk) {
#pragma unroll
              for (uint32_t j = 0; j < kChunk; j++)
                if (c0 + j >= valid) r[j] = 0xff800000u;  // -inf: v = +inf, never a candidate
            }
            // four independent 3-input max chains, then their max: a short
            // dependency chain between the two reads of the block
            float m4[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
#pragma unroll
            for (uint32_t j = 0; j < kChunk; j += 8)
#pragma unroll
              for (uint32_t i = 0; i < 4; i++)
                m4[i] = fmax3(m4[i], __uint_as_float(r[j + 2 * i]), __uint_as_float(r[j + 2 * i + 1]));
            const float mx = fmaxf(fmaxf(m4[0], m4[1]), fmaxf(m4[2], m4[3]));
            if (!__any_sync(0xffffffffu, mx >= tD)) continue;
#pragma unroll
            for (uint32_t j = 0; j < kChunk; j++) r[j] = __float_as_uint(-2.f * __uint_as_float(r[j]));
            candidates(r, p + c0);
          }
        } else {
          const uint32_t slot = bi % NSLOT;
          if (!(ok = mbar_wait(&bar_t_full[slot], (bi / NSLOT) & 1, a.err))) break;
          if (!(ok = mbar_wait(&bar_x_full[slot], (bi / NSLOT) & 1, a.err))) break;
          if (arow < item.nq) thv = fminf(thv, v_threshold(th_now, dq));
          tc_fence_after();
          const float *xr = xs + slot * kBN;
          const uint32_t taddr = tmem + ((32u * ew) << 16) + (slot * MT + (MT == 2 ? grp : 0)) * ACC * kBN;
          // 32 columns of both accumulators per tensor-memory read: approx,
          // filter, candidates
          constexpr uint32_t CW = 32;
#pragma unroll 1
          for (uint32_t c = 0; c < kBN / CW; c++) {
            uint32_t r[CW], r2[CW];
            __syncwarp();
            tmem_ld32(taddr + c * CW, r);
            tmem_ld32(taddr + kBN + c * CW, r2);
            tmem_wait_ld();
            // v in place of the accumulator values
            float mn = INFINITY;
#pragma unroll
            for (uint32_t j4 = 0; j4 < CW / 4; j4++) {
              const float4 x4 = *reinterpret_cast<const float4 *>(xr + c * CW + 4 * j4);
              const float xw[4] = {x4.x, x4.y, x4.z, x4.w};
#pragma unroll
              for (int e = 0; e < 4; e++) {
                float tv = fmaf(alpha, __uint_as_float(r[4 * j4 + e]), xw[e]);
                tv = fmaf(alpha, __uint_as_float(r2[4 * j4 + e]), tv);
                r[4 * j4 + e] = __float_as_uint(tv);
              }
              mn = fminf(mn, fminf(fminf(__uint_as_float(r[4 * j4]), __uint_as_float(r[4 * j4 + 1])),
                                   fminf(__uint_as_float(r[4 * j4 + 2]), __uint_as_float(r[4 * j4 + 3]))));
            }
            // the slot goes back (to the MMA warp and to warp 2, which then
            // restages its row constants) once the tile's last accumulator
            // read is in registers and its row constants have been read,
            // before this chunk's candidates (and any shortlist merge) are
            // handled
            if (c == kBN / CW - 1) {
              tc_fence_before();
              __syncwarp();
              if (lane == 0) mbar_arrive(&bar_t_empty[slot]);
            }
            if (!__any_sync(0xffffffffu, mn <= thv)) continue;
            candidates(r, p + c * CW);
          }
        }
      }
      if (keep && dropped && arow < item.nq)
        atomicMin(a.drop + q, __float_as_uint(fmaxf(myla[LOC - 1], 0.f)));  // non-negative: bits order
      flush(__ballot_sync(0xffffffffu, nl > 0), q, nl, thv, dq);
      __syncwarp();
      if (lane == 0) mbar_arrive(&bar_r_empty[rslot]);
    }
    if (a.trace && warp == 4 && lane == 0) {
      for (int j = 0; j < 3; j++) a.trace[cta * kTcTraceWords + 11 + j] = ep[j];
      a.trace[cta * kTcTraceWords + 14] = tclk() - t_all;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// One instance: tensor maps and arguments from the launch's parameters.
// PROBE: the split format's probe-round variant (wider candidate buffers).
template <int MT, bool SPLIT, bool PROBE>
__global__ void __launch_bounds__(kThreads, 1)
    tc_search_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const __grid_constant__ TcArgs a) {
  tc_search_body<MT, SPLIT, PROBE>(&tmA, &tmB, a, blockIdx.x, gridDim.x);
}

// Many instances in one launch: CTA blockIdx.x works for the instance whose
// range [cta0, cta0 + ctas) holds it (the table ascends by cta0), on that
// instance's items with that instance's tensor maps and arguments, which a
// host copy wrote to global memory before the launch.
template <int MT, bool SPLIT, bool PROBE>
__global__ void __launch_bounds__(kThreads, 1)
    tc_search_batch_kernel(const TcBatchEntry *__restrict__ tab, uint32_t ninst) {
  uint32_t lo = 0, hi = ninst;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (tab[mid].cta0 <= blockIdx.x)
      lo = mid;
    else
      hi = mid;
  }
  const TcBatchEntry &e = tab[lo];
  if (blockIdx.x < e.cta0 || blockIdx.x - e.cta0 >= e.ctas) return;
  fence_tensormap_acquire(&e.tmA);
  fence_tensormap_acquire(&e.tmB);
  tc_search_body<MT, SPLIT, PROBE>(&e.tmA, &e.tmB, e.a, blockIdx.x - e.cta0, e.ctas);
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

// One warp per row: whether every x' = x - c (FP32) value is exact in BF16,
// and the largest |x'_i| of the list.
__global__ void tc_center_kernel(const float *__restrict__ Xp, uint32_t ld, const uint64_t *__restrict__ off,
                                 uint32_t nr, const float *__restrict__ R, uint64_t n, uint32_t d,
                                 uint32_t *__restrict__ inexact, uint32_t *__restrict__ lmax_bits) {
  const uint64_t p = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (p >= n) return;
  const uint32_t r = list_of(off, nr, p);
  const float *x = Xp + p * ld, *c = R + (uint64_t)r * ld;
  float mx = 0.f;
  uint32_t bad = 0;
  for (uint32_t i = lane; i < d; i += 32) {
    const float v = __fsub_rn(x[i], c[i]);
    bad |= __bfloat162float(__float2bfloat16_rn(v)) != v;
    mx = fmaxf(mx, fabsf(v));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if (lane == 0) {
    if (bad) atomicOr(inexact, 1u);
    atomicMax(lmax_bits + r, __float_as_uint(mx));
  }
}

// mu: the mean of the representatives per coordinate (split format; zero in
// the exact format, whose operands must stay exact), zero past d.
__global__ void tc_mu_kernel(const float *__restrict__ R, uint32_t ld, uint32_t nr, uint32_t d, uint32_t kp,
                             uint32_t format, float *__restrict__ mu) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kp) return;
  double s = 0.0;
  if (format == kTcSplit && i < d)
    for (uint32_t r = 0; r < nr; r++) s += R[(uint64_t)r * ld + i];
  mu[i] = (float)(s / nr);
}

// Per list: the operand scale, a bound on ||x'|| from the list radius (the
// largest member distance, relative error <= gamma_{d+1}) and ||c - mu||.
__global__ void tc_list_params_kernel(const float *__restrict__ R, uint32_t ld, uint32_t nr, uint32_t d,
                                      const float *__restrict__ radius, const uint32_t *__restrict__ lmax_bits,
                                      const float *__restrict__ mu, uint32_t format, float *__restrict__ lscale,
                                      float *__restrict__ lxmax, float *__restrict__ lcnorm) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nr) return;
  const double u = 5.9604644775390625e-08, g = (d + 3) * u / (1.0 - (d + 3) * u);
  lscale[r] = format == kTcSplit ? half_scale(__uint_as_float(lmax_bits[r])) : 1.f;
  lxmax[r] = __double2float_ru(sqrt((double)radius[r] / (1.0 - g)) * (1.0 + g));
  double cc = 0.0;
  for (uint32_t i = 0; i < d; i++) {
    const double t = (double)R[(uint64_t)r * ld + i] - (double)mu[i];
    cc += t * t;
  }
  lcnorm[r] = __double2float_ru(sqrt(cc) * (1.0 + 4.0 * u));
}

// One warp per row of the padded operand: BF16 x' (exact format) or FP16
// hi | lo of s_r x' (split format), and w = ||x'||^2 + 2 (c - mu).x'; rows
// past n are zero.
__global__ void tc_convert_kernel(const float *__restrict__ Xp, uint32_t ld, const uint64_t *__restrict__ off,
                                  uint32_t nr, const float *__restrict__ R, const float *__restrict__ mu, uint64_t n,
                                  uint64_t n_pad, uint32_t d, uint32_t kp, uint32_t format,
                                  const float *__restrict__ lscale, uint16_t *__restrict__ Xh,
                                  float *__restrict__ w) {
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
  float sxx = 0.f, scx = 0.f;
  for (uint32_t i = lane; i < kp; i += 32) {
    const float v = i < d ? __fsub_rn(x[i], c[i]) : 0.f;
    if (i < d) {
      sxx = fmaf(v, v, sxx);
      scx = fmaf(c[i] - mu[i], v, scx);
    }
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
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sxx += __shfl_xor_sync(0xffffffffu, sxx, o);
    scx += __shfl_xor_sync(0xffffffffu, scx, o);
  }
  if (lane == 0) w[p] = sxx + 2.f * scx;
}

// One thread per padded row: the w operand of the BF16 format's folded
// product.  w is split into three BF16 pieces, w1 = bf16(w), w2 = bf16(w -
// w1), w3 = bf16(w - w1 - w2) (both differences exact in FP32), so |w - w1 -
// w2 - w3| <= 2^-24 |w|.  The 16-half row holds w1 w2 w3 0 0 0 0 0 twice; with
// the constant tile's -1/4 at the same places the product is -(w1 + w2 + w3)
// / 2, whichever order the two 8-half chunks take in the swizzled layout.
__global__ void tc_wrows_kernel(const float *__restrict__ w, uint64_t n_pad, uint4 *__restrict__ Wh) {
  const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (p >= n_pad) return;
  const float v = w[p];
  const __nv_bfloat16 b1 = __float2bfloat16_rn(v);
  // a representative's row (w = +inf): D = -inf, never a candidate
  const float r1 = isinf(v) ? 0.f : __fsub_rn(v, __bfloat162float(b1));
  const __nv_bfloat16 b2 = __float2bfloat16_rn(r1);
  const float r2 = __fsub_rn(r1, __bfloat162float(b2));
  const __nv_bfloat16 b3 = __float2bfloat16_rn(r2);
  const uint32_t lo = (uint32_t)__bfloat16_as_ushort(b1) | ((uint32_t)__bfloat16_as_ushort(b2) << 16);
  const uint4 c = make_uint4(lo, (uint32_t)__bfloat16_as_ushort(b3), 0u, 0u);
  Wh[2 * p] = c;
  Wh[2 * p + 1] = c;
}

// One warp per query row (row m is the zero row): the operand row of q - mu,
// its scale, ||q - mu|| and whether some value is not exact in BF16.
__device__ __forceinline__ void tc_query_warp(const float *__restrict__ Q, uint32_t ld, uint64_t m, uint32_t d,
                                              uint32_t kp, uint32_t format, const float *__restrict__ mu,
                                              uint16_t *__restrict__ Qh, float *__restrict__ qscale,
                                              float *__restrict__ qnorm, uint8_t *__restrict__ qinex, uint64_t q,
                                              uint32_t lane) {
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
    const float v = __fsub_rn(x[i], mu[i]);
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
    const float v = i < d ? __fsub_rn(x[i], mu[i]) : 0.f;
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

__global__ void tc_query_kernel(const float *__restrict__ Q, uint32_t ld, uint64_t m, uint32_t d, uint32_t kp,
                                uint32_t format, const float *__restrict__ mu, uint16_t *__restrict__ Qh,
                                float *__restrict__ qscale, float *__restrict__ qnorm, uint8_t *__restrict__ qinex) {
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (q > m) return;
  tc_query_warp(Q, ld, m, d, kp, format, mu, Qh, qscale, qnorm, qinex, q, threadIdx.x & 31);
}

// Both shortlist buffers empty, buffer 0 current, thresholds open, locks free,
// error bounds zero.
__global__ void sl_init_kernel(float *sl_a, uint32_t *sl_row, uint32_t *sel, uint32_t *theta, uint32_t *lock,
                               uint32_t *emax, uint64_t m, uint32_t sl) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < 2 * m * sl) {
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

// One thread per query: the shortlist's current buffer (sel = 0 after
// sl_init_kernel) takes the query's exact top-sl over its probed lists.
// Those rows are exact, so they add nothing to the error bound; a probed row
// left out ranks after the sl-th under (distance, id), hence after every
// shortlist entry's value, which the certificate already covers.
template <bool BATCH>
__global__ void sl_seed_kernel(const __grid_constant__ SlSeedArgs a0, const SlSeedArgs *__restrict__ tab) {
  const SlSeedArgs &a = BATCH ? tab[blockIdx.y] : a0;
  const uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (q >= a.m) return;
  const float *__restrict__ res_d = a.res_d, *__restrict__ seed_a = a.seed_a;
  const uint32_t *__restrict__ res_i = a.res_i, *__restrict__ iperm = a.iperm, *__restrict__ seed_row = a.seed_row;
  const uint32_t kw = a.kw, sl = a.sl, k = a.k;
  float *__restrict__ sl_a = a.sl_a;
  uint32_t *__restrict__ sl_row = a.sl_row, *__restrict__ theta = a.theta, *__restrict__ tau = a.tau,
                        *__restrict__ cap = a.cap;
  const float *rd = res_d + q * kw;
  const uint32_t *ri = res_i + q * kw;
  const float *sa = seed_a + q * sl;
  const uint32_t *sr = seed_row + q * sl;
  float *oa = sl_a + q * sl;
  uint32_t *orow = sl_row + q * sl;
  // two sorted lists (by distance) merged; a row in both (a representative
  // in a probed list) has the same exact distance in both and is kept once
  uint32_t i = 0, j = 0, n = 0;
  while (n < sl) {
    const bool ha = i < sl && ri[i] != RBC_DUMMY, hb = j < sl && sr[j] != RBC_DUMMY;
    if (!ha && !hb) break;
    const float va = ha ? rd[i] : INFINITY, vb = hb ? sa[j] : INFINITY;
    const bool take_a = ha && (!hb || va <= vb);
    const float v = take_a ? va : vb;
    const uint32_t r = take_a ? iperm[ri[i]] : sr[j];
    if (take_a)
      i++;
    else
      j++;
    bool dup = false;
    for (uint32_t t = n; t > 0 && oa[t - 1] == v && !dup; t--) dup = orow[t - 1] == r;
    if (!dup) {
      oa[n] = v;
      orow[n] = r;
      n++;
    }
  }
  for (uint32_t t = n; t < sl; t++) {
    oa[t] = INFINITY;
    orow[t] = RBC_DUMMY;
  }
  const float kth = n >= k ? oa[k - 1] : FLT_MAX;
  float th = n == sl ? oa[sl - 1] : FLT_MAX;
  tau[q] = fbits(kth);
  if (cap) {
    const float c = tau_cap(kth);
    cap[q] = __float_as_uint(c);
    th = fminf(th, c);
  }
  theta[q] = __float_as_uint(th);
}

// The representatives' list-major rows, and w = +inf there (the tensor
// search leaves them to the shortlist seed).
__global__ void rep_mask_kernel(const uint32_t *__restrict__ rep_ids, uint32_t nr, const uint32_t *__restrict__ iperm,
                                float *__restrict__ w, uint32_t *__restrict__ rep_rows) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nr) return;
  const uint32_t p = iperm[rep_ids[r]];
  rep_rows[r] = p;
  w[p] = INFINITY;
}

// One warp per query: its sl (<= 64) nearest representatives under (Dqr,
// representative index).  Each lane keeps the 8 nearest of its own entries
// (sorted, in registers); the lanes' lists then merge into a sorted 64-entry
// warp list (entry 32 w + lane in register w).  That list is exact unless a
// lane that dropped entries holds an 8th entry ahead of the list's last; such
// queries (rare) redo the merge over every 32-wide chunk of Dqr.  The first P
// entries are the query's probed lists (the same (distance, index) order as
// the plain form's probe table).
__device__ __forceinline__ void rep_seed_warp(const float *__restrict__ Dqr, uint32_t nr,
                                              const uint32_t *__restrict__ rep_rows, uint32_t sl,
                                              float *__restrict__ seed_a, uint32_t *__restrict__ seed_row, uint32_t P,
                                              uint32_t *__restrict__ probe, float *__restrict__ probed, uint64_t q,
                                              uint32_t lane) {
  constexpr int L = 8;
  const float *row = Dqr + q * nr;
  float pd[L];
  uint32_t pi[L];
#pragma unroll
  for (int j = 0; j < L; j++) {
    pd[j] = INFINITY;
    pi[j] = RBC_DUMMY;
  }
  // entries lane, lane + 32, ... in turn, read kU at a time so that each
  // lane keeps several loads in flight (the row is read once, from DRAM)
  constexpr int kU = 8;
  uint32_t seen = 0;
  for (uint32_t r0 = 0; r0 < nr; r0 += 32 * kU) {
    float v[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const uint32_t r = r0 + 32 * u + lane;
      v[u] = r < nr ? __ldg(row + r) : INFINITY;
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      float cv = v[u];
      uint32_t ci = r0 + 32 * u + lane;
      if (ci >= nr) break;
      seen++;
      if (!pair_less(cv, ci, pd[L - 1], pi[L - 1])) continue;
#pragma unroll
      for (int j = 0; j < L; j++)
        if (pair_less(cv, ci, pd[j], pi[j])) {
          const float td = pd[j];
          const uint32_t ti = pi[j];
          pd[j] = cv;
          pi[j] = ci;
          cv = td;
          ci = ti;
        }
    }
  }
  float ld[2] = {INFINITY, INFINITY};
  uint32_t li[2] = {RBC_DUMMY, RBC_DUMMY};
  // each lane's j-th entries in turn, while some lane still has one ahead of
  // the list's last (the lanes' lists ascend)
  float wd = INFINITY;
  uint32_t wi = RBC_DUMMY;
#pragma unroll
  for (int j = 0; j < L; j++) {
    if (!__any_sync(0xffffffffu, pair_less(pd[j], pi[j], wd, wi))) break;
    warp_merge_into_w<2>(ld, li, pd[j], pi[j]);
    wd = __shfl_sync(0xffffffffu, ld[1], 31);
    wi = __shfl_sync(0xffffffffu, li[1], 31);
  }
  // a lane that saw more than L entries dropped only entries behind its L-th
  const bool unsure = seen > (uint32_t)L && pair_less(pd[L - 1], pi[L - 1], wd, wi);
  if (__any_sync(0xffffffffu, unsure)) {
    ld[0] = ld[1] = INFINITY;
    li[0] = li[1] = RBC_DUMMY;
    for (uint32_t r0 = 0; r0 < nr; r0 += 32) {
      const uint32_t r = r0 + lane;
      const float v = r < nr ? row[r] : INFINITY;
      const uint32_t id = r < nr ? r : RBC_DUMMY;
      const float td = __shfl_sync(0xffffffffu, ld[1], 31);
      const uint32_t ti = __shfl_sync(0xffffffffu, li[1], 31);
      if (!__any_sync(0xffffffffu, pair_less(v, id, td, ti))) continue;
      warp_merge_into_w<2>(ld, li, v, id);
    }
  }
#pragma unroll
  for (int w = 0; w < 2; w++) {
    const uint32_t j = 32 * w + lane;
    if (j < sl) {
      seed_a[q * sl + j] = li[w] != RBC_DUMMY ? ld[w] : INFINITY;
      seed_row[q * sl + j] = li[w] != RBC_DUMMY ? rep_rows[li[w]] : RBC_DUMMY;
    }
  }
  if (lane < P) {  // P <= 32
    probe[q * P + lane] = li[0];
    probed[q * P + lane] = li[0] != RBC_DUMMY ? ld[0] : FLT_MAX;
  }
}

__global__ void rep_seed_kernel(const float *__restrict__ Dqr, uint64_t m, uint32_t nr,
                                const uint32_t *__restrict__ rep_rows, uint32_t sl, float *__restrict__ seed_a,
                                uint32_t *__restrict__ seed_row, uint32_t P, uint32_t *__restrict__ probe,
                                float *__restrict__ probed) {
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (q >= m) return;
  rep_seed_warp(Dqr, nr, rep_rows, sl, seed_a, seed_row, P, probe, probed, q, threadIdx.x & 31);
}

// Batched set-up of the tensor query (rbc_batch), instance blockIdx.y, one
// warp per query row (row m: the zero operand row): the nearest
// representatives and the probe table, the query's operand row, empty
// shortlists, FP32 probe-round lists and candidate-drop bound; block 0 also
// zeroes the instance's control words and counters.
__global__ void tc_prep_batch_kernel(const TcPrepArgs *__restrict__ tab) {
  const TcPrepArgs &a = tab[blockIdx.y];
  if (blockIdx.x == 0 && threadIdx.x < 16)
    for (int c = 0; c < 4; c++)
      if (a.ctl[c]) a.ctl[c][threadIdx.x] = 0;
  if (blockIdx.x == 0 && threadIdx.x < 4) a.stats[threadIdx.x] = 0;
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (q > a.m) return;
  tc_query_warp(a.Qp, a.ld, a.m, a.d, a.kp, a.format, a.mu, a.Qh, a.qscale, a.qnorm, a.qinex, q, lane);
  if (q == a.m) return;
  rep_seed_warp(a.Dqr, a.nr, a.rep_rows, a.sl, a.seed_a, a.seed_row, a.P, a.probe, a.probed, q, lane);
  for (uint32_t j = lane; j < a.sl; j += 32)
    for (uint64_t b = 0; b < 2; b++) {
      a.sl_a[(b * a.m + q) * a.sl + j] = INFINITY;
      a.sl_row[(b * a.m + q) * a.sl + j] = RBC_DUMMY;
    }
  for (uint32_t j = lane; j < a.kw; j += 32) {
    a.res_d[q * a.kw + j] = FLT_MAX;
    a.res_i[q * a.kw + j] = RBC_DUMMY;
  }
  if (lane == 0) {
    a.sl_sel[q] = 0;
    a.sl_theta[q] = __float_as_uint(FLT_MAX);
    a.sl_lock[q] = 0;
    a.emax[q] = 0;
    a.drop[q] = 0x7F7F7F7Fu;  // a finite float above every distance
    a.tau[q] = __float_as_uint(FLT_MAX);
    a.lock[q] = 0;
  }
}

// Per query: the planning threshold tau = min(tau, predicted) when a
// prediction is given (the speculative plan), then the shortlist cap
// tau (1 + 2^-10) and the shortlist threshold lowered to it.  A row whose
// approx exceeds the cap cannot reach the top k once the final k-th distance
// is at most tau and the error bound at most 2^-10 tau; the certificate
// checks both.
__global__ void cap_kernel(uint32_t *__restrict__ tau, const float *__restrict__ predicted, uint64_t m,
                           uint32_t *__restrict__ cap, uint32_t *__restrict__ theta) {
  const uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (q >= m) return;
  float t = __uint_as_float(tau[q]);
  if (predicted) {
    const float p = predicted[q];
    if (p >= 0.f && p < t) t = p;  // a NaN or negative prediction is ignored
    tau[q] = __float_as_uint(t);
  }
  const float c = t < FLT_MAX ? fminf(__fmul_ru(t, 1.0009765625f), FLT_MAX) : FLT_MAX;
  cap[q] = __float_as_uint(c);
  theta[q] = __float_as_uint(fminf(__uint_as_float(theta[q]), c));
}

__global__ void iperm_kernel(const uint32_t *__restrict__ perm, uint64_t n, uint32_t *__restrict__ iperm) {
  const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (p < n) iperm[perm[p]] = (uint32_t)p;
}

// Exact rerank of each query's shortlist (one warp per query): the k-th exact
// distance as a pruning threshold, or the results and the certificate.
template <int METRIC, bool BATCH>
__global__ void rerank_kernel(const __grid_constant__ RerankArgs a0, const RerankArgs *__restrict__ tab) {
  const RerankArgs &a = BATCH ? tab[blockIdx.y] : a0;
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= a.m) return;
  const float *qrow = a.Q + q * a.ld;
  const uint64_t slot = ((uint64_t)a.sl_sel[q] * a.m + q) * a.sl;
  const float *sa_q = a.sl_a + slot;
  const uint32_t *sr_q = a.sl_row + slot;
  float ld = FLT_MAX, cd = FLT_MAX;
  uint32_t li = RBC_DUMMY, ci = RBC_DUMMY;
  uint32_t valid = 0;
  for (int round = 0; round < 2; round++) {
    const int t = round * 32 + lane;
    float dv = FLT_MAX;
    uint32_t id = RBC_DUMMY;
    if (t < (int)a.sl) {
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
  if (a.tau && lane == 0) {
    const float t = fminf(__uint_as_float(atomicMin(a.tau + q, fbits(kth))), kth);
    if (a.cap_out) {  // the final k-th distance is at most t
      const float c = tau_cap(t);
      a.cap_out[q] = __float_as_uint(c);
      atomicMin(a.theta + q, __float_as_uint(c));
    }
  }
  if (!a.ids && !a.dists) return;
  // certificate: every row searched but not in the shortlist has approx >=
  // T = min(cap, drop, a_last) (a_last only when the shortlist is full:
  // otherwise only the cap and the candidate buffers turned rows away), so
  // its exact distance is >= T - E > kth
  // when certified; rows of pruned lists are beyond the plan's threshold,
  // which must then be at least kth
  bool certified = true;
  const float cap = fminf(a.sl_cap ? __uint_as_float(a.sl_cap[q]) : FLT_MAX,
                          a.drop ? __uint_as_float(a.drop[q]) : FLT_MAX);  // rows left out of buffers too
  const float T = valid == a.sl ? fminf(sa_q[a.sl - 1], cap) : cap;
  if (T < FLT_MAX) {
    const double E = (double)__uint_as_float(a.emax[q]);
    certified = (double)T - E > (double)kth;
  }
  if (a.tplan && !(kth <= __uint_as_float(a.tplan[q]))) certified = false;
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
size_t smem_bytes(uint32_t kb, uint32_t as, uint32_t bs, uint32_t stage_words, uint32_t stage_lanes = 32) {
  const size_t kbh = SPLIT ? 2 * kb : kb;
  const size_t nslot = 4 / (MT * (SPLIT ? 2 : 1));
  const size_t b_stage = kbh * kTile16K + (SPLIT ? 0 : kWTile);
  const size_t consts = SPLIT ? nslot * kBN * 4 : kWTile;  // row constants, or the w product's constant tile
  const size_t states = 2 * 2 * kBM * (SPLIT ? sizeof(RowState) : sizeof(RowStateF));
  return 1024 + (size_t)as * MT * kbh * kTile16K + (size_t)bs * b_stage + consts + states +
         (size_t)kEpiGroups * 4 * stage_lanes * stage_words * 4;
}

template <int MT, bool SPLIT>
size_t plan_stages(TcArgs &a) {
  // Shared-memory plan.  BF16 format with two query tiles (the pruned round):
  // its query tiles live in tensor memory, so one query stage suffices, and
  // three B stages with staging areas for half of each warp's lanes measured
  // faster than two B stages with staging for all (c3: 22.1 against 23.5 ms
  // per launch; the two MMA warps wait on B tiles otherwise).  Otherwise the
  // deepest pipeline that fits with merge staging (2 SL + 1 words) for every
  // epilogue thread -- the lane-parallel shortlist merges matter more than
  // pipeline depth: B depth first (it hides the L2 latency of every tile),
  // then a second query stage (it hides the gather at item starts).
  static const uint32_t pref[][2] = {{2, 4}, {2, 3}, {1, 4}, {1, 3}, {2, 2}, {1, 2}};
  uint32_t as = 0, bs = 0;
  a.stage_lanes = 32;
  if (!SPLIT && MT == 2 && smem_bytes<MT, SPLIT>(a.kb, 1, 3, 2 * a.sl + 1, 16) <= kSmemLimit) {
    as = 1;
    bs = 3;
    a.stage_words = 2 * a.sl + 1;
    a.stage_lanes = 16;
  }
  for (uint32_t sw : {2 * a.sl + 1, 0u}) {
    if (as) break;
    for (const auto &c : pref)
      if (smem_bytes<MT, SPLIT>(a.kb, c[0], c[1], sw) <= kSmemLimit) {
        as = c[0];
        bs = c[1];
        break;
      }
    if (as) a.stage_words = sw;
  }
  // RBC_TC_STAGES="a,b[,s]" overrides the choice (tuning experiments) when it
  // fits: a query stages, b B stages, s staging areas per epilogue warp (32,
  // 16, or 0: without the merge staging, warp merges one lane at a time)
  if (const char *env = std::getenv("RBC_TC_STAGES")) {
    unsigned ea = 0, eb = 0, es = 32;
    const int got = std::sscanf(env, "%u,%u,%u", &ea, &eb, &es);
    const uint32_t lanes = got == 3 ? (es >= 32 || es == 1 ? 32u : es >= 16 ? 16u : 0u) : 32u;
    const uint32_t sw = lanes ? 2 * a.sl + 1 : 0u;
    if (got >= 2 && ea >= 1 && ea <= kMaxA && eb >= 2 && eb <= kMaxB &&
        smem_bytes<MT, SPLIT>(a.kb, ea, eb, sw, lanes) <= kSmemLimit) {
      as = ea;
      bs = eb;
      a.stage_words = sw;
      a.stage_lanes = lanes;
    }
  }
  if (!as) return 0;
  a.a_stages = as;
  a.b_stages = bs;
  return smem_bytes<MT, SPLIT>(a.kb, as, bs, a.stage_words, a.stage_lanes);
}

template <int MT, bool SPLIT, bool PROBE = false>
cudaError_t launch_tc(const CUtensorMap &tmA, const CUtensorMap &tmB, TcArgs a, int grid, cudaStream_t s) {
  const size_t smem = plan_stages<MT, SPLIT>(a);
  if (!smem) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(tc_search_kernel<MT, SPLIT, PROBE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  tc_search_kernel<MT, SPLIT, PROBE><<<grid, kThreads, smem, s>>>(tmA, tmB, a);
  return launched();
}

template <int MT, bool SPLIT, bool PROBE = false>
cudaError_t launch_tc_batch(const TcBatchEntry *tab, uint32_t ninst, uint32_t ctas, size_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(tc_search_batch_kernel<MT, SPLIT, PROBE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  tc_search_batch_kernel<MT, SPLIT, PROBE><<<ctas, kThreads, smem, s>>>(tab, ninst);
  return launched();
}

}  // namespace

// ------------------------------------------------------------------ host side
bool tc_supported(uint32_t dp) { return dp <= 128; }

uint32_t tc_kp(uint32_t d) { return (d + 63) / 64 * 64; }

uint32_t tc_query_tile(uint32_t format) { return format == kTcSplit ? kBM : 2 * kBM; }

namespace {
cudaError_t resolve_encode() {
  if (!g_encode) {
    cudaDriverEntryPointQueryResult qr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void **)&g_encode, 12000,
                                                     cudaEnableDefault, &qr);
    if (e != cudaSuccess) return e;
    if (qr != cudaDriverEntryPointSuccess || !g_encode) return cudaErrorNotSupported;
  }
  return cudaSuccess;
}
}  // namespace

cudaError_t tc_make_map(CUtensorMap *map, const void *ptr, uint64_t rows, uint32_t cols, uint32_t box_rows) {
  cudaError_t e = resolve_encode();
  if (e != cudaSuccess) return e;
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void *>(ptr), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

int tc_build(const float *Xp, const uint32_t *perm, const uint64_t *offsets, const float *R, const float *radius,
             const uint32_t *rep_ids, uint64_t n, uint64_t n_pad, uint32_t nr, uint32_t d, uint32_t ld, uint32_t kp,
             TcBuild *out, uint64_t *bytes, cudaStream_t s) {
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
  tc_center_kernel<<<grid_n, 256, 0, s>>>(Xp, ld, offsets, nr, R, n, d, fl.as<uint32_t>(), lmax.as<uint32_t>());
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
  if (e == cudaSuccess) e = cudaMalloc(&t.mu, kp * 4);
  if (e == cudaSuccess) e = cudaMalloc(&t.iperm, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&t.rep_rows, nr * 4);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_build: tensor-form operands");
  *bytes += xh_bytes + (n_pad + kBN) * 4 + 4ull * nr * 4 + kp * 4 + n * 4;
  iperm_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(perm, n, t.iperm);
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_build: row map");
  tc_mu_kernel<<<(kp + 127) / 128, 128, 0, s>>>(R, ld, nr, d, kp, t.format, t.mu);
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_build: centering vector");
  tc_list_params_kernel<<<(nr + 127) / 128, 128, 0, s>>>(R, ld, nr, d, radius, lmax.as<uint32_t>(), t.mu, t.format,
                                                        t.lscale, t.lxmax, t.lcnorm);
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_build: list parameters");
  tc_convert_kernel<<<(unsigned)((n_pad * 32 + 255) / 256), 256, 0, s>>>(
      Xp, ld, offsets, nr, R, t.mu, n, n_pad, d, kp, t.format, t.lscale, static_cast<uint16_t *>(t.Xh), t.w);
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_build: operand rows");
  rep_mask_kernel<<<(nr + 127) / 128, 128, 0, s>>>(rep_ids, nr, t.iperm, t.w, t.rep_rows);
  if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_build: representative rows");
  if (t.format == kTcExact) {
    // a tile's 128 rows are read whole: kBN rows of padding past n_pad
    if ((e = cudaMalloc(&t.Wh, (n_pad + kBN) * 32)) != cudaSuccess) return cuda_fail(e, "rbc_build: w operand rows");
    *bytes += (n_pad + kBN) * 32;
    tc_wrows_kernel<<<(unsigned)((n_pad + kBN + 255) / 256), 256, 0, s>>>(t.w, n_pad + kBN, static_cast<uint4 *>(t.Wh));
    if ((e = launched()) != cudaSuccess) return cuda_fail(e, "rbc_build: w operand rows");
  }
  return RBC_OK;
}

cudaError_t launch_tc_queries(const float *Q, uint32_t ld, uint64_t m, uint32_t d, uint32_t kp, uint32_t format,
                              const float *mu, void *Qh, float *qscale, float *qnorm, uint8_t *q_inexact,
                              cudaStream_t s) {
  const uint64_t threads = (m + 1) * 32;
  tc_query_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(Q, ld, m, d, kp, format, mu,
                                                                    static_cast<uint16_t *>(Qh), qscale, qnorm,
                                                                    q_inexact);
  return launched();
}

cudaError_t launch_rep_seed(const float *Dqr, uint64_t m, uint32_t nr, const uint32_t *rep_rows, uint32_t sl,
                            float *seed_a, uint32_t *seed_row, uint32_t P, uint32_t *probe, float *probed,
                            cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  if (sl > 64 || P > 32) return cudaErrorInvalidValue;
  const uint64_t threads = m * 32;
  rep_seed_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(Dqr, m, nr, rep_rows, sl, seed_a, seed_row, P,
                                                                    probe, probed);
  return launched();
}

cudaError_t launch_sl_seed(const float *res_d, const uint32_t *res_i, uint32_t kw, const uint32_t *iperm,
                           const float *seed_a, const uint32_t *seed_row, uint64_t m, uint32_t sl, uint32_t k,
                           float *sl_a, uint32_t *sl_row, uint32_t *theta, uint32_t *tau, uint32_t *cap,
                           cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  const SlSeedArgs a{res_d, res_i, kw, iperm, seed_a, seed_row, m, sl, k, sl_a, sl_row, theta, tau, cap};
  sl_seed_kernel<false><<<(unsigned)((m + 127) / 128), 128, 0, s>>>(a, nullptr);
  return launched();
}

cudaError_t launch_sl_seed_batch(const SlSeedArgs *tab, uint32_t ninst, uint64_t m_max, cudaStream_t s) {
  if (ninst == 0 || m_max == 0) return cudaSuccess;
  sl_seed_kernel<true><<<dim3((unsigned)((m_max + 127) / 128), ninst), 128, 0, s>>>(SlSeedArgs{}, tab);
  return launched();
}

cudaError_t launch_tc_prep_batch(const TcPrepArgs *tab, uint32_t ninst, uint64_t m_max, cudaStream_t s) {
  if (ninst == 0) return cudaSuccess;
  const uint64_t threads = (m_max + 1) * 32;
  tc_prep_batch_kernel<<<dim3((unsigned)((threads + 255) / 256), ninst), 256, 0, s>>>(tab);
  return launched();
}

cudaError_t launch_cap(uint32_t *tau, const float *predicted, uint64_t m, uint32_t *cap, uint32_t *theta,
                       cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  cap_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(tau, predicted, m, cap, theta);
  return launched();
}

cudaError_t launch_sl_init(float *sl_a, uint32_t *sl_row, uint32_t *sel, uint32_t *theta, uint32_t *lock,
                           uint32_t *emax, uint64_t m, uint32_t sl, cudaStream_t s) {
  const uint64_t total = std::max<uint64_t>(2 * m * sl, 1);
  sl_init_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(sl_a, sl_row, sel, theta, lock, emax, m, sl);
  return launched();
}

int tc_grid() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

namespace {
// RBC_TC_TRACE set: each launch records where every role's cycles went
// (per-CTA clock64 counters) and prints the CTAs' averages to stderr.  The
// launch then synchronises its stream: profiling runs only, not inside a
// graph capture.
cudaError_t launch_tc_traced(const CUtensorMap &tmA, const CUtensorMap &tmB, TcArgs a, int grid, cudaStream_t s,
                             bool narrow) {
  const size_t words = (size_t)grid * kTcTraceWords + 6 * kTcTraceEvents + (size_t)grid * 4;
  unsigned long long *buf = nullptr;
  cudaError_t e = cudaMallocAsync(&buf, words * 8, s);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(buf, 0, words * 8, s)) != cudaSuccess) return e;
  a.trace = buf;
  const int mt = (a.format == kTcSplit || narrow) ? 1 : 2;
  if (a.format == kTcSplit)
    e = narrow ? launch_tc<1, true, true>(tmA, tmB, a, grid, s) : launch_tc<1, true>(tmA, tmB, a, grid, s);
  else
    e = narrow ? launch_tc<1, false>(tmA, tmB, a, grid, s) : launch_tc<2, false>(tmA, tmB, a, grid, s);
  if (e != cudaSuccess) return e;
  std::vector<unsigned long long> h(words);
  if ((e = cudaMemcpyAsync(h.data(), buf, words * 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  cudaFreeAsync(buf, s);
  {
    // CTA 0's window of blocks: clocks relative to the first issue
    const long long *ev = reinterpret_cast<const long long *>(h.data() + (size_t)grid * kTcTraceWords);
    const long long base = ev[0];
    if (base) {
      std::fprintf(stderr, "tc_events MT=%d (u: issue-start commit full release | B-wait start end)\n",
                   (a.format == kTcSplit || narrow) ? 1 : 2);
      for (uint32_t i = 0; i < kTcTraceEvents; i++) {
        auto rel = [&](int j) { return ev[j * kTcTraceEvents + i] ? ev[j * kTcTraceEvents + i] - base : -1ll; };
        std::fprintf(stderr, "ev %u %lld %lld %lld %lld | %lld %lld\n", kTcTraceFirst + i, rel(0), rel(1), rel(2),
                     rel(3), rel(4), rel(5));
      }
    }
  }
  {
    const unsigned long long *f = h.data() + (size_t)grid * kTcTraceWords + 6 * kTcTraceEvents;
    int shown = 0;
    for (int c = 0; c < grid && shown < 12; c++)
      for (int j = 0; j < 4; j++)
        if (f[c * 4 + j] >> 63) {
          const unsigned long long v = f[c * 4 + j];
          std::fprintf(stderr, "tc_wait_failed cta=%d role=%d site=%llu item=%llu tile=%llu parity=%llu\n", c, j,
                       (v >> 56) & 0x7f, (v >> 32) & 0xffffff, (v & 0xffffffffull) >> 1, v & 1);
          shown++;
        }
  }
  double m[kTcTraceWords] = {0};
  for (int c = 0; c < grid; c++)
    for (uint32_t j = 0; j < kTcTraceWords; j++) m[j] += (double)h[(size_t)c * kTcTraceWords + j] / grid;
  auto pct = [&](int j, int of) { return m[of] > 0 ? 100.0 * m[j] / m[of] : 0.0; };
  std::fprintf(stderr,
               "tc_trace MT=%d format=%u grid=%d | mma: %.0f cyc, wait query %.1f%% prev-item %.1f%% B %.1f%% "
               "slot %.1f%%, %.0f MMAs (%.1f cyc each) | producer: wait stage %.1f%%, %.0f tiles | gather warp: "
               "wait rows %.1f%% stage %.1f%% | epilogue: wait rows %.1f%% acc %.1f%% merge %.1f%% of %.0f cyc\n",
               mt, a.format, grid, m[0], pct(1, 0), pct(2, 0), pct(3, 0), pct(4, 0), m[5],
               m[5] > 0 ? m[0] / m[5] : 0.0, pct(6, 7), m[15], pct(8, 10), pct(9, 10), pct(11, 14), pct(12, 14),
               pct(13, 14), m[14]);
  return cudaSuccess;
}
}  // namespace

cudaError_t launch_tc_search(const CUtensorMap &tmA, const CUtensorMap &tmB, const TcArgs &a, int grid,
                             cudaStream_t s, bool narrow) {
  if (a.kb < 1 || a.kb > 2) return cudaErrorInvalidValue;
  if (a.format != kTcSplit && !a.wh) return cudaErrorInvalidValue;
  static const bool trace = std::getenv("RBC_TC_TRACE") != nullptr;
  if (trace) return launch_tc_traced(tmA, tmB, a, grid, s, narrow);
  if (a.format == kTcSplit)
    return narrow ? launch_tc<1, true, true>(tmA, tmB, a, grid, s) : launch_tc<1, true>(tmA, tmB, a, grid, s);
  return narrow ? launch_tc<1, false>(tmA, tmB, a, grid, s) : launch_tc<2, false>(tmA, tmB, a, grid, s);
}

size_t tc_stage_plan(TcArgs &a, bool narrow) {
  if (a.format == kTcSplit) return plan_stages<1, true>(a);
  return narrow ? plan_stages<1, false>(a) : plan_stages<2, false>(a);
}

cudaError_t launch_tc_search_batch(const TcBatchEntry *tab, uint32_t ninst, uint32_t total_ctas, uint32_t format,
                                   bool narrow, size_t smem, cudaStream_t s) {
  if (ninst == 0 || total_ctas == 0) return cudaSuccess;
  if (smem == 0 || smem > kSmemLimit) return cudaErrorInvalidConfiguration;
  if (format == kTcSplit)
    return narrow ? launch_tc_batch<1, true, true>(tab, ninst, total_ctas, smem, s)
                  : launch_tc_batch<1, true>(tab, ninst, total_ctas, smem, s);
  return narrow ? launch_tc_batch<1, false>(tab, ninst, total_ctas, smem, s)
                : launch_tc_batch<2, false>(tab, ninst, total_ctas, smem, s);
}

cudaError_t launch_rerank(int metric, const RerankArgs &a, cudaStream_t s) {
  if (a.m == 0) return cudaSuccess;
  const uint64_t threads = a.m * 32;
  const unsigned grid = (unsigned)((threads + 255) / 256);
  if (metric == RBC_L1)
    rerank_kernel<RBC_L1, false><<<grid, 256, 0, s>>>(a, nullptr);
  else
    rerank_kernel<RBC_L2, false><<<grid, 256, 0, s>>>(a, nullptr);
  return launched();
}

cudaError_t launch_rerank_batch(int metric, const RerankArgs *tab, uint32_t ninst, uint64_t m_max, cudaStream_t s) {
  if (ninst == 0 || m_max == 0) return cudaSuccess;
  const dim3 grid((unsigned)((m_max * 32 + 255) / 256), ninst);
  if (metric == RBC_L1)
    rerank_kernel<RBC_L1, true><<<grid, 256, 0, s>>>(RerankArgs{}, tab);
  else
    rerank_kernel<RBC_L2, true><<<grid, 256, 0, s>>>(RerankArgs{}, tab);
  return launched();
}

}  // namespace rbc
