// search.cu -- exact list search: the engine's hot kernel.
//
// Counterpart of planKNNKernel / planNNKernel / knnKernel (kernels.cu:15-282
// of the reference): queries are compared against runs of database rows and a
// sorted (dist, id) list of KW = 32, 64 or 128 entries (the smallest width
// >= k) is kept per query.  GB300 design:
//   * persistent CTAs pull SearchItems from a device work counter, so no host
//     round trip sits between the plan and the search and the whole query
//     pipeline can run inside one CUDA graph;
//   * list rows are contiguous (the build reorders the database by list) and
//     are double-buffered into shared memory with cp.async;
//   * a 256-thread CTA computes 16*TQ x 32 distance tiles in registers on the
//     FP32 pipe with the reference's rounding (tile.cuh);
//   * candidates are filtered against the query's current k-th distance and
//     merged into the per-query list with warp-shuffle bitonic networks in
//     place of the reference's shared-memory Batcher network (kernels.cu:479-625);
//   * each CTA merges its lists into the global per-query lists under a short
//     per-query lock whose wait is bounded (error word, never a hang).
#include <algorithm>

#include "kernels.cuh"
#include "tile.cuh"

namespace rbc {

namespace {

constexpr uint32_t kLockSpinLimit = 1u << 22;
// Largest tile that still lets two search CTAs share an SM (228 KB per SM,
// 1 KB reserved per CTA).
constexpr size_t kTwoCtaSmem = 113 * 1024;

struct SearchSmem {
  float *Qs, *Xs0, *Xs1, *cand_d, *list_d, *tau_s;
  uint32_t *cand_i, *list_i, *cand_n;
};

template <int TQ, int W>
__device__ __forceinline__ SearchSmem carve(unsigned char *base, uint32_t S) {
  constexpr int BQ = 16 * TQ, KW = 32 * W;
  SearchSmem sm;
  float *f = reinterpret_cast<float *>(base);
  sm.Qs = f;
  f += BQ * S;
  sm.Xs0 = f;
  f += kTileCols * S;
  sm.Xs1 = f;
  f += kTileCols * S;
  sm.cand_d = f;
  f += BQ * kTileCols;
  sm.list_d = f;
  f += BQ * KW;
  sm.tau_s = f;
  f += BQ;
  uint32_t *u = reinterpret_cast<uint32_t *>(f);
  sm.cand_i = u;
  u += BQ * kTileCols;
  sm.list_i = u;
  u += BQ * KW;
  sm.cand_n = u;
  return sm;
}

size_t smem_bytes(int tq, uint32_t dp, uint32_t kw) {
  const size_t BQ = 16 * (size_t)tq, S = dp + 4;
  size_t floats = BQ * S + 2 * kTileCols * S + BQ * kTileCols + BQ * kw + BQ;
  size_t words = BQ * kTileCols + BQ * kw + BQ;
  return (floats + words) * 4;
}

// The kth entry (0-based) of a KW list held W registers per lane.
template <int W>
__device__ __forceinline__ float list_entry(const float (&ld)[W], uint32_t kth) {
  float v = ld[0];
#pragma unroll
  for (int w = 1; w < W; w++) v = kth >= 32u * w ? ld[w] : v;  // selects, no indexed local array
  return __shfl_sync(0xffffffffu, v, kth & 31);
}

// g holds the work queue; each item's data come from g itself or, in a
// batched launch over many independent indexes, from g.insts[item.inst].
template <int METRIC, int TQ, int W>
__global__ void __launch_bounds__(kTileThreads, 2) search_kernel(const __grid_constant__ SearchArgs g) {
  constexpr int BQ = 16 * TQ, KW = 32 * W;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint32_t s_item;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tq = tid >> 4, tx = tid & 15;
  unsigned long long my_pairs = 0, my_lists = 0;

  for (;;) {
    if (tid == 0) s_item = atomicAdd(g.work, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    if (it >= *g.nitems) break;
    const SearchItem item = g.items[it];
    const SearchArgs &a = g.insts ? g.insts[item.inst] : g;
    const uint32_t S = a.dp + 4;
    const SearchSmem sm = carve<TQ, W>(smem_raw, S);
    const uint32_t kk = a.k;

    // ---- stage the query tile, thresholds and empty lists ----
    for (uint32_t t = tid; t < BQ; t += kTileThreads) {
      float ts = -1.f;  // < 0 marks an inactive slot
      if (t < item.nq) {
        uint32_t q = a.qidx[item.q0 + t];
        float tq_now = __uint_as_float(__ldcg(a.tau + q));
        ts = tq_now;
        if (a.qthr && a.qthr[item.q0 + t] > tq_now) ts = -1.f;  // pruned since planning
      }
      sm.tau_s[t] = ts;
      sm.cand_n[t] = 0;
    }
    for (uint32_t t = tid; t < BQ * KW; t += kTileThreads) {
      sm.list_d[t] = FLT_MAX;
      sm.list_i[t] = RBC_DUMMY;
    }
    __syncthreads();
    const int nactive = __syncthreads_count(tid < BQ && sm.tau_s[tid] >= 0.f);
    if (nactive == 0) continue;
    {
      const uint32_t chunks = a.dp >> 2;
      for (uint32_t t = tid; t < BQ * chunks; t += kTileThreads) {
        uint32_t r = t / chunks, c = t - r * chunks;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r < item.nq && sm.tau_s[r] >= 0.f)
          v = __ldg(reinterpret_cast<const float4 *>(a.Q + (uint64_t)a.qidx[item.q0 + r] * a.ld) + c);
        *reinterpret_cast<float4 *>(sm.Qs + r * S + 4 * c) = v;
      }
    }

    // ---- stream the rows in tiles of 32 ----
    const uint32_t ntiles = (item.np + kTileCols - 1) / kTileCols;
    stage_rows_async(sm.Xs0, S, a.X, a.ld, item.p0, min((uint32_t)kTileCols, item.np), a.dp);
    cp_async_commit();
    for (uint32_t t = 0; t < ntiles; t++) {
      float *cur = (t & 1) ? sm.Xs1 : sm.Xs0;
      float *nxt = (t & 1) ? sm.Xs0 : sm.Xs1;
      if (t + 1 < ntiles) {
        uint32_t r0 = (t + 1) * kTileCols;
        stage_rows_async(nxt, S, a.X, a.ld, item.p0 + r0, min((uint32_t)kTileCols, item.np - r0), a.dp);
      }
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();

      const uint32_t base = t * kTileCols;
      const uint32_t valid = min((uint32_t)kTileCols, item.np - base);
      float acc[TQ][2];
      tile_distances<METRIC, TQ>(sm.Qs, cur, S, a.dp, tq, tx, acc);
#pragma unroll
      for (int i = 0; i < TQ; i++) {
        const int slot = tq + 16 * i;
        const float thr = sm.tau_s[slot];
#pragma unroll
        for (int j = 0; j < 2; j++) {
          const uint32_t col = tx + 16 * j;
          if (col < valid && thr >= 0.f && acc[i][j] <= thr) {
            uint32_t pos = atomicAdd(&sm.cand_n[slot], 1u);
            uint64_t row = item.p0 + base + col;
            sm.cand_d[slot * kTileCols + pos] = acc[i][j];
            sm.cand_i[slot * kTileCols + pos] = a.pid ? a.pid[row] : (uint32_t)row;
          }
        }
      }
      __syncthreads();

      // ---- merge each slot's candidates into its list (one warp per slot) ----
      for (int slot = warp; slot < BQ; slot += kTileThreads / 32) {
        const uint32_t n = sm.cand_n[slot];
        if (n == 0) continue;
        float ld[W];
        uint32_t li[W];
#pragma unroll
        for (int w = 0; w < W; w++) {
          ld[w] = sm.list_d[slot * KW + 32 * w + lane];
          li[w] = sm.list_i[slot * KW + 32 * w + lane];
        }
        for (uint32_t b = 0; b < n; b += 32) {
          float cd = FLT_MAX;
          uint32_t ci = RBC_DUMMY;
          if (b + lane < n) {
            cd = sm.cand_d[slot * kTileCols + b + lane];
            ci = sm.cand_i[slot * kTileCols + b + lane];
          }
          warp_merge_into_w<W>(ld, li, cd, ci);
        }
#pragma unroll
        for (int w = 0; w < W; w++) {
          sm.list_d[slot * KW + 32 * w + lane] = ld[w];
          sm.list_i[slot * KW + 32 * w + lane] = li[w];
        }
        const float kth = list_entry<W>(ld, kk - 1);
        if (lane == 0) {
          sm.cand_n[slot] = 0;
          if (kth < sm.tau_s[slot]) sm.tau_s[slot] = kth;
        }
      }
      __syncthreads();
    }
    if (tid == 0) {
      my_pairs += (unsigned long long)item.np * nactive;
      my_lists += nactive;
    }

    // ---- publish: merge into the global per-query lists ----
    for (int slot = warp; slot < (int)item.nq; slot += kTileThreads / 32) {
      if (sm.tau_s[slot] < 0.f) continue;
      const uint32_t q = a.qidx[item.q0 + slot];
      // the slot's list cut to k entries (still sorted: the tail is the maximum pair)
      float cd[W];
      uint32_t ci[W];
#pragma unroll
      for (int w = 0; w < W; w++) {
        const bool keep = 32 * w + lane < (int)kk;
        cd[w] = keep ? sm.list_d[slot * KW + 32 * w + lane] : FLT_MAX;
        ci[w] = keep ? sm.list_i[slot * KW + 32 * w + lane] : RBC_DUMMY;
      }
      float first = __shfl_sync(0xffffffffu, cd[0], 0);
      uint32_t first_id = __shfl_sync(0xffffffffu, ci[0], 0);
      float gtau = __shfl_sync(0xffffffffu, __uint_as_float(__ldcg(a.tau + q)), 0);
      if (first_id == RBC_DUMMY || first > gtau) continue;
      int got = 0;
      if (lane == 0) got = lock_bounded(a.lock + q, kLockSpinLimit, g.err);
      got = __shfl_sync(0xffffffffu, got, 0);
      if (!got) continue;
      __threadfence();
      float gd[W];
      uint32_t gi[W];
#pragma unroll
      for (int w = 0; w < W; w++) {
        gd[w] = __ldcg(a.res_d + (uint64_t)q * KW + 32 * w + lane);
        gi[w] = __ldcg(a.res_i + (uint64_t)q * KW + 32 * w + lane);
      }
      warp_merge_lists_w<W>(gd, gi, cd, ci);
#pragma unroll
      for (int w = 0; w < W; w++) {
        a.res_d[(uint64_t)q * KW + 32 * w + lane] = gd[w];
        a.res_i[(uint64_t)q * KW + 32 * w + lane] = gi[w];
      }
      const float kth = list_entry<W>(gd, kk - 1);
      __threadfence();
      if (lane == 0) {
        atomicMin(a.tau + q, fbits(kth));
        __threadfence();
        atomicExch(a.lock + q, 0u);
      }
    }
    __syncthreads();
  }
  if (g.stats && tid == 0 && my_lists) {
    atomicAdd(g.stats, my_pairs);
    atomicAdd(g.stats + 1, my_lists);
  }
}

template <int METRIC, int TQ, int W>
cudaError_t launch_tq(const SearchArgs &a, int grid, cudaStream_t s) {
  size_t smem = smem_bytes(TQ, a.dp, 32 * W);
  cudaError_t e = cudaFuncSetAttribute(search_kernel<METRIC, TQ, W>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  search_kernel<METRIC, TQ, W><<<grid, kTileThreads, smem, s>>>(a);
  return launched();
}

template <int METRIC, int TQ, int W>
int grid_tq(uint32_t dp) {
  size_t smem = smem_bytes(TQ, dp, 32 * W);
  cudaFuncSetAttribute(search_kernel<METRIC, TQ, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  int per_sm = 0, dev = 0, sms = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, search_kernel<METRIC, TQ, W>, kTileThreads,
                                                smem);
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (per_sm < 1) per_sm = 1;
  return per_sm * sms;
}

__global__ void init_results_kernel(float *res_d, uint32_t *res_i, uint32_t *tau, uint32_t *lock,
                                    uint64_t m, uint32_t kw) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < m * kw) {
    res_d[i] = FLT_MAX;
    res_i[i] = RBC_DUMMY;
  }
  if (i < m) {
    tau[i] = fbits(FLT_MAX);
    lock[i] = 0;
  }
}

__global__ void write_results_kernel(const float *res_d, const uint32_t *res_i, uint64_t m, uint32_t k,
                                     uint32_t kw, uint32_t *ids, float *dists, uint32_t ldo) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= m * k) return;
  uint64_t q = i / k;
  uint32_t j = (uint32_t)(i - q * k);
  if (ids) ids[q * ldo + j] = res_i[q * kw + j];
  if (dists) dists[q * ldo + j] = res_d[q * kw + j];
}

// ---------------------------------------------------------------- batched query set-up (rbc_batch)
// instance blockIdx.z of the table
__global__ void batch_pad_kernel(const BatchQuery *tab) {
  const BatchQuery &bq = tab[blockIdx.z];
  const uint64_t total = bq.m * bq.ld;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = i / bq.ld;
    const uint32_t c = (uint32_t)(i - r * bq.ld);
    bq.Qp[i] = c < bq.d ? bq.Q[r * bq.ldq + c] : 0.f;
  }
}

// one warp per query: the nearest representative under (distance, index),
// then the query's empty result list
__global__ void batch_nearest_kernel(const BatchQuery *tab) {
  const BatchQuery &bq = tab[blockIdx.z];
  if (blockIdx.x == 0 && threadIdx.x < 16) bq.ctl[threadIdx.x] = 0;
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (q >= bq.m) return;
  const float *row = bq.Dqr + q * bq.nr;
  float bd = FLT_MAX;
  uint32_t bi = RBC_DUMMY;
  for (uint32_t r = lane; r < bq.nr; r += 32) {
    const float v = row[r];
    if (pair_less(v, r, bd, bi)) {
      bd = v;
      bi = r;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float od = __shfl_xor_sync(0xffffffffu, bd, o);
    const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (pair_less(od, oi, bd, bi)) {
      bd = od;
      bi = oi;
    }
  }
  if (lane == 0) {
    bq.probe[q] = bi;
    bq.probed[q] = bd;
    bq.tau[q] = fbits(FLT_MAX);
    bq.lock[q] = 0;
  }
  for (uint32_t j = lane; j < bq.kw; j += 32) {
    bq.res_d[q * bq.kw + j] = FLT_MAX;
    bq.res_i[q * bq.kw + j] = RBC_DUMMY;
  }
}

__global__ void batch_write_kernel(const BatchQuery *tab) {
  const BatchQuery &bq = tab[blockIdx.z];
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= bq.m * bq.k) return;
  const uint64_t q = i / bq.k;
  const uint32_t j = (uint32_t)(i - q * bq.k);
  if (bq.ids) bq.ids[q * bq.ldo + j] = bq.res_i[q * bq.kw + j];
  if (bq.dists) bq.dists[q * bq.ldo + j] = bq.res_d[q * bq.kw + j];
}

__global__ void scatter_results_kernel(const uint32_t *src_i, const float *src_d, const uint32_t *rows, uint32_t nrows,
                                       uint32_t k, uint32_t *ids, float *dists, uint32_t ldo) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= (uint64_t)nrows * k) return;
  uint32_t r = (uint32_t)(i / k), j = (uint32_t)(i - (uint64_t)r * k);
  if (ids) ids[(uint64_t)rows[r] * ldo + j] = src_i[i];
  if (dists) dists[(uint64_t)rows[r] * ldo + j] = src_d[i];
}

__global__ void brute_items_kernel(SearchItem *items, uint32_t *nitems, uint32_t *qidx, uint64_t n,
                                   uint32_t chunk, uint64_t m, uint32_t qtile) {
  const uint64_t nchunks = (n + chunk - 1) / chunk;
  const uint64_t ntile = (m + qtile - 1) / qtile;
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < m) qidx[i] = (uint32_t)i;
  if (i < nchunks * ntile) {
    uint64_t c = i / ntile, t = i - c * ntile;  // chunk-major: a chunk stays hot in L2
    SearchItem it;
    it.p0 = c * chunk;
    it.np = (uint32_t)min((uint64_t)chunk, n - c * chunk);
    it.list = RBC_DUMMY;
    it.q0 = (uint32_t)(t * qtile);
    it.nq = (uint32_t)min((uint64_t)qtile, m - t * qtile);
    it.inst = 0;
    it.pad = 0;
    items[i] = it;
  }
  if (i == 0) *nitems = (uint32_t)(nchunks * ntile);
}

// Work items of the search over every row for the queries listed first in a
// slot array, their number (*count) known only on the device: every (row
// chunk, tile of listed queries) pair, chunk-major.  A count whose items
// would not fit cap gives no items and records RBC_ERR_NOMEM (the caller
// sizes cap for every query of the batch, so this cannot happen).
__global__ void listed_items_kernel(SearchItem *items, uint32_t *nitems, const uint32_t *count, uint64_t n,
                                    uint32_t chunk, uint32_t qtile, uint64_t cap, uint32_t *err) {
  const uint32_t c = *count;
  const uint64_t nchunks = (n + chunk - 1) / chunk, ntile = (c + (uint64_t)qtile - 1) / qtile;
  const uint64_t total = nchunks * ntile;
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i == 0) {
    *nitems = total <= cap ? (uint32_t)total : 0u;
    if (total > cap) atomicMax(err, (uint32_t)RBC_ERR_NOMEM);
  }
  if (total > cap || i >= total) return;
  const uint64_t ch = i / ntile, t = i - ch * ntile;
  SearchItem it;
  it.p0 = ch * chunk;
  it.np = (uint32_t)min((uint64_t)chunk, n - ch * chunk);
  it.list = RBC_DUMMY;
  it.q0 = (uint32_t)(t * qtile);
  it.nq = (uint32_t)min((uint64_t)qtile, (uint64_t)c - t * qtile);
  it.inst = 0;
  it.pad = 0;
  items[i] = it;
}

// ids / dists rows of the *count queries listed in rows[] from the per-query lists.
__global__ void listed_results_kernel(const float *res_d, const uint32_t *res_i, uint32_t kw, const uint32_t *rows,
                                      const uint32_t *count, uint64_t cap, uint32_t k, uint32_t *ids, float *dists,
                                      uint32_t ldo) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t r = i / k;
  if (r >= cap || r >= *count) return;
  const uint32_t j = (uint32_t)(i - r * k), q = rows[r];
  if (ids) ids[(uint64_t)q * ldo + j] = res_i[(uint64_t)q * kw + j];
  if (dists) dists[(uint64_t)q * ldo + j] = res_d[(uint64_t)q * kw + j];
}

__global__ void fold_errors_kernel(ErrWords src, uint32_t *dst) {
  uint32_t v = 0;
  for (int i = 0; i < 4; i++)
    if (src.w[i]) v = max(v, *src.w[i]);
  if (v) atomicMax(dst, v);
}

// ---------------------------------------------------------------- batched device fallback (rbc_batch)
// Instance blockIdx.y of the table.  Empty kw-wide lists and open thresholds
// for every query, control words zeroed.
__global__ void listed_init_batch_kernel(const ListedArgs *__restrict__ tab) {
  const ListedArgs &a = tab[blockIdx.y];
  if (blockIdx.x == 0 && threadIdx.x < 16) a.ctl[threadIdx.x] = 0;
  const uint64_t total = a.m * a.kw;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    a.res_d[i] = FLT_MAX;
    a.res_i[i] = RBC_DUMMY;
    if (i % a.kw == 0) {
      a.tau[i / a.kw] = fbits(FLT_MAX);
      a.lock[i / a.kw] = 0;
    }
  }
}

// The work items of the search over every row for the instance's listed
// queries (as listed_items_kernel), grid-stride: the count is usually small.
__global__ void listed_items_batch_kernel(const ListedArgs *__restrict__ tab) {
  const ListedArgs &a = tab[blockIdx.y];
  const uint32_t c = *a.count;
  const uint64_t nchunks = (a.n + a.chunk - 1) / a.chunk, ntile = (c + (uint64_t)a.qtile - 1) / a.qtile;
  const uint64_t total = nchunks * ntile;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.ctl[1] = total <= a.cap ? (uint32_t)total : 0u;
    if (total > a.cap) atomicMax(a.ctl + 2, (uint32_t)RBC_ERR_NOMEM);
  }
  if (total > a.cap) return;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t ch = i / ntile, t = i - ch * ntile;
    SearchItem it;
    it.p0 = ch * a.chunk;
    it.np = (uint32_t)min((uint64_t)a.chunk, a.n - ch * a.chunk);
    it.list = RBC_DUMMY;
    it.q0 = (uint32_t)(t * a.qtile);
    it.nq = (uint32_t)min((uint64_t)a.qtile, (uint64_t)c - t * a.qtile);
    it.inst = 0;
    it.pad = 0;
    a.items[i] = it;
  }
}

// The listed queries' results written over the instance's outputs.
__global__ void listed_results_batch_kernel(const ListedArgs *__restrict__ tab) {
  const ListedArgs &a = tab[blockIdx.y];
  const uint64_t total = min((uint64_t)*a.count, a.m) * a.k;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = i / a.k;
    const uint32_t j = (uint32_t)(i - r * a.k), q = a.rows[r];
    if (a.ids) a.ids[(uint64_t)q * a.ldo + j] = a.res_i[(uint64_t)q * a.kw + j];
    if (a.dists) a.dists[(uint64_t)q * a.ldo + j] = a.res_d[(uint64_t)q * a.kw + j];
  }
}

// One thread per table entry: its error words folded into *dst.
__global__ void fold_errors_batch_kernel(const ErrWords *__restrict__ tab, uint32_t n, uint32_t *dst) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  uint32_t v = 0;
  for (int i = 0; i < 4; i++)
    if (tab[e].w[i]) v = max(v, *tab[e].w[i]);
  if (v) atomicMax(dst, v);
}

}  // namespace

cudaError_t launch_fold_errors(ErrWords src, uint32_t *dst, cudaStream_t s) {
  fold_errors_kernel<<<1, 1, 0, s>>>(src, dst);
  return launched();
}

cudaError_t launch_fold_errors_batch(const ErrWords *tab, uint32_t n, uint32_t *dst, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  fold_errors_batch_kernel<<<(n + 127) / 128, 128, 0, s>>>(tab, n, dst);
  return launched();
}

cudaError_t launch_listed_init_batch(const ListedArgs *tab, uint32_t ninst, uint64_t mkw_max, cudaStream_t s) {
  if (ninst == 0 || mkw_max == 0) return cudaSuccess;
  const unsigned grid = (unsigned)std::min<uint64_t>((mkw_max + 255) / 256, 512);
  listed_init_batch_kernel<<<dim3(grid, ninst), 256, 0, s>>>(tab);
  return launched();
}

cudaError_t launch_listed_items_batch(const ListedArgs *tab, uint32_t ninst, cudaStream_t s) {
  if (ninst == 0) return cudaSuccess;
  listed_items_batch_kernel<<<dim3(8, ninst), 256, 0, s>>>(tab);
  return launched();
}

cudaError_t launch_listed_results_batch(const ListedArgs *tab, uint32_t ninst, cudaStream_t s) {
  if (ninst == 0) return cudaSuccess;
  listed_results_batch_kernel<<<dim3(8, ninst), 256, 0, s>>>(tab);
  return launched();
}

cudaError_t launch_listed_items(SearchItem *items, uint32_t *nitems, const uint32_t *count, uint64_t n, uint32_t chunk,
                                uint32_t qtile, uint64_t cap, uint32_t *err, cudaStream_t s) {
  const uint64_t threads = std::max<uint64_t>(cap, 1);
  listed_items_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(items, nitems, count, n, chunk, qtile, cap,
                                                                        err);
  return launched();
}

cudaError_t launch_listed_results(const float *res_d, const uint32_t *res_i, uint32_t kw, const uint32_t *rows,
                                  const uint32_t *count, uint64_t cap, uint32_t k, uint32_t *ids, float *dists,
                                  uint32_t ldo, cudaStream_t s) {
  const uint64_t total = std::max<uint64_t>(cap * k, 1);
  listed_results_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(res_d, res_i, kw, rows, count, cap, k, ids,
                                                                        dists, ldo);
  return launched();
}

// Rows per thread in the query dimension (query tile = 16 TQ).  The default
// keeps the shared-memory tile under ~100 KB; `tq` (1, 2 or 4) overrides it
// when that tile still fits (the autotuner's knob).  Wider lists (kw 64, 128)
// take TQ <= 2, halved further while the tile would keep two CTAs off an SM.
int search_tq_for(uint32_t dp, int tq, uint32_t kw) {
  int t = (tq == 1 || tq == 2 || tq == 4) && (tq == 1 || dp <= 256u / (uint32_t)(tq / 2))
              ? tq
              : (dp <= 128 ? 4 : (dp <= 256 ? 2 : 1));
  if (kw > 32) {
    t = std::min(t, 2);
    while (t > 1 && smem_bytes(t, dp, kw) > kTwoCtaSmem) t /= 2;
  }
  return t;
}
int search_query_tile(uint32_t dp, int tq, uint32_t kw) { return 16 * search_tq_for(dp, tq, kw); }

size_t search_smem_bytes(uint32_t dp, int tq, uint32_t kw) {
  return smem_bytes(search_tq_for(dp, tq, kw), dp, list_width_for(kw));
}

#define RBC_SEARCH_DISPATCH(metric, tqv, w, FN, ...)                                                   \
  do {                                                                                                 \
    if ((w) == 1) {                                                                                    \
      if ((metric) == RBC_L1)                                                                          \
        return (tqv) == 4 ? FN<RBC_L1, 4, 1>(__VA_ARGS__)                                              \
                          : (tqv) == 2 ? FN<RBC_L1, 2, 1>(__VA_ARGS__) : FN<RBC_L1, 1, 1>(__VA_ARGS__); \
      return (tqv) == 4 ? FN<RBC_L2, 4, 1>(__VA_ARGS__)                                                \
                        : (tqv) == 2 ? FN<RBC_L2, 2, 1>(__VA_ARGS__) : FN<RBC_L2, 1, 1>(__VA_ARGS__);   \
    }                                                                                                  \
    if ((w) == 2) {                                                                                    \
      if ((metric) == RBC_L1) return (tqv) == 2 ? FN<RBC_L1, 2, 2>(__VA_ARGS__) : FN<RBC_L1, 1, 2>(__VA_ARGS__); \
      return (tqv) == 2 ? FN<RBC_L2, 2, 2>(__VA_ARGS__) : FN<RBC_L2, 1, 2>(__VA_ARGS__);               \
    }                                                                                                  \
    if ((metric) == RBC_L1) return (tqv) == 2 ? FN<RBC_L1, 2, 4>(__VA_ARGS__) : FN<RBC_L1, 1, 4>(__VA_ARGS__); \
    return (tqv) == 2 ? FN<RBC_L2, 2, 4>(__VA_ARGS__) : FN<RBC_L2, 1, 4>(__VA_ARGS__);                 \
  } while (0)

int search_grid(int metric, uint32_t dp, int tq, uint32_t kw) {
  const uint32_t w = list_width_for(kw) / 32;
  const int tqv = search_tq_for(dp, tq, 32 * w);
  RBC_SEARCH_DISPATCH(metric, tqv, w, grid_tq, dp);
}

cudaError_t launch_search(int metric, const SearchArgs &a, int grid, cudaStream_t s, int tq) {
  const uint32_t w = list_width_for(a.k) / 32;
  const int tqv = search_tq_for(a.dp, tq, 32 * w);
  RBC_SEARCH_DISPATCH(metric, tqv, w, launch_tq, a, grid, s);
}

cudaError_t launch_batch_pad(const BatchQuery *tab, uint32_t ninst, uint64_t elems_max, cudaStream_t s) {
  if (ninst == 0 || elems_max == 0) return cudaSuccess;
  const unsigned grid = (unsigned)std::min<uint64_t>((elems_max + 255) / 256, 1024);
  batch_pad_kernel<<<dim3(grid, 1, ninst), 256, 0, s>>>(tab);
  return launched();
}

cudaError_t launch_batch_nearest(const BatchQuery *tab, uint32_t ninst, uint64_t m_max, cudaStream_t s) {
  if (ninst == 0) return cudaSuccess;
  const unsigned grid = (unsigned)std::max<uint64_t>((m_max * 32 + 255) / 256, 1);
  batch_nearest_kernel<<<dim3(grid, 1, ninst), 256, 0, s>>>(tab);
  return launched();
}

cudaError_t launch_batch_write(const BatchQuery *tab, uint32_t ninst, uint64_t mk_max, cudaStream_t s) {
  if (ninst == 0 || mk_max == 0) return cudaSuccess;
  batch_write_kernel<<<dim3((unsigned)((mk_max + 255) / 256), 1, ninst), 256, 0, s>>>(tab);
  return launched();
}

cudaError_t launch_init_results(float *res_d, uint32_t *res_i, uint32_t *tau, uint32_t *lock,
                                uint64_t m, uint32_t kw, cudaStream_t s) {
  uint64_t total = std::max<uint64_t>(m * kw, 1);
  init_results_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(res_d, res_i, tau, lock, m, kw);
  return launched();
}

cudaError_t launch_write_results(const float *res_d, const uint32_t *res_i, uint64_t m, uint32_t k,
                                 uint32_t kw, uint32_t *ids, float *dists, uint32_t ldo, cudaStream_t s) {
  uint64_t total = m * k;
  if (total == 0) return cudaSuccess;
  write_results_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(res_d, res_i, m, k, kw, ids,
                                                                       dists, ldo);
  return launched();
}

cudaError_t launch_scatter_results(const uint32_t *src_i, const float *src_d, const uint32_t *rows, uint32_t nrows,
                                   uint32_t k, uint32_t *ids, float *dists, uint32_t ldo, cudaStream_t s) {
  uint64_t total = (uint64_t)nrows * k;
  if (total == 0) return cudaSuccess;
  scatter_results_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(src_i, src_d, rows, nrows, k, ids, dists, ldo);
  return launched();
}

cudaError_t launch_brute_items(SearchItem *items, uint32_t *nitems, uint32_t *qidx, uint64_t n,
                               uint32_t chunk, uint64_t m, uint32_t qtile, cudaStream_t s) {
  uint64_t nchunks = (n + chunk - 1) / chunk;
  uint64_t total = nchunks * ((m + qtile - 1) / qtile);
  if (m > total) total = m;
  if (total == 0) total = 1;
  brute_items_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(items, nitems, qidx, n, chunk, m,
                                                                     qtile);
  return launched();
}

}  // namespace rbc
