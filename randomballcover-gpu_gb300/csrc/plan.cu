// plan.cu -- query planning: which (list, query) pairs to search.
//
// The reference plans on the host (computeCounts / buildQMap / idIntersection
// / initCompPlan, rbc.cu:260-440): queries grouped by nearest representative
// are matched to one list each.  Here the plan is built on the device, list
// major, in two rounds:
//   probe round   each query searches the lists of its P nearest
//                 representatives (P = 1 is the reference's one-shot plan);
//   prune round   every other (query, list) pair survives only if its lower
//                 bound on the distance of any list member can still beat the
//                 query's k-th distance after the probe round.
// For list r with radius psi_r (largest member distance) and the query's
// nearest representative r0, any member x obeys
//     D(q,x) >= D(q,r) - psi_r               (ball bound)
//     D(q,x) >= (D(q,r) - c D(q,r0)) / (1+c) (x is closer to r than to r0)
// with D the metric (sqrt of the squared L2 sum, or the L1 sum).  Computed
// distances differ from exact ones by a relative error below
// gamma = (dp+8) 2^-23 (twice the bound for a sequential float sum of dp
// non-negative rounded terms), so every bound is taken on the safe side of
// gamma, c = 1 + 3 gamma covers the owner test being made on computed
// distances, and the final threshold is rounded down to float.  A pair is
// pruned only when that threshold is strictly above the k-th distance, so a
// pruned point can never enter the (dist, id)-ordered result, ties included.
#include "kernels.cuh"
#include "rbc_common.cuh"

namespace rbc {

namespace {

constexpr uint32_t kPlanQueries = 64;  // queries per plan CTA (one rep per thread)

// Per query: the P nearest reps under (dist, rep index), one warp per query.
__global__ void row_topp_kernel(const float *__restrict__ D, uint64_t m, uint32_t nr, uint32_t P,
                                uint32_t *__restrict__ probe, float *__restrict__ probed) {
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (q >= m) return;
  const float *row = D + q * nr;
  float ld[8];
  uint32_t li[8];
#pragma unroll
  for (int p = 0; p < 8; p++) {
    ld[p] = FLT_MAX;
    li[p] = RBC_DUMMY;
  }
  for (uint32_t r = lane; r < nr; r += 32) {
    float v = row[r];
    if (!pair_less(v, r, ld[P - 1], li[P - 1])) continue;
    // insertion into the sorted local list of length P
    float cv = v;
    uint32_t ci = r;
#pragma unroll
    for (int p = 0; p < 8; p++) {
      if (p < (int)P && pair_less(cv, ci, ld[p], li[p])) {
        float td = ld[p];
        uint32_t ti = li[p];
        ld[p] = cv;
        li[p] = ci;
        cv = td;
        ci = ti;
      }
    }
  }
  // P rounds of a warp-wide minimum over the lanes' list heads
  int head = 0;
  for (uint32_t p = 0; p < P; p++) {
    float hd = FLT_MAX;
    uint32_t hi = RBC_DUMMY;
#pragma unroll
    for (int t = 0; t < 8; t++)
      if (t == head) {
        hd = ld[t];
        hi = li[t];
      }
    float bd = hd;
    uint32_t bi = hi;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      float od = __shfl_xor_sync(0xffffffffu, bd, o);
      uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (pair_less(od, oi, bd, bi)) {
        bd = od;
        bi = oi;
      }
    }
    if (hi == bi && hd == bd && bi != RBC_DUMMY) head++;
    if (lane == 0) {
      probe[q * P + p] = bi;
      probed[q * P + p] = bd;
    }
  }
}

// Lower bound on the computed distance of any member of list r, in the
// comparison space (squared L2 or L1), evaluated in FP32 with every operation
// rounded in the safe direction (divisions as products with reciprocals
// rounded the safe way, a fraction of an ulp looser):
//   lo   = D(q,r)/(1+g) (sqrt for L2), rounded down
//   hi0  = D(q,r0)/(1-g) (sqrt for L2), rounded up; c hi0 rounded up is the
//          per-query term chi0 (query_term)
//   hpsi = psi_r/(1-g) (sqrt for L2), rounded up
//   lb   = max(lo - hpsi, (lo - c hi0) / (1 + c)), rounded down
//   thr  = lb^2 (1-g) (L2) or lb (1-g) (L1), rounded down.
__device__ __forceinline__ float query_term(float dq0, const PlanArgs &a) {
  const float t = __fmul_ru(dq0, a.inv_omg_ru);
  return __fmul_ru(a.c_ru, a.metric == RBC_L1 ? t : __fsqrt_ru(t));
}

__device__ __forceinline__ float prune_threshold(float dqr, float chi0, float hpsi, const PlanArgs &a) {
  const float t = __fmul_rd(dqr, a.inv_opg_rd);
  const float lo = a.metric == RBC_L1 ? t : __fsqrt_rd(t);
  const float lb1 = __fsub_rd(lo, hpsi);
  const float num = __fsub_rd(lo, chi0);
  const float lb2 = num > 0.f ? __fmul_rd(num, a.inv_opc_rd) : 0.f;
  const float lb = fmaxf(lb1, lb2);
  if (!(lb > 0.f)) return 0.f;
  return a.metric == RBC_L1 ? __fmul_rd(lb, a.omg_rd) : __fmul_rd(__fmul_rd(lb, lb), a.omg_rd);
}

// A cheaper test that prunes only pairs prune_threshold prunes too, for the
// bulk of them.  With s = sqrt(tau / (1-g)) (L2; tau / (1-g) for L1) and a
// margin m = 1 + 2^-16 on every step: lb > s m gives thr > tau, and lb > s m
// follows from lo > L = min(s m + hpsi, s m (1 + c) + chi0) m, which in turn
// follows from D(q,r) > L^2 (1+g) m (L2; L (1+g) m for L1).  The margins
// exceed every rounding of these float evaluations (a few units in 2^-24
// relative), s is kept at least 1e-18 (L2; 1e-30 for L1) so that lb > s m
// cannot underflow thr to zero, and tau = FLT_MAX (or NaN, which the full
// test never prunes against) gives s = +inf: no pair.
constexpr float kFastMargin = 1.0000152587890625f;  // 1 + 2^-16
__device__ __forceinline__ float fast_s(float tau, const PlanArgs &a) {
  if (!(tau < FLT_MAX)) return INFINITY;
  const float t = __fdiv_ru(tau, a.omg_rd);
  return fmaxf(a.metric == RBC_L1 ? t : __fsqrt_ru(t), a.metric == RBC_L1 ? 1e-30f : 1e-18f) * kFastMargin;
}
// D(q,r) above this value: the pair is pruned (sm = fast_s, lb2 = sm (1 + c) + chi0).
__device__ __forceinline__ float fast_reject(float sm, float lb2, float hpsi, const PlanArgs &a) {
  const float L = fminf(sm + hpsi, lb2) * kFastMargin;
  return (a.metric == RBC_L1 ? L : L * L) * a.opg_ru * kFastMargin;
}

// Bound on the radius term of list r (see prune_threshold), rounded up.
__device__ __forceinline__ float psi_bound(float psi, const PlanArgs &a) {
  const float t = __fdiv_ru(psi, a.omg_rd);
  return a.metric == RBC_L1 ? t : __fsqrt_ru(t);
}

// A batched launch takes instance blockIdx.z's arguments from the table, its
// list counters by phase.
template <bool BATCH>
__device__ __forceinline__ PlanArgs plan_args_of(const PlanArgs &a0, const BatchPlan *tab, uint32_t phase) {
  if (!BATCH) return a0;
  const BatchPlan &bp = tab[blockIdx.z];
  PlanArgs a = bp.a;
  a.phase = phase;
  a.list_cnt = phase == 0 ? bp.cnt : bp.start;
  a.list_cursor = bp.cursor;
  return a;
}

// mode 1: every (query, list) pair except the probed ones whose bound
// survives; pass 0 counts per list, pass 1 writes the list-major entries.
template <bool BATCH>
__global__ void plan_kernel(PlanArgs a0, const BatchPlan *tab, uint32_t phase) {
  __shared__ float s_tau[kPlanQueries], s_chi0[kPlanQueries], s_sm[kPlanQueries], s_lb2[kPlanQueries];
  const PlanArgs a = plan_args_of<BATCH>(a0, tab, phase);
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t q0 = (uint64_t)blockIdx.y * kPlanQueries;
  if (q0 >= a.m) return;  // a batched grid's blocks past this instance's queries
  const uint64_t q1 = min(a.m, q0 + kPlanQueries);
  // the per-query terms, once per block
  for (uint32_t j = threadIdx.x; j < q1 - q0; j += blockDim.x) {
    const float tau = __uint_as_float(a.tau[q0 + j]);
    const float chi0 = query_term(a.dq0 ? a.dq0[q0 + j] : a.probed[(q0 + j) * a.P], a);
    const float sm = fast_s(tau, a);
    s_tau[j] = tau;
    s_chi0[j] = chi0;
    s_sm[j] = sm;
    s_lb2[j] = sm * a.opc_ru * kFastMargin + chi0;
  }
  __syncthreads();
  const bool rv = r < a.nr;
  const bool nonempty = rv && a.offsets[r + 1] > a.offsets[r];
  const float hpsi = rv ? psi_bound(a.radius[r], a) : 0.f;
  uint32_t cnt = 0;
  for (int sweep = 0; sweep < (a.phase == 0 ? 1 : 2); sweep++) {
    uint32_t pos = 0;
    if (sweep == 1) {
      if (cnt == 0) break;
      pos = a.list_cnt[r] + atomicAdd(a.list_cursor + r, cnt);  // list_cnt holds the scanned starts
    }
    for (uint64_t q = q0; q < q1; q++) {
      if (!nonempty) break;
      bool member = false;
      for (uint32_t p = 0; p < a.P_excl; p++) member |= a.probe[q * a.P + p] == r;
      if (member) continue;
      const float dqr = a.Dqr[q * a.nr + r];
      if (dqr > fast_reject(s_sm[q - q0], s_lb2[q - q0], hpsi, a)) continue;  // pruned (by the full bound too)
      const float thr = prune_threshold(dqr, s_chi0[q - q0], hpsi, a);
      if (thr > s_tau[q - q0]) continue;
      if (sweep == 0) {
        cnt++;
      } else {
        a.pair_q[pos] = (uint32_t)q;
        a.pair_thr[pos] = thr;
        pos++;
      }
    }
    if (sweep == 0 && a.phase == 0 && cnt) atomicAdd(a.list_cnt + r, cnt);
  }
}

// mode 0: the probe pairs (q, probe[q][p]) of non-empty lists, each list once
// per query; one thread per probe entry.
template <bool BATCH>
__global__ void plan_probe_kernel(PlanArgs a0, const BatchPlan *tab, uint32_t phase) {
  const PlanArgs a = plan_args_of<BATCH>(a0, tab, phase);
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= a.m * a.P) return;
  const uint64_t q = i / a.P;
  const uint32_t p = (uint32_t)(i - q * a.P);
  const uint32_t r = a.probe[i];
  if (r >= a.nr || a.offsets[r + 1] == a.offsets[r]) return;
  for (uint32_t t = 0; t < p; t++)
    if (a.probe[q * a.P + t] == r) return;
  if (a.phase == 0) {
    atomicAdd(a.list_cnt + r, 1u);
  } else {
    const uint32_t pos = a.list_cnt[r] + atomicAdd(a.list_cursor + r, 1u);
    a.pair_q[pos] = (uint32_t)q;
    a.pair_thr[pos] = 0.f;
  }
}

// The rows of list r the filter's window keeps: [lo, lo + n) list-relative.
__device__ __forceinline__ void row_window(const uint64_t *offsets, uint32_t r, const ListFilter &f, uint64_t &lo,
                                           uint64_t &n) {
  const uint64_t np = offsets[r + 1] - offsets[r];
  lo = min(f.skip, np);
  n = min(np - lo, f.take);
}

// Work items per list: query tiles x row chunks of at most max_rows rows
// (long lists are cut so one item cannot hold up the whole launch).
__device__ __forceinline__ uint32_t row_chunks(const uint64_t *offsets, uint32_t r, uint32_t max_rows,
                                               const ListFilter &f) {
  uint64_t lo, n;
  row_window(offsets, r, f, lo, n);
  return n == 0 ? 1u : (uint32_t)((n + max_rows - 1) / max_rows);
}

// Lists the filter leaves out get no items (nor do lists whose window is
// empty when the window skips rows).
__device__ __forceinline__ bool list_selected(const uint64_t *offsets, const uint32_t *list_cnt, uint32_t r,
                                              const ListFilter &f) {
  const uint64_t np = offsets[r + 1] - offsets[r];
  const uint32_t c = list_cnt[r];
  return np >= f.rows_lo && np < f.rows_hi && c >= f.cnt_lo && c < f.cnt_hi && (f.skip == 0 || np > f.skip);
}

__device__ __forceinline__ void tiles_per_list(const uint32_t *__restrict__ list_cnt,
                                               const uint64_t *__restrict__ offsets, uint32_t nr, uint32_t qtile,
                                               uint32_t max_rows, const ListFilter &f,
                                               uint32_t *__restrict__ tile_cnt, uint32_t r) {
  if (r < nr)
    tile_cnt[r] = list_selected(offsets, list_cnt, r, f)
                      ? (list_cnt[r] + qtile - 1) / qtile * row_chunks(offsets, r, max_rows, f)
                      : 0;
  if (r == nr) tile_cnt[nr] = 0;
}

__global__ void tiles_per_list_kernel(const uint32_t *__restrict__ list_cnt, const uint64_t *__restrict__ offsets,
                                      uint32_t nr, uint32_t qtile, uint32_t max_rows, ListFilter f,
                                      uint32_t *__restrict__ tile_cnt) {
  tiles_per_list(list_cnt, offsets, nr, qtile, max_rows, f, tile_cnt, blockIdx.x * blockDim.x + threadIdx.x);
}

// items for list r: its query tiles x row chunks, in list order.  A plan
// with more items than the buffer holds writes none, records RBC_ERR_NOMEM
// and leaves an empty work list (the caller sizes the buffer so this cannot
// happen; the check keeps every write in bounds regardless).
__device__ __forceinline__ void plan_items(const uint32_t *__restrict__ list_cnt,
                                           const uint32_t *__restrict__ list_start,
                                           const uint32_t *__restrict__ tile_start,
                                           const uint64_t *__restrict__ offsets, uint32_t nr, uint32_t qtile,
                                           uint32_t max_rows, const ListFilter &f, SearchItem *__restrict__ items,
                                           uint64_t cap, uint32_t *__restrict__ nitems, uint32_t *__restrict__ err,
                                           uint32_t r) {
  const uint32_t total = tile_start[nr];
  if (r == nr) {
    *nitems = total <= cap ? total : 0u;
    if (total > cap) raise_error(err, RBC_ERR_NOMEM);
  }
  if (total > cap || r >= nr || !list_selected(offsets, list_cnt, r, f)) return;
  const uint32_t cnt = list_cnt[r];
  const uint32_t nt = (cnt + qtile - 1) / qtile, nc = row_chunks(offsets, r, max_rows, f);
  uint64_t lo, np;
  row_window(offsets, r, f, lo, np);
  const uint64_t p0 = offsets[r] + lo;
  uint32_t slot = tile_start[r];
  for (uint32_t c = 0; c < nc; c++) {
    for (uint32_t t = 0; t < nt; t++) {
      SearchItem it;
      it.p0 = p0 + (uint64_t)c * max_rows;
      it.np = (uint32_t)min((uint64_t)max_rows, np - (uint64_t)c * max_rows);
      it.list = r;
      it.q0 = list_start[r] + t * qtile;
      it.nq = min(qtile, cnt - t * qtile);
      it.inst = 0;
      it.pad = 0;
      items[slot++] = it;
    }
  }
}

__global__ void plan_items_kernel(const uint32_t *__restrict__ list_cnt, const uint32_t *__restrict__ list_start,
                                  const uint32_t *__restrict__ tile_start, const uint64_t *__restrict__ offsets,
                                  uint32_t nr, uint32_t qtile, uint32_t max_rows, ListFilter f,
                                  SearchItem *__restrict__ items, uint64_t cap, uint32_t *__restrict__ nitems,
                                  uint32_t *__restrict__ err) {
  plan_items(list_cnt, list_start, tile_start, offsets, nr, qtile, max_rows, f, items, cap, nitems, err,
             blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------- batched plan rounds (rbc_batch)
// Instance blockIdx.z (blockIdx.y for the one-block scans) of the table.
__global__ void batch_zero_kernel(const BatchPlan *tab) {
  const BatchPlan &bp = tab[blockIdx.z];
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r <= bp.a.nr) {
    bp.cnt[r] = 0;
    bp.cursor[r] = 0;
  }
}

// Exclusive scan of nr + 1 counters, one block per instance, in 256-entry
// steps with a running carry (the lists of one instance number thousands at
// most).
__global__ void batch_scan_kernel(const BatchPlan *tab, uint32_t which) {
  __shared__ uint32_t wsum[8];
  const BatchPlan &bp = tab[blockIdx.y];
  const uint32_t *in = which ? bp.tcnt : bp.cnt;
  uint32_t *out = which ? bp.tstart : bp.start;
  const uint32_t n = bp.a.nr + 1, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t carry = 0;
  for (uint32_t base = 0; base < n; base += 256) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if ((int)lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      uint32_t t = lane < 8 ? wsum[lane] : 0u;
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
        if ((int)lane >= o) t += y;
      }
      if (lane < 8) wsum[lane] = t;
    }
    __syncthreads();
    if (i < n) out[i] = carry + (w ? wsum[w - 1] : 0u) + x - v;
    carry += wsum[7];
    __syncthreads();
  }
}

__global__ void batch_tiles_kernel(const BatchPlan *tab) {
  const BatchPlan &bp = tab[blockIdx.z];
  tiles_per_list(bp.cnt, bp.a.offsets, bp.a.nr, bp.qtile, bp.max_rows, bp.f, bp.tcnt,
                 blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void batch_items_kernel(const BatchPlan *tab) {
  const BatchPlan &bp = tab[blockIdx.z];
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > bp.a.nr) return;
  plan_items(bp.cnt, bp.start, bp.tstart, bp.a.offsets, bp.a.nr, bp.qtile, bp.max_rows, bp.f, bp.items,
             bp.cap, bp.nitems, bp.err, r);
}

}  // namespace

cudaError_t launch_row_topp(const float *D, uint64_t m, uint32_t nr, uint32_t P, uint32_t *probe, float *probed,
                            cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  uint64_t threads = m * 32;
  row_topp_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(D, m, nr, P, probe, probed);
  return launched();
}

// pass 0 (a.phase == 0): list_cnt[r] += surviving pairs; pass 1: fill, with
// a.list_cnt pointing at the scanned list starts and list_cursor zeroed.
cudaError_t launch_plan_pass(const PlanArgs &a, uint32_t mode, cudaStream_t s) {
  if (a.m == 0) return cudaSuccess;
  if (mode == 0) {
    const uint64_t total = a.m * a.P;
    plan_probe_kernel<false><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(a, nullptr, a.phase);
  } else {
    dim3 grid((a.nr + 255) / 256, (unsigned)((a.m + kPlanQueries - 1) / kPlanQueries));
    plan_kernel<false><<<grid, 256, 0, s>>>(a, nullptr, a.phase);
  }
  return launched();
}

cudaError_t launch_plan_batch(const BatchPlan *tab, uint32_t ninst, uint32_t mode, uint32_t nr_max, uint64_t m_max,
                              uint32_t P_max, cudaStream_t s) {
  if (ninst == 0 || m_max == 0) return cudaSuccess;
  const unsigned lists = (nr_max + 1 + 255) / 256;
  batch_zero_kernel<<<dim3(lists, 1, ninst), 256, 0, s>>>(tab);
  cudaError_t e = launched();
  for (uint32_t phase = 0; phase < 2 && e == cudaSuccess; phase++) {
    if (mode == 0) {
      plan_probe_kernel<true><<<dim3((unsigned)((m_max * P_max + 255) / 256), 1, ninst), 256, 0, s>>>(
          PlanArgs{}, tab, phase);
    } else {
      plan_kernel<true><<<dim3((nr_max + 255) / 256, (unsigned)((m_max + kPlanQueries - 1) / kPlanQueries), ninst),
                          256, 0, s>>>(PlanArgs{}, tab, phase);
    }
    if ((e = launched()) != cudaSuccess) break;
    if (phase == 0) {
      batch_scan_kernel<<<dim3(1, ninst), 256, 0, s>>>(tab, 0);
      e = launched();
    }
  }
  if (e != cudaSuccess) return e;
  batch_tiles_kernel<<<dim3(lists, 1, ninst), 256, 0, s>>>(tab);
  if ((e = launched()) != cudaSuccess) return e;
  batch_scan_kernel<<<dim3(1, ninst), 256, 0, s>>>(tab, 1);
  if ((e = launched()) != cudaSuccess) return e;
  batch_items_kernel<<<dim3(lists, 1, ninst), 256, 0, s>>>(tab);
  return launched();
}

cudaError_t launch_tiles_per_list(const uint32_t *list_cnt, const uint64_t *offsets, uint32_t nr, uint32_t qtile,
                                  uint32_t max_rows, ListFilter f, uint32_t *tile_cnt, cudaStream_t s) {
  tiles_per_list_kernel<<<(nr + 1 + 255) / 256, 256, 0, s>>>(list_cnt, offsets, nr, qtile, max_rows, f, tile_cnt);
  return launched();
}

cudaError_t launch_plan_items(const uint32_t *list_cnt, const uint32_t *list_start, const uint32_t *tile_start,
                              const uint64_t *offsets, uint32_t nr, uint32_t qtile, uint32_t max_rows, ListFilter f,
                              SearchItem *items, uint64_t cap, uint32_t *nitems, uint32_t *err, cudaStream_t s) {
  plan_items_kernel<<<(nr + 1 + 255) / 256, 256, 0, s>>>(list_cnt, list_start, tile_start, offsets, nr, qtile,
                                                         max_rows, f, items, cap, nitems, err);
  return launched();
}

}  // namespace rbc
