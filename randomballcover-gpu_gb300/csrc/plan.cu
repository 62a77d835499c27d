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

__device__ __forceinline__ float prune_threshold(float dqr, float dq0, float psi, uint32_t metric,
                                                 double g) {
  const double c = 1.0 + 3.0 * g;
  double lo, hi0, hpsi;
  if (metric == RBC_L1) {
    lo = (double)dqr / (1.0 + g);
    hi0 = (double)dq0 / (1.0 - g);
    hpsi = (double)psi / (1.0 - g);
  } else {
    lo = sqrt((double)dqr / (1.0 + g));
    hi0 = sqrt((double)dq0 / (1.0 - g));
    hpsi = sqrt((double)psi / (1.0 - g));
  }
  double lb = fmax(lo - hpsi, (lo - c * hi0) / (1.0 + c));
  if (!(lb > 0.0)) return 0.f;
  double t = (metric == RBC_L1 ? lb : lb * lb) * (1.0 - g) * (1.0 - 1e-12);
  return __double2float_rd(t);
}

// mode 0: the pairs (q, probe[q][p]); mode 1: all other pairs whose bound
// survives.  pass 0 counts per list, pass 1 writes the list-major entries.
__global__ void plan_kernel(PlanArgs a, uint32_t mode) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t q0 = (uint64_t)blockIdx.y * kPlanQueries;
  const uint64_t q1 = min(a.m, q0 + kPlanQueries);
  const bool rv = r < a.nr;
  const bool nonempty = rv && a.offsets[r + 1] > a.offsets[r];
  const float psi = (rv && mode == 1) ? a.radius[r] : 0.f;
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
      for (uint32_t p = 0; p < a.P; p++) member |= a.probe[q * a.P + p] == r;
      bool surv;
      float thr = 0.f;
      if (mode == 0) {
        surv = member;
      } else {
        surv = !member;
        if (surv) {
          float tau = __uint_as_float(a.tau[q]);
          thr = prune_threshold(a.Dqr[q * a.nr + r], a.probed[q * a.P], psi, a.metric, a.gamma);
          surv = !(thr > tau);
        }
      }
      if (!surv) continue;
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

// Work items per list: query tiles x row chunks of at most max_rows rows
// (long lists are cut so one item cannot hold up the whole launch).
__device__ __forceinline__ uint32_t row_chunks(const uint64_t *offsets, uint32_t r, uint32_t max_rows) {
  const uint64_t np = offsets[r + 1] - offsets[r];
  return np == 0 ? 1u : (uint32_t)((np + max_rows - 1) / max_rows);
}

__global__ void tiles_per_list_kernel(const uint32_t *__restrict__ list_cnt, const uint64_t *__restrict__ offsets,
                                      uint32_t nr, uint32_t qtile, uint32_t max_rows, uint32_t *__restrict__ tile_cnt) {
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nr) tile_cnt[r] = (list_cnt[r] + qtile - 1) / qtile * row_chunks(offsets, r, max_rows);
  if (r == nr) tile_cnt[nr] = 0;
}

// items for list r: its query tiles x row chunks, in list order.
__global__ void plan_items_kernel(const uint32_t *__restrict__ list_cnt, const uint32_t *__restrict__ list_start,
                                  const uint32_t *__restrict__ tile_start, const uint64_t *__restrict__ offsets,
                                  uint32_t nr, uint32_t qtile, uint32_t max_rows, SearchItem *__restrict__ items,
                                  uint32_t *__restrict__ nitems) {
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r == nr) *nitems = tile_start[nr];
  if (r >= nr) return;
  const uint32_t cnt = list_cnt[r];
  const uint32_t nt = (cnt + qtile - 1) / qtile, nc = row_chunks(offsets, r, max_rows);
  const uint64_t p0 = offsets[r], np = offsets[r + 1] - offsets[r];
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

// Counting sort of query indices by key (their nearest list): order[slot] = q.
__global__ void key_hist_kernel(const uint32_t *__restrict__ key, uint32_t stride, uint64_t m,
                                uint32_t *__restrict__ hist) {
  uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (q < m) atomicAdd(hist + key[q * stride], 1u);
}

__global__ void key_scatter_kernel(const uint32_t *__restrict__ key, uint32_t stride, uint64_t m,
                                   const uint32_t *__restrict__ start, uint32_t *__restrict__ cursor,
                                   uint32_t *__restrict__ order, uint32_t *__restrict__ slot_of) {
  uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (q >= m) return;
  const uint32_t k = key[q * stride];
  const uint32_t slot = start[k] + atomicAdd(cursor + k, 1u);
  order[slot] = (uint32_t)q;
  slot_of[q] = slot;
}

// flags[tile][list] = 1 for every surviving (list, query) pair of the plan
// (one block per list) and for every probed (query, list) pair.
__global__ void mark_pairs_kernel(const uint32_t *__restrict__ list_start, const uint32_t *__restrict__ list_cnt,
                                  const uint32_t *__restrict__ pair_q, const uint32_t *__restrict__ slot_of,
                                  uint32_t nr, uint8_t *__restrict__ flags) {
  const uint32_t r = blockIdx.x;
  const uint32_t s0 = list_start[r], c = list_cnt[r];
  for (uint32_t i = threadIdx.x; i < c; i += blockDim.x) flags[(uint64_t)(slot_of[pair_q[s0 + i]] / 128) * nr + r] = 1;
}

__global__ void mark_probes_kernel(const uint32_t *__restrict__ probe, uint64_t m, uint32_t P,
                                   const uint32_t *__restrict__ slot_of, uint32_t nr, uint8_t *__restrict__ flags) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= m * P) return;
  const uint64_t q = i / P;
  const uint32_t r = probe[i];
  if (r < nr) flags[(uint64_t)(slot_of[q] / 128) * nr + r] = 1;
}

}  // namespace

cudaError_t launch_sort_by_key(const uint32_t *key, uint32_t stride, uint64_t m, uint32_t nbins, uint32_t *hist,
                               uint32_t *start, uint32_t *cursor, void *scan_tmp, uint32_t *order, uint32_t *slot_of,
                               cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(hist, 0, (nbins + 1) * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(cursor, 0, (nbins + 1) * 4, s);
  if (e != cudaSuccess) return e;
  key_hist_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(key, stride, m, hist);
  if ((e = launched()) != cudaSuccess) return e;
  if ((e = launch_exclusive_scan(hist, start, nbins + 1, scan_tmp, nullptr, s)) != cudaSuccess) return e;
  key_scatter_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(key, stride, m, start, cursor, order, slot_of);
  return launched();
}

cudaError_t launch_mark_tiles(const uint32_t *list_start, const uint32_t *list_cnt, const uint32_t *pair_q,
                              const uint32_t *probe, uint64_t m, uint32_t P, const uint32_t *slot_of, uint32_t nr,
                              uint8_t *flags, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  if (list_cnt) {
    mark_pairs_kernel<<<nr, 128, 0, s>>>(list_start, list_cnt, pair_q, slot_of, nr, flags);
    if ((e = launched()) != cudaSuccess) return e;
  }
  mark_probes_kernel<<<(unsigned)((m * P + 255) / 256), 256, 0, s>>>(probe, m, P, slot_of, nr, flags);
  return launched();
}

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
  dim3 grid((a.nr + 255) / 256, (unsigned)((a.m + kPlanQueries - 1) / kPlanQueries));
  plan_kernel<<<grid, 256, 0, s>>>(a, mode);
  return launched();
}

cudaError_t launch_tiles_per_list(const uint32_t *list_cnt, const uint64_t *offsets, uint32_t nr, uint32_t qtile,
                                  uint32_t max_rows, uint32_t *tile_cnt, cudaStream_t s) {
  tiles_per_list_kernel<<<(nr + 1 + 255) / 256, 256, 0, s>>>(list_cnt, offsets, nr, qtile, max_rows, tile_cnt);
  return launched();
}

cudaError_t launch_plan_items(const uint32_t *list_cnt, const uint32_t *list_start, const uint32_t *tile_start,
                              const uint64_t *offsets, uint32_t nr, uint32_t qtile, uint32_t max_rows, SearchItem *items,
                              uint32_t *nitems, cudaStream_t s) {
  plan_items_kernel<<<(nr + 1 + 255) / 256, 256, 0, s>>>(list_cnt, list_start, tile_start, offsets, nr, qtile,
                                                         max_rows, items, nitems);
  return launched();
}

}  // namespace rbc
