// kernels.cuh -- launch interface between the host engine and the kernels.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

namespace rbc {

// Kernels launched by this library in this process (benchmark evidence).
inline std::atomic<unsigned long long> g_kernel_launches{0};

// Every launch wrapper ends with this: counts the launch, reports its error.
inline cudaError_t launched() {
  g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

// One unit of list-search work: a contiguous run of database rows searched
// for up to one tile of queries.
struct SearchItem {
  uint64_t p0;    // first row in the (reordered) database
  uint32_t np;    // number of rows
  uint32_t list;  // list (representative) index, or RBC_DUMMY for brute chunks
  uint32_t q0;    // offset of the tile's first query slot in the slot arrays
  uint32_t nq;    // query slots in the tile
  uint32_t inst;  // instance of a batched launch (0 otherwise)
  uint32_t pad;
};

struct SearchArgs {
  const float *X;         // database rows, stride ld, zero-padded to dp
  const uint32_t *pid;    // row -> original id (nullptr: the row itself)
  const float *Q;         // query rows, stride ld, zero-padded to dp
  const uint32_t *qidx;   // query index of every slot
  const float *qthr;      // per-slot pruning threshold or nullptr
  const SearchItem *items;
  const uint32_t *nitems; // device-side item count
  uint32_t *work;         // work counter, zero at launch
  float *res_d;           // per-query lists [m][KW], sorted by (dist, id); KW = list_width_for(k)
  uint32_t *res_i;
  uint32_t *tau;          // per-query k-th distance (float bits)
  uint32_t *lock;         // per-query lock words, zero at rest
  uint32_t *err;          // error word
  unsigned long long *stats;  // [0] (query, point) pairs, [1] (query, list) pairs
  uint32_t ld, dp, k;
  // batched launch: per-instance arguments (device array) indexed by item.inst;
  // the work queue fields (items, nitems, work, err, stats) stay in this struct
  const SearchArgs *insts;
};

// Tile geometry of the list-search kernel for a dimensionality and list
// width kw (32, 64, 128); tq (1, 2, 4) overrides the default rows-per-thread
// when it fits, 0 keeps the default.  launch_search takes kw from a.k.
int search_tq_for(uint32_t dp, int tq = 0, uint32_t kw = 32);
int search_query_tile(uint32_t dp, int tq = 0, uint32_t kw = 32);  // 16 * TQ
size_t search_smem_bytes(uint32_t dp, int tq = 0, uint32_t kw = 32);
cudaError_t launch_search(int metric, const SearchArgs &a, int grid, cudaStream_t s, int tq = 0);
int search_grid(int metric, uint32_t dp, int tq = 0, uint32_t kw = 32);

// Per-query lists of kw entries: m x kw (dist, id) pairs, tau and lock words.
cudaError_t launch_init_results(float *res_d, uint32_t *res_i, uint32_t *tau, uint32_t *lock,
                                uint64_t m, uint32_t kw, cudaStream_t s);
cudaError_t launch_write_results(const float *res_d, const uint32_t *res_i, uint64_t m, uint32_t k,
                                 uint32_t kw, uint32_t *ids, float *dists, uint32_t ldo, cudaStream_t s);
// ids[rows[r] * ldo + j] = src_i[r * k + j] (and the distances likewise).
cudaError_t launch_scatter_results(const uint32_t *src_i, const float *src_d, const uint32_t *rows,
                                   uint32_t nrows, uint32_t k, uint32_t *ids, float *dists, uint32_t ldo,
                                   cudaStream_t s);
cudaError_t launch_brute_items(SearchItem *items, uint32_t *nitems, uint32_t *qidx, uint64_t n,
                               uint32_t chunk, uint64_t m, uint32_t qtile, cudaStream_t s);
// The same over every row for the queries listed first in a slot array, their
// number *count read on the device; at most cap items (RBC_ERR_NOMEM otherwise).
cudaError_t launch_listed_items(SearchItem *items, uint32_t *nitems, const uint32_t *count, uint64_t n, uint32_t chunk,
                                uint32_t qtile, uint64_t cap, uint32_t *err, cudaStream_t s);
// ids[rows[r] * ldo + j] = res_i[rows[r] * kw + j] (and the distances) for r < *count (<= cap).
cudaError_t launch_listed_results(const float *res_d, const uint32_t *res_i, uint32_t kw, const uint32_t *rows,
                                  const uint32_t *count, uint64_t cap, uint32_t k, uint32_t *ids, float *dists,
                                  uint32_t ldo, cudaStream_t s);
// *dst = max(*dst, *src.w[i]) over the non-null src.w[i] (error words folded into one).
struct ErrWords {
  const uint32_t *w[4];
};
cudaError_t launch_fold_errors(ErrWords src, uint32_t *dst, cudaStream_t s);
// Each entry's words folded into *dst (one launch for n entries).
cudaError_t launch_fold_errors_batch(const ErrWords *tab, uint32_t n, uint32_t *dst, cudaStream_t s);
// One instance of a batched device fallback (rbc_batch): the *count queries
// listed first in rows[] searched again over all n database rows.
struct ListedArgs {
  float *res_d;         // m x kw per-query lists, thresholds and locks (reset first)
  uint32_t *res_i, *tau, *lock;
  uint64_t m;
  uint32_t kw;
  uint32_t *ctl;        // 16 control words, zeroed by the reset: [1] items, [2] error
  SearchItem *items;    // (row chunk, tile of listed queries) items, at most cap
  uint64_t n, cap;
  uint32_t chunk, qtile;
  const uint32_t *rows;
  const uint32_t *count;
  uint32_t k, ldo;      // results of the listed queries written to ids / dists
  uint32_t *ids;
  float *dists;
};
// Per instance: the reset (launch_init_results over m x kw entries, control
// words zeroed), the work items (launch_listed_items) and the results
// (launch_listed_results), each one launch over the whole table.
cudaError_t launch_listed_init_batch(const ListedArgs *tab, uint32_t ninst, uint64_t mkw_max, cudaStream_t s);
cudaError_t launch_listed_items_batch(const ListedArgs *tab, uint32_t ninst, cudaStream_t s);
cudaError_t launch_listed_results_batch(const ListedArgs *tab, uint32_t ninst, cudaStream_t s);

// Row-matrix utilities.
cudaError_t launch_pad_rows(const float *src, uint64_t ld_src, float *dst, uint32_t ld_dst,
                            uint64_t rows, uint32_t d, cudaStream_t s);
cudaError_t launch_gather_rows(const float *src, uint32_t ld, const uint32_t *rows, uint64_t n,
                               float *dst, cudaStream_t s);

// Dense distances: D[i][j] = dist(A row i, B row j) for i < na, j < nb.
cudaError_t launch_dense_dist(int metric, const float *A, uint64_t na, const float *B, uint64_t nb,
                              uint32_t ld, uint32_t dp, float *D, uint64_t ldD, cudaStream_t s);
// The same in double, the double build's arithmetic (f64.cu).
cudaError_t launch_dense_dist64(int metric, const double *A, uint64_t na, const double *B, uint64_t nb, uint32_t ld,
                                uint32_t d, double *D, uint64_t ldD, cudaStream_t s);
// Nearest row of B for every row of A under (dist, index).
cudaError_t launch_argmin(int metric, const float *A, uint64_t na, const float *B, uint32_t nb,
                          uint32_t ld, uint32_t dp, uint32_t *best, float *bestd, cudaStream_t s);
// Range counts: counts[i] = #{j : dist(Q_i, X_j) < ranges[i]}.
cudaError_t launch_range_count(int metric, const float *Q, uint64_t m, const float *X, uint64_t n,
                               uint32_t ld, uint32_t dp, const float *ranges, uint32_t *counts,
                               cudaStream_t s);

// Partition build: stable counting sort of row ids by owner.
uint32_t owner_tile_rows();
cudaError_t launch_owner_hist(const uint32_t *owner, uint64_t n, uint32_t nr, uint32_t *hist,
                              uint32_t ntiles, cudaStream_t s);
cudaError_t launch_owner_scatter(const uint32_t *owner, uint64_t n, uint32_t nr,
                                 const uint32_t *hist_scan, uint32_t ntiles, uint32_t *perm,
                                 cudaStream_t s);
cudaError_t launch_list_offsets(const uint32_t *hist_scan, uint32_t nr, uint32_t ntiles, uint64_t n,
                                uint64_t *offsets, cudaStream_t s);
cudaError_t launch_list_radius(const uint64_t *offsets, const uint32_t *perm, const float *odist,
                               uint32_t nr, float *radius, cudaStream_t s);

// Device-wide exclusive scan of 32-bit counts (decoupled look-back).
size_t scan_temp_bytes(uint64_t n);
cudaError_t launch_exclusive_scan(const uint32_t *in, uint32_t *out, uint64_t n, void *temp,
                                  uint32_t *err, cudaStream_t s);

// One-shot lists (the reference's build): exact s-selection per row of a
// rep x point distance block, then compaction in increasing point order.
cudaError_t launch_row_select(const float *D, uint64_t ldD, uint32_t rows, uint64_t n, uint32_t s,
                              uint32_t *thr_bits, uint32_t *need, cudaStream_t st);
cudaError_t launch_row_compact(const float *D, uint64_t ldD, uint32_t rows, uint64_t n,
                               const uint32_t *thr_bits, const uint32_t *need, uint32_t *lists,
                               uint32_t lds, uint32_t *counts, cudaStream_t st);

// Query planning.
cudaError_t launch_row_topp(const float *D, uint64_t m, uint32_t nr, uint32_t P, uint32_t *probe,
                            float *probed, cudaStream_t s);
cudaError_t launch_group_by_list(const uint32_t *probe, uint64_t m, uint32_t P, uint32_t nr,
                                 uint32_t *list_cnt, cudaStream_t s);
struct PlanArgs {
  const float *Dqr;        // m x nr query-to-rep distances (computed form)
  const float *radius;     // nr list radii (computed form, max member distance)
  const uint64_t *offsets; // nr+1 list offsets
  const uint32_t *probe;   // m x P probed lists (first column = nearest rep)
  const float *probed;     // m x P their distances
  const float *dq0;        // per query: distance to its nearest representative (nullptr: probed[q P],
                           // the probe table then starting with the nearest representative)
  const uint32_t *tau;     // per-query k-th distance bits after the probe phase
  uint64_t m;
  uint32_t nr, P, metric, qtile;
  uint32_t P_excl;         // mode 1 leaves out the first P_excl probe-table lists (searched already)
  float opg_ru, omg_rd;    // 1 + gamma rounded up, 1 - gamma rounded down (gamma: relative
                           // error bound of a computed distance)
  float c_ru, opc_ru;      // c = 1 + 3 gamma and 1 + c, rounded up
  float inv_opg_rd, inv_omg_ru, inv_opc_rd;  // 1/(1+gamma) and 1/(1+c) rounded down, 1/(1-gamma) up
  uint32_t *list_cnt;      // nr+1 counters (surviving queries per list)
  uint32_t *list_cursor;   // nr fill cursors
  uint32_t *pair_q;        // list-major surviving (query) entries
  float *pair_thr;         // matching prune thresholds
  uint32_t *tile_cnt;      // nr+1 query tiles per list
  SearchItem *items;
  uint32_t *nitems;
  uint32_t phase;          // 0 = count, 1 = fill
};
// mode 0: the probe pairs (q, probe[q][p]); mode 1: every other pair whose
// pruning bound survives.  a.phase 0 counts per list into a.list_cnt; phase 1
// fills pair_q / pair_thr with a.list_cnt pointing at the scanned starts.
cudaError_t launch_plan_pass(const PlanArgs &a, uint32_t mode, cudaStream_t s);
// One instance of a batched query set-up and result write-back (rbc_batch).
struct BatchQuery {
  const float *Q;        // m rows of d floats, stride ldq
  uint64_t ldq, m;
  float *Qp;             // padded copy, stride ld
  uint32_t ld, d;
  const float *Dqr;      // m x nr query-representative distances
  uint32_t nr;
  uint32_t *probe;       // per query: the nearest representative, and its distance
  float *probed;
  float *res_d;          // per query kw result entries, threshold, lock
  uint32_t *res_i, *tau, *lock;
  uint32_t kw;
  uint32_t *ctl;         // 16 control words, zeroed by the set-up
  uint32_t k, ldo;       // write-back: the first k entries of each list
  uint32_t *ids;
  float *dists;
};
// Padded query copies of every instance in one launch.
cudaError_t launch_batch_pad(const BatchQuery *tab, uint32_t ninst, uint64_t elems_max, cudaStream_t s);
// Every instance's nearest representatives (ties to the lower index, as
// launch_row_topp with P = 1), empty result lists and zeroed control words.
cudaError_t launch_batch_nearest(const BatchQuery *tab, uint32_t ninst, uint64_t m_max, cudaStream_t s);
// Every instance's results written out (as launch_write_results).
cudaError_t launch_batch_write(const BatchQuery *tab, uint32_t ninst, uint64_t mk_max, cudaStream_t s);
// One instance of a batched dense distance block: D (na x nb, row stride ldD)
// = distances of A's rows to B's rows.
struct DenseInst {
  const float *A;
  uint64_t na;
  const float *B;
  uint64_t nb;
  float *D;
  uint64_t ldD;
};
// Every instance of the table in one launch; all share the row stride ld and
// the padded dimension dp (the maxima size the grid).
cudaError_t launch_dense_dist_batch(int metric, const DenseInst *tab, uint32_t ninst, uint64_t na_max,
                                    uint64_t nb_max, uint32_t ld, uint32_t dp, cudaStream_t s);
// Which lists of a plan get work items: rows_lo <= rows < rows_hi and
// cnt_lo <= planned queries < cnt_hi.
// Of each selected list, only rows [skip, skip + take) (list-relative) get
// items; a list with no rows there gets none.
struct ListFilter {
  uint64_t rows_lo = 0, rows_hi = UINT64_MAX;
  uint32_t cnt_lo = 0, cnt_hi = UINT32_MAX;
  uint64_t skip = 0, take = UINT64_MAX;
};
// One instance of a batched plan round (rbc_batch): its plan arguments
// (list_cnt and phase are set per step) and its plan buffers.
struct BatchPlan {
  PlanArgs a;
  uint32_t *cnt, *start, *cursor, *tcnt, *tstart;  // nr + 1 each
  uint32_t qtile, max_rows;
  ListFilter f;  // the lists (and rows of them) that get work items
  SearchItem *items;
  uint64_t cap;
  uint32_t *nitems, *err;
};
// A whole plan round (count, scan, fill, tiles per list, scan, items) of
// every instance in the device table, each step one launch over all of them;
// the maxima size the grids (blocks past an instance's sizes return).
cudaError_t launch_plan_batch(const BatchPlan *tab, uint32_t ninst, uint32_t mode, uint32_t nr_max, uint64_t m_max,
                              uint32_t P_max, cudaStream_t s);
// Items per list: query tiles x chunks of at most max_rows list rows, for
// the lists the filter selects only.
cudaError_t launch_tiles_per_list(const uint32_t *list_cnt, const uint64_t *offsets, uint32_t nr,
                                  uint32_t qtile, uint32_t max_rows, ListFilter f, uint32_t *tile_cnt,
                                  cudaStream_t s);
cudaError_t launch_plan_items(const uint32_t *list_cnt, const uint32_t *list_start,
                              const uint32_t *tile_start, const uint64_t *offsets, uint32_t nr,
                              uint32_t qtile, uint32_t max_rows, ListFilter f, SearchItem *items,
                              uint64_t cap, uint32_t *nitems, uint32_t *err, cudaStream_t s);

// Synthetic data.
cudaError_t launch_synth(int kind, uint64_t seed, uint64_t stream_id, uint64_t r0, uint64_t rows,
                         uint32_t d, uint32_t ld, float *out, uint32_t ncomp, float sigma_lo,
                         float sigma_hi, cudaStream_t s);
void geometric_table(uint32_t num, uint32_t den, uint32_t *T);

}  // namespace rbc
