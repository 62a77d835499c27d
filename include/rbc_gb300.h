/*
 * rbc_gb300.h -- C ABI of the GB300 Random Ball Cover k-NN engine.
 *
 * Plain C types only (pointers, sizes, status codes) so any FFI can bind it.
 * Every function returns RBC_OK (0) or an RBC_ERR_* code; the message of the
 * last failure on the calling thread is rbc_last_error().  Device pointers
 * (prefix d) must be 16-byte aligned; `stream` is a cudaStream_t passed as
 * void* (NULL = legacy default stream).  Calls on one index handle must not
 * overlap: use one handle per host thread or serialise the calls.
 *
 * The entry points replace the reference's interface as follows (reference
 * file:line in brackets):
 *   rbc_build / rbc_build_host     buildRBC + setupReps   [rbc.h:11, rbc.cu:126-229]
 *   rbc_query / rbc_query_host     kqueryRBC / queryRBC   [rbc.h:12-13, rbc.cu:19-123]
 *   rbc_destroy                    destroyRBC             [rbc.h:14, rbc.cu:363-368]
 *   rbc_brute_knn                  bruteK / bruteSearch   [brute.h:11-13, brute.cu:43-88]
 *   rbc_brute_range_count          bruteRangeCount        [brute.h:10, brute.cu:19-40]
 *   rbc_read_matrix_bin/_text      readData / readDataText [driver.cu:201-245]
 *   rbc_write_neighbors_bin/_text  writeNeighbs           [driver.cu:352-393]
 * The reference's own C++ names and by-value struct signatures are exported
 * too, from rbc.h / brute.h / utils.h in this directory.
 */
#ifndef RBC_GB300_H
#define RBC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define RBC_OK 0
#define RBC_ERR_INVALID 1     /* bad argument (sizes, k, pointers, reps)      */
#define RBC_ERR_CUDA 2        /* a CUDA runtime call or kernel launch failed  */
#define RBC_ERR_NOMEM 3       /* device or host allocation failed             */
#define RBC_ERR_ITER_LIMIT 4  /* a bounded device wait ran out                */
#define RBC_ERR_UNSUPPORTED 5 /* shape outside what this build handles        */
#define RBC_ERR_IO 6          /* file open/read/write failure                 */

/* ---- metrics: the per-coordinate term of defs.h:20-21, summed in order ---- */
#define RBC_L2 0 /* sum of (q-x)^2: squared Euclidean, never square-rooted */
#define RBC_L1 1 /* sum of |q-x|                                           */

#define RBC_KMAX 32 /* neighbours per query of the reference's engine (defs.h:9) */
#define RBC_K_LIMIT 128 /* largest k of rbc_query / rbc_brute_knn; RBC_KMAX for
                           rbc_query_batch, rbc_brute_knn_noalloc and the
                           tensor-core search (wider k there takes the FP32 one) */

/* ---- build flags ---- */
#define RBC_BUILD_PARTITION 1u /* nearest-representative lists for exact search */
#define RBC_BUILD_ONESHOT 2u   /* the reference's lists: s nearest points per rep */
#define RBC_BUILD_BF16 4u      /* half-precision tensor-core operands of the lists:
                                  rows centered on their representative, in BF16
                                  when every value is exact in it, else FP16
                                  hi + lo halves (RBC_TC_* in rbc_index_info)     */
#define RBC_BUILD_F64 8u       /* set (never passed) on indexes built by rbc_build_f64 */

/* ---- tensor-core operand formats (rbc_index_info.tc_format) ---- */
#define RBC_TC_BF16 0u       /* one BF16 product per pair (data exact in BF16)   */
#define RBC_TC_FP16_SPLIT 1u /* three FP16 products (hi.hi + hi.lo + lo.hi)      */

/* ---- query modes ---- */
#define RBC_QUERY_EXACT 0u    /* exact k-NN: triangle-inequality pruning of lists */
#define RBC_QUERY_ONESHOT 1u  /* reference one-shot: only the nearest rep's list  */
#define RBC_QUERY_EXACT_TC 2u /* exact k-NN whose list search runs on the tensor
                                 cores (operands of RBC_BUILD_BF16), an FP32 rerank
                                 of a 40-row shortlist and a certified error bound
                                 (falls back per query when uncertain); L2 only    */
#define RBC_QUERY_ROUTED 0x1000u /* flag for RBC_QUERY_EXACT: search the attached
                                    router's top lists (and the nearest
                                    representative's) before pruning; results stay
                                    exact whatever the router predicts               */

/* ---- synthetic data kinds (counter-based, identical bits on host and GPU) ---- */
#define RBC_SYNTH_UNIFORM 0   /* i.i.d. U[0,1)                                     */
#define RBC_SYNTH_MIXTURE 1   /* isotropic Gaussian mixture, means U[0,1)^d        */
#define RBC_SYNTH_GEOMETRIC 2 /* integer geometric(p=1/21), mean 20, clipped 255   */

typedef struct rbc_index rbc_index; /* opaque handle */

typedef struct {
  uint32_t num_reps;       /* representatives; 1 <= num_reps <= n            */
  uint32_t s;              /* one-shot list length (RBC_BUILD_ONESHOT)        */
  int metric;              /* RBC_L2 or RBC_L1                                */
  uint32_t flags;          /* RBC_BUILD_*; 0 means RBC_BUILD_PARTITION        */
  uint64_t seed;           /* representative sampling seed                    */
  const uint32_t *rep_ids; /* optional host array of num_reps distinct ids    */
} rbc_build_params;

typedef struct {
  uint64_t n;
  uint32_t d, ld, num_reps, s;
  int metric;
  uint32_t flags;
  uint64_t min_list, max_list; /* partition list sizes                  */
  uint64_t device_bytes;       /* device memory held by the index        */
  uint32_t tc_format;          /* RBC_TC_* (with RBC_BUILD_BF16)         */
  uint32_t tc_plain;           /* 1: rbc_autotune_tc found the plain FP32
                                  search faster, and RBC_QUERY_EXACT_TC
                                  calls run it                          */
  uint32_t router_picks;       /* lists routed calls take from the router */
  uint32_t tc_unrouted;        /* 1: rbc_autotune_tc found routed tensor-form
                                  calls faster without the router's picks
                                  (the nearest lists alone), and they skip
                                  the router                             */
  uint64_t tc_probe_cap;       /* rbc_set_tc_probe_cap (0: none)          */
} rbc_index_info;

typedef struct {               /* work done by the last rbc_query on an index */
  uint64_t queries;
  uint64_t rep_pairs;          /* query-to-representative distances           */
  uint64_t lists_probed;       /* (query, list) pairs searched                */
  uint64_t point_pairs;        /* (query, point) distances computed in lists  */
  uint64_t fallback_queries;   /* tensor-core mode: queries recomputed in FP32;
                                  rbc_query_f64: queries searched in double    */
} rbc_query_stats;

const char *rbc_status_string(int status);
const char *rbc_last_error(void);
int rbc_version(void);

/* Build an index over n rows of d floats at dX (row stride ldx >= d floats).
 * The index keeps its own reordered device copy; dX may be freed after. */
int rbc_build(const float *dX, uint64_t n, uint32_t d, uint32_t ldx, const rbc_build_params *params,
              void *stream, rbc_index **out);
/* Same from host memory (the copy to the device is part of the call). */
int rbc_build_host(const float *hX, uint64_t n, uint32_t d, uint32_t ldx,
                   const rbc_build_params *params, rbc_index **out);
int rbc_destroy(rbc_index *index);

int rbc_get_info(const rbc_index *index, rbc_index_info *info);

/* Index files (no counterpart in the reference, whose rbcStruct lives only in
 * device memory, rbc.cu:363-368): build once, query from other processes.
 * The file holds every list structure the index was built with; loading
 * needs no rebuild.  Format: a fixed header (magic "RBCGB300", version,
 * sizes, flags) followed by the arrays, little-endian. */
int rbc_save(const rbc_index *index, const char *path);
int rbc_load(const char *path, rbc_index **out);
/* Copies of the index structure to host memory (for tests and tooling). */
int rbc_get_reps(const rbc_index *index, uint32_t *h_rep_ids /* num_reps */);
int rbc_get_partition(const rbc_index *index, uint64_t *h_offsets /* num_reps+1 */,
                      uint32_t *h_members /* n */, float *h_radius /* num_reps */);
int rbc_get_oneshot(const rbc_index *index, uint32_t *h_lists /* num_reps x s */,
                    uint32_t *h_counts /* num_reps */);

/* k-NN of m queries (rows of d floats, stride ldq).  Results are sorted by
 * (distance, id); row i of dIds/dDists (stride ldo >= k) holds query i.
 * Missing neighbours are (FLT_MAX, 0xFFFFFFFF).  1 <= k <= RBC_K_LIMIT; the
 * tensor-core mode answers k > RBC_KMAX with the FP32 exact search. */
int rbc_query(rbc_index *index, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
              uint32_t *dIds, float *dDists, uint32_t ldo, void *stream);
int rbc_query_host(rbc_index *index, const float *hQ, uint64_t m, uint32_t ldq, uint32_t k,
                   uint32_t mode, uint32_t *hIds, float *hDists, uint32_t ldo);
int rbc_get_query_stats(const rbc_index *index, rbc_query_stats *stats);
/* The queries (indices into that call's batch, increasing) that the last
 * RBC_QUERY_EXACT_TC call on this index answered a second time: recomputed
 * on the FP32 path because the tensor form's certificate left them open,
 * or, in a routed call without a probe round (rbc_set_router with probes =
 * 0), searched again with the probe round because their k-th distance
 * exceeded the prediction.  *count receives how many there were and
 * min(count, cap) of them go to h_ids.  No counterpart in the reference: it
 * lets a caller check those answers on their own. */
int rbc_get_fallback_queries(const rbc_index *index, uint32_t *h_ids, uint64_t cap, uint64_t *count);

/* ---- batched queries over many indexes (no counterpart in the reference) ----
 * Instances (index, device queries, k, outputs) are added, then rbc_batch_run
 * answers all of them exactly: each round plans every FP32 instance, then
 * one persistent search launch serves all their work; tensor-form instances
 * (rbc_batch_add_mode with RBC_QUERY_EXACT_TC, BF16 indexes, k <= 32) run
 * their rounds on the tensor cores the same way, one tensor-search launch
 * per round in which each instance owns a range of CTAs, the queries their
 * certificates leave open searched again on the device (an instance whose
 * index the autotuner set to the plain search, info.tc_plain, runs with the
 * FP32 instances).  The first run captures the
 * whole sequence into a CUDA graph; later runs replay it, so new query
 * values written into the same buffers are answered by one graph launch.
 * Instances must share the metric; m x num_reps <= 2^28 each. */
typedef struct rbc_batch rbc_batch;
int rbc_batch_create(rbc_batch **out);
int rbc_batch_add(rbc_batch *batch, rbc_index *index, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k,
                  uint32_t *dIds, float *dDists, uint32_t ldo);
int rbc_batch_add_mode(rbc_batch *batch, rbc_index *index, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k,
                       uint32_t mode, uint32_t *dIds, float *dDists, uint32_t ldo);
int rbc_batch_run(rbc_batch *batch, void *stream);
int rbc_batch_destroy(rbc_batch *batch);

/* Search tuning of an index: rows per thread of the FP32 list-search tile
 * (tq = 1, 2 or 4; 0 keeps the default) and the longest run of list rows
 * one work item covers.  rbc_autotune times the candidates on sample queries
 * and keeps the fastest; with cache_path non-NULL the choice is stored in
 * and reused from that file, keyed by the index shape. */
int rbc_set_tuning(rbc_index *index, int tq, uint32_t item_rows);
int rbc_autotune(rbc_index *index, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k,
                 const char *cache_path, void *stream);
/* Tuning of the tensor-core form: nearest lists searched in its probe round
 * (1-16; 0 keeps the default, 4; RBC_TC_ROUTER_ONLY: none in routed calls,
 * whose probe round then searches the router's picks alone, and one in
 * others) and how many rows of each probed list the FP32 path searches
 * first (whole lists when shorter; the rest of a longer list goes to the
 * tensor cores; 0 keeps the default, 8192; RBC_TC_PREFIX_NONE: none, the
 * tensor cores search whole probed lists).
 * rbc_autotune_tc times 1, 2, 4, 8 probes (and RBC_TC_ROUTER_ONLY in routed
 * mode) x RBC_TC_PREFIX_NONE, 512, 2048, 8192, 32768 rows on sample
 * queries in the given mode (RBC_QUERY_EXACT_TC, optionally
 * | RBC_QUERY_ROUTED, where it also tries one and two router picks, and the
 * nearest lists without the router, when the router was attached with picks;
 * the last makes routed tensor-form calls skip the router, info.tc_unrouted)
 * and keeps the fastest; it also times the plain FP32
 * search (RBC_QUERY_EXACT with the same routing) and, when that is faster,
 * makes RBC_QUERY_EXACT_TC calls on this index run it (info.tc_plain).
 * rbc_set_tc_tuning selects the tensor form, routed as asked, again; so does
 * attaching a router.  Results never change.
 * rbc_set_tc_probe_cap: the probe round's tensor search takes at most `rows`
 * rows of each probed list past the FP32 prefix (0: all of them); the rest
 * of a longer list is searched after the probe round's threshold update, by
 * the tensor search with two query tiles per B tile.  rbc_autotune_tc tries
 * 32768, 65536 and 131072 rows with its best probe count and with 8 probes
 * once the other knobs are chosen, and keeps one when it is faster. */
#define RBC_TC_ROUTER_ONLY 0xFFu
#define RBC_TC_PREFIX_NONE 0xFFFFFFFFFFFFFFFFull
int rbc_set_tc_tuning(rbc_index *index, uint32_t probes, uint64_t probe_rows);
int rbc_get_tc_tuning(const rbc_index *index, uint32_t *probes, uint64_t *probe_rows);
int rbc_set_tc_probe_cap(rbc_index *index, uint64_t rows);
int rbc_autotune_tc(rbc_index *index, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
                    void *stream);

/* ---- learned list router (no counterpart in the reference) ----
 * An MLP d -> hidden -> hidden -> num_lists (GELU), FP32 master weights with a
 * BF16 copy used by its GEMMs (FP32 accumulation), trained on the GPU with
 * softmax cross-entropy and Adam.  Parameters are one flat FP32 array
 * [W1 (hidden x d), b1, W2 (hidden x hidden), b2, W3 (num_lists x hidden), b3]. */
typedef struct rbc_router rbc_router;
int rbc_router_create(uint32_t d, uint32_t hidden, uint32_t num_lists, uint64_t seed, rbc_router **out);
int rbc_router_destroy(rbc_router *router);
int rbc_router_num_params(const rbc_router *router, uint64_t *count);
int rbc_router_get_params(const rbc_router *router, float *h_params);
int rbc_router_set_params(rbc_router *router, const float *h_params);
/* Mean loss and the gradients of one batch (no update). */
int rbc_router_gradients(rbc_router *router, const float *dQ, uint32_t batch, uint32_t ldq,
                         const uint32_t *dLabels, float *loss, float *h_grads, void *stream);
/* Epochs of Adam over n labelled queries in shuffled batches. */
int rbc_router_train(rbc_router *router, const float *dQ, uint64_t n, uint32_t ldq,
                     const uint32_t *dLabels, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                     float *final_loss, void *stream);
/* Logits of m queries into dLogits (m x num_lists): the inference the routed
 * queries use -- tensor-core GEMMs with BF16 activations when hidden is a
 * multiple of 64, else the training kernels' FP32-activation forward. */
int rbc_router_logits(rbc_router *router, const float *dQ, uint64_t m, uint32_t ldq, float *dLogits,
                      void *stream);
/* The router's P (1..16) most likely lists per query, largest logit first,
 * ties to the lower list: m x P into dLists -- the picks routed queries
 * probe.  With hidden a multiple of 64 and at most 512 the last layer runs
 * fused with the selection on the tensor cores (no logits are formed in
 * memory). */
int rbc_router_top_lists(rbc_router *router, const float *dQ, uint64_t m, uint32_t ldq, uint32_t P,
                         uint32_t *dLists, void *stream);
/* Training labels produced by the RBC: the list owning each query's exact
 * nearest neighbour. */
int rbc_owner_labels(rbc_index *index, const float *dQ, uint64_t m, uint32_t ldq, uint32_t *dLabels,
                     void *stream);
/* Attach (or detach, router = NULL) a router to an index; RBC_QUERY_ROUTED
 * queries then probe its top `probes` (1..7) lists first.  probes = 0 (a
 * router with a distance head): the tensor form skips its probe round and
 * plans with the predicted k-th distance (see below). */
int rbc_set_router(rbc_index *index, rbc_router *router, uint32_t probes);

/* The router's distance head: one more output of the last layer, a
 * regression of the normalised log ratio of the query's k-th neighbour
 * distance to the distance of its nearest representative (which every query
 * computes exactly), trained beside the list classifier (squared error, same
 * Adam steps).  A
 * routed tensor-form query with probes = 0 skips the probe round: it prunes
 * every list with tau = min(prediction, k-th nearest representative), caps
 * each shortlist at tau (1 + 2^-10) and searches.  The answer is accepted
 * only when its exact k-th distance is at most tau (nothing pruned or turned
 * away can then be in the top k); the other queries are answered again by
 * the tensor form with its probe round.  Results stay exact; a good
 * prediction saves the probe round.  No counterpart in the reference.
 * Parameters: as rbc_router_create, with W3 and b3 one row longer (the
 * head's weights last). */
int rbc_router_create_with_distance(uint32_t d, uint32_t hidden, uint32_t num_lists, uint64_t seed,
                                    rbc_router **out);
/* Labels for both heads from one exact k-NN query: the list owning each
 * query's nearest neighbour (dLabels), its k-th distance (dDist, as
 * rbc_query reports distances) and its nearest representative's distance
 * (dNear); any output may be NULL.  k <= 32. */
int rbc_router_labels(rbc_index *index, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k,
                      uint32_t *dLabels, float *dDist, float *dNear, void *stream);
/* Training of both heads on n labelled queries.  The distance targets
 * log(dDist / dNear) are normalised (mean and spread); rows where either
 * distance is zero or not finite train the list head only.  The last 2 % of
 * the rows (when n >= 1000) are held out: the margin added to every
 * prediction is the 99.5th percentile of (target - prediction) over them. */
int rbc_router_train_with_distance(rbc_router *router, const float *dQ, uint64_t n, uint32_t ldq,
                                   const uint32_t *dLabels, const float *dDist, const float *dNear,
                                   uint32_t epochs, uint32_t batch, float lr, uint64_t seed, float *final_loss,
                                   void *stream);
/* Loss and gradients of one batch with both heads; dTargets are the distance
 * head's targets in its own (normalised) units, NaN for none. */
int rbc_router_gradients_with_distance(rbc_router *router, const float *dQ, uint32_t batch, uint32_t ldq,
                                       const uint32_t *dLabels, const float *dTargets, float *loss,
                                       float *h_grads, void *stream);
/* Predicted k-th distances (margin included) of m queries whose nearest
 * representatives are at dNear. */
int rbc_router_predict_distance(rbc_router *router, const float *dQ, uint64_t m, uint32_t ldq, const float *dNear,
                                float *dDist, void *stream);
/* The head's normalisation (log(distance / nearest representative's) =
 * mu + sigma (output + margin)) and
 * margin; the margin can be set (a larger one: fewer queries answered twice,
 * more lists searched). */
int rbc_router_distance_params(const rbc_router *router, float *mu, float *sigma, float *margin);
int rbc_router_set_distance_margin(rbc_router *router, float margin);

/* Benchmark instrumentation (no counterpart in the reference): with profiling
 * on, every list-search kernel launch of a query call is bracketed by CUDA
 * events on the call's stream and its duration is summed. */
typedef struct {
  uint64_t search_launches; /* list-search kernel launches in the last query call */
  double search_ms;         /* their summed duration in milliseconds            */
  /* tensor form: the pruned round's launches alone (the probe round's large
   * lists are the rest of the launches above) and the (query, row) pairs
   * they evaluated; zero for the other forms */
  uint64_t pruned_launches;
  double pruned_ms;
  uint64_t pruned_pairs;
} rbc_profile;
int rbc_set_profiling(rbc_index *index, int enable);
int rbc_get_profile(const rbc_index *index, rbc_profile *profile);
/* Number of kernels this library has launched in this process. */
uint64_t rbc_kernel_launches(void);
/* Exercises the failure path of the kernels' bounded waits without a fault:
 * one kernel waits on an mbarrier nobody arrives on (50 ms limit), one on a
 * lock nobody releases (16,384 attempts); each records its error word and
 * returns.  Both statuses come back as RBC_ERR_ITER_LIMIT, and the context
 * stays usable for the next call. */
int rbc_selftest_bounded_wait(uint32_t *mbar_status, uint32_t *lock_status, void *stream);

/* Brute-force exact k-NN of every query over every database row;
 * 1 <= k <= RBC_K_LIMIT. */
int rbc_brute_knn(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m,
                  uint32_t ldq, uint32_t d, uint32_t k, int metric, uint32_t *dIds, float *dDists,
                  uint32_t ldo, void *stream);
/* Brute-force exact k-NN that allocates no memory (no counterpart in the
 * reference).  For callers that cannot allocate device memory at call time:
 * services whose memory budget is fully reserved up front by their own
 * allocator, latency-bound callers that must not wait on an allocator, and
 * code running inside another allocator's callback.  Results equal
 * rbc_brute_knn's.  Its working memory is one fixed device array of about
 * 2.4 MB, part of the library's device code: CUDA loads that code lazily, so
 * a device gives the array its memory at the library's first call there and
 * keeps it until the process exits.  A call with m = 0 takes the array and
 * looks its address up, nothing else: make one on every device at start-up,
 * before any stream capture.  Limits: m <= 8192 queries per call, d a
 * multiple of 4 and at most 512, ldx == ldq a multiple of 4, dX and dQ
 * 16-byte aligned; other shapes return RBC_ERR_UNSUPPORTED.  All calls share
 * the array, so calls that overlap on the GPU race: order them on one
 * stream. */
int rbc_brute_knn_noalloc(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m,
                          uint32_t ldq, uint32_t d, uint32_t k, int metric, uint32_t *dIds,
                          float *dDists, uint32_t ldo, void *stream);
/* counts[i] = number of database rows with distance strictly below ranges[i]. */
int rbc_brute_range_count(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m,
                          uint32_t ldq, uint32_t d, int metric, const float *dRanges,
                          uint32_t *dCounts, void *stream);

/* ---- double-precision variant: the reference built with real = double
 * (defs.h:27-31, readme.txt:134-152).  Inputs, distances and results are
 * double, equal to the double build's sequential arithmetic (each subtract,
 * multiply and add rounded to double; ties to the lower id).  The FP32 engine
 * searches float-rounded copies for a shortlist of max(2k, k+16) rows per
 * query (at most 128), the shortlist is reranked in double, and a certified
 * error bound proves the double top k lies inside it; a query the bound
 * cannot settle is searched in double over the whole database.  Missing
 * neighbours are (DBL_MAX, 0xFFFFFFFF).  1 <= k <= RBC_K_LIMIT. */
/* Index over n double rows (stride ldx).  Values must be finite and within
 * +-2^56 (else RBC_ERR_UNSUPPORTED); RBC_BUILD_ONESHOT is not available.  The
 * index keeps a double copy of the rows (n x d x 8 bytes) besides the FP32
 * structures; info.flags carries RBC_BUILD_F64.  rbc_query refuses it. */
int rbc_build_f64(const double *dX, uint64_t n, uint32_t d, uint32_t ldx, const rbc_build_params *params,
                  void *stream, rbc_index **out);
/* Exact k-NN in double over an rbc_build_f64 index: mode RBC_QUERY_EXACT or
 * RBC_QUERY_EXACT_TC (optionally | RBC_QUERY_ROUTED) selects the FP32 search
 * behind the shortlists.  rbc_get_query_stats' fallback_queries counts the
 * queries searched in double. */
int rbc_query_f64(rbc_index *index, const double *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
                  uint32_t *dIds, double *dDists, uint32_t ldo, void *stream);
/* Brute-force exact k-NN in double; *open_queries (optional) receives the
 * number of queries searched in double (all of them when a value is outside
 * the float range). */
int rbc_brute_knn_f64(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m, uint32_t ldq,
                      uint32_t d, uint32_t k, int metric, uint32_t *dIds, double *dDists, uint32_t ldo,
                      uint64_t *open_queries, void *stream);
/* counts[i] = number of rows whose double distance is strictly below ranges[i]. */
int rbc_brute_range_count_f64(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m,
                              uint32_t ldq, uint32_t d, int metric, const double *dRanges, uint32_t *dCounts,
                              void *stream);

/* Rows [r0, r0+rows) of a synthetic matrix into dOut (stride ld, padding
 * columns zeroed).  stream_id separates independent draws (database 0,
 * queries 1, ...).  ncomp/sigma_* apply to RBC_SYNTH_MIXTURE. */
int rbc_synth(int kind, uint64_t seed, uint64_t stream_id, uint64_t r0, uint64_t rows, uint32_t d,
              uint32_t ld, float *dOut, uint32_t ncomp, float sigma_lo, float sigma_hi,
              void *stream);

/* Headerless float32 row-major files (driver.cu:201-221): rows x cols values
 * read into a buffer of stride ld; text files hold whitespace-separated
 * numbers (driver.cu:224-245). */
int rbc_read_matrix_bin(const char *path, float *hBuf, uint64_t rows, uint32_t cols, uint32_t ld);
int rbc_read_matrix_text(const char *path, float *hBuf, uint64_t rows, uint32_t cols, uint32_t ld);
int rbc_write_matrix_bin(const char *path, const float *hBuf, uint64_t rows, uint32_t cols,
                         uint32_t ld);
/* Neighbour output (driver.cu:352-393): all m rows of k ids (uint32), then
 * all m rows of k distances (float32); text writes the same order. */
int rbc_write_neighbors_bin(const char *path, const uint32_t *hIds, const float *hDists, uint64_t m,
                            uint32_t k, uint32_t ld);
int rbc_write_neighbors_text(const char *path, const uint32_t *hIds, const float *hDists,
                             uint64_t m, uint32_t k, uint32_t ld);
/* The same formats in the double build (real = double): 8-byte values. */
int rbc_read_matrix_bin_f64(const char *path, double *hBuf, uint64_t rows, uint32_t cols, uint32_t ld);
int rbc_read_matrix_text_f64(const char *path, double *hBuf, uint64_t rows, uint32_t cols, uint32_t ld);
int rbc_write_matrix_bin_f64(const char *path, const double *hBuf, uint64_t rows, uint32_t cols,
                             uint32_t ld);
int rbc_write_neighbors_bin_f64(const char *path, const uint32_t *hIds, const double *hDists, uint64_t m,
                                uint32_t k, uint32_t ld);
int rbc_write_neighbors_text_f64(const char *path, const uint32_t *hIds, const double *hDists,
                                 uint64_t m, uint32_t k, uint32_t ld);

#ifdef __cplusplus
}
#endif

#endif /* RBC_GB300_H */
