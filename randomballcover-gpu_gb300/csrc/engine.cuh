// engine.cuh -- host-side state of the RBC engine (internal).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rbc_gb300.h"
#include "kernels.cuh"
#include "router.cuh"
#include "tc.cuh"

namespace rbc {

// Internal build flag: keep the padded copy of the input in original row
// order (the legacy rbcStruct exposes it as rbcS.dx).
constexpr uint32_t kBuildKeepInput = 0x100u;
// Internal query flag: do not wait for the stream at the end of the call.
constexpr uint32_t kQueryNoSync = 0x100u;

void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

// Stream-ordered device buffer released on scope exit.
struct DevBuf {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  cudaError_t alloc(size_t bytes, cudaStream_t st) {
    s = st;
    return cudaMallocAsync(&p, bytes ? bytes : 16, st);
  }
  template <typename T>
  T *as() const {
    return reinterpret_cast<T *>(p);
  }
};

// Per-call buffers of one query batch; items holds item_cap work items.
struct QueryBufs {
  DevBuf Qp, Dqr, probe, probed, res_d, res_i, tau, lock, cnt, start, cursor, tcnt, tstart, pair_q,
      pair_thr, items, ctl, scan_tmp;
  uint64_t item_cap = 0;
  const float *dq0 = nullptr;  // nearest-representative distances when the probe table lacks them
  bool plan_all = false;       // the pruning round plans every list (no probe round ran)
};

// One tensor-form query round set up for batches of up to mb queries: the
// host-side choices and every buffer (tc_setup), then the kernels of one
// batch (tc_enqueue).  In graph mode tc_enqueue synchronises nothing: the
// queries the certificate leaves open are searched again on the device (the
// FP32 search over the whole database, its work list sized by their count on
// the device) and the error words are folded into err_sink.
// The tensor form's probe round searches the first this many rows of every
// probed list on the FP32 path (whole lists when shorter: few queries share a
// probed list, and small tensor items are dominated by fixed costs and
// shortlist merges) and the rest of longer lists on the tensor cores, into
// shortlists those exact rows already hold.  RBC_TC_PROBE_ROWS overrides it.
constexpr uint64_t kTcProbeRows = 8192;

struct TcQuery {
  bool routed = false, spec = false;
  bool cap = false;  // shortlists capped at tau (1 + 2^-7) once the seed or a rerank knows tau
  uint32_t k = 0, Pn = 0, Pnear = 0, P = 0, sl = 0, kw = 0, qtile = 0;
  uint64_t probe_rows = 0, probe_cap = 0, mb = 0;
  int grid = 0, sgrid = 0, ptq = 0, pgrid = 0;
  QueryBufs b;
  DevBuf near, near_d, logits, Qh, qscale, qnorm, qinex, sl_a, sl_row, sl_sel, sl_theta, sl_lock, emax, ctl, failq,
      stats, seed_a, seed_row, sl_cap, tpred, drop;
  // graph mode: the device fallback's work list and control words
  DevBuf fb_items, fb_ctl;
  uint32_t fb_chunk = 0, fb_qtile = 0;
  uint64_t fb_cap = 0;
  int fb_grid = 0;
};

}  // namespace rbc

struct rbc_index;

namespace rbc {
// Plan one query round (mode 0 probe pairs, mode 1 pruned pairs); stage 0
// stops after the plan, 1 after the work items, 2 also runs the search.
// tq < 0 uses the index's tuned tile.
// qtile > 0 overrides the query tile of the work items; only the lists the
// filter selects get items.
int plan_and_search(rbc_index *idx, QueryBufs &b, uint64_t m, uint32_t P, uint32_t k, uint32_t mode,
                    const float *X, const uint32_t *pid, const uint64_t *offsets, const float *radius,
                    int grid, unsigned long long *stats, cudaStream_t s, int stage = 2, int tq = -1,
                    uint32_t qtile = 0, ListFilter filter = ListFilter());
// The plan arguments of one query round (the per-index directed-rounding
// constants of the pruning bound, the round's buffers); list_cnt and phase
// are left to the caller.
void fill_plan_args(const rbc_index *idx, QueryBufs &b, uint64_t m, uint32_t P, uint32_t qtile,
                    const uint64_t *offsets, const float *radius, PlanArgs &a);
// Build the tensor-core operands of an index that has its partition.
int build_tc(rbc_index *idx, cudaStream_t s);
// Work items a plan of mb queries can produce with query tiles of qtile
// (query tiles x row chunks); probes > 0 bounds a probe-round plan, whose
// (query, list) pairs number at most mb x probes.
uint64_t item_capacity(const rbc_index *idx, uint64_t mb, uint32_t qtile, uint32_t probes = 0);
int query_index(rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
                uint32_t *dIds, float *dDists, uint32_t ldo, cudaStream_t s);
int tc_setup(rbc_index *idx, uint64_t mb, uint32_t k, uint32_t mode, bool graph, TcQuery &t, cudaStream_t s);
int tc_enqueue(rbc_index *idx, TcQuery &t, const float *dQ, uint64_t mq, uint32_t ldq, uint32_t *dIds, float *dDists,
               uint32_t ldo, bool graph, uint32_t *err_sink, bool *tc_probe, cudaStream_t s);
int build_index(const float *dX, uint64_t n, uint32_t d, uint32_t ldx, const rbc_build_params *p,
                cudaStream_t s, rbc_index **out);
int brute_knn(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t d,
              uint32_t k, int metric, uint32_t *dIds, float *dDists, uint32_t ldo, cudaStream_t s);
}  // namespace rbc

struct rbc_index {
  int device = 0;
  uint64_t n = 0;
  uint32_t d = 0, ld = 0, dp = 0;
  int metric = RBC_L2;
  uint32_t flags = 0;
  uint32_t nr = 0, s = 0, lds = 0;
  std::vector<uint32_t> rep_ids;
  // partition (exact search)
  uint32_t *owner = nullptr;    // original id -> list (nearest representative)
  float *Xp = nullptr;          // n x ld rows, list-major
  uint32_t *perm = nullptr;     // list-major row -> original id
  uint64_t *offsets = nullptr;  // nr + 1
  std::vector<uint64_t> h_offsets;  // host copy of offsets (tensor-form work units)
  float *radius = nullptr;      // nr
  // representatives
  float *R = nullptr;           // pad16(nr) x ld
  // one-shot lists (the reference's structure)
  uint32_t *os_lists = nullptr;   // pad16(nr) x lds original ids, increasing (rbcStruct.dxMap)
  uint32_t *os_counts = nullptr;  // nr
  uint32_t *os_ids = nullptr;     // nr x s packed ids: row -> id map of Xo
  uint64_t *os_offsets = nullptr; // nr + 1 rows of Xo per list
  float *Xo = nullptr;            // list-major copy of the one-shot lists' rows
  // tensor-core operands of the partition rows (RBC_BUILD_BF16): rows centered
  // on their representative, in BF16 (exact data) or FP16 hi|lo (tc.cuh)
  rbc::TcBuild tc{};
  uint64_t n_pad = 0;
  uint32_t kp = 0;
  CUtensorMap tmB;                // TMA map of tc.Xh (128-row boxes, 128-byte swizzle)
  // double-precision variant (rbc_build_f64, flag RBC_BUILD_F64): the double
  // rows in original order (stride ld64) and their largest L2 / L1 norms
  double *X64 = nullptr;
  uint32_t ld64 = 0;
  unsigned long long *norm64 = nullptr;
  // padded copy of the input in original order (legacy rbcStruct.dx)
  float *Xi = nullptr;
  uint64_t xi_rows = 0;
  uint64_t min_list = 0, max_list = 0;
  uint64_t device_bytes = 0;
  rbc_query_stats stats{};
  std::vector<uint32_t> fallback_ids;  // queries the last tensor-form call recomputed in FP32
  // search tuning (rbc_set_tuning / the autotuner): rows-per-thread of the
  // list-search tile (0 = default) and the longest row run of one work item
  int tune_tq = 0;
  uint32_t item_rows = 16384;
  // tensor-form tuning (rbc_set_tc_tuning / rbc_autotune_tc): nearest lists
  // searched in the probe round and the row count from which a probed list
  // goes to the tensor cores (0: the defaults)
  uint32_t tc_probes = 0;
  uint64_t tc_probe_rows = 0;
  uint64_t tc_probe_cap = 0;      // rows past the FP32 prefix the tensor probe round takes (0: all)
  bool tc_plain = false;          // the plain FP32 search answers RBC_QUERY_EXACT_TC (it was faster)
  // learned router (rbc_set_router): probes its top router_probes lists
  rbc_router *router = nullptr;
  uint32_t router_probes = 0;
  bool tc_unrouted = false;  // rbc_autotune_tc: routed tensor-form calls skip the router
  // benchmark instrumentation (rbc_set_profiling)
  bool profile = false;
  std::vector<cudaEvent_t> ev_pool;  // pairs of events around search launches
  size_t ev_used = 0;
  rbc_profile prof{};
};
