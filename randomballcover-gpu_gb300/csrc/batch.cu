// batch.cu -- many independent (index, query set) instances answered by one
// persistent search launch per round, the whole sequence captured once into
// a CUDA graph and replayed.
//
// Each instance keeps its own plan buffers and per-query results.  A round
// (probe, then pruned) plans every instance (small kernels), concatenates all
// instances' work items into one queue tagged with the instance, and runs a
// single persistent list-search launch over the queue: the kernel reads the
// instance's database, queries, lists and results from a device table.  The
// captured graph replays the rounds for new query values in the same
// buffers.  The reference runs one (database, query set) per call with a
// host round trip between every kernel (rbc.cu:72-123).
#include <algorithm>
#include <memory>
#include <vector>

#include "engine.cuh"
#include "rbc_common.cuh"

namespace rbc {

namespace {

__global__ void batch_offsets_kernel(uint32_t *const *counts, uint32_t ninst, uint32_t *offsets, uint32_t *total) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint32_t s = 0;
  for (uint32_t i = 0; i < ninst; i++) {
    offsets[i] = s;
    s += *counts[i];
  }
  *total = s;
}

__global__ void batch_concat_kernel(const SearchItem *const *src, uint32_t *const *counts, const uint32_t *offsets,
                                    SearchItem *dst) {
  const uint32_t i = blockIdx.y;
  const uint32_t c = *counts[i];
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < c; j += gridDim.x * blockDim.x) {
    SearchItem it = src[i][j];
    it.inst = i;
    dst[offsets[i] + j] = it;
  }
}

template <typename T>
T *dalloc(size_t n, std::vector<void *> &owned) {
  void *p = nullptr;
  if (cudaMalloc(&p, n ? n * sizeof(T) : 16) != cudaSuccess) return nullptr;
  owned.push_back(p);
  return static_cast<T *>(p);
}

}  // namespace

}  // namespace rbc

using namespace rbc;

struct BatchInstance {
  rbc_index *idx;
  const float *Q;
  uint64_t m;
  uint32_t ldq, k, ldo;
  uint32_t mode;  // RBC_QUERY_EXACT (the shared FP32 search) or RBC_QUERY_EXACT_TC
  uint32_t *ids;
  float *dists;
  QueryBufs b;
  std::unique_ptr<TcQuery> tc;  // the tensor form's buffers (RBC_QUERY_EXACT_TC)
};

struct rbc_batch {
  std::vector<std::unique_ptr<BatchInstance>> inst;
  std::vector<void *> owned;
  std::vector<cudaStream_t> branch;  // capture-time side streams (tensor-form instances)
  std::vector<cudaEvent_t> marks;
  bool ready = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  uint32_t *ctl = nullptr;  // [0] work, [1] items, [2] error
  unsigned long long graph_kernels = 0;  // kernel nodes one replay runs
  ~rbc_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    inst.clear();  // releases the per-instance buffers on the capture stream
    if (cap) {
      cudaStreamSynchronize(cap);
      cudaStreamDestroy(cap);
    }
    for (void *p : owned) cudaFree(p);
    for (cudaStream_t b : branch) cudaStreamDestroy(b);
    for (cudaEvent_t e : marks) cudaEventDestroy(e);
  }
};

namespace {

#define BCK(expr)                                       \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #expr); \
  } while (0)
#define BTRY(expr)                  \
  do {                              \
    int rc_ = (expr);               \
    if (rc_ != RBC_OK) return rc_;  \
  } while (0)

// Allocate every buffer, then record the whole sequence on a capture stream
// into a graph: the FP32 instances' set-up (one launch each for the padded
// queries, the nearest representatives and empty results, one distance launch
// per padded dimension), their two rounds (each one batched plan round and
// one persistent search launch over all of them) and their write-back; then
// every tensor-form instance's round (its uncertified queries searched again
// on the device), those on parallel branches.
int prepare(rbc_batch *bt) {
  std::vector<BatchInstance *> fp, tcv;
  for (auto &ip : bt->inst) (ip->mode == RBC_QUERY_EXACT_TC ? tcv : fp).push_back(ip.get());
  const uint32_t N = (uint32_t)fp.size();
  const int metric = bt->inst[0]->idx->metric;
  // one tile geometry for the shared launch: the smallest query tile any instance needs
  int tq = 4;
  uint32_t dp_max = 0;
  for (BatchInstance *ip : fp) {
    tq = std::min(tq, search_tq_for(ip->idx->dp, ip->idx->tune_tq));
    dp_max = std::max(dp_max, ip->idx->dp);
  }
  const uint32_t qtile = (uint32_t)search_query_tile(dp_max, tq);
  uint64_t item_total = 0;
  cudaStream_t s;
  BCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  bt->cap = s;
  std::vector<SearchArgs> args0(N), args1(N);
  std::vector<SearchItem *> srcs(N);
  std::vector<uint32_t *> counts(N);
  for (uint32_t i = 0; i < N; i++) {
    BatchInstance &in = *fp[i];
    rbc_index *idx = in.idx;
    const uint32_t nr = idx->nr, ld = idx->ld;
    QueryBufs &b = in.b;
    const uint64_t mb = in.m, pair_cap = mb * nr, item_cap = item_capacity(idx, mb, qtile);
    item_total += item_cap;
    BCK(b.Qp.alloc(mb * ld * 4, s));
    BCK(b.Dqr.alloc(mb * nr * 4, s));
    BCK(b.probe.alloc(mb * 4, s));
    BCK(b.probed.alloc(mb * 4, s));
    BCK(b.res_d.alloc(mb * kListWidth * 4, s));
    BCK(b.res_i.alloc(mb * kListWidth * 4, s));
    BCK(b.tau.alloc(mb * 4, s));
    BCK(b.lock.alloc(mb * 4, s));
    BCK(b.cnt.alloc((nr + 1) * 4, s));
    BCK(b.start.alloc((nr + 1) * 4, s));
    BCK(b.cursor.alloc((nr + 1) * 4, s));
    BCK(b.tcnt.alloc((nr + 1) * 4, s));
    BCK(b.tstart.alloc((nr + 1) * 4, s));
    BCK(b.pair_q.alloc(pair_cap * 4, s));
    BCK(b.pair_thr.alloc(pair_cap * 4, s));
    BCK(b.items.alloc(item_cap * sizeof(SearchItem), s));
    b.item_cap = item_cap;
    BCK(b.ctl.alloc(64, s));
    BCK(b.scan_tmp.alloc(scan_temp_bytes(nr + 1), s));
    srcs[i] = b.items.as<SearchItem>();
    counts[i] = b.ctl.as<uint32_t>() + 1;
    SearchArgs a{};
    a.X = idx->Xp;
    a.pid = idx->perm;
    a.Q = b.Qp.as<float>();
    a.qidx = b.pair_q.as<uint32_t>();
    a.res_d = b.res_d.as<float>();
    a.res_i = b.res_i.as<uint32_t>();
    a.tau = b.tau.as<uint32_t>();
    a.lock = b.lock.as<uint32_t>();
    a.ld = ld;
    a.dp = idx->dp;
    a.k = in.k;
    args0[i] = a;
    a.qthr = b.pair_thr.as<float>();
    args1[i] = a;
  }
  // the FP32 instances' set-up, plan rounds and write-back run as batched
  // launches over device tables of per-instance arguments (the distance
  // blocks once per padded dimension)
  std::vector<BatchQuery> qtab(N);
  std::vector<BatchPlan> ptab(N);
  std::vector<std::vector<DenseInst>> dgroups;
  std::vector<std::pair<uint32_t, uint32_t>> dkeys;  // (ld, dp) of each group
  uint64_t m_max = 0, elems_max = 0, mk_max = 0;
  uint32_t nr_max = 0;
  for (uint32_t i = 0; i < N; i++) {
    BatchInstance &in = *fp[i];
    rbc_index *idx = in.idx;
    QueryBufs &b = in.b;
    BatchQuery q{};
    q.Q = in.Q;
    q.ldq = in.ldq;
    q.m = in.m;
    q.Qp = b.Qp.as<float>();
    q.ld = idx->ld;
    q.d = idx->d;
    q.Dqr = b.Dqr.as<float>();
    q.nr = idx->nr;
    q.probe = b.probe.as<uint32_t>();
    q.probed = b.probed.as<float>();
    q.res_d = b.res_d.as<float>();
    q.res_i = b.res_i.as<uint32_t>();
    q.tau = b.tau.as<uint32_t>();
    q.lock = b.lock.as<uint32_t>();
    q.kw = kListWidth;
    q.ctl = b.ctl.as<uint32_t>();
    q.k = in.k;
    q.ldo = in.ldo;
    q.ids = in.ids;
    q.dists = in.dists;
    qtab[i] = q;
    BatchPlan bp{};
    // the query tile the single-index planner would take for this instance
    bp.qtile = (uint32_t)search_query_tile(idx->dp, tq, list_width_for(in.k));
    fill_plan_args(idx, b, in.m, 1, bp.qtile, idx->offsets, idx->radius, bp.a);
    bp.cnt = b.cnt.as<uint32_t>();
    bp.start = b.start.as<uint32_t>();
    bp.cursor = b.cursor.as<uint32_t>();
    bp.tcnt = b.tcnt.as<uint32_t>();
    bp.tstart = b.tstart.as<uint32_t>();
    bp.max_rows = idx->item_rows;
    bp.items = b.items.as<SearchItem>();
    bp.cap = b.item_cap;
    bp.nitems = b.ctl.as<uint32_t>() + 1;
    bp.err = b.ctl.as<uint32_t>() + 2;
    ptab[i] = bp;
    const std::pair<uint32_t, uint32_t> key(idx->ld, idx->dp);
    size_t g = std::find(dkeys.begin(), dkeys.end(), key) - dkeys.begin();
    if (g == dkeys.size()) {
      dkeys.push_back(key);
      dgroups.emplace_back();
    }
    dgroups[g].push_back(DenseInst{b.Qp.as<float>(), in.m, idx->R, idx->nr, b.Dqr.as<float>(), idx->nr});
    m_max = std::max<uint64_t>(m_max, in.m);
    nr_max = std::max(nr_max, idx->nr);
    elems_max = std::max<uint64_t>(elems_max, in.m * idx->ld);
    mk_max = std::max<uint64_t>(mk_max, in.m * in.k);
  }
  for (BatchInstance *ip : tcv) {
    ip->tc = std::make_unique<TcQuery>();
    BTRY(tc_setup(ip->idx, ip->m, ip->k, RBC_QUERY_EXACT_TC, true, *ip->tc, s));
  }
  // The tensor-form instances are captured on side streams forked from the
  // capture stream and joined back, so the graph holds them as parallel
  // branches instead of running them in turn.  The instances of one index
  // share a branch (its router's scratch is the index's); distinct indexes go
  // round the branches.
  const uint32_t nbranch = (uint32_t)std::min<size_t>(tcv.size(), 8);
  for (uint32_t i = 0; i < nbranch; i++) {
    cudaStream_t b;
    BCK(cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking));
    bt->branch.push_back(b);
  }
  for (size_t i = 0; i < 3 * (nbranch + 1); i++) {
    cudaEvent_t e;
    BCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    bt->marks.push_back(e);
  }
  std::vector<std::pair<rbc_index *, cudaStream_t>> lanes;
  auto lane_of = [&](rbc_index *idx) {
    auto it = std::find_if(lanes.begin(), lanes.end(), [&](const auto &e) { return e.first == idx; });
    if (it == lanes.end()) it = lanes.insert(lanes.end(), {idx, bt->branch[lanes.size() % nbranch]});
    return it->second;
  };
  BCK(cudaStreamSynchronize(s));
  SearchArgs *t0 = dalloc<SearchArgs>(N, bt->owned), *t1 = dalloc<SearchArgs>(N, bt->owned);
  SearchItem **dsrc = dalloc<SearchItem *>(N, bt->owned);
  uint32_t **dcnt = dalloc<uint32_t *>(N, bt->owned);
  uint32_t *offs = dalloc<uint32_t>(N, bt->owned);
  SearchItem *all = dalloc<SearchItem>(item_total, bt->owned);
  bt->ctl = dalloc<uint32_t>(16, bt->owned);
  if (!t0 || !t1 || !dsrc || !dcnt || !offs || !all || !bt->ctl)
    return fail(RBC_ERR_NOMEM, "rbc_batch_run: device allocation failed");
  BCK(cudaMemcpy(t0, args0.data(), N * sizeof(SearchArgs), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(t1, args1.data(), N * sizeof(SearchArgs), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(dsrc, srcs.data(), N * sizeof(void *), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(dcnt, counts.data(), N * sizeof(void *), cudaMemcpyHostToDevice));
  BatchQuery *dq = dalloc<BatchQuery>(N, bt->owned);
  BatchPlan *dp_tab = dalloc<BatchPlan>(N, bt->owned);
  if (N && (!dq || !dp_tab)) return fail(RBC_ERR_NOMEM, "rbc_batch_run: device allocation failed");
  BCK(cudaMemcpy(dq, qtab.data(), N * sizeof(BatchQuery), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(dp_tab, ptab.data(), N * sizeof(BatchPlan), cudaMemcpyHostToDevice));
  std::vector<DenseInst *> ddev(dgroups.size());
  for (size_t g = 0; g < dgroups.size(); g++) {
    ddev[g] = dalloc<DenseInst>(dgroups[g].size(), bt->owned);
    if (!ddev[g]) return fail(RBC_ERR_NOMEM, "rbc_batch_run: device allocation failed");
    BCK(cudaMemcpy(ddev[g], dgroups[g].data(), dgroups[g].size() * sizeof(DenseInst), cudaMemcpyHostToDevice));
  }
  const int grid = N ? search_grid(metric, dp_max, tq) : 1;
  SearchArgs g{};
  g.items = all;
  g.nitems = bt->ctl + 1;
  g.work = bt->ctl;
  g.err = bt->ctl + 2;
  g.dp = dp_max;  // sizes the shared-memory tile of the shared launch
  g.k = 1;  // every instance has k <= 32: lists of 32 entries

  // launches recorded during capture run only when the graph replays:
  // the launch counter is charged per replay instead
  const unsigned long long l0 = g_kernel_launches.load();
  BCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = RBC_OK;
  cudaEvent_t *mark = bt->marks.data();
  auto fork = [&]() -> int {
    BCK(cudaEventRecord(*mark, s));
    for (cudaStream_t b : bt->branch) BCK(cudaStreamWaitEvent(b, *mark, 0));
    mark++;
    return RBC_OK;
  };
  auto join = [&]() -> int {
    for (cudaStream_t b : bt->branch) {
      BCK(cudaEventRecord(*mark, b));
      BCK(cudaStreamWaitEvent(s, *mark, 0));
      mark++;
    }
    return RBC_OK;
  };
  auto capture = [&]() -> int {
    BCK(cudaMemsetAsync(bt->ctl, 0, 64, s));
    if (N) {
      BCK(launch_batch_pad(dq, N, elems_max, s));
      for (size_t gi = 0; gi < dgroups.size(); gi++) {
        uint64_t na = 0, nb = 0;
        for (const DenseInst &di : dgroups[gi]) {
          na = std::max(na, di.na);
          nb = std::max(nb, di.nb);
        }
        BCK(launch_dense_dist_batch(metric, ddev[gi], (uint32_t)dgroups[gi].size(), na, nb, dkeys[gi].first,
                                    dkeys[gi].second, s));
      }
      BCK(launch_batch_nearest(dq, N, m_max, s));
    }
    for (uint32_t round = 0; round < 2 && N; round++) {
      BCK(launch_plan_batch(dp_tab, N, round, nr_max, m_max, 1, s));
      batch_offsets_kernel<<<1, 1, 0, s>>>(dcnt, N, offs, bt->ctl + 1);
      BCK(launched());
      batch_concat_kernel<<<dim3(64, N), 256, 0, s>>>(dsrc, dcnt, offs, all);
      BCK(launched());
      BCK(cudaMemsetAsync(bt->ctl, 0, 4, s));
      g.insts = round == 0 ? t0 : t1;
      BCK(launch_search(metric, g, grid, s, tq));
    }
    if (N) BCK(launch_batch_write(dq, N, mk_max, s));
    // the tensor-form instances, each a whole round with its device fallback
    // on a branch; their error words fold into the batch's
    if (tcv.empty()) return RBC_OK;
    BTRY(fork());
    for (BatchInstance *ip : tcv)
      BTRY(tc_enqueue(ip->idx, *ip->tc, ip->Q, ip->m, ip->ldq, ip->ids, ip->dists, ip->ldo, true, bt->ctl + 2,
                      nullptr, lane_of(ip->idx)));
    return join();
  };
  rc = capture();
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  bt->graph_kernels = g_kernel_launches.load() - l0;
  g_kernel_launches.fetch_sub(bt->graph_kernels);
  if (rc != RBC_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "rbc_batch_run: graph capture");
  bt->graph = graph;
  BCK(cudaGraphInstantiate(&bt->exec, graph, 0));
  bt->ready = true;
  return RBC_OK;
}

}  // namespace

extern "C" {

int rbc_batch_create(rbc_batch **out) {
  if (!out) return fail(RBC_ERR_INVALID, "rbc_batch_create: out is NULL");
  *out = new rbc_batch();
  return RBC_OK;
}

int rbc_batch_add(rbc_batch *bt, rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k,
                  uint32_t *dIds, float *dDists, uint32_t ldo) {
  return rbc_batch_add_mode(bt, idx, dQ, m, ldq, k, RBC_QUERY_EXACT, dIds, dDists, ldo);
}

int rbc_batch_add_mode(rbc_batch *bt, rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k,
                       uint32_t mode, uint32_t *dIds, float *dDists, uint32_t ldo) {
  if (!bt || !idx) return fail(RBC_ERR_INVALID, "rbc_batch_add: NULL argument");
  if (bt->ready) return fail(RBC_ERR_INVALID, "rbc_batch_add: the batch already ran; create a new one");
  if (!(idx->flags & RBC_BUILD_PARTITION)) return fail(RBC_ERR_INVALID, "rbc_batch_add: index has no partition");
  if (mode != RBC_QUERY_EXACT && mode != RBC_QUERY_EXACT_TC)
    return fail(RBC_ERR_INVALID, "rbc_batch_add: mode must be RBC_QUERY_EXACT or RBC_QUERY_EXACT_TC");
  if (mode == RBC_QUERY_EXACT_TC && !(idx->flags & RBC_BUILD_BF16))
    return fail(RBC_ERR_INVALID, "rbc_batch_add: RBC_QUERY_EXACT_TC needs an index built with RBC_BUILD_BF16");
  if (idx->flags & RBC_BUILD_F64) return fail(RBC_ERR_INVALID, "rbc_batch_add: index holds doubles: rbc_query_f64");
  if (k < 1 || k > (uint32_t)kListWidth || ldo < k || ldq < idx->d || m == 0 || !dQ || (!dIds && !dDists))
    return fail(RBC_ERR_INVALID, "rbc_batch_add: bad query arguments");
  if (m * (uint64_t)idx->nr > (1ull << 28))
    return fail(RBC_ERR_UNSUPPORTED, "rbc_batch_add: m x num_reps above 2^28 (split the query set)");
  if (!bt->inst.empty() && bt->inst[0]->idx->metric != idx->metric)
    return fail(RBC_ERR_INVALID, "rbc_batch_add: all instances must share the metric");
  auto in = std::make_unique<BatchInstance>();
  in->idx = idx;
  in->Q = dQ;
  in->m = m;
  in->ldq = ldq;
  in->k = k;
  in->ldo = ldo;
  in->mode = mode;
  in->ids = dIds;
  in->dists = dDists;
  bt->inst.push_back(std::move(in));
  return RBC_OK;
}

int rbc_batch_run(rbc_batch *bt, void *stream) {
  if (!bt || bt->inst.empty()) return fail(RBC_ERR_INVALID, "rbc_batch_run: empty batch");
  if (!bt->ready) BTRY(prepare(bt));
  cudaStream_t s = (cudaStream_t)stream;
  BCK(cudaGraphLaunch(bt->exec, s));
  g_kernel_launches.fetch_add(bt->graph_kernels, std::memory_order_relaxed);
  uint32_t err = 0;
  BCK(cudaMemcpyAsync(&err, bt->ctl + 2, 4, cudaMemcpyDeviceToHost, s));
  BCK(cudaStreamSynchronize(s));
  if (err) return fail(RBC_ERR_ITER_LIMIT, "rbc_batch_run: a bounded device wait ran out");
  return RBC_OK;
}

int rbc_batch_destroy(rbc_batch *bt) {
  delete bt;
  return RBC_OK;
}

}  // extern "C"
