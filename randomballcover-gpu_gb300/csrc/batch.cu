// batch.cu -- many independent (index, query set) instances answered by one
// persistent search launch per round, the whole sequence captured once into
// a CUDA graph and replayed.
//
// Each instance keeps its own plan buffers and per-query results.  A round
// (probe, then pruned) plans every instance (small kernels), concatenates all
// instances' work items into one queue tagged with the instance, and runs a
// single persistent list-search launch over the queue: the kernel reads the
// instance's database, queries, lists and results from a device table.
// Tensor-form instances run their three rounds the same way, their tensor
// searches one grid per round in which each instance owns a range of CTAs
// and its tensor maps come from the table.  The captured graph replays the
// rounds for new query values in the same buffers.  The reference runs one (database, query set) per call with a
// host round trip between every kernel (rbc.cu:72-123).
#include <algorithm>
#include <cstdlib>
#include <memory>
#include <vector>

#include "engine.cuh"
#include "rbc_common.cuh"

namespace rbc {

namespace {

// The instances' item offsets in the concatenated queue, its length, and the
// search's work counter zeroed.
__global__ void batch_offsets_kernel(uint32_t *const *counts, uint32_t ninst, uint32_t *offsets, uint32_t *total,
                                     uint32_t *work) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint32_t s = 0;
  for (uint32_t i = 0; i < ninst; i++) {
    offsets[i] = s;
    s += *counts[i];
  }
  *total = s;
  *work = 0;
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
  DevBuf fb_items, fb_ctl;      // tensor form: the batched device fallback's items and control words
};

struct rbc_batch {
  std::vector<std::unique_ptr<BatchInstance>> inst;
  std::vector<void *> owned;
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

template <typename T>
T *to_dev(const std::vector<T> &v, std::vector<void *> &owned) {
  T *d = dalloc<T>(v.size(), owned);
  if (d && !v.empty() && cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    return nullptr;
  return d;
}

// The tensor-form instances of a batch.  Each step of their query -- set-up,
// the probe round on the FP32 path (the first rows of the probed lists) and
// on the tensor cores (the rest), the pruned round, both reranks and the
// device fallback for uncertified queries -- is one launch over a device
// table of per-instance arguments; the FP32 searches run over the
// instances' concatenated work items, the tensor searches over per-instance
// CTA ranges of one grid per operand format.
struct TcTables {
  uint32_t T = 0;
  uint64_t m_max = 0, elems_max = 0, mkw_max = 0;
  uint32_t nr_max = 0, P_max = 0, dp_max = 0;
  BatchQuery *pad = nullptr;
  std::vector<std::pair<uint32_t, uint32_t>> dkeys;  // (ld, dp) of each distance group
  std::vector<std::vector<DenseInst>> dgroups;
  std::vector<DenseInst *> ddev;
  TcPrepArgs *prep = nullptr;
  // FP32 probe round, tensor probe round, pruned round, the rest of capped
  // probed lists (rbc_set_tc_probe_cap)
  BatchPlan *plan[4] = {};
  bool fp_probe = false, tc_probe = false, rest = false;
  SearchArgs *sp = nullptr, *sf = nullptr;  // the FP32 searches: probe round, fallback
  SearchItem **src_p = nullptr, **src_f = nullptr;
  uint32_t **cnt_p = nullptr, **cnt_f = nullptr;
  uint32_t *offs = nullptr;
  SearchItem *all = nullptr;
  int tq_p = 1, grid_p = 1, tq_f = 1, grid_f = 1;
  SlSeedArgs *seed = nullptr;
  struct Launch {
    TcBatchEntry *tab;
    uint32_t n, ctas, format;
    size_t smem;
  };
  std::vector<Launch> tc[3];  // probe round (one query tile per B tile), pruned round, capped lists' rest
  RerankArgs *rr[2] = {};
  ListedArgs *listed = nullptr;
  ErrWords *errs = nullptr;
};

int prepare_tc(rbc_batch *bt, const std::vector<BatchInstance *> &tcv, cudaStream_t s, TcTables &x) {
  const uint32_t T = x.T = (uint32_t)tcv.size();
  if (!T) return RBC_OK;
  const int metric = tcv[0]->idx->metric;
  constexpr uint32_t kwp = 64, kwf = 32;  // list widths: shortlists (40-56 rows), results (k <= 32)
  int tq_p = 4, tq_f = 4;
  for (BatchInstance *ip : tcv) {
    ip->tc = std::make_unique<TcQuery>();
    BTRY(tc_setup(ip->idx, ip->m, ip->k, RBC_QUERY_EXACT_TC, false, *ip->tc, s));
    if (ip->tc->kw != kwp) return fail(RBC_ERR_UNSUPPORTED, "rbc_batch_run: tensor shortlist wider than 64");
    x.dp_max = std::max(x.dp_max, ip->idx->dp);
    tq_p = std::min(tq_p, search_tq_for(ip->idx->dp, ip->tc->ptq, kwp));
    tq_f = std::min(tq_f, search_tq_for(ip->idx->dp, 0, kwf));
  }
  // the shared FP32 launches: one tile geometry, the one the widest rows allow
  x.tq_p = search_tq_for(x.dp_max, tq_p, kwp);
  x.tq_f = search_tq_for(x.dp_max, tq_f, kwf);
  x.grid_p = search_grid(metric, x.dp_max, x.tq_p, kwp);
  x.grid_f = search_grid(metric, x.dp_max, x.tq_f, kwf);
  const uint32_t qtile_p = 16 * x.tq_p, qtile_f = 16 * x.tq_f;

  std::vector<BatchQuery> pad(T);
  std::vector<TcPrepArgs> prep(T);
  std::vector<BatchPlan> plan[4] = {std::vector<BatchPlan>(T), std::vector<BatchPlan>(T), std::vector<BatchPlan>(T),
                                    std::vector<BatchPlan>(T)};
  std::vector<SearchArgs> sp(T), sf(T);
  std::vector<SearchItem *> src_p(T), src_f(T);
  std::vector<uint32_t *> cnt_p(T), cnt_f(T);
  std::vector<SlSeedArgs> seed(T);
  std::vector<RerankArgs> rr[2] = {std::vector<RerankArgs>(T), std::vector<RerankArgs>(T)};
  std::vector<ListedArgs> listed(T);
  std::vector<ErrWords> errs(T);
  std::vector<TcBatchEntry> ent[3] = {std::vector<TcBatchEntry>(T), std::vector<TcBatchEntry>(T),
                                     std::vector<TcBatchEntry>(T)};
  std::vector<size_t> smem[3] = {std::vector<size_t>(T), std::vector<size_t>(T), std::vector<size_t>(T)};
  std::vector<double> weight(T);
  std::vector<bool> probes(T), rests(T);
  uint64_t all_p = 0, all_f = 0;
  for (uint32_t i = 0; i < T; i++) {
    BatchInstance &in = *tcv[i];
    rbc_index *idx = in.idx;
    TcQuery &t = *in.tc;
    QueryBufs &b = t.b;
    const uint64_t mq = in.m;
    const uint32_t ld = idx->ld, fmt = idx->tc.format;
    x.m_max = std::max(x.m_max, mq);
    x.nr_max = std::max(x.nr_max, idx->nr);
    x.P_max = std::max(x.P_max, t.P);
    x.elems_max = std::max<uint64_t>(x.elems_max, mq * ld);
    x.mkw_max = std::max<uint64_t>(x.mkw_max, mq * kwf);
    BatchQuery q{};
    q.Q = in.Q;
    q.ldq = in.ldq;
    q.m = mq;
    q.Qp = b.Qp.as<float>();
    q.ld = ld;
    q.d = idx->d;
    pad[i] = q;
    const std::pair<uint32_t, uint32_t> key(ld, idx->dp);
    size_t g = std::find(x.dkeys.begin(), x.dkeys.end(), key) - x.dkeys.begin();
    if (g == x.dkeys.size()) {
      x.dkeys.push_back(key);
      x.dgroups.emplace_back();
    }
    x.dgroups[g].push_back(DenseInst{b.Qp.as<float>(), mq, idx->R, idx->nr, b.Dqr.as<float>(), idx->nr});
    // the device fallback: every (row chunk, listed query tile) pair for as
    // many queries as the instance holds
    uint32_t chunk = (uint32_t)std::max<uint64_t>(4096, (idx->n + 4ull * x.grid_f - 1) / (4ull * x.grid_f));
    chunk = (chunk + 31) / 32 * 32;
    const uint64_t fcap = ((idx->n + chunk - 1) / chunk) * ((mq + qtile_f - 1) / qtile_f);
    BCK(in.fb_items.alloc(std::max<uint64_t>(fcap, 1) * sizeof(SearchItem), s));
    BCK(in.fb_ctl.alloc(64, s));
    uint32_t *fctl = in.fb_ctl.as<uint32_t>();
    all_f += fcap;

    TcPrepArgs pa{};
    pa.Dqr = b.Dqr.as<float>();
    pa.m = mq;
    pa.nr = idx->nr;
    pa.sl = t.sl;
    pa.P = t.P;
    pa.rep_rows = idx->tc.rep_rows;
    pa.seed_a = t.seed_a.as<float>();
    pa.seed_row = t.seed_row.as<uint32_t>();
    pa.probe = b.probe.as<uint32_t>();
    pa.probed = b.probed.as<float>();
    pa.Qp = b.Qp.as<float>();
    pa.ld = ld;
    pa.d = idx->d;
    pa.kp = idx->kp;
    pa.format = fmt;
    pa.mu = idx->tc.mu;
    pa.Qh = t.Qh.as<uint16_t>();
    pa.qscale = t.qscale.as<float>();
    pa.qnorm = t.qnorm.as<float>();
    pa.qinex = t.qinex.as<uint8_t>();
    pa.sl_a = t.sl_a.as<float>();
    pa.sl_row = t.sl_row.as<uint32_t>();
    pa.sl_sel = t.sl_sel.as<uint32_t>();
    pa.sl_theta = t.sl_theta.as<uint32_t>();
    pa.sl_lock = t.sl_lock.as<uint32_t>();
    pa.emax = t.emax.as<uint32_t>();
    pa.drop = t.drop.as<uint32_t>();
    pa.res_d = b.res_d.as<float>();
    pa.res_i = b.res_i.as<uint32_t>();
    pa.tau = b.tau.as<uint32_t>();
    pa.lock = b.lock.as<uint32_t>();
    pa.kw = t.kw;
    pa.ctl[0] = b.ctl.as<uint32_t>();
    pa.ctl[1] = t.ctl.as<uint32_t>();
    pa.ctl[2] = fctl;
    pa.stats = t.stats.as<unsigned long long>();
    prep[i] = pa;

    // the plan rounds, as tc_enqueue plans them
    probes[i] = idx->max_list > t.probe_rows;
    rests[i] = probes[i] && t.probe_cap && idx->max_list > t.probe_rows + t.probe_cap;
    x.fp_probe |= t.probe_rows > 0;
    x.tc_probe |= probes[i];
    x.rest |= rests[i];
    // plan[0] FP32 probe round, [1] tensor probe round, [2] pruned round,
    // [3] the rest of capped probed lists (nothing selected without a cap)
    for (int r = 0; r < 4; r++) {
      BatchPlan bp{};
      bp.qtile = r == 0 ? qtile_p : (r == 1 ? tc_query_tile(kTcSplit) : t.qtile);
      fill_plan_args(idx, b, mq, t.P, bp.qtile, idx->offsets, idx->radius, bp.a);
      bp.cnt = b.cnt.as<uint32_t>();
      bp.start = b.start.as<uint32_t>();
      bp.cursor = b.cursor.as<uint32_t>();
      bp.tcnt = b.tcnt.as<uint32_t>();
      bp.tstart = b.tstart.as<uint32_t>();
      bp.max_rows = r == 1 ? (uint32_t)std::min<uint64_t>(2ull * idx->item_rows, 1u << 30) : idx->item_rows;
      bp.items = b.items.as<SearchItem>();
      bp.cap = b.item_cap;
      bp.nitems = b.ctl.as<uint32_t>() + 1;
      bp.err = b.ctl.as<uint32_t>() + 2;
      if (r == 0) bp.f.take = t.probe_rows;
      if (r == 1) {
        bp.f.rows_lo = t.probe_rows + 1;
        bp.f.skip = t.probe_rows;
        if (t.probe_cap) bp.f.take = t.probe_cap;
      }
      if (r == 3) {
        bp.f.rows_lo = rests[i] ? t.probe_rows + t.probe_cap + 1 : UINT64_MAX;
        bp.f.skip = rests[i] ? t.probe_rows + t.probe_cap : 0;
      }
      plan[r][i] = bp;
    }
    all_p += item_capacity(idx, mq, qtile_p, t.P);

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
    a.k = t.sl;
    sp[i] = a;
    a.qidx = t.failq.as<uint32_t>();
    a.k = in.k;
    sf[i] = a;
    src_p[i] = b.items.as<SearchItem>();
    cnt_p[i] = b.ctl.as<uint32_t>() + 1;
    src_f[i] = in.fb_items.as<SearchItem>();
    cnt_f[i] = fctl + 1;
    SlSeedArgs sa{};
    sa.res_d = b.res_d.as<float>();
    sa.res_i = b.res_i.as<uint32_t>();
    sa.kw = t.kw;
    sa.iperm = idx->tc.iperm;
    sa.seed_a = t.seed_a.as<float>();
    sa.seed_row = t.seed_row.as<uint32_t>();
    sa.m = mq;
    sa.sl = t.sl;
    sa.k = in.k;
    sa.sl_a = t.sl_a.as<float>();
    sa.sl_row = t.sl_row.as<uint32_t>();
    sa.theta = t.sl_theta.as<uint32_t>();
    sa.tau = b.tau.as<uint32_t>();
    sa.cap = t.cap ? t.sl_cap.as<uint32_t>() : nullptr;
    seed[i] = sa;

    TcArgs ta{};
    ta.items = b.items.as<SearchItem>();
    ta.nitems = b.ctl.as<uint32_t>() + 1;
    ta.qidx = b.pair_q.as<uint32_t>();
    ta.Dqr = b.Dqr.as<float>();
    ta.nr = idx->nr;
    ta.kb = idx->kp / 64;
    ta.zero_row = (uint32_t)mq;
    ta.d = idx->d;
    ta.w = idx->tc.w;
    ta.wh = static_cast<const uint4 *>(idx->tc.Wh);
    ta.lscale = idx->tc.lscale;
    ta.lxmax = idx->tc.lxmax;
    ta.lcnorm = idx->tc.lcnorm;
    ta.qscale = t.qscale.as<float>();
    ta.qnorm = t.qnorm.as<float>();
    ta.q_inexact = t.qinex.as<uint8_t>();
    ta.x_inexact = idx->tc.x_inexact;
    ta.format = fmt;
    ta.sl = t.sl;
    ta.sl_a = t.sl_a.as<float>();
    ta.sl_row = t.sl_row.as<uint32_t>();
    ta.sl_sel = t.sl_sel.as<uint32_t>();
    ta.sl_theta = t.sl_theta.as<uint32_t>();
    ta.sl_cap = sa.cap;
    ta.drop = t.drop.as<uint32_t>();
    ta.sl_lock = t.sl_lock.as<uint32_t>();
    ta.emax = t.emax.as<uint32_t>();
    ta.m = mq;
    ta.offsets = idx->offsets;
    ta.stats = t.stats.as<unsigned long long>();
    ta.err = t.ctl.as<uint32_t>();
    TcArgs tp = ta;
    tp.stats = ta.stats + 2;
    tp.keep_k = in.k;
    TcBatchEntry e{};
    BCK(tc_make_map(&e.tmA, t.Qh.p, mq + 1, idx->tc.cols, 1));
    e.tmB = idx->tmB;
    e.a = tp;
    smem[0][i] = tc_stage_plan(e.a, true);
    ent[0][i] = e;
    e.a = ta;
    smem[1][i] = tc_stage_plan(e.a, false);
    ent[1][i] = e;
    e.a.stats = ta.stats + 2;  // the capped lists' rest counts with the probe round
    smem[2][i] = smem[1][i];
    ent[2][i] = e;
    if (!smem[0][i] || !smem[1][i]) return fail(RBC_ERR_UNSUPPORTED, "rbc_batch_run: no shared-memory plan fits");
    weight[i] = (double)mq * (double)idx->n * (double)ta.kb * (fmt == kTcSplit ? 2.0 : 1.0);

    RerankArgs ra{};
    ra.X = idx->Xp;
    ra.pid = idx->perm;
    ra.Q = b.Qp.as<float>();
    ra.ld = ld;
    ra.dp = idx->dp;
    ra.k = in.k;
    ra.sl = t.sl;
    ra.m = mq;
    ra.sl_a = t.sl_a.as<float>();
    ra.sl_row = t.sl_row.as<uint32_t>();
    ra.sl_sel = t.sl_sel.as<uint32_t>();
    ra.emax = t.emax.as<uint32_t>();
    ra.drop = t.drop.as<uint32_t>();
    ra.sl_cap = sa.cap;
    ra.cap_out = sa.cap;
    ra.theta = t.sl_theta.as<uint32_t>();
    ra.ldo = in.ldo;
    ra.nfail = t.ctl.as<uint32_t>() + 1;
    ra.fail = t.failq.as<uint32_t>();
    RerankArgs r0 = ra;
    r0.tau = b.tau.as<uint32_t>();
    if (!probes[i]) r0.m = 0;  // no tensor probe round: its threshold update does not run either
    rr[0][i] = r0;
    ra.ids = in.ids;
    ra.dists = in.dists;
    rr[1][i] = ra;

    ListedArgs la{};
    la.res_d = b.res_d.as<float>();
    la.res_i = b.res_i.as<uint32_t>();
    la.tau = b.tau.as<uint32_t>();
    la.lock = b.lock.as<uint32_t>();
    la.m = mq;
    la.kw = kwf;
    la.ctl = fctl;
    la.items = in.fb_items.as<SearchItem>();
    la.n = idx->n;
    la.cap = fcap;
    la.chunk = chunk;
    la.qtile = qtile_f;
    la.rows = t.failq.as<uint32_t>();
    la.count = t.ctl.as<uint32_t>() + 1;
    la.k = in.k;
    la.ldo = in.ldo;
    la.ids = in.ids;
    la.dists = in.dists;
    listed[i] = la;
    errs[i] = ErrWords{{t.ctl.as<uint32_t>(), b.ctl.as<uint32_t>() + 2, fctl + 2, nullptr}};
  }
  BCK(cudaStreamSynchronize(s));
  std::vector<void *> &o = bt->owned;
  x.pad = to_dev(pad, o);
  x.prep = to_dev(prep, o);
  for (int r = 0; r < 4; r++) x.plan[r] = to_dev(plan[r], o);
  x.sp = to_dev(sp, o);
  x.sf = to_dev(sf, o);
  x.src_p = to_dev(src_p, o);
  x.src_f = to_dev(src_f, o);
  x.cnt_p = to_dev(cnt_p, o);
  x.cnt_f = to_dev(cnt_f, o);
  x.offs = dalloc<uint32_t>(T, o);
  x.all = dalloc<SearchItem>(std::max(x.fp_probe ? all_p : 0, all_f), o);
  x.seed = to_dev(seed, o);
  x.rr[0] = to_dev(rr[0], o);
  x.rr[1] = to_dev(rr[1], o);
  x.listed = to_dev(listed, o);
  x.errs = to_dev(errs, o);
  if (!x.pad || !x.prep || !x.plan[0] || !x.plan[1] || !x.plan[2] || !x.plan[3] || !x.sp || !x.sf || !x.src_p ||
      !x.src_f || !x.cnt_p || !x.cnt_f || !x.offs || !x.all || !x.seed || !x.rr[0] || !x.rr[1] || !x.listed || !x.errs)
    return fail(RBC_ERR_NOMEM, "rbc_batch_run: device allocation failed");
  for (const auto &gr : x.dgroups) {
    x.ddev.push_back(to_dev(gr, o));
    if (!x.ddev.back()) return fail(RBC_ERR_NOMEM, "rbc_batch_run: device allocation failed");
  }
  // the tensor searches: per round and operand format one grid, each
  // instance a CTA range sized by its share of the work (about four waves in
  // all: c4 4.19M / 4.67M / 4.86M / 4.85M / 4.82M queries/s at 1 / 2 / 4 / 6
  // / 8), the largest first; RBC_BATCH_WAVES overrides
  const uint32_t sms = (uint32_t)tc_grid();
  double waves = 4.0;
  if (const char *env = std::getenv("RBC_BATCH_WAVES")) waves = std::max(0.25, std::atof(env));
  for (int r = 0; r < 3; r++)
    for (uint32_t fmt : {(uint32_t)kTcExact, (uint32_t)kTcSplit}) {
      std::vector<uint32_t> mem;
      double wsum = 0;
      for (uint32_t i = 0; i < T; i++)
        if (tcv[i]->idx->tc.format == fmt && (r == 0 ? probes[i] : (r == 1 || rests[i]))) {
          mem.push_back(i);
          wsum += weight[i];
        }
      if (mem.empty()) continue;
      std::stable_sort(mem.begin(), mem.end(), [&](uint32_t a, uint32_t b) { return weight[a] > weight[b]; });
      std::vector<TcBatchEntry> tab;
      uint32_t cta = 0;
      size_t sm = 0;
      for (uint32_t i : mem) {
        TcBatchEntry e = ent[r][i];
        const double share = wsum > 0 ? weight[i] / wsum : 1.0;
        e.ctas = (uint32_t)std::min<double>(sms, std::max(1.0, std::ceil(waves * sms * share)));
        e.cta0 = cta;
        cta += e.ctas;
        sm = std::max(sm, smem[r][i]);
        tab.push_back(e);
      }
      TcBatchEntry *d = to_dev(tab, o);
      if (!d) return fail(RBC_ERR_NOMEM, "rbc_batch_run: device allocation failed");
      x.tc[r].push_back(TcTables::Launch{d, (uint32_t)tab.size(), cta, fmt, sm});
    }
  return RBC_OK;
}

// Record the tensor-form instances' query (see TcTables) on stream s.
int capture_tc(const TcTables &x, int metric, uint32_t *ctl, cudaStream_t s) {
  const uint32_t T = x.T;
  if (!T) return RBC_OK;
  BCK(launch_batch_pad(x.pad, T, x.elems_max, s));
  for (size_t gi = 0; gi < x.dgroups.size(); gi++) {
    uint64_t na = 0, nb = 0;
    for (const DenseInst &di : x.dgroups[gi]) {
      na = std::max(na, di.na);
      nb = std::max(nb, di.nb);
    }
    BCK(launch_dense_dist_batch(metric, x.ddev[gi], (uint32_t)x.dgroups[gi].size(), na, nb, x.dkeys[gi].first,
                                x.dkeys[gi].second, s));
  }
  BCK(launch_tc_prep_batch(x.prep, T, x.m_max, s));
  SearchArgs g{};
  g.items = x.all;
  g.nitems = ctl + 1;
  g.work = ctl;
  g.err = ctl + 2;
  g.dp = x.dp_max;  // sizes the shared-memory tile of the shared launches
  if (x.fp_probe) {
    BCK(launch_plan_batch(x.plan[0], T, 0, x.nr_max, x.m_max, x.P_max, s));
    batch_offsets_kernel<<<1, 1, 0, s>>>(x.cnt_p, T, x.offs, ctl + 1, ctl);
    BCK(launched());
    batch_concat_kernel<<<dim3(64, T), 256, 0, s>>>(x.src_p, x.cnt_p, x.offs, x.all);
    BCK(launched());
    g.insts = x.sp;
    g.k = 64;  // shortlist-wide lists
    BCK(launch_search(metric, g, x.grid_p, s, x.tq_p));
  }
  BCK(launch_sl_seed_batch(x.seed, T, x.m_max, s));
  if (x.tc_probe) {
    BCK(launch_plan_batch(x.plan[1], T, 0, x.nr_max, x.m_max, x.P_max, s));
    for (const auto &L : x.tc[0]) BCK(launch_tc_search_batch(L.tab, L.n, L.ctas, L.format, true, L.smem, s));
    BCK(launch_rerank_batch(metric, x.rr[0], T, x.m_max, s));
  }
  if (x.rest) {
    BCK(launch_plan_batch(x.plan[3], T, 0, x.nr_max, x.m_max, x.P_max, s));
    for (const auto &L : x.tc[2]) BCK(launch_tc_search_batch(L.tab, L.n, L.ctas, L.format, false, L.smem, s));
    BCK(launch_rerank_batch(metric, x.rr[0], T, x.m_max, s));
  }
  BCK(launch_plan_batch(x.plan[2], T, 1, x.nr_max, x.m_max, x.P_max, s));
  for (const auto &L : x.tc[1]) BCK(launch_tc_search_batch(L.tab, L.n, L.ctas, L.format, false, L.smem, s));
  BCK(launch_rerank_batch(metric, x.rr[1], T, x.m_max, s));
  // the uncertified queries (their count on the device) searched again over
  // every row on the FP32 path, their answers written over the tensor form's
  BCK(launch_listed_init_batch(x.listed, T, x.mkw_max, s));
  BCK(launch_listed_items_batch(x.listed, T, s));
  batch_offsets_kernel<<<1, 1, 0, s>>>(x.cnt_f, T, x.offs, ctl + 1, ctl);
  BCK(launched());
  batch_concat_kernel<<<dim3(64, T), 256, 0, s>>>(x.src_f, x.cnt_f, x.offs, x.all);
  BCK(launched());
  g.insts = x.sf;
  g.k = 32;
  BCK(launch_search(metric, g, x.grid_f, s, x.tq_f));
  BCK(launch_listed_results_batch(x.listed, T, s));
  BCK(launch_fold_errors_batch(x.errs, T, ctl + 2, s));
  return RBC_OK;
}

// Allocate every buffer, then record the whole sequence on a capture stream
// into a graph: the FP32 instances' set-up (one launch each for the padded
// queries, the nearest representatives and empty results, one distance launch
// per padded dimension), their two rounds (each one batched plan round and
// one persistent search launch over all of them) and their write-back; then
// the tensor-form instances' rounds, each step one launch over all of them
// (TcTables).
int prepare(rbc_batch *bt) {
  // a tensor-form instance whose index the autotuner set to the plain search
  // (rbc_index_info.tc_plain) joins the FP32 instances, as its single query
  // call would run the FP32 search
  std::vector<BatchInstance *> fp, tcv;
  for (auto &ip : bt->inst) (ip->mode == RBC_QUERY_EXACT_TC && !ip->idx->tc_plain ? tcv : fp).push_back(ip.get());
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
  TcTables tx;
  BTRY(prepare_tc(bt, tcv, s, tx));
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
      batch_offsets_kernel<<<1, 1, 0, s>>>(dcnt, N, offs, bt->ctl + 1, bt->ctl);
      BCK(launched());
      batch_concat_kernel<<<dim3(64, N), 256, 0, s>>>(dsrc, dcnt, offs, all);
      BCK(launched());
      g.insts = round == 0 ? t0 : t1;
      BCK(launch_search(metric, g, grid, s, tq));
    }
    if (N) BCK(launch_batch_write(dq, N, mk_max, s));
    // the tensor-form instances; their error words fold into the batch's
    return capture_tc(tx, metric, bt->ctl, s);
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
