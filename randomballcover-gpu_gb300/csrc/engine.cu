// engine.cu -- host orchestration of build, query and brute force, and the
// C ABI of include/rbc_gb300.h.
//
// Everything runs on the caller's stream with stream-ordered temporaries
// (cudaMallocAsync), so a call adds no device-wide synchronisation; the
// public calls wait for their stream once at the end to report the device
// error word.  There is no CPU fallback: if a kernel cannot run, the call
// fails with RBC_ERR_CUDA.
#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <unordered_map>

#include "engine.cuh"
#include "rbc_common.cuh"

namespace rbc {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}
int cuda_fail(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? RBC_ERR_NOMEM : RBC_ERR_CUDA;
}

#define CK(expr)                                        \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #expr); \
  } while (0)
#define TRY(expr)                      \
  do {                                 \
    int rc_ = (expr);                  \
    if (rc_ != RBC_OK) return rc_;     \
  } while (0)

namespace {

constexpr uint32_t kDefaultProbes = 1;  // lists searched before planning (the one-shot plan)
constexpr uint32_t kTcProbes = 4;       // the tensor form: a tighter start for its shortlists

void pool_setup() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done[dev] = true;
}

uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// nr distinct ids of [0, n): a partial Fisher-Yates shuffle over a virtual
// identity array (O(nr) memory), driven by a seeded 64-bit counter hash.
// Plays the role of setupReps/subRandPerm (rbc.cu:212-229, utils.cu:17-37),
// whose seed is the wall clock; here the seed is an argument.
void sample_reps(uint64_t n, uint32_t nr, uint64_t seed, std::vector<uint32_t> &out) {
  std::unordered_map<uint64_t, uint32_t> moved;
  moved.reserve(nr * 2);
  auto get = [&](uint64_t i) {
    auto it = moved.find(i);
    return it == moved.end() ? (uint32_t)i : it->second;
  };
  const uint64_t key = mix64(seed ^ 0xA0761D6478BD642Full);
  out.resize(nr);
  for (uint32_t i = 0; i < nr; i++) {
    uint64_t j = i + mix64(key + i) % (n - i);
    uint32_t vi = get(i), vj = get(j);
    moved[j] = vi;
    out[i] = vj;
  }
}

int check_dims(uint32_t d, uint32_t ld, const char *what) {
  if (d == 0) return fail(RBC_ERR_INVALID, std::string(what) + ": d must be >= 1");
  if (ld < d) return fail(RBC_ERR_INVALID, std::string(what) + ": leading dimension smaller than d");
  if (pad4(d) > kMaxDim)
    return fail(RBC_ERR_UNSUPPORTED, std::string(what) + ": d larger than " + std::to_string(kMaxDim));
  return RBC_OK;
}

}  // namespace

// Build the list-major plan for one mode, then (stage >= 1) its work items
// and (stage 2) run the search over them.  The plan stays in b.cnt / b.start
// / b.pair_q / b.pair_thr, the items in b.items with their count in b.ctl[1].
// The float nearest to v on the side away from (up) or towards (down) zero,
// for positive v.
static float round_up_f(double v) {
  float f = (float)v;
  return (double)f < v ? std::nextafter(f, INFINITY) : f;
}
static float round_down_f(double v) {
  float f = (float)v;
  return (double)f > v ? std::nextafter(f, 0.f) : f;
}

void fill_plan_args(const rbc_index *idx, QueryBufs &b, uint64_t m, uint32_t P, uint32_t qtile,
                    const uint64_t *offsets, const float *radius, PlanArgs &a) {
  const uint32_t nr = idx->nr;
  a = PlanArgs{};
  a.Dqr = b.Dqr.as<float>();
  a.radius = radius;
  a.offsets = offsets;
  a.probe = b.probe.as<uint32_t>();
  a.probed = b.probed.as<float>();
  a.dq0 = b.dq0;
  a.tau = b.tau.as<uint32_t>();
  a.m = m;
  a.nr = nr;
  a.P = P;
  a.P_excl = b.plan_all ? 0 : P;
  a.metric = (uint32_t)idx->metric;
  a.qtile = qtile;
  const double g = (double)(idx->dp + 8) * 1.1920928955078125e-07;
  a.opg_ru = round_up_f(1.0 + g);
  a.omg_rd = round_down_f(1.0 - g);
  a.c_ru = round_up_f(1.0 + 3.0 * g);
  a.opc_ru = round_up_f(2.0 + 3.0 * g);
  // reciprocals, nudged by 2^-50 so the float rounding lands on the safe side
  // of the exact value whatever the double evaluation's last bit
  a.inv_opg_rd = round_down_f(1.0 / (1.0 + g) * (1.0 - 0x1p-50));
  a.inv_omg_ru = round_up_f(1.0 / (1.0 - g) * (1.0 + 0x1p-50));
  a.inv_opc_rd = round_down_f(1.0 / (2.0 + 3.0 * g) * (1.0 - 0x1p-50));
  a.list_cursor = b.cursor.as<uint32_t>();
  a.pair_q = b.pair_q.as<uint32_t>();
  a.pair_thr = b.pair_thr.as<float>();
}

int plan_and_search(rbc_index *idx, QueryBufs &b, uint64_t m, uint32_t P, uint32_t k, uint32_t mode,
                    const float *X, const uint32_t *pid, const uint64_t *offsets, const float *radius,
                    int grid, unsigned long long *stats, cudaStream_t s, int stage, int tq, uint32_t qtile_over,
                    ListFilter filter) {
  const int tqv = tq < 0 ? idx->tune_tq : tq;
  const uint32_t nr = idx->nr, qtile = qtile_over ? qtile_over : (uint32_t)search_query_tile(idx->dp, tqv, list_width_for(k));
  uint32_t *ctl = b.ctl.as<uint32_t>();  // [0] work, [1] nitems, [2] err
  PlanArgs a;
  fill_plan_args(idx, b, m, P, qtile, offsets, radius, a);
  uint32_t *cnt = b.cnt.as<uint32_t>(), *start = b.start.as<uint32_t>();
  uint32_t *tcnt = b.tcnt.as<uint32_t>(), *tstart = b.tstart.as<uint32_t>();

  CK(cudaMemsetAsync(cnt, 0, (nr + 1) * sizeof(uint32_t), s));
  CK(cudaMemsetAsync(b.cursor.p, 0, (nr + 1) * sizeof(uint32_t), s));
  a.list_cnt = cnt;
  a.phase = 0;
  CK(launch_plan_pass(a, mode, s));
  CK(launch_exclusive_scan(cnt, start, nr + 1, b.scan_tmp.p, ctl + 2, s));
  a.list_cnt = start;
  a.phase = 1;
  CK(launch_plan_pass(a, mode, s));
  if (stage == 0) return RBC_OK;
  CK(launch_tiles_per_list(cnt, offsets, nr, qtile, idx->item_rows, filter, tcnt, s));
  CK(launch_exclusive_scan(tcnt, tstart, nr + 1, b.scan_tmp.p, ctl + 2, s));
  CK(launch_plan_items(cnt, start, tstart, offsets, nr, qtile, idx->item_rows, filter, b.items.as<SearchItem>(),
                       b.item_cap, ctl + 1, ctl + 2, s));
  if (stage == 1) return RBC_OK;

  SearchArgs sa{};
  sa.X = X;
  sa.pid = pid;
  sa.Q = b.Qp.as<float>();
  sa.qidx = b.pair_q.as<uint32_t>();
  sa.qthr = mode == 0 ? nullptr : b.pair_thr.as<float>();
  sa.items = b.items.as<SearchItem>();
  sa.nitems = ctl + 1;
  sa.work = ctl;
  sa.res_d = b.res_d.as<float>();
  sa.res_i = b.res_i.as<uint32_t>();
  sa.tau = b.tau.as<uint32_t>();
  sa.lock = b.lock.as<uint32_t>();
  sa.err = ctl + 2;
  sa.stats = stats;
  sa.ld = idx->ld;
  sa.dp = idx->dp;
  sa.k = k;
  CK(cudaMemsetAsync(ctl, 0, sizeof(uint32_t), s));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (idx->profile) {
    while (idx->ev_pool.size() < idx->ev_used + 2) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      idx->ev_pool.push_back(e);
    }
    e0 = idx->ev_pool[idx->ev_used++];
    e1 = idx->ev_pool[idx->ev_used++];
    CK(cudaEventRecord(e0, s));
  }
  CK(launch_search(idx->metric, sa, grid, s, tqv));
  if (e1) CK(cudaEventRecord(e1, s));
  return RBC_OK;
}

// List r contributes ceil(cnt_r / qtile) x c_r items, c_r = its row chunks
// (sum over lists <= n / item_rows + nr + 1); cnt_r <= mb, and in a probe
// round sum cnt_r <= mb x probes, which bounds the tiles by
// mb x probes / qtile + nr and each list's chunks by the largest list's.
uint64_t item_capacity(const rbc_index *idx, uint64_t mb, uint32_t qtile, uint32_t probes) {
  const uint64_t rows = std::max<uint32_t>(idx->item_rows, 1);
  const uint64_t chunks = idx->n / rows + idx->nr + 1;
  const uint64_t any = (mb / qtile + 1) * chunks + idx->nr + 1;
  if (!probes) return any;
  const uint64_t max_chunks = idx->max_list / rows + 1;
  return std::min(any, (mb * probes / qtile + idx->nr + 1) * max_chunks + idx->nr + 1);
}

namespace {

}  // namespace

// ------------------------------------------------------------------ build
int build_tc(rbc_index *idx, cudaStream_t s) {
  if (idx->metric != RBC_L2) return fail(RBC_ERR_UNSUPPORTED, "rbc_build: the tensor-core form is L2 only");
  if (!tc_supported(idx->dp)) return fail(RBC_ERR_UNSUPPORTED, "rbc_build: the tensor-core form needs d <= 128");
  idx->kp = tc_kp(idx->d);
  idx->n_pad = (idx->n + 127) / 128 * 128;
  DevBuf rid;
  CK(rid.alloc(idx->nr * 4ull, s));
  CK(cudaMemcpyAsync(rid.p, idx->rep_ids.data(), idx->nr * 4ull, cudaMemcpyHostToDevice, s));
  TRY(tc_build(idx->Xp, idx->perm, idx->offsets, idx->R, idx->radius, rid.as<uint32_t>(), idx->n, idx->n_pad,
               idx->nr, idx->d, idx->ld, idx->kp, &idx->tc, &idx->device_bytes, s));
  CK(tc_make_map(&idx->tmB, idx->tc.Xh, idx->n_pad, idx->tc.cols, 128));
  CK(cudaStreamSynchronize(s));
  return RBC_OK;
}

int build_index(const float *dX, uint64_t n, uint32_t d, uint32_t ldx, const rbc_build_params *p,
                cudaStream_t s, rbc_index **out) {
  if (!out) return fail(RBC_ERR_INVALID, "rbc_build: out is NULL");
  *out = nullptr;
  if (!p) return fail(RBC_ERR_INVALID, "rbc_build: params is NULL");
  if (!dX) return fail(RBC_ERR_INVALID, "rbc_build: X is NULL");
  TRY(check_dims(d, ldx, "rbc_build"));
  if (n == 0 || n >= 0xFFFFFFFFull) return fail(RBC_ERR_INVALID, "rbc_build: n must be in [1, 2^32-1)");
  if (p->metric != RBC_L2 && p->metric != RBC_L1) return fail(RBC_ERR_INVALID, "rbc_build: unknown metric");
  if (p->num_reps == 0 || p->num_reps > n)
    return fail(RBC_ERR_INVALID, "rbc_build: num_reps must be in [1, n]");
  if (p->num_reps > 32768) return fail(RBC_ERR_UNSUPPORTED, "rbc_build: num_reps above 32768");
  uint32_t flags = p->flags ? p->flags : RBC_BUILD_PARTITION;
  if ((flags & RBC_BUILD_ONESHOT) && p->s == 0) return fail(RBC_ERR_INVALID, "rbc_build: s must be >= 1");
  pool_setup();

  rbc_index *idx = new rbc_index();
  struct Guard {
    rbc_index *&i;
    ~Guard() {
      if (i) rbc_destroy(i);
    }
  } guard{idx};
  CK(cudaGetDevice(&idx->device));
  idx->n = n;
  idx->d = d;
  idx->ld = pad16(d);
  idx->dp = pad4(d);
  idx->metric = p->metric;
  idx->flags = flags;
  idx->nr = p->num_reps;
  const uint32_t nr = idx->nr, ld = idx->ld;

  // representatives
  if (p->rep_ids) {
    idx->rep_ids.assign(p->rep_ids, p->rep_ids + nr);
    std::vector<uint32_t> sorted = idx->rep_ids;
    std::sort(sorted.begin(), sorted.end());
    if (sorted.back() >= n) return fail(RBC_ERR_INVALID, "rbc_build: rep id out of range");
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
      return fail(RBC_ERR_INVALID, "rbc_build: rep ids are not distinct");
  } else {
    sample_reps(n, nr, p->seed, idx->rep_ids);
  }

  // padded copy of the input (zero columns past d, zero rows up to pad16(n))
  idx->xi_rows = pad16((uint32_t)std::min<uint64_t>(n, 0xFFFFFFF0ull));
  if (idx->xi_rows < n) idx->xi_rows = n;
  DevBuf xi_tmp;
  float *Xi = nullptr;
  size_t xi_bytes = (size_t)idx->xi_rows * ld * 4;
  if (flags & kBuildKeepInput) {
    CK(cudaMalloc(&idx->Xi, xi_bytes));
    Xi = idx->Xi;
    idx->device_bytes += xi_bytes;
  } else {
    CK(xi_tmp.alloc(xi_bytes, s));
    Xi = xi_tmp.as<float>();
  }
  CK(cudaMemsetAsync(Xi + n * ld, 0, (idx->xi_rows - n) * ld * 4, s));
  CK(launch_pad_rows(dX, ldx, Xi, ld, n, d, s));

  DevBuf rid;
  CK(rid.alloc(nr * 4, s));
  CK(cudaMemcpyAsync(rid.p, idx->rep_ids.data(), nr * 4, cudaMemcpyHostToDevice, s));
  size_t r_bytes = (size_t)pad16(nr) * ld * 4;
  CK(cudaMalloc(&idx->R, r_bytes));
  idx->device_bytes += r_bytes;
  CK(cudaMemsetAsync(idx->R, 0, r_bytes, s));
  CK(launch_gather_rows(Xi, ld, rid.as<uint32_t>(), nr, idx->R, s));

  if (flags & RBC_BUILD_PARTITION) {
    DevBuf odist, hist, hscan, tmp;
    const uint32_t ntiles = (uint32_t)((n + owner_tile_rows() - 1) / owner_tile_rows());
    const uint64_t hn = (uint64_t)nr * ntiles;
    CK(odist.alloc(n * 4, s));
    CK(hist.alloc(hn * 4, s));
    CK(hscan.alloc(hn * 4, s));
    CK(tmp.alloc(scan_temp_bytes(hn), s));
    CK(cudaMalloc(&idx->owner, n * 4));
    CK(cudaMalloc(&idx->perm, n * 4));
    CK(cudaMalloc(&idx->offsets, (nr + 1) * 8));
    CK(cudaMalloc(&idx->radius, nr * 4));
    CK(cudaMalloc(&idx->Xp, (size_t)n * ld * 4));
    idx->device_bytes += 2 * n * 4 + (nr + 1) * 8 + nr * 4 + (size_t)n * ld * 4;
    CK(launch_argmin(idx->metric, Xi, n, idx->R, nr, ld, idx->dp, idx->owner, odist.as<float>(), s));
    CK(launch_owner_hist(idx->owner, n, nr, hist.as<uint32_t>(), ntiles, s));
    CK(launch_exclusive_scan(hist.as<uint32_t>(), hscan.as<uint32_t>(), hn, tmp.p, nullptr, s));
    CK(launch_owner_scatter(idx->owner, n, nr, hscan.as<uint32_t>(), ntiles, idx->perm, s));
    CK(launch_list_offsets(hscan.as<uint32_t>(), nr, ntiles, n, idx->offsets, s));
    CK(launch_list_radius(idx->offsets, idx->perm, odist.as<float>(), nr, idx->radius, s));
    CK(launch_gather_rows(Xi, ld, idx->perm, n, idx->Xp, s));
    std::vector<uint64_t> &off = idx->h_offsets;
    off.resize(nr + 1);
    CK(cudaMemcpyAsync(off.data(), idx->offsets, (nr + 1) * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    idx->min_list = UINT64_MAX;
    idx->max_list = 0;
    for (uint32_t r = 0; r < nr; r++) {
      uint64_t c = off[r + 1] - off[r];
      idx->min_list = std::min(idx->min_list, c);
      idx->max_list = std::max(idx->max_list, c);
    }
  }

  if (flags & RBC_BUILD_BF16) {
    if (!(flags & RBC_BUILD_PARTITION))
      return fail(RBC_ERR_INVALID, "rbc_build: RBC_BUILD_BF16 needs RBC_BUILD_PARTITION");
    TRY(build_tc(idx, s));
  }

  if (flags & RBC_BUILD_ONESHOT) {
    const uint32_t s_eff = (uint32_t)std::min<uint64_t>(p->s, n);
    idx->s = s_eff;
    idx->lds = pad16(p->s);
    size_t lists_bytes = (size_t)pad16(nr) * idx->lds * 4;
    const uint64_t total = (uint64_t)nr * s_eff;
    CK(cudaMalloc(&idx->os_lists, lists_bytes));
    CK(cudaMemsetAsync(idx->os_lists, 0, lists_bytes, s));
    CK(cudaMalloc(&idx->os_counts, nr * 4));
    CK(cudaMalloc(&idx->os_offsets, (nr + 1) * 8));
    CK(cudaMalloc(&idx->os_ids, total * 4));
    CK(cudaMalloc(&idx->Xo, total * ld * 4));
    idx->device_bytes += lists_bytes + nr * 4 + (nr + 1) * 8 + total * 4 + total * ld * 4;
    // distance block per group of representatives, bounded to ~4 GiB
    const uint64_t ldD = (n + 3) / 4 * 4;
    uint64_t rows_per = std::max<uint64_t>(1, (4ull << 30) / (ldD * 4));
    rows_per = std::min<uint64_t>(rows_per, nr);
    DevBuf Dbuf, thr, need;
    CK(Dbuf.alloc(rows_per * ldD * 4, s));
    CK(thr.alloc(nr * 4, s));
    CK(need.alloc(nr * 4, s));
    for (uint64_t r0 = 0; r0 < nr; r0 += rows_per) {
      uint32_t rows = (uint32_t)std::min<uint64_t>(rows_per, nr - r0);
      CK(launch_dense_dist(idx->metric, idx->R + r0 * ld, rows, Xi, n, ld, idx->dp, Dbuf.as<float>(), ldD, s));
      CK(launch_row_select(Dbuf.as<float>(), ldD, rows, n, s_eff, thr.as<uint32_t>() + r0,
                           need.as<uint32_t>() + r0, s));
      CK(launch_row_compact(Dbuf.as<float>(), ldD, rows, n, thr.as<uint32_t>() + r0, need.as<uint32_t>() + r0,
                            idx->os_lists + r0 * idx->lds, idx->lds, idx->os_counts + r0, s));
    }
    // every list holds exactly s_eff ids: list r is rows [r s_eff, (r+1) s_eff) of Xo
    std::vector<uint64_t> off(nr + 1);
    for (uint32_t r = 0; r <= nr; r++) off[r] = (uint64_t)r * s_eff;
    CK(cudaMemcpyAsync(idx->os_offsets, off.data(), (nr + 1) * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpy2DAsync(idx->os_ids, (size_t)s_eff * 4, idx->os_lists, (size_t)idx->lds * 4, (size_t)s_eff * 4,
                         nr, cudaMemcpyDeviceToDevice, s));
    CK(launch_gather_rows(Xi, ld, idx->os_ids, total, idx->Xo, s));
    CK(cudaStreamSynchronize(s));  // off[] is a host array
  }
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  *out = idx;
  idx = nullptr;
  return RBC_OK;
}

// ------------------------------------------------------------------ query
int query_tc(rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode, uint32_t *dIds,
             float *dDists, uint32_t ldo, cudaStream_t s);

// Exact mode: nearest-rep probe round, then the pruned round over every other
// list (plan.cu).  One-shot mode: the probe round alone over the one-shot
// lists, which is the reference's kqueryRBC algorithm (rbc.cu:72-123).
// Tensor mode: query_tc.
int query_index(rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
                uint32_t *dIds, float *dDists, uint32_t ldo, cudaStream_t s) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_query: index is NULL");
  if (k < 1 || k > (uint32_t)kMaxListWidth) return fail(RBC_ERR_INVALID, "rbc_query: k must be in [1, 128]");
  if (ldo < k) return fail(RBC_ERR_INVALID, "rbc_query: ldo < k");
  if (ldq < idx->d) return fail(RBC_ERR_INVALID, "rbc_query: ldq < d");
  if (m == 0) return RBC_OK;
  if (!dQ || (!dIds && !dDists)) return fail(RBC_ERR_INVALID, "rbc_query: NULL buffer");
  if (m >= 0xFFFFFFFFull) return fail(RBC_ERR_INVALID, "rbc_query: m must be below 2^32-1");
  const bool nosync = (mode & kQueryNoSync) != 0;
  const uint32_t base = mode & 0xFFu;
  const float *X;
  const uint32_t *pid;
  const uint64_t *offsets;
  if (base == RBC_QUERY_EXACT) {
    if (!(idx->flags & RBC_BUILD_PARTITION)) return fail(RBC_ERR_INVALID, "rbc_query: index has no partition lists");
    X = idx->Xp;
    pid = idx->perm;
    offsets = idx->offsets;
  } else if (base == RBC_QUERY_ONESHOT) {
    if (!(idx->flags & RBC_BUILD_ONESHOT)) return fail(RBC_ERR_INVALID, "rbc_query: index has no one-shot lists");
    X = idx->Xo;
    pid = idx->os_ids;
    offsets = idx->os_offsets;
  } else if (base == RBC_QUERY_EXACT_TC) {
    if (!(idx->flags & RBC_BUILD_BF16)) return fail(RBC_ERR_INVALID, "rbc_query: index has no BF16 lists");
    // the autotuner may have found the router's picks not worth their cost
    if (idx->tc_unrouted) mode &= ~(uint32_t)RBC_QUERY_ROUTED;
    if (k <= kTcMaxK && !idx->tc_plain) return query_tc(idx, dQ, m, ldq, k, mode, dIds, dDists, ldo, s);
    // wider k (the shortlists stop at 56 entries), or the autotuner found the
    // plain search faster: the FP32 exact search over the same partition
    // lists answers (a BF16 index always has them); no query falls back
    idx->fallback_ids.clear();
    return query_index(idx, dQ, m, ldq, k, (mode & ~0xFFu) | RBC_QUERY_EXACT, dIds, dDists, ldo, s);
  } else {
    return fail(RBC_ERR_INVALID, "rbc_query: unknown mode");
  }
  pool_setup();
  const uint32_t nr = idx->nr, ld = idx->ld;
  const bool routed = (mode & RBC_QUERY_ROUTED) && base == RBC_QUERY_EXACT;
  if (routed && !idx->router) return fail(RBC_ERR_INVALID, "rbc_query: RBC_QUERY_ROUTED without a router");
  // probe table: the nearest representative, then (routed) the router's picks
  const uint32_t Pn = std::min(kDefaultProbes, nr);
  const uint32_t P = routed ? Pn + std::min(idx->router_probes, nr - Pn) : Pn;
  const uint32_t kw = list_width_for(k);
  const uint32_t qtile = (uint32_t)search_query_tile(idx->dp, idx->tune_tq, kw);
  const int grid = search_grid(idx->metric, idx->dp, idx->tune_tq, kw);
  // batch so the m x nr plan arrays stay near 2^29 entries (~10 bytes each)
  const uint64_t mb = std::min<uint64_t>(m, std::max<uint64_t>(qtile, (1ull << 29) / nr));
  QueryBufs b;
  const uint64_t pair_cap = mb * nr;
  const uint64_t item_cap = item_capacity(idx, mb, qtile);
  CK(b.Qp.alloc(mb * ld * 4, s));
  CK(b.Dqr.alloc(mb * nr * 4, s));
  CK(b.probe.alloc(mb * P * 4, s));
  CK(b.probed.alloc(mb * P * 4, s));
  CK(b.res_d.alloc(mb * kw * 4, s));
  CK(b.res_i.alloc(mb * kw * 4, s));
  CK(b.tau.alloc(mb * 4, s));
  CK(b.lock.alloc(mb * 4, s));
  CK(b.cnt.alloc((nr + 1) * 4, s));
  CK(b.start.alloc((nr + 1) * 4, s));
  CK(b.cursor.alloc((nr + 1) * 4, s));
  CK(b.tcnt.alloc((nr + 1) * 4, s));
  CK(b.tstart.alloc((nr + 1) * 4, s));
  CK(b.pair_q.alloc(pair_cap * 4, s));
  CK(b.pair_thr.alloc(pair_cap * 4, s));
  CK(b.items.alloc(item_cap * sizeof(SearchItem), s));
  b.item_cap = item_cap;
  CK(b.ctl.alloc(64, s));
  CK(b.scan_tmp.alloc(scan_temp_bytes(nr + 1), s));
  DevBuf stats, near, near_d, logits;
  if (routed) {
    CK(near.alloc(mb * Pn * 4, s));
    CK(near_d.alloc(mb * Pn * 4, s));
    if (!idx->router->r.top_ok(P)) CK(logits.alloc(mb * nr * 4, s));
  }
  CK(stats.alloc(2 * sizeof(unsigned long long), s));
  CK(cudaMemsetAsync(stats.p, 0, 2 * sizeof(unsigned long long), s));
  CK(cudaMemsetAsync(b.ctl.p, 0, 64, s));
  idx->ev_used = 0;
  for (uint64_t b0 = 0; b0 < m; b0 += mb) {
    const uint64_t mq = std::min(mb, m - b0);
    CK(launch_pad_rows(dQ + b0 * ldq, ldq, b.Qp.as<float>(), ld, mq, idx->d, s));
    CK(launch_dense_dist(idx->metric, b.Qp.as<float>(), mq, idx->R, nr, ld, idx->dp, b.Dqr.as<float>(), nr, s));
    if (routed) {
      CK(launch_row_topp(b.Dqr.as<float>(), mq, nr, Pn, near.as<uint32_t>(), near_d.as<float>(), s));
      Router &rt = idx->router->r;
      if (rt.top_ok(P)) {
        // the last layer fused with the selection: no logits written
        CK(rt.probes_tc(b.Qp.as<float>(), ld, (uint32_t)mq, P - Pn, Pn, near.as<uint32_t>(), near_d.as<float>(),
                        b.probe.as<uint32_t>(), b.probed.as<float>(), b.ctl.as<uint32_t>() + 2, s));
      } else {
        if (rt.tc_ok()) {
          CK(rt.forward_tc(b.Qp.as<float>(), ld, (uint32_t)mq, logits.as<float>(), b.ctl.as<uint32_t>() + 2, s));
        } else {
          const uint32_t chunk = 4096;
          CK(rt.alloc_batch(chunk, s));
          for (uint64_t i = 0; i < mq; i += chunk) {
            const uint32_t cb = (uint32_t)std::min<uint64_t>(chunk, mq - i);
            CK(rt.forward(b.Qp.as<float>() + i * ld, ld, cb, logits.as<float>() + i * nr, s));
          }
        }
        CK(launch_router_probes(logits.as<float>(), mq, nr, P - Pn, Pn, near.as<uint32_t>(), near_d.as<float>(),
                                b.probe.as<uint32_t>(), b.probed.as<float>(), s));
      }
    } else {
      CK(launch_row_topp(b.Dqr.as<float>(), mq, nr, P, b.probe.as<uint32_t>(), b.probed.as<float>(), s));
    }
    CK(launch_init_results(b.res_d.as<float>(), b.res_i.as<uint32_t>(), b.tau.as<uint32_t>(),
                           b.lock.as<uint32_t>(), mq, kw, s));
    TRY(plan_and_search(idx, b, mq, P, k, 0, X, pid, offsets, idx->radius, grid, stats.as<unsigned long long>(), s));
    if (base == RBC_QUERY_EXACT)
      TRY(plan_and_search(idx, b, mq, P, k, 1, X, pid, offsets, idx->radius, grid, stats.as<unsigned long long>(), s));
    CK(launch_write_results(b.res_d.as<float>(), b.res_i.as<uint32_t>(), mq, k, kw, dIds ? dIds + b0 * ldo : nullptr,
                            dDists ? dDists + b0 * ldo : nullptr, ldo, s));
  }
  idx->stats.queries = m;
  idx->stats.rep_pairs = m * nr;
  idx->stats.fallback_queries = 0;
  if (!nosync) {
    unsigned long long st[2] = {0, 0};
    uint32_t ctl[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(st, stats.p, sizeof(st), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ctl, b.ctl.p, sizeof(ctl), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    idx->stats.point_pairs = st[0];
    idx->stats.lists_probed = st[1];
    if (ctl[2]) return fail((int)ctl[2], "rbc_query: a device-side check failed (bounded wait or work-list size)");
    if (idx->profile) {
      idx->prof.search_launches = idx->ev_used / 2;
      idx->prof.search_ms = 0;
      idx->prof.pruned_launches = 0;
      idx->prof.pruned_ms = 0;
      idx->prof.pruned_pairs = 0;
      for (size_t i = 0; i + 1 < idx->ev_used; i += 2) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, idx->ev_pool[i], idx->ev_pool[i + 1]));
        idx->prof.search_ms += ms;
      }
    }
  }
  return RBC_OK;
}

// Tensor-core exact query (tc_search.cu): an RBC query whose bulk list search
// runs on the tensor cores, in two rounds like the plain form:
//   1. query x representative distances, probe table (the nearest
//      representatives, plus the router's picks when routed);
//   2. probe round: the probed lists searched exactly on the FP32 path for
//      each query's top-sl (a probed list holds few queries, so the tensor
//      tiles would run nearly empty); that list seeds the query's shortlist
//      and its k-th distance (an upper bound on the true one) is the pruning
//      threshold;
//   3. pruned round: the pruning plan over every other list, tensor search of
//      the surviving (list, query) items into the same shortlists, exact
//      rerank and certificate; uncertified queries are recomputed by the
//      plain exact path.
// Rows of pruned lists cannot be in the top k (exact bounds), so the
// certificate covers everything.  The rounds need no host round trip.
// The host-side choices and every buffer of a tensor-form round for batches
// of up to mb queries (see TcQuery).
int tc_setup(rbc_index *idx, uint64_t mb, uint32_t k, uint32_t mode, bool graph, TcQuery &t, cudaStream_t s) {
  const uint32_t nr = idx->nr, ld = idx->ld, cols = idx->tc.cols;
  t.routed = (mode & RBC_QUERY_ROUTED) != 0;
  if (t.routed && !idx->router) return fail(RBC_ERR_INVALID, "rbc_query: RBC_QUERY_ROUTED without a router");
  if (graph && t.routed) return fail(RBC_ERR_UNSUPPORTED, "rbc_query: routed tensor-form queries in a graph");
  // lists searched in the probe round: the nearest representatives' (plus,
  // routed, the router's picks among the others); RBC_TC_PROBES overrides the
  // number of nearest ones; RBC_TC_ROUTER_ONLY (routed calls): none, the
  // router's picks alone.
  // A routed call whose router has a distance head and probes = 0 skips the
  // probe round: every list is planned with tau = min(predicted k-th
  // distance, k-th nearest representative), the shortlists are capped at
  // tau (1 + 2^-10), and a query is accepted only if its exact k-th distance
  // is at most tau; the others are answered again with the probe round.
  t.spec = t.routed && idx->router->r.T && idx->router_probes == 0;
  uint32_t Pn = idx->tc_probes ? idx->tc_probes : kTcProbes;
  if (Pn == RBC_TC_ROUTER_ONLY) Pn = t.routed ? 0 : 1;
  if (const char *env = std::getenv("RBC_TC_PROBES")) Pn = std::max(1, std::min(16, std::atoi(env)));
  if (t.spec) Pn = 1;  // the nearest representative only: the bound needs its distance
  t.Pn = Pn = std::min(Pn, nr);
  t.Pnear = std::max(Pn, 1u);  // nearest representatives found (the bound needs the first)
  t.P = t.routed && !t.spec ? Pn + std::min(idx->router_probes, nr - Pn) : Pn;
  t.k = k;
  t.mb = mb;
  t.grid = tc_grid();
  t.sgrid = search_grid(idx->metric, idx->dp, idx->tune_tq);
  // the probe round's FP32 lists hold a whole shortlist; its query tiles
  // follow the probed queries per list (16 wide when few share a list)
  t.sl = tc_shortlist(k);
  t.kw = list_width_for(t.sl);
  t.probe_rows = idx->tc_probe_rows == RBC_TC_PREFIX_NONE ? 0 : idx->tc_probe_rows ? idx->tc_probe_rows : kTcProbeRows;
  if (const char *env = std::getenv("RBC_TC_PROBE_ROWS")) t.probe_rows = std::strtoull(env, nullptr, 10);
  t.probe_cap = idx->tc_probe_cap;
  t.qtile = tc_query_tile(idx->tc.format);
  const uint64_t probe_per_list = mb * t.P / nr;
  t.ptq = search_tq_for(idx->dp, probe_per_list >= 48 ? 4 : (probe_per_list >= 24 ? 2 : 1), t.kw);
  t.pgrid = search_grid(idx->metric, idx->dp, t.ptq, t.kw);
  const uint32_t P = t.P, sl = t.sl, kw = t.kw;
  QueryBufs &b = t.b;
  // work items of the three plans: pruned round (query tiles of qtile), probe
  // round on the FP32 path (16) and on the tensor cores (128)
  const uint64_t pair_cap = mb * nr,
                 item_cap = std::max({item_capacity(idx, mb, t.qtile), item_capacity(idx, mb, 16, P),
                                      item_capacity(idx, mb, tc_query_tile(kTcSplit), P)});
  CK(b.Qp.alloc(mb * ld * 4, s));
  CK(b.Dqr.alloc(mb * nr * 4, s));
  CK(b.probe.alloc(mb * P * 4, s));
  CK(b.probed.alloc(mb * P * 4, s));
  CK(b.res_d.alloc(mb * kw * 4, s));
  CK(b.res_i.alloc(mb * kw * 4, s));
  CK(b.tau.alloc(mb * 4, s));
  CK(b.lock.alloc(mb * 4, s));
  CK(b.cnt.alloc((nr + 1) * 4, s));
  CK(b.start.alloc((nr + 1) * 4, s));
  CK(b.cursor.alloc((nr + 1) * 4, s));
  CK(b.tcnt.alloc((nr + 1) * 4, s));
  CK(b.tstart.alloc((nr + 1) * 4, s));
  CK(b.pair_q.alloc(pair_cap * 4, s));
  CK(b.pair_thr.alloc(pair_cap * 4, s));
  CK(b.items.alloc(item_cap * sizeof(SearchItem), s));
  b.item_cap = item_cap;
  CK(b.ctl.alloc(64, s));
  CK(b.scan_tmp.alloc(scan_temp_bytes(nr + 1), s));
  b.plan_all = t.spec;
  if (t.spec) {
    CK(t.tpred.alloc(mb * 4, s));
  } else if (t.routed) {
    CK(t.near.alloc(mb * t.Pnear * 4, s));
    CK(t.near_d.alloc(mb * t.Pnear * 4, s));
    if (!idx->router->r.top_ok(P)) CK(t.logits.alloc(mb * nr * 4, s));
    // without nearest lists in the probe table the pruning bound takes the
    // nearest representative's distance from here
    if (Pn == 0) b.dq0 = t.near_d.as<float>();
  }
  CK(t.Qh.alloc((mb + 1) * cols * 2, s));
  CK(t.qscale.alloc((mb + 1) * 4, s));
  CK(t.qnorm.alloc((mb + 1) * 4, s));
  CK(t.qinex.alloc(mb + 1, s));
  CK(t.sl_a.alloc(2 * mb * sl * 4, s));
  CK(t.seed_a.alloc(mb * sl * 4, s));
  CK(t.seed_row.alloc(mb * sl * 4, s));
  CK(t.sl_row.alloc(2 * mb * sl * 4, s));
  CK(t.sl_sel.alloc(mb * 4, s));
  CK(t.sl_theta.alloc(mb * 4, s));
  CK(t.sl_lock.alloc(mb * 4, s));
  // the BF16 format's error bound is small next to 2^-7 tau, so its
  // certificate passes under the cap; the FP16 hi/lo format's bound can be
  // larger (RBC_TC_TAU_CAP=0 or 1 overrides)
  t.cap = idx->tc.format == kTcExact;
  if (const char *env = std::getenv("RBC_TC_TAU_CAP")) t.cap = std::atoi(env) != 0;
  CK(t.sl_cap.alloc(mb * 4, s));
  CK(t.drop.alloc(mb * 4, s));
  CK(t.emax.alloc(mb * 4, s));
  CK(t.ctl.alloc(64, s));
  CK(t.failq.alloc(mb * 4, s));
  CK(t.stats.alloc(4 * sizeof(unsigned long long), s));  // pruned round [0, 1], probe round [2, 3]
  if (graph) {
    // the device fallback: every (row chunk, 16 TQ listed queries) pair for
    // as many queries as the batch holds
    const uint32_t fkw = list_width_for(k);
    t.fb_qtile = (uint32_t)search_query_tile(idx->dp, 0, fkw);
    t.fb_grid = search_grid(idx->metric, idx->dp, 0, fkw);
    t.fb_chunk = (uint32_t)std::max<uint64_t>(4096, (idx->n + 4ull * t.fb_grid - 1) / (4ull * t.fb_grid));
    t.fb_chunk = (t.fb_chunk + 31) / 32 * 32;
    t.fb_cap = ((idx->n + t.fb_chunk - 1) / t.fb_chunk) * ((mb + t.fb_qtile - 1) / t.fb_qtile);
    CK(t.fb_items.alloc(std::max<uint64_t>(t.fb_cap, 1) * sizeof(SearchItem), s));
    CK(t.fb_ctl.alloc(64, s));
  }
  return RBC_OK;
}

// The kernels of one batch of mq <= t.mb queries (their rows at dQ, results
// to dIds / dDists).  Outside graph mode the caller reads the control words
// and answers the uncertified queries; *tc_probe tells whether a tensor probe
// round ran (its launch was timed into events 2 and 3 when profiling).
int tc_enqueue(rbc_index *idx, TcQuery &t, const float *dQ, uint64_t mq, uint32_t ldq, uint32_t *dIds, float *dDists,
               uint32_t ldo, bool graph, uint32_t *err_sink, bool *tc_probe, cudaStream_t s) {
  const uint32_t nr = idx->nr, ld = idx->ld, kp = idx->kp, fmt = idx->tc.format, cols = idx->tc.cols;
  const uint32_t k = t.k, sl = t.sl, kw = t.kw, P = t.P, Pn = t.Pn;
  const bool spec = t.spec, prof = idx->profile && !graph;
  QueryBufs &b = t.b;
  if (tc_probe) *tc_probe = false;
  CK(cudaMemsetAsync(b.ctl.p, 0, 64, s));
  CK(cudaMemsetAsync(t.ctl.p, 0, 64, s));
  CK(cudaMemsetAsync(t.drop.p, 0x7F, mq * 4, s));  // 0x7F7F7F7F: a finite float above every distance
  if (graph) CK(cudaMemsetAsync(t.stats.p, 0, 4 * sizeof(unsigned long long), s));
  // 1. distances to the representatives, probe table
  CK(launch_pad_rows(dQ, ldq, b.Qp.as<float>(), ld, mq, idx->d, s));
  CK(launch_dense_dist(idx->metric, b.Qp.as<float>(), mq, idx->R, nr, ld, idx->dp, b.Dqr.as<float>(), nr, s));
  // the nearest representatives: the shortlist seed and, first, the probe table
  if (t.routed && !spec) {
    CK(launch_rep_seed(b.Dqr.as<float>(), mq, nr, idx->tc.rep_rows, sl, t.seed_a.as<float>(),
                       t.seed_row.as<uint32_t>(), t.Pnear, t.near.as<uint32_t>(), t.near_d.as<float>(), s));
    Router &rt = idx->router->r;
    if (rt.top_ok(P)) {
      // the last layer fused with the selection: no logits written
      CK(rt.probes_tc(b.Qp.as<float>(), ld, (uint32_t)mq, P - Pn, Pn, t.near.as<uint32_t>(), t.near_d.as<float>(),
                      b.probe.as<uint32_t>(), b.probed.as<float>(), b.ctl.as<uint32_t>() + 2, s));
    } else {
      if (rt.tc_ok()) {
        CK(rt.forward_tc(b.Qp.as<float>(), ld, (uint32_t)mq, t.logits.as<float>(), b.ctl.as<uint32_t>() + 2, s));
      } else {
        const uint32_t chunk = 4096;
        CK(rt.alloc_batch(chunk, s));
        for (uint64_t i = 0; i < mq; i += chunk) {
          const uint32_t cb = (uint32_t)std::min<uint64_t>(chunk, mq - i);
          CK(rt.forward(b.Qp.as<float>() + i * ld, ld, cb, t.logits.as<float>() + i * nr, s));
        }
      }
      CK(launch_router_probes(t.logits.as<float>(), mq, nr, P - Pn, Pn, t.near.as<uint32_t>(), t.near_d.as<float>(),
                              b.probe.as<uint32_t>(), b.probed.as<float>(), s));
    }
  } else {
    CK(launch_rep_seed(b.Dqr.as<float>(), mq, nr, idx->tc.rep_rows, sl, t.seed_a.as<float>(),
                       t.seed_row.as<uint32_t>(), P, b.probe.as<uint32_t>(), b.probed.as<float>(), s));
    if (spec)
      CK(idx->router->r.predict_tau(b.Qp.as<float>(), ld, (uint32_t)mq, b.probed.as<float>(), t.tpred.as<float>(),
                                    b.ctl.as<uint32_t>() + 2, s));
  }
  CK(launch_init_results(b.res_d.as<float>(), b.res_i.as<uint32_t>(), b.tau.as<uint32_t>(), b.lock.as<uint32_t>(), mq,
                         kw, s));
  // query operands (row mq is the zero row gathered for empty item slots)
  CK(launch_tc_queries(b.Qp.as<float>(), ld, mq, idx->d, kp, fmt, idx->tc.mu, t.Qh.p, t.qscale.as<float>(),
                       t.qnorm.as<float>(), t.qinex.as<uint8_t>(), s));
  CUtensorMap tmA;
  CK(tc_make_map(&tmA, t.Qh.p, mq + 1, cols, 1));
  CK(launch_sl_init(t.sl_a.as<float>(), t.sl_row.as<uint32_t>(), t.sl_sel.as<uint32_t>(), t.sl_theta.as<uint32_t>(),
                    t.sl_lock.as<uint32_t>(), t.emax.as<uint32_t>(), mq, sl, s));
  TcArgs ta{};
  ta.items = b.items.as<SearchItem>();
  ta.nitems = b.ctl.as<uint32_t>() + 1;
  ta.qidx = b.pair_q.as<uint32_t>();
  ta.Dqr = b.Dqr.as<float>();
  ta.nr = nr;
  ta.kb = kp / 64;
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
  ta.sl = sl;
  ta.sl_a = t.sl_a.as<float>();
  ta.sl_row = t.sl_row.as<uint32_t>();
  ta.sl_sel = t.sl_sel.as<uint32_t>();
  ta.sl_theta = t.sl_theta.as<uint32_t>();
  // the shortlist cap: from the prediction (speculative plan) or, once the
  // seed or a rerank knows an exact bound tau on the k-th distance, tau
  // (1 + 2^-7) -- rows above it cannot reach the top k, and fewer rows then
  // queue on the shortlists' merges
  uint32_t *sl_cap = spec || t.cap ? t.sl_cap.as<uint32_t>() : nullptr;
  ta.sl_cap = sl_cap;
  ta.drop = t.drop.as<uint32_t>();
  ta.keep_k = 0;
  ta.sl_lock = t.sl_lock.as<uint32_t>();
  ta.emax = t.emax.as<uint32_t>();
  ta.m = mq;
  ta.offsets = idx->offsets;
  ta.stats = t.stats.as<unsigned long long>();
  ta.err = t.ctl.as<uint32_t>();
  RerankArgs ra{};
  ra.X = idx->Xp;
  ra.pid = idx->perm;
  ra.Q = b.Qp.as<float>();
  ra.ld = ld;
  ra.dp = idx->dp;
  ra.k = k;
  ra.sl = sl;
  ra.m = mq;
  ra.sl_a = t.sl_a.as<float>();
  ra.sl_row = t.sl_row.as<uint32_t>();
  ra.sl_sel = t.sl_sel.as<uint32_t>();
  ra.emax = t.emax.as<uint32_t>();
  ra.sl_cap = sl_cap;
  ra.cap_out = t.cap ? sl_cap : nullptr;
  ra.theta = t.sl_theta.as<uint32_t>();
  ra.drop = t.drop.as<uint32_t>();
  ra.tplan = nullptr;
  ra.ldo = ldo;
  ra.nfail = t.ctl.as<uint32_t>() + 1;
  ra.fail = t.failq.as<uint32_t>();
  // probe round, small lists: searched exactly on the FP32 path; every
  // query's exact top-sl there seeds its shortlist, and its k-th distance
  // the pruning threshold (none in the speculative plan: the seed is the
  // nearest representatives, the threshold the prediction)
  if (!spec) {
    const bool keep = idx->profile;
    idx->profile = false;
    // the first probe_rows rows of every probed list (whole lists when
    // shorter): exact seeds that give the tensor round a tight threshold
    ListFilter small;
    small.take = t.probe_rows;
    const int rc = plan_and_search(idx, b, mq, P, sl, 0, idx->Xp, idx->perm, idx->offsets, idx->radius, t.pgrid,
                                   nullptr, s, 2, t.ptq, 0, small);
    idx->profile = keep;
    TRY(rc);
  }
  CK(launch_sl_seed(b.res_d.as<float>(), b.res_i.as<uint32_t>(), kw, idx->tc.iperm, t.seed_a.as<float>(),
                    t.seed_row.as<uint32_t>(), mq, sl, k, t.sl_a.as<float>(), t.sl_row.as<uint32_t>(),
                    t.sl_theta.as<uint32_t>(), b.tau.as<uint32_t>(), sl_cap, s));
  // the speculative plan: the predicted k-th distance lowers the planning
  // threshold and caps every shortlist (only rows that can still reach the
  // top k pass the tensor search's filter); the certificate then also
  // checks the k-th distance against it
  if (spec) {
    CK(launch_cap(b.tau.as<uint32_t>(), t.tpred.as<float>(), mq, t.sl_cap.as<uint32_t>(), t.sl_theta.as<uint32_t>(),
                  s));
    ra.tplan = b.tau.as<uint32_t>();
  }
  // probe round, large lists: tensor search into the seeded shortlists, one
  // 128-query tile per B tile (measured faster than two-tile items even for
  // the busiest probed lists), then the k-th exact distance of each
  // shortlist tightens the threshold
  // a probe cap c (rbc_set_tc_probe_cap): the tensor probe round takes rows
  // [probe_rows, probe_rows + c) of each probed list; the rest of the longer
  // lists follows, once the threshold is tight, in a launch of the kernel
  // with two query tiles per B tile (hub lists hold most probed rows and
  // hundreds of probing queries: c3, 8 probed lists, 65,536 rows: 370k ->
  // 376k queries/s)
  const uint64_t cap = t.probe_cap;
  if (!spec && idx->max_list > t.probe_rows) {
    ListFilter large;  // the rest of the longer lists
    large.rows_lo = t.probe_rows + 1;
    large.skip = t.probe_rows;
    if (cap) large.take = cap;
    // items twice the index's row run: each query's buffers merge once per
    // item, and the probed lists' few queries leave the launch short of work
    // items anyway (c3: 16,384 / 32,768 / 65,536 / 131,072 rows gave a 5.16 /
    // 4.48 / 4.91 / 5.09 ms probe launch; whole lists 10.2 ms)
    const uint32_t keep_rows = idx->item_rows;
    idx->item_rows = (uint32_t)std::min<uint64_t>(2ull * keep_rows, 1u << 30);
    const int prc = plan_and_search(idx, b, mq, P, k, 0, idx->Xp, idx->perm, idx->offsets, idx->radius, t.sgrid,
                                    nullptr, s, 1, -1, tc_query_tile(kTcSplit), large);
    idx->item_rows = keep_rows;
    TRY(prc);
    // the probe round's candidate buffers keep each query's best and merge
    // once per item (its lists hold few queries, many of them busy hubs,
    // where merges per buffer-full queued on the queries' locks: c3 probe
    // launch 7.7 -> 5.0 ms; the same in the pruned round measured no gain)
    TcArgs tp = ta;
    tp.stats = ta.stats + 2;
    tp.keep_k = k;
    if (prof) CK(cudaEventRecord(idx->ev_pool[2], s));
    CK(launch_tc_search(tmA, idx->tmB, tp, t.grid, s, true));
    if (prof) CK(cudaEventRecord(idx->ev_pool[3], s));
    if (tc_probe) *tc_probe = true;
    ra.tau = b.tau.as<uint32_t>();
    ra.ids = nullptr;
    ra.dists = nullptr;
    CK(launch_rerank(idx->metric, ra, s));
    if (cap && idx->max_list > t.probe_rows + cap) {
      ListFilter rest;
      rest.rows_lo = t.probe_rows + cap + 1;
      rest.skip = t.probe_rows + cap;
      TRY(plan_and_search(idx, b, mq, P, k, 0, idx->Xp, idx->perm, idx->offsets, idx->radius, t.sgrid, nullptr, s, 1,
                          -1, t.qtile, rest));
      TcArgs tr = ta;
      tr.stats = ta.stats + 2;
      CK(launch_tc_search(tmA, idx->tmB, tr, t.grid, s));
      CK(launch_rerank(idx->metric, ra, s));
    }
  }
  // pruned round: every other list whose bound survives, on the tensor
  // cores, into the same shortlists; exact rerank and certificate
  TRY(plan_and_search(idx, b, mq, P, k, 1, idx->Xp, idx->perm, idx->offsets, idx->radius, t.sgrid, nullptr, s, 1, -1,
                      t.qtile));
  if (prof) CK(cudaEventRecord(idx->ev_pool[0], s));
  CK(launch_tc_search(tmA, idx->tmB, ta, t.grid, s));
  if (prof) CK(cudaEventRecord(idx->ev_pool[1], s));
  ra.tau = nullptr;
  ra.ids = dIds;
  ra.dists = dDists;
  CK(launch_rerank(idx->metric, ra, s));
  if (!graph) return RBC_OK;
  // graph mode: the queries the certificate left open (their count and rows
  // on the device) searched again over every row on the FP32 path, their
  // answers written over the tensor form's
  const uint32_t fkw = list_width_for(k);
  uint32_t *fctl = t.fb_ctl.as<uint32_t>();  // [0] work, [1] items, [2] error
  CK(cudaMemsetAsync(fctl, 0, 64, s));
  CK(launch_init_results(b.res_d.as<float>(), b.res_i.as<uint32_t>(), b.tau.as<uint32_t>(), b.lock.as<uint32_t>(), mq,
                         fkw, s));
  CK(launch_listed_items(t.fb_items.as<SearchItem>(), fctl + 1, t.ctl.as<uint32_t>() + 1, idx->n, t.fb_chunk,
                         t.fb_qtile, t.fb_cap, fctl + 2, s));
  SearchArgs fa{};
  fa.X = idx->Xp;
  fa.pid = idx->perm;
  fa.Q = b.Qp.as<float>();
  fa.qidx = t.failq.as<uint32_t>();
  fa.items = t.fb_items.as<SearchItem>();
  fa.nitems = fctl + 1;
  fa.work = fctl;
  fa.res_d = b.res_d.as<float>();
  fa.res_i = b.res_i.as<uint32_t>();
  fa.tau = b.tau.as<uint32_t>();
  fa.lock = b.lock.as<uint32_t>();
  fa.err = fctl + 2;
  fa.ld = ld;
  fa.dp = idx->dp;
  fa.k = k;
  CK(launch_search(idx->metric, fa, t.fb_grid, s));
  CK(launch_listed_results(b.res_d.as<float>(), b.res_i.as<uint32_t>(), fkw, t.failq.as<uint32_t>(),
                           t.ctl.as<uint32_t>() + 1, mq, k, dIds, dDists, ldo, s));
  if (err_sink) {
    ErrWords w{};
    w.w[0] = t.ctl.as<uint32_t>();
    w.w[1] = b.ctl.as<uint32_t>() + 2;
    w.w[2] = fctl + 2;
    CK(launch_fold_errors(w, err_sink, s));
  }
  return RBC_OK;
}

// Tensor-core exact query: tc_setup, then per batch tc_enqueue, the control
// words read back, and the uncertified queries answered again on the host's
// command (the FP32 exact search, or for a speculative plan the tensor form
// with its probe round).
int query_tc(rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode, uint32_t *dIds,
             float *dDists, uint32_t ldo, cudaStream_t s) {
  pool_setup();
  const uint32_t nr = idx->nr, ld = idx->ld;
  // query batches of up to 2^29 (query, representative) pairs: the distances
  // and the plan take ~10 bytes a pair (5 GB at most), and a larger batch puts
  // more queries on each probed list (wider FP32 probe tiles, fuller tensor
  // tiles, fewer launches)
  const uint64_t mb = std::min<uint64_t>(m, std::max<uint64_t>(tc_query_tile(idx->tc.format), (1ull << 29) / nr));
  TcQuery t;
  TRY(tc_setup(idx, mb, k, mode, false, t, s));
  CK(cudaMemsetAsync(t.stats.p, 0, 4 * sizeof(unsigned long long), s));
  uint64_t nfail_total = 0;
  idx->fallback_ids.clear();
  double tc_ms = 0, pruned_ms = 0;
  uint32_t tc_launches = 0, pruned_launches = 0;
  while (idx->ev_pool.size() < 4 && idx->profile) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    idx->ev_pool.push_back(e);
  }
  idx->ev_used = 0;
  for (uint64_t b0 = 0; b0 < m; b0 += mb) {
    const uint64_t mq = std::min(mb, m - b0);
    bool tc_probe = false;
    TRY(tc_enqueue(idx, t, dQ + b0 * ldq, mq, ldq, dIds ? dIds + b0 * ldo : nullptr,
                   dDists ? dDists + b0 * ldo : nullptr, ldo, false, nullptr, &tc_probe, s));
    uint32_t hc[2], bc[3];
    CK(cudaMemcpyAsync(hc, t.ctl.p, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(bc, t.b.ctl.p, 12, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (hc[0] || bc[2])
      return fail(hc[0] ? (int)hc[0] : (int)bc[2], "rbc_query: a device-side check failed (bounded wait or work-list size)");
    if (idx->profile) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, idx->ev_pool[0], idx->ev_pool[1]));
      tc_ms += ms;
      tc_launches += 1;
      pruned_ms += ms;
      pruned_launches += 1;
      if (tc_probe) {
        CK(cudaEventElapsedTime(&ms, idx->ev_pool[2], idx->ev_pool[3]));
        tc_ms += ms;
        tc_launches += 1;
      }
    }
    const uint32_t nfail = hc[1];
    nfail_total += nfail;
    if (nfail) {
      std::vector<uint32_t> f(nfail);
      CK(cudaMemcpy(f.data(), t.failq.p, nfail * 4ull, cudaMemcpyDeviceToHost));
      std::sort(f.begin(), f.end());
      for (uint32_t q : f) idx->fallback_ids.push_back((uint32_t)(b0 + q));
    }
    if (nfail && (dIds || dDists)) {
      DevBuf Qf, fi, fd;
      CK(Qf.alloc((uint64_t)nfail * ld * 4, s));
      CK(fi.alloc((uint64_t)nfail * k * 4, s));
      CK(fd.alloc((uint64_t)nfail * k * 4, s));
      CK(launch_gather_rows(t.b.Qp.as<float>(), ld, t.failq.as<uint32_t>(), nfail, Qf.as<float>(), s));
      rbc_profile keep = idx->prof;
      rbc_query_stats keep_stats = idx->stats;
      const int keep_tq = idx->tune_tq;
      const bool keep_profile = idx->profile;
      int rc;
      if (t.spec) {
        // a prediction that fell short (or a certificate left open): the
        // tensor form again, with its probe round this time
        std::vector<uint32_t> keep_fb;
        keep_fb.swap(idx->fallback_ids);
        idx->profile = false;
        rc = query_tc(idx, Qf.as<float>(), nfail, ld, k, RBC_QUERY_EXACT_TC, fi.as<uint32_t>(), fd.as<float>(), k, s);
        idx->fallback_ids.swap(keep_fb);
      } else {
        idx->tune_tq = 1;  // a handful of queries: 16-query tiles
        rc = query_index(idx, Qf.as<float>(), nfail, ld, k, RBC_QUERY_EXACT, fi.as<uint32_t>(), fd.as<float>(), k, s);
      }
      idx->profile = keep_profile;
      idx->tune_tq = keep_tq;
      idx->prof = keep;
      idx->stats = keep_stats;
      TRY(rc);
      CK(launch_scatter_results(fi.as<uint32_t>(), fd.as<float>(), t.failq.as<uint32_t>(), nfail, k,
                                dIds ? dIds + b0 * ldo : nullptr, dDists ? dDists + b0 * ldo : nullptr, ldo, s));
      CK(cudaStreamSynchronize(s));
    }
  }
  unsigned long long st[4] = {0, 0, 0, 0};
  CK(cudaMemcpy(st, t.stats.p, sizeof(st), cudaMemcpyDeviceToHost));
  idx->stats.queries = m;
  idx->stats.rep_pairs = m * nr;
  idx->stats.point_pairs = st[0] + st[2];
  idx->stats.lists_probed = st[1] + st[3];
  idx->stats.fallback_queries = nfail_total;
  if (idx->profile) {
    idx->prof.search_launches = tc_launches;
    idx->prof.search_ms = tc_ms;
    idx->prof.pruned_launches = pruned_launches;
    idx->prof.pruned_ms = pruned_ms;
    idx->prof.pruned_pairs = st[0];
  }
  return RBC_OK;
}

// ------------------------------------------------------------------ brute force
// One search over the whole database split into chunks (bruteK / bruteSearch,
// brute.cu:43-88): every (chunk, query tile) pair is a work item.
int brute_knn(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t d,
              uint32_t k, int metric, uint32_t *dIds, float *dDists, uint32_t ldo, cudaStream_t s) {
  TRY(check_dims(d, std::min(ldx, ldq), "rbc_brute_knn"));
  if (k < 1 || k > (uint32_t)kMaxListWidth) return fail(RBC_ERR_INVALID, "rbc_brute_knn: k must be in [1, 128]");
  if (ldo < k) return fail(RBC_ERR_INVALID, "rbc_brute_knn: ldo < k");
  if (metric != RBC_L2 && metric != RBC_L1) return fail(RBC_ERR_INVALID, "rbc_brute_knn: unknown metric");
  if (m == 0) return RBC_OK;
  if (!dQ || (!dIds && !dDists) || (n && !dX)) return fail(RBC_ERR_INVALID, "rbc_brute_knn: NULL buffer");
  if (n >= 0xFFFFFFFFull || m >= 0xFFFFFFFFull) return fail(RBC_ERR_INVALID, "rbc_brute_knn: n, m must be below 2^32-1");
  pool_setup();
  const uint32_t ld = pad16(d), dp = pad4(d);
  const uint32_t kw = list_width_for(k);
  const uint32_t qtile = (uint32_t)search_query_tile(dp, 0, kw);
  const int grid = search_grid(metric, dp, 0, kw);
  DevBuf Xp, Qp, res_d, res_i, tau, lock, qidx, items, ctl;
  CK(Xp.alloc(std::max<uint64_t>(n, 1) * ld * 4, s));
  CK(Qp.alloc(m * ld * 4, s));
  CK(res_d.alloc(m * kw * 4, s));
  CK(res_i.alloc(m * kw * 4, s));
  CK(tau.alloc(m * 4, s));
  CK(lock.alloc(m * 4, s));
  CK(qidx.alloc(m * 4, s));
  CK(ctl.alloc(64, s));
  CK(cudaMemsetAsync(ctl.p, 0, 64, s));
  CK(launch_pad_rows(dX, ldx, Xp.as<float>(), ld, n, d, s));
  CK(launch_pad_rows(dQ, ldq, Qp.as<float>(), ld, m, d, s));
  CK(launch_init_results(res_d.as<float>(), res_i.as<uint32_t>(), tau.as<uint32_t>(), lock.as<uint32_t>(), m, kw, s));
  const uint64_t qtiles = (m + qtile - 1) / qtile;
  uint64_t nchunks = std::max<uint64_t>(1, (4ull * grid + qtiles - 1) / qtiles);
  nchunks = std::min<uint64_t>(nchunks, std::max<uint64_t>(1, n / 256));
  uint32_t chunk = (uint32_t)(((n + nchunks - 1) / nchunks + 31) / 32 * 32);
  if (chunk == 0) chunk = 32;
  nchunks = (n + chunk - 1) / chunk;
  const uint64_t nitems = nchunks * qtiles;
  CK(items.alloc(std::max<uint64_t>(nitems, 1) * sizeof(SearchItem), s));
  CK(launch_brute_items(items.as<SearchItem>(), ctl.as<uint32_t>() + 1, qidx.as<uint32_t>(), n, chunk, m, qtile, s));
  SearchArgs sa{};
  sa.X = Xp.as<float>();
  sa.pid = nullptr;
  sa.Q = Qp.as<float>();
  sa.qidx = qidx.as<uint32_t>();
  sa.qthr = nullptr;
  sa.items = items.as<SearchItem>();
  sa.nitems = ctl.as<uint32_t>() + 1;
  sa.work = ctl.as<uint32_t>();
  sa.res_d = res_d.as<float>();
  sa.res_i = res_i.as<uint32_t>();
  sa.tau = tau.as<uint32_t>();
  sa.lock = lock.as<uint32_t>();
  sa.err = ctl.as<uint32_t>() + 2;
  sa.stats = nullptr;
  sa.ld = ld;
  sa.dp = dp;
  sa.k = k;
  if (n) CK(launch_search(metric, sa, grid, s));
  CK(launch_write_results(res_d.as<float>(), res_i.as<uint32_t>(), m, k, kw, dIds, dDists, ldo, s));
  uint32_t hctl[3];
  CK(cudaMemcpyAsync(hctl, ctl.p, sizeof(hctl), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (hctl[2]) return fail((int)hctl[2], "rbc_brute_knn: a bounded device wait ran out");
  return RBC_OK;
}

int brute_range_count(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m, uint32_t ldq,
                      uint32_t d, int metric, const float *dRanges, uint32_t *dCounts, cudaStream_t s) {
  TRY(check_dims(d, std::min(ldx, ldq), "rbc_brute_range_count"));
  if (metric != RBC_L2 && metric != RBC_L1) return fail(RBC_ERR_INVALID, "rbc_brute_range_count: unknown metric");
  if (m == 0) return RBC_OK;
  if (!dQ || !dRanges || !dCounts || (n && !dX)) return fail(RBC_ERR_INVALID, "rbc_brute_range_count: NULL buffer");
  pool_setup();
  const uint32_t ld = pad16(d), dp = pad4(d);
  DevBuf Xp, Qp;
  CK(Xp.alloc(std::max<uint64_t>(n, 1) * ld * 4, s));
  CK(Qp.alloc(m * ld * 4, s));
  CK(launch_pad_rows(dX, ldx, Xp.as<float>(), ld, n, d, s));
  CK(launch_pad_rows(dQ, ldq, Qp.as<float>(), ld, m, d, s));
  CK(launch_range_count(metric, Qp.as<float>(), m, Xp.as<float>(), n, ld, dp, dRanges, dCounts, s));
  CK(cudaStreamSynchronize(s));
  return RBC_OK;
}

}  // namespace rbc

// ====================================================================== C ABI
using namespace rbc;

extern "C" {

const char *rbc_status_string(int status) {
  switch (status) {
    case RBC_OK: return "ok";
    case RBC_ERR_INVALID: return "invalid argument";
    case RBC_ERR_CUDA: return "CUDA error";
    case RBC_ERR_NOMEM: return "out of memory";
    case RBC_ERR_ITER_LIMIT: return "bounded device wait ran out";
    case RBC_ERR_UNSUPPORTED: return "unsupported shape";
    case RBC_ERR_IO: return "I/O error";
    default: return "unknown status";
  }
}

const char *rbc_last_error(void) { return g_last_error.c_str(); }

int rbc_version(void) { return 10000; }

int rbc_build(const float *dX, uint64_t n, uint32_t d, uint32_t ldx, const rbc_build_params *params, void *stream,
              rbc_index **out) {
  return build_index(dX, n, d, ldx, params, (cudaStream_t)stream, out);
}

int rbc_build_host(const float *hX, uint64_t n, uint32_t d, uint32_t ldx, const rbc_build_params *params,
                   rbc_index **out) {
  if (!hX) return fail(RBC_ERR_INVALID, "rbc_build_host: X is NULL");
  if (ldx < d || n == 0) return build_index(hX, n, d, ldx, params, nullptr, out);  // reports the error
  void *dX = nullptr;
  CK(cudaMalloc(&dX, (size_t)n * ldx * 4));
  cudaError_t e = cudaMemcpy(dX, hX, (size_t)n * ldx * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(dX);
    return cuda_fail(e, "rbc_build_host: copy of X");
  }
  int rc = build_index((const float *)dX, n, d, ldx, params, nullptr, out);
  cudaFree(dX);
  return rc;
}

int rbc_destroy(rbc_index *idx) {
  if (!idx) return RBC_OK;
  void *ptrs[] = {idx->Xp,      idx->perm,   idx->offsets, idx->radius,     idx->R,  idx->os_lists, idx->os_counts,
                  idx->os_ids, idx->os_offsets, idx->Xo,   idx->Xi,        idx->tc.Xh, idx->tc.w,  idx->tc.Wh, idx->tc.rep_rows, idx->owner,
                  idx->tc.lscale, idx->tc.lxmax, idx->tc.lcnorm, idx->tc.mu, idx->tc.iperm, idx->X64, idx->norm64};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (cudaEvent_t e : idx->ev_pool) cudaEventDestroy(e);
  delete idx;
  return RBC_OK;
}

int rbc_get_info(const rbc_index *idx, rbc_index_info *info) {
  if (!idx || !info) return fail(RBC_ERR_INVALID, "rbc_get_info: NULL argument");
  info->n = idx->n;
  info->d = idx->d;
  info->ld = idx->ld;
  info->num_reps = idx->nr;
  info->s = idx->s;
  info->metric = idx->metric;
  info->flags = idx->flags & 0xFFu;
  info->min_list = idx->min_list;
  info->max_list = idx->max_list;
  info->device_bytes = idx->device_bytes;
  info->tc_format = idx->tc.format;
  info->tc_plain = idx->tc_plain ? 1u : 0u;
  info->router_picks = idx->router ? idx->router_probes : 0u;
  info->tc_unrouted = idx->tc_unrouted ? 1u : 0u;
  info->tc_probe_cap = idx->tc_probe_cap;
  return RBC_OK;
}

int rbc_get_reps(const rbc_index *idx, uint32_t *h) {
  if (!idx || !h) return fail(RBC_ERR_INVALID, "rbc_get_reps: NULL argument");
  std::memcpy(h, idx->rep_ids.data(), idx->nr * 4);
  return RBC_OK;
}

int rbc_get_partition(const rbc_index *idx, uint64_t *h_offsets, uint32_t *h_members, float *h_radius) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_get_partition: NULL index");
  if (!(idx->flags & RBC_BUILD_PARTITION)) return fail(RBC_ERR_INVALID, "rbc_get_partition: no partition lists");
  if (h_offsets) CK(cudaMemcpy(h_offsets, idx->offsets, (idx->nr + 1) * 8, cudaMemcpyDeviceToHost));
  if (h_members) CK(cudaMemcpy(h_members, idx->perm, idx->n * 4, cudaMemcpyDeviceToHost));
  if (h_radius) CK(cudaMemcpy(h_radius, idx->radius, idx->nr * 4, cudaMemcpyDeviceToHost));
  return RBC_OK;
}

int rbc_get_oneshot(const rbc_index *idx, uint32_t *h_lists, uint32_t *h_counts) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_get_oneshot: NULL index");
  if (!(idx->flags & RBC_BUILD_ONESHOT)) return fail(RBC_ERR_INVALID, "rbc_get_oneshot: no one-shot lists");
  if (h_lists) CK(cudaMemcpy(h_lists, idx->os_ids, (size_t)idx->nr * idx->s * 4, cudaMemcpyDeviceToHost));
  if (h_counts) CK(cudaMemcpy(h_counts, idx->os_counts, idx->nr * 4, cudaMemcpyDeviceToHost));
  return RBC_OK;
}

int rbc_query(rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode, uint32_t *dIds,
              float *dDists, uint32_t ldo, void *stream) {
  if (idx && (idx->flags & RBC_BUILD_F64)) return fail(RBC_ERR_INVALID, "rbc_query: index holds doubles: rbc_query_f64");
  return query_index(idx, dQ, m, ldq, k, mode, dIds, dDists, ldo, (cudaStream_t)stream);
}

int rbc_query_host(rbc_index *idx, const float *hQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
                   uint32_t *hIds, float *hDists, uint32_t ldo) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_query_host: index is NULL");
  if (idx->flags & RBC_BUILD_F64) return fail(RBC_ERR_INVALID, "rbc_query_host: index holds doubles: rbc_query_f64");
  if (m == 0) return RBC_OK;
  if (!hQ || (!hIds && !hDists)) return fail(RBC_ERR_INVALID, "rbc_query_host: NULL buffer");
  if (ldq < idx->d || ldo < k) return query_index(idx, hQ, m, ldq, k, mode, nullptr, nullptr, ldo, nullptr);
  cudaStream_t s = nullptr;
  DevBuf q, ids, dists;
  CK(q.alloc(m * ldq * 4, s));
  CK(ids.alloc(m * ldo * 4, s));
  CK(dists.alloc(m * ldo * 4, s));
  CK(cudaMemcpyAsync(q.p, hQ, m * ldq * 4, cudaMemcpyHostToDevice, s));
  TRY(query_index(idx, q.as<float>(), m, ldq, k, mode | kQueryNoSync, ids.as<uint32_t>(), dists.as<float>(), ldo, s));
  if (hIds) CK(cudaMemcpyAsync(hIds, ids.p, m * ldo * 4, cudaMemcpyDeviceToHost, s));
  if (hDists) CK(cudaMemcpyAsync(hDists, dists.p, m * ldo * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return RBC_OK;
}

int rbc_get_query_stats(const rbc_index *idx, rbc_query_stats *st) {
  if (!idx || !st) return fail(RBC_ERR_INVALID, "rbc_get_query_stats: NULL argument");
  *st = idx->stats;
  return RBC_OK;
}

int rbc_get_fallback_queries(const rbc_index *idx, uint32_t *h_ids, uint64_t cap, uint64_t *count) {
  if (!idx || !count || (cap && !h_ids)) return fail(RBC_ERR_INVALID, "rbc_get_fallback_queries: NULL argument");
  *count = idx->fallback_ids.size();
  if (cap && *count) std::memcpy(h_ids, idx->fallback_ids.data(), std::min<uint64_t>(cap, *count) * 4);
  return RBC_OK;
}

int rbc_set_router(rbc_index *idx, rbc_router *router, uint32_t probes) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_set_router: NULL index");
  if (router && (router->r.d != idx->d || router->r.L != idx->nr))
    return fail(RBC_ERR_INVALID, "rbc_set_router: router shape does not match the index (d, number of lists)");
  if (router && probes == 0 && !router->r.T)
    return fail(RBC_ERR_INVALID, "rbc_set_router: probes = 0 needs a router with a distance head");
  if (router && probes > 7) return fail(RBC_ERR_INVALID, "rbc_set_router: probes must be in [0, 7]");
  idx->router = router;
  idx->router_probes = router ? probes : 0;
  idx->tc_unrouted = false;  // a tuning decision about another router does not carry over
  return RBC_OK;
}

int rbc_owner_labels(rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t *dLabels, void *stream) {
  if (!idx || (m && (!dQ || !dLabels))) return fail(RBC_ERR_INVALID, "rbc_owner_labels: bad argument");
  if (!(idx->flags & RBC_BUILD_PARTITION)) return fail(RBC_ERR_INVALID, "rbc_owner_labels: index has no partition");
  if (m == 0) return RBC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf ids;
  CK(ids.alloc(m * 4, s));
  // exact either way; the tensor form is faster when the index has it
  const uint32_t mode = (idx->flags & RBC_BUILD_BF16) ? RBC_QUERY_EXACT_TC : RBC_QUERY_EXACT;
  TRY(query_index(idx, dQ, m, ldq, 1, mode, ids.as<uint32_t>(), nullptr, 1, s));
  CK(launch_owner_lookup(ids.as<uint32_t>(), m, 1, idx->owner, dLabels, s));
  CK(cudaStreamSynchronize(s));
  return RBC_OK;
}

int rbc_router_labels(rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t *dLabels,
                      float *dDist, float *dNear, void *stream) {
  if (!idx || (m && (!dQ || (!dLabels && !dDist && !dNear))))
    return fail(RBC_ERR_INVALID, "rbc_router_labels: bad argument");
  if (!(idx->flags & RBC_BUILD_PARTITION)) return fail(RBC_ERR_INVALID, "rbc_router_labels: index has no partition");
  if (k < 1 || k > kTcMaxK) return fail(RBC_ERR_INVALID, "rbc_router_labels: k must be in [1, 32]");
  if (m == 0) return RBC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf ids, dd;
  CK(ids.alloc(m * k * 4, s));
  CK(dd.alloc(m * k * 4, s));
  const uint32_t mode = (idx->flags & RBC_BUILD_BF16) ? RBC_QUERY_EXACT_TC : RBC_QUERY_EXACT;
  TRY(query_index(idx, dQ, m, ldq, k, mode, ids.as<uint32_t>(), dd.as<float>(), k, s));
  if (dLabels) CK(launch_owner_lookup(ids.as<uint32_t>(), m, k, idx->owner, dLabels, s));
  if (dDist)
    CK(cudaMemcpy2DAsync(dDist, 4, dd.as<float>() + (k - 1), (size_t)k * 4, 4, m, cudaMemcpyDeviceToDevice, s));
  if (dNear) {  // the nearest representative's distance, as the queries compute it
    DevBuf Qp, best;
    CK(Qp.alloc(m * idx->ld * 4, s));
    CK(best.alloc(m * 4, s));
    CK(launch_pad_rows(dQ, ldq, Qp.as<float>(), idx->ld, m, idx->d, s));
    CK(launch_argmin(idx->metric, Qp.as<float>(), m, idx->R, idx->nr, idx->ld, idx->dp, best.as<uint32_t>(), dNear,
                     s));
  }
  CK(cudaStreamSynchronize(s));
  return RBC_OK;
}

int rbc_set_profiling(rbc_index *idx, int enable) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_set_profiling: NULL index");
  idx->profile = enable != 0;
  return RBC_OK;
}

int rbc_get_profile(const rbc_index *idx, rbc_profile *out) {
  if (!idx || !out) return fail(RBC_ERR_INVALID, "rbc_get_profile: NULL argument");
  *out = idx->prof;
  return RBC_OK;
}

uint64_t rbc_kernel_launches(void) { return g_kernel_launches.load(); }

int rbc_brute_knn(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t d,
                  uint32_t k, int metric, uint32_t *dIds, float *dDists, uint32_t ldo, void *stream) {
  return brute_knn(dX, n, ldx, dQ, m, ldq, d, k, metric, dIds, dDists, ldo, (cudaStream_t)stream);
}

int rbc_brute_range_count(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m, uint32_t ldq,
                          uint32_t d, int metric, const float *dRanges, uint32_t *dCounts, void *stream) {
  return brute_range_count(dX, n, ldx, dQ, m, ldq, d, metric, dRanges, dCounts, (cudaStream_t)stream);
}

int rbc_synth(int kind, uint64_t seed, uint64_t stream_id, uint64_t r0, uint64_t rows, uint32_t d, uint32_t ld,
              float *dOut, uint32_t ncomp, float sigma_lo, float sigma_hi, void *stream) {
  if (kind < RBC_SYNTH_UNIFORM || kind > RBC_SYNTH_GEOMETRIC) return fail(RBC_ERR_INVALID, "rbc_synth: unknown kind");
  if (ld < d || (rows && !dOut)) return fail(RBC_ERR_INVALID, "rbc_synth: bad buffer");
  CK(launch_synth(kind, seed, stream_id, r0, rows, d, ld, dOut, ncomp, sigma_lo, sigma_hi, (cudaStream_t)stream));
  return RBC_OK;
}

}  // extern "C"
