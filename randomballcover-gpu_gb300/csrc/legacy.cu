// legacy.cu -- the reference's C++ API (rbc.h, brute.h, utils.h, utilsGPU.h)
// implemented over the engine, so programs written against the reference
// (e.g. its driver.cu) link unchanged.
//
// buildRBC keeps the reference's observable structure: rbcS.dx is the padded
// device copy of the database, rbcS.dr the representatives, rbcS.dxMap the
// one-shot lists (s nearest points of each representative, ids increasing,
// rbc.cu:126-208) and rbcS.groupCount their sizes.  The engine's index that
// also holds the partition for exact search is found again from rbcS.dx.mat,
// so the caller-allocated rbcStruct layout is unchanged.  Errors follow the
// reference's checkErr convention: a message on stderr and exit(1).
//
// Compiled a second time with RBC_REAL_DOUBLE (librbcgb_f64.so), this file is
// the API of the reference's double build (real = double, defs.h:27-31): the
// same functions over double matrices, answered by the library's double-
// precision calls.  The one-shot lists are float-only there: rbcS.dxMap stays
// empty and the one-shot query mode is refused.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/brute.h"
#include "../../include/rbc.h"
#include "../../include/rbc_gb300.h"
#include "../../include/utils.h"
#include "../../include/utilsGPU.h"
#include "engine.cuh"
#include "rbc_common.cuh"

namespace {

std::mutex g_mu;
std::map<const void *, rbc_index *> g_indexes;
unsigned g_query_mode = RBC_QUERY_EXACT;
int g_metric = RBC_L2;
unsigned long long g_seed = 0x5EEDull;
bool g_seed_from_env = false;

[[noreturn]] void die(const char *where, int rc) {
  std::fprintf(stderr, "GPU-related error:\n\t%s: %s (%s)\nexiting ..\n", where, rbc_status_string(rc),
               rbc_last_error());
  std::exit(1);
}

void check(const char *where, int rc) {
  if (rc != RBC_OK) die(where, rc);
}

unsigned long long legacy_seed() {
  if (!g_seed_from_env) {
    if (const char *e = std::getenv("RBC_SEED")) g_seed = std::strtoull(e, nullptr, 0);
    if (const char *e = std::getenv("RBC_LEGACY_MODE"))
      if (!std::strcmp(e, "oneshot")) g_query_mode = RBC_QUERY_ONESHOT;
    g_seed_from_env = true;
  }
  return g_seed;
}

rbc_index *lookup(const rbcStruct &r) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_indexes.find(r.dx.mat);
  if (it == g_indexes.end()) {
    std::fprintf(stderr, "rbcStruct was not built by buildRBC.. exiting\n");
    std::exit(1);
  }
  return it->second;
}

real dist_host(const real *a, const real *b, unint d) {
  real acc = 0;
  for (unint i = 0; i < d; i++) {
    volatile real t = a[i] - b[i];  // keep each operation rounded on its own
    volatile real term = g_metric == RBC_L1 ? std::fabs(t) : t * t;
    acc = acc + term;
  }
  return acc;
}

// The engine's calls of each precision, chosen by the type of `real`.
int eng_brute_knn(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t d,
                  uint32_t k, uint32_t *ids, float *dists, uint32_t ldo) {
  return rbc_brute_knn(dX, n, ldx, dQ, m, ldq, d, k, g_metric, ids, dists, ldo, nullptr);
}
int eng_brute_knn(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m, uint32_t ldq, uint32_t d,
                  uint32_t k, uint32_t *ids, double *dists, uint32_t ldo) {
  return rbc_brute_knn_f64(dX, n, ldx, dQ, m, ldq, d, k, g_metric, ids, dists, ldo, nullptr, nullptr);
}
int eng_range_count(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t d,
                    const float *r, uint32_t *c) {
  return rbc_brute_range_count(dX, n, ldx, dQ, m, ldq, d, g_metric, r, c, nullptr);
}
int eng_range_count(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m, uint32_t ldq,
                    uint32_t d, const double *r, uint32_t *c) {
  return rbc_brute_range_count_f64(dX, n, ldx, dQ, m, ldq, d, g_metric, r, c, nullptr);
}
int eng_query_host(rbc_index *idx, const float *hQ, uint64_t m, uint32_t ldq, uint32_t k, unsigned mode,
                   uint32_t *hIds, float *hD, uint32_t ldo) {
  return rbc_query_host(idx, hQ, m, ldq, k, mode, hIds, hD, ldo);
}
int eng_query_host(rbc_index *idx, const double *hQ, uint64_t m, uint32_t ldq, uint32_t k, unsigned mode,
                   uint32_t *hIds, double *hD, uint32_t ldo) {
  void *q = nullptr, *ids = nullptr, *dd = nullptr;
  cudaError_t e = cudaMalloc(&q, m * ldq * 8 + 16);
  if (e == cudaSuccess) e = cudaMalloc(&ids, m * ldo * 4 + 16);
  if (e == cudaSuccess) e = cudaMalloc(&dd, m * ldo * 8 + 16);
  if (e == cudaSuccess) e = cudaMemcpy(q, hQ, m * ldq * 8, cudaMemcpyHostToDevice);
  int rc = e == cudaSuccess ? RBC_OK : RBC_ERR_CUDA;
  if (rc == RBC_OK) rc = rbc_query_f64(idx, (const double *)q, m, ldq, k, mode, (uint32_t *)ids, (double *)dd, ldo, nullptr);
  if (rc == RBC_OK && cudaMemcpy(hIds, ids, m * ldo * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = RBC_ERR_CUDA;
  if (rc == RBC_OK && cudaMemcpy(hD, dd, m * ldo * 8, cudaMemcpyDeviceToHost) != cudaSuccess) rc = RBC_ERR_CUDA;
  cudaFree(q);
  cudaFree(ids);
  cudaFree(dd);
  return rc;
}

}  // namespace

extern "C" {
void rbc_set_legacy_query_mode(unsigned mode) { g_query_mode = mode; }
void rbc_set_legacy_metric(int metric) { g_metric = metric; }
void rbc_set_legacy_seed(unsigned long long seed) {
  g_seed = seed;
  g_seed_from_env = true;
}
}

// ------------------------------------------------------------------ rbc.h
void buildRBC(const matrix x, rbcStruct *rbcS, unint numReps, unint s) {
  if (!rbcS) die("buildRBC", RBC_ERR_INVALID);
  rbc_build_params p{};
  p.num_reps = numReps;
  p.s = s;
  p.metric = g_metric;
  p.seed = legacy_seed();
  rbc_index *idx = nullptr;
#ifdef RBC_REAL_DOUBLE
  // the double build: the partition over double rows (kept in the padded
  // legacy layout as rbcS.dx); no one-shot lists
  p.flags = RBC_BUILD_PARTITION | rbc::kBuildKeepInput;
  double *dX = nullptr;
  checkErr(cudaMalloc(&dX, (size_t)x.r * x.ld * sizeof(real) + 16));
  checkErr(cudaMemcpy(dX, x.mat, (size_t)x.r * x.ld * sizeof(real), cudaMemcpyHostToDevice));
  int rc = rbc_build_f64(dX, x.r, x.c, x.ld, &p, nullptr, &idx);
  cudaFree(dX);
  check("buildRBC", rc);
  rbcS->dx.mat = idx->X64;
  rbcS->dx.r = x.r;
  rbcS->dx.c = x.c;
  rbcS->dx.pr = PAD(x.r);
  rbcS->dx.pc = rbcS->dx.ld = idx->ld64;
  {
    matrix r;
    r.r = numReps;
    r.pr = PAD(numReps);
    r.c = x.c;
    r.pc = r.ld = PAD(x.c);
    std::vector<real> buf((size_t)r.pr * r.pc, 0);
    r.mat = buf.data();
    for (unint i = 0; i < numReps; i++)
      copyVector(&r.mat[IDX(i, 0, r.ld)], &x.mat[IDX(idx->rep_ids[i], 0, x.ld)], x.c);
    copyAndMove(&rbcS->dr, &r);
  }
  rbcS->dxMap.mat = nullptr;
  rbcS->dxMap.r = numReps;
  rbcS->dxMap.c = 0;
  rbcS->dxMap.pr = PAD(numReps);
  rbcS->dxMap.pc = rbcS->dxMap.ld = 0;
  rbcS->groupCount = (unint *)std::calloc(PAD(numReps), sizeof(unint));
  std::lock_guard<std::mutex> lk(g_mu);
  g_indexes[idx->X64] = idx;
  (void)s;
#else
  p.flags = RBC_BUILD_PARTITION | RBC_BUILD_ONESHOT | rbc::kBuildKeepInput;
  check("buildRBC", rbc_build_host(x.mat, x.r, x.c, x.ld, &p, &idx));
  rbcS->dx.mat = idx->Xi;
  rbcS->dx.r = x.r;
  rbcS->dx.c = x.c;
  rbcS->dx.pr = (unint)idx->xi_rows;
  rbcS->dx.pc = rbcS->dx.ld = idx->ld;
  rbcS->dr.mat = idx->R;
  rbcS->dr.r = numReps;
  rbcS->dr.c = x.c;
  rbcS->dr.pr = PAD(numReps);
  rbcS->dr.pc = rbcS->dr.ld = idx->ld;
  rbcS->dxMap.mat = idx->os_lists;
  rbcS->dxMap.r = numReps;
  rbcS->dxMap.c = s;
  rbcS->dxMap.pr = PAD(numReps);
  rbcS->dxMap.pc = rbcS->dxMap.ld = idx->lds;
  rbcS->groupCount = (unint *)std::calloc(PAD(numReps), sizeof(unint));
  check("buildRBC", rbc_get_oneshot(idx, nullptr, rbcS->groupCount));
  std::lock_guard<std::mutex> lk(g_mu);
  g_indexes[idx->Xi] = idx;
#endif
}

void queryRBC(const matrix q, const rbcStruct rbcS, unint *NNs, real *NNdists) {
  rbc_index *idx = lookup(rbcS);
  std::vector<real> d(q.r);
  check("queryRBC", eng_query_host(idx, q.mat, q.r, q.ld, 1, g_query_mode, NNs, NNdists ? NNdists : d.data(), 1));
}

void kqueryRBC(const matrix q, const rbcStruct rbcS, intMatrix NNs, matrix NNdists) {
  rbc_index *idx = lookup(rbcS);
  check("kqueryRBC", eng_query_host(idx, q.mat, q.r, q.ld, KMAX, g_query_mode, NNs.mat, NNdists.mat, NNs.ld));
  if (NNdists.ld != NNs.ld)
    die("kqueryRBC: NNs and NNdists must share the leading dimension", RBC_ERR_INVALID);
}

void destroyRBC(rbcStruct *rbcS) {
  if (!rbcS) return;
  rbc_index *idx = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_indexes.find(rbcS->dx.mat);
    if (it != g_indexes.end()) {
      idx = it->second;
      g_indexes.erase(it);
    }
  }
  rbc_destroy(idx);
#ifdef RBC_REAL_DOUBLE
  cudaFree(rbcS->dr.mat);  // the double representatives belong to this layer
#endif
  std::free(rbcS->groupCount);
  rbcS->groupCount = nullptr;
  rbcS->dx.mat = nullptr;
  rbcS->dr.mat = nullptr;
  rbcS->dxMap.mat = nullptr;
}

// Distances from rows [start, start+length) of dr to every row of dx, into
// the device matrix dD (rbc.cu:356-360).
void distSubMat(matrix dr, matrix dx, matrix dD, unint start, unint length) {
  if (dr.ld != dx.ld || dr.ld % 4) die("distSubMat: operands must share a padded leading dimension", RBC_ERR_INVALID);
#ifdef RBC_REAL_DOUBLE
  cudaError_t e = rbc::launch_dense_dist64(g_metric, dr.mat + (size_t)start * dr.ld, length, dx.mat, dx.pr, dx.ld, dx.c,
                                           dD.mat, dD.ld, nullptr);
#else
  cudaError_t e = rbc::launch_dense_dist(g_metric, dr.mat + (size_t)start * dr.ld, length, dx.mat, dx.pr, dx.ld,
                                         rbc::pad4(dx.c), dD.mat, dD.ld, nullptr);
#endif
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) checkErr(e);
}

// Nearest row of dr for every row of dq, results on the host (rbc.cu:233-247).
void computeReps(matrix dq, matrix dr, unint *repIDs, real *distToReps) {
  unint *dIds = nullptr;
  real *dD = nullptr;
  checkErr(cudaMalloc(&dIds, (size_t)dq.r * 4));
  checkErr(cudaMalloc(&dD, (size_t)dq.r * sizeof(real)));
#ifdef RBC_REAL_DOUBLE
  // nearest representative under (dist, index) in double
  const int rc = rbc_brute_knn_f64(dr.mat, dr.r, dr.ld, dq.mat, dq.r, dq.ld, dq.c, 1, g_metric, dIds, dD, 1, nullptr,
                                   nullptr);
  if (rc != RBC_OK) die("computeReps", rc);
  cudaError_t e = cudaSuccess;
#else
  cudaError_t e = rbc::launch_argmin(g_metric, dq.mat, dq.r, dr.mat, dr.r, dq.ld, rbc::pad4(dq.c), dIds, dD, nullptr);
#endif
  if (e == cudaSuccess) e = cudaMemcpy(repIDs, dIds, (size_t)dq.r * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && distToReps) e = cudaMemcpy(distToReps, dD, (size_t)dq.r * sizeof(real), cudaMemcpyDeviceToHost);
  cudaFree(dIds);
  cudaFree(dD);
  if (e != cudaSuccess) checkErr(e);
}

// radii[r] = max distance of the points assigned to r (rbc.cu:251-256).
void computeRadii(unint *repIDs, real *distToReps, real *radii, unint n, unint numReps) {
  for (unint i = 0; i < n; i++)
    if (repIDs[i] < numReps) radii[repIDs[i]] = MAX(distToReps[i], radii[repIDs[i]]);
}

void computeCounts(unint *repIDs, unint n, unint *groupCount) {
  for (unint i = 0; i < n; i++) groupCount[repIDs[i]]++;
}

// Queries grouped by representative, each group padded to 16 with DUMMY_IDX
// (rbc.cu:268-294).
void buildQMap(matrix q, unint *qMap, unint *repIDs, unint numReps, unint *compLength) {
  std::vector<unint> gs(numReps + 1, 0);
  for (unint i = 0; i < q.r; i++) gs[repIDs[i] + 1]++;
  for (unint i = 0; i <= numReps; i++) gs[i] = PAD(gs[i]);
  for (unint i = 1; i <= numReps; i++) gs[i] += gs[i - 1];
  *compLength = gs[numReps];
  for (unint i = 0; i < *compLength; i++) qMap[i] = DUMMY_IDX;
  for (unint i = 0; i < q.r; i++) qMap[gs[repIDs[i]]++] = i;
}

void idIntersection(charMatrix cM) {
  for (unint i = 0; i < cM.r && i < cM.c; i++) cM.mat[IDX(i, i, cM.ld)] = 1;
}

void fullIntersection(charMatrix cM) {
  for (unint i = 0; i < cM.r; i++)
    for (unint j = 0; j < cM.c; j++) cM.mat[IDX(i, j, cM.ld)] = 1;
}

// ------------------------------------------------------------------ compPlan
// The reference's query plan (rbc.cu:375-440): query group g (the queries
// whose nearest representative is g, laid out in 16-slot blocks by
// buildQMap) is compared with the database groups j where cM[g][j] is set.
// Row g of qGroupToXGroup lists those j, groupCountX their list lengths;
// qToQGroup maps every query slot to its group.  Built on the host and moved
// to the device like the reference's; freeCompPlan releases it.
namespace {

template <typename T>
__global__ void gather_pad_kernel(const T *__restrict__ src, uint64_t ld_src, const uint32_t *__restrict__ rows,
                                  uint64_t n, uint32_t d, T *__restrict__ dst, uint32_t ld_dst) {
  const uint64_t total = n * ld_dst;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = i / ld_dst;
    const uint32_t c = (uint32_t)(i - r * ld_dst);
    dst[i] = c < d ? src[(uint64_t)rows[r] * ld_src + c] : T(0);
  }
}

// dst row r = src row rows[r] (columns past d zeroed); rows is on the device.
template <typename T>
cudaError_t gather_pad(const T *src, uint64_t ld_src, const uint32_t *rows, uint64_t n, uint32_t d, T *dst,
                       uint32_t ld_dst) {
  if (n == 0) return cudaSuccess;
  const uint64_t total = n * ld_dst;
  const unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, 152ull * 32);
  gather_pad_kernel<T><<<grid, 256>>>(src, ld_src, rows, n, d, dst, ld_dst);
  return rbc::launched();
}

template <typename T>
T *dev_alloc(size_t count) {
  T *p = nullptr;
  checkErr(cudaMalloc((void **)&p, std::max<size_t>(count, 1) * sizeof(T)));
  return p;
}

template <typename T>
std::vector<T> to_host(const T *d, size_t count) {
  std::vector<T> h(count);
  if (count) checkErr(cudaMemcpy(h.data(), d, count * sizeof(T), cudaMemcpyDeviceToHost));
  return h;
}

// One run of consecutive query blocks of the same group: its real queries and
// the database groups (list, length) it is compared with.
struct PlanRun {
  unint g;
  std::vector<unint> queries;
  std::vector<std::pair<unint, unint>> groups;
};

// The plan read back from the device and checked against the matrices it
// indexes (ids, lists and lengths in range), as runs of query blocks.
std::vector<PlanRun> read_plan(const matrix &dx, const intMatrix &dxMap, const matrix &dq, const unint *dqMap,
                               const compPlan &dcP, unint compLength, const char *who) {
  if (compLength % BLOCK_SIZE) die(who, RBC_ERR_INVALID);
  const std::vector<unint> qmap = to_host(dqMap, compLength);
  const std::vector<unint> q2g = to_host(dcP.qToQGroup, compLength);
  unint gmax = 0;
  for (unint b = 0; b < compLength; b += BLOCK_SIZE) gmax = std::max(gmax, q2g[b]);
  const std::vector<unint> num = to_host(dcP.numGroups, compLength ? gmax + 1 : 0);
  const size_t width = (size_t)(compLength ? gmax + 1 : 0) * dcP.ld;
  const std::vector<unint> xg = to_host(dcP.qGroupToXGroup, width), cnt = to_host(dcP.groupCountX, width);
  std::vector<PlanRun> runs;
  for (unint b = 0; b < compLength; b += BLOCK_SIZE) {
    const unint g = q2g[b];
    if (runs.empty() || runs.back().g != g) {
      PlanRun r;
      r.g = g;
      if (num[g] > dcP.ld) die(who, RBC_ERR_INVALID);
      for (unint i = 0; i < num[g]; i++) {
        const unint j = xg[(size_t)g * dcP.ld + i], c = cnt[(size_t)g * dcP.ld + i];
        if (j >= dxMap.r || c > dxMap.ld) die(who, RBC_ERR_INVALID);
        r.groups.push_back({j, c});
      }
      runs.push_back(std::move(r));
    }
    for (unint t = 0; t < BLOCK_SIZE; t++) {
      const unint q = qmap[b + t];
      if (q == DUMMY_IDX) continue;
      if (q >= dq.r) die(who, RBC_ERR_INVALID);
      runs.back().queries.push_back(q);
    }
  }
  (void)dx;
  return runs;
}

// Database ids of the lists a plan uses, each list once: rows, and the first
// row of every list in it (UINT64_MAX for unused lists).
void plan_rows(const std::vector<PlanRun> &runs, const matrix &dx, const intMatrix &dxMap,
               std::vector<unint> &rows, std::vector<uint64_t> &first, const char *who) {
  unint jmax = 0;
  for (const PlanRun &r : runs)
    for (auto &gc : r.groups) jmax = std::max(jmax, gc.first + 1);
  const std::vector<unint> lists = to_host(dxMap.mat, (size_t)jmax * dxMap.ld);
  first.assign(jmax, UINT64_MAX);
  std::vector<unint> len(jmax, 0);
  for (const PlanRun &r : runs)
    for (auto &gc : r.groups) len[gc.first] = std::max(len[gc.first], gc.second);
  for (unint j = 0; j < jmax; j++) {
    if (!len[j]) continue;
    first[j] = rows.size();
    for (unint t = 0; t < len[j]; t++) {
      const unint id = lists[(size_t)j * dxMap.ld + t];
      if (id >= dx.r) die(who, RBC_ERR_INVALID);
      rows.push_back(id);
    }
  }
}

#ifndef RBC_REAL_DOUBLE
// The plan's searches in one persistent list-search launch: the lists' rows
// gathered (zero-padded) into one buffer, work items (query tile of a run,
// row chunk of one of its lists), per-query sorted (dist, id) lists of the
// engine's exact FP32 search.
void plan_search(const matrix &dx, const intMatrix &dxMap, const matrix &dq, const unint *dqMap, const compPlan &dcP,
                 unint compLength, unint k, unint *hIds, real *hDists, unint ldo, const char *who) {
  const std::vector<PlanRun> runs = read_plan(dx, dxMap, dq, dqMap, dcP, compLength, who);
  std::vector<unint> rows;
  std::vector<uint64_t> first;
  plan_rows(runs, dx, dxMap, rows, first, who);
  const uint32_t d = dq.c, ld = rbc::pad16(d), dp = rbc::pad4(d), m = dq.r;
  if (dx.c != d || d > rbc::kMaxDim) die(who, RBC_ERR_UNSUPPORTED);
  const uint32_t kw = rbc::list_width_for(k), qtile = (uint32_t)rbc::search_query_tile(dp, 0, kw);
  constexpr uint32_t kChunk = 16384;
  std::vector<unint> qidx;
  std::vector<rbc::SearchItem> items;
  for (const PlanRun &r : runs) {
    const uint32_t q0 = (uint32_t)qidx.size(), nq = (uint32_t)r.queries.size();
    qidx.insert(qidx.end(), r.queries.begin(), r.queries.end());
    for (auto &gc : r.groups)
      for (uint32_t c0 = 0; c0 < gc.second; c0 += kChunk)
        for (uint32_t t0 = 0; t0 < nq; t0 += qtile) {
          rbc::SearchItem it{};
          it.p0 = first[gc.first] + c0;
          it.np = std::min(kChunk, gc.second - c0);
          it.list = gc.first;
          it.q0 = q0 + t0;
          it.nq = std::min(qtile, nq - t0);
          items.push_back(it);
        }
  }
  float *Xg = dev_alloc<float>(rows.size() * ld), *Qp = dev_alloc<float>((size_t)m * ld);
  float *res_d = dev_alloc<float>((size_t)m * kw), *out_d = dev_alloc<float>((size_t)m * k);
  unint *d_rows = dev_alloc<unint>(rows.size()), *d_qidx = dev_alloc<unint>(qidx.size());
  unint *res_i = dev_alloc<unint>((size_t)m * kw), *out_i = dev_alloc<unint>((size_t)m * k);
  unint *tau = dev_alloc<unint>(m), *lock = dev_alloc<unint>(m), *ctl = dev_alloc<unint>(16);
  rbc::SearchItem *d_items = dev_alloc<rbc::SearchItem>(items.size());
  checkErr(cudaMemcpy(d_rows, rows.data(), rows.size() * 4, cudaMemcpyHostToDevice));
  checkErr(cudaMemcpy(d_qidx, qidx.data(), qidx.size() * 4, cudaMemcpyHostToDevice));
  checkErr(cudaMemcpy(d_items, items.data(), items.size() * sizeof(rbc::SearchItem), cudaMemcpyHostToDevice));
  checkErr(cudaMemset(ctl, 0, 64));
  const uint32_t nitems = (uint32_t)items.size();
  checkErr(cudaMemcpy(ctl + 1, &nitems, 4, cudaMemcpyHostToDevice));
  checkErr(gather_pad<float>(dx.mat, dx.ld, d_rows, rows.size(), d, Xg, ld));
  checkErr(rbc::launch_pad_rows(dq.mat, dq.ld, Qp, ld, m, d, nullptr));
  checkErr(rbc::launch_init_results(res_d, res_i, tau, lock, m, kw, nullptr));
  rbc::SearchArgs sa{};
  sa.X = Xg;
  sa.pid = d_rows;
  sa.Q = Qp;
  sa.qidx = d_qidx;
  sa.items = d_items;
  sa.nitems = ctl + 1;
  sa.work = ctl;
  sa.res_d = res_d;
  sa.res_i = res_i;
  sa.tau = tau;
  sa.lock = lock;
  sa.err = ctl + 2;
  sa.ld = ld;
  sa.dp = dp;
  sa.k = k;
  if (nitems) checkErr(rbc::launch_search(g_metric, sa, rbc::search_grid(g_metric, dp, 0, kw), nullptr));
  checkErr(rbc::launch_write_results(res_d, res_i, m, k, kw, out_i, out_d, k, nullptr));
  unint err_word = 0;
  checkErr(cudaMemcpy(&err_word, ctl + 2, 4, cudaMemcpyDeviceToHost));
  if (err_word) die(who, (int)err_word);
  const std::vector<unint> hi = to_host(out_i, (size_t)m * k);
  const std::vector<float> hd = to_host(out_d, (size_t)m * k);
  for (unint q = 0; q < m; q++)
    for (unint j = 0; j < k; j++) {
      hIds[(size_t)q * ldo + j] = hi[(size_t)q * k + j];
      if (hDists) hDists[(size_t)q * ldo + j] = hd[(size_t)q * k + j];
    }
  void *ptrs[] = {Xg, Qp, res_d, out_d, d_rows, d_qidx, res_i, out_i, tau, lock, ctl, d_items};
  for (void *p : ptrs) cudaFree(p);
}
#else
// The double build: each run of query blocks answered by the double brute
// force over its lists' rows (gathered), ids mapped back through the lists.
void plan_search(const matrix &dx, const intMatrix &dxMap, const matrix &dq, const unint *dqMap, const compPlan &dcP,
                 unint compLength, unint k, unint *hIds, real *hDists, unint ldo, const char *who) {
  const std::vector<PlanRun> runs = read_plan(dx, dxMap, dq, dqMap, dcP, compLength, who);
  std::vector<unint> all_rows;
  std::vector<uint64_t> first;
  plan_rows(runs, dx, dxMap, all_rows, first, who);
  const uint32_t d = dq.c, ld = rbc::pad16(d);
  if (dx.c != d) die(who, RBC_ERR_UNSUPPORTED);
  for (unint q = 0; q < dq.r; q++)
    for (unint j = 0; j < k; j++) {
      hIds[(size_t)q * ldo + j] = DUMMY_IDX;
      if (hDists) hDists[(size_t)q * ldo + j] = MAX_REAL;
    }
  for (const PlanRun &r : runs) {
    if (r.queries.empty()) continue;
    std::vector<unint> rows;
    for (auto &gc : r.groups)
      rows.insert(rows.end(), all_rows.begin() + first[gc.first], all_rows.begin() + first[gc.first] + gc.second);
    if (rows.empty()) continue;
    const size_t nq = r.queries.size(), nx = rows.size();
    unint *d_rows = dev_alloc<unint>(nx), *d_q = dev_alloc<unint>(nq), *ids = dev_alloc<unint>(nq * k);
    real *Xg = dev_alloc<real>(nx * ld), *Qg = dev_alloc<real>(nq * ld), *dd = dev_alloc<real>(nq * k);
    checkErr(cudaMemcpy(d_rows, rows.data(), nx * 4, cudaMemcpyHostToDevice));
    checkErr(cudaMemcpy(d_q, r.queries.data(), nq * 4, cudaMemcpyHostToDevice));
    checkErr(gather_pad<real>(dx.mat, dx.ld, d_rows, nx, d, Xg, ld));
    checkErr(gather_pad<real>(dq.mat, dq.ld, d_q, nq, d, Qg, ld));
    const int rc = rbc_brute_knn_f64(Xg, nx, ld, Qg, nq, ld, d, k, g_metric, ids, dd, k, nullptr, nullptr);
    if (rc != RBC_OK) die(who, rc);
    const std::vector<unint> hi = to_host(ids, nq * k);
    const std::vector<real> hd = to_host(dd, nq * k);
    for (size_t t = 0; t < nq; t++)
      for (unint j = 0; j < k; j++) {
        const unint pos = hi[t * k + j];
        hIds[(size_t)r.queries[t] * ldo + j] = pos < nx ? rows[pos] : DUMMY_IDX;
        if (hDists) hDists[(size_t)r.queries[t] * ldo + j] = hd[t * k + j];
      }
    void *ptrs[] = {d_rows, d_q, ids, Xg, Qg, dd};
    for (void *p : ptrs) cudaFree(p);
  }
}
#endif

}  // namespace

void initCompPlan(compPlan *dcP, charMatrix cM, unint *groupCountQ, unint *groupCountX, unint numReps) {
  if (!dcP || (numReps && (!cM.mat || !groupCountQ || !groupCountX))) die("initCompPlan", RBC_ERR_INVALID);
  std::vector<unint> num(numReps, 0);
  unint width = 0;
  for (unint g = 0; g < numReps; g++) {
    for (unint j = 0; j < numReps; j++) num[g] += cM.mat[IDX(g, j, cM.ld)] ? 1u : 0u;
    width = std::max(width, num[g]);
  }
  std::vector<unint> q2g;
  for (unint g = 0; g < numReps; g++) q2g.insert(q2g.end(), PAD(groupCountQ[g]), g);
  std::vector<unint> xg((size_t)numReps * width, 0), cnt((size_t)numReps * width, 0);
  for (unint g = 0; g < numReps; g++)
    for (unint j = 0, t = 0; j < numReps; j++)
      if (cM.mat[IDX(g, j, cM.ld)]) {
        xg[IDX(g, t, width)] = j;
        cnt[IDX(g, t++, width)] = groupCountX[j];
      }
  auto up = [](const std::vector<unint> &h) {
    unint *p = dev_alloc<unint>(h.size());
    if (!h.empty()) checkErr(cudaMemcpy(p, h.data(), h.size() * 4, cudaMemcpyHostToDevice));
    return p;
  };
  dcP->numGroups = up(num);
  dcP->groupCountX = up(cnt);
  dcP->qToQGroup = up(q2g);
  dcP->qGroupToXGroup = up(xg);
  dcP->ld = width;
}

void freeCompPlan(compPlan *dcP) {
  if (!dcP) return;
  cudaFree(dcP->numGroups);
  cudaFree(dcP->groupCountX);
  cudaFree(dcP->qToQGroup);
  cudaFree(dcP->qGroupToXGroup);
  dcP->numGroups = dcP->groupCountX = dcP->qToQGroup = dcP->qGroupToXGroup = nullptr;
}

// 1-NN of every query over the lists its plan names, into host NNs / NNdists
// (rbc.cu:317-330).  dx, dxMap, dq and dqMap are device data.
void computeNNs(matrix dx, intMatrix dxMap, matrix dq, unint *dqMap, compPlan dcP, unint *NNs, real *NNdists,
                unint compLength) {
  if (!NNs) die("computeNNs", RBC_ERR_INVALID);
  plan_search(dx, dxMap, dq, dqMap, dcP, compLength, 1, NNs, NNdists, 1, "computeNNs");
}

// KMAX nearest neighbours of every query over the lists its plan names,
// sorted by (dist, id), into the host matrices NNs / NNdists (rbc.cu:333-348).
void computeKNNs(matrix dx, intMatrix dxMap, matrix dq, unint *dqMap, compPlan dcP, intMatrix NNs, matrix NNdists,
                 unint compLength) {
  if (!NNs.mat || (NNdists.mat && NNdists.ld != NNs.ld) || NNs.ld < KMAX) die("computeKNNs", RBC_ERR_INVALID);
  plan_search(dx, dxMap, dq, dqMap, dcP, compLength, KMAX, NNs.mat, NNdists.mat, NNs.ld, "computeKNNs");
}

// Random representatives copied to a padded device matrix rbcS->dr (rbc.cu:212-229).
void setupReps(matrix x, rbcStruct *rbcS, unint numReps) {
  std::vector<unint> ids(PAD(numReps), 0);
  subRandPerm(numReps, x.r, ids.data());
  matrix r;
  r.r = numReps;
  r.pr = PAD(numReps);
  r.c = x.c;
  r.pc = r.ld = PAD(x.c);
  std::vector<real> buf((size_t)r.pr * r.pc, 0);
  r.mat = buf.data();
  for (unint i = 0; i < numReps; i++) copyVector(&r.mat[IDX(i, 0, r.ld)], &x.mat[IDX(ids[i], 0, x.ld)], x.c);
  copyAndMove(&rbcS->dr, &r);
}

// ------------------------------------------------------------------ brute.h
namespace {
struct DevMat {
  real *p = nullptr;
  DevMat(const matrix &m) {
    size_t b = (size_t)m.pr * m.pc * sizeof(real);
    checkErr(cudaMalloc(&p, b ? b : 16));
    checkErr(cudaMemcpy(p, m.mat, b, cudaMemcpyHostToDevice));
  }
  ~DevMat() { cudaFree(p); }
};
}  // namespace

void bruteRangeCount(matrix x, matrix q, real *ranges, unint *cnts) {
  DevMat dx(x), dq(q);
  real *dr = nullptr;
  unint *dc = nullptr;
  checkErr(cudaMalloc(&dr, (size_t)q.pr * sizeof(real)));
  checkErr(cudaMalloc(&dc, (size_t)q.pr * 4));
  checkErr(cudaMemcpy(dr, ranges, (size_t)q.r * sizeof(real), cudaMemcpyHostToDevice));
  int rc = eng_range_count(dx.p, x.r, x.ld, dq.p, q.r, q.ld, x.c, dr, dc);
  if (rc == RBC_OK) checkErr(cudaMemcpy(cnts, dc, (size_t)q.r * 4, cudaMemcpyDeviceToHost));
  cudaFree(dr);
  cudaFree(dc);
  check("bruteRangeCount", rc);
}

void bruteSearch(matrix x, matrix q, unint *NNs) {
  DevMat dx(x), dq(q);
  unint *di = nullptr;
  checkErr(cudaMalloc(&di, (size_t)q.pr * 4));
  int rc = eng_brute_knn(dx.p, x.r, x.ld, dq.p, q.r, q.ld, x.c, 1, di, (real *)nullptr, 1);
  if (rc == RBC_OK) checkErr(cudaMemcpy(NNs, di, (size_t)q.r * 4, cudaMemcpyDeviceToHost));
  cudaFree(di);
  check("bruteSearch", rc);
}

void bruteK(matrix x, matrix q, intMatrix NNs, matrix NNdists) {
  DevMat dx(x), dq(q);
  unint *di = nullptr;
  real *dd = nullptr;
  checkErr(cudaMalloc(&di, (size_t)q.pr * NNs.ld * 4));
  checkErr(cudaMalloc(&dd, (size_t)q.pr * NNs.ld * sizeof(real)));
  int rc = eng_brute_knn(dx.p, x.r, x.ld, dq.p, q.r, q.ld, x.c, KMAX, di, dd, NNs.ld);
  if (rc == RBC_OK) {
    checkErr(cudaMemcpy(NNs.mat, di, (size_t)q.r * NNs.ld * 4, cudaMemcpyDeviceToHost));
    checkErr(cudaMemcpy2D(NNdists.mat, NNdists.ld * sizeof(real), dd, NNs.ld * sizeof(real), KMAX * sizeof(real), q.r,
                          cudaMemcpyDeviceToHost));
  }
  cudaFree(di);
  cudaFree(dd);
  check("bruteK", rc);
}

// Host 1-NN, ids scanned upward with a strict '<' (brute.cu:91-112).
void bruteCPU(matrix X, matrix Q, unint *NNs) {
  for (unint i = 0; i < Q.r; i++) {
    real best = MAX_REAL;
    NNs[i] = 0;
    for (unint j = 0; j < X.r; j++) {
      real t = dist_host(&Q.mat[IDX(i, 0, Q.ld)], &X.mat[IDX(j, 0, X.ld)], Q.c);
      if (t < best) {
        best = t;
        NNs[i] = j;
      }
    }
  }
}

// ------------------------------------------------------------------ utils.h
void swap(unint *a, unint *b) {
  unint t = *a;
  *a = *b;
  *b = t;
}

// Uniform integer in [a, b) from the C library generator (utils.cu:57-67).
unint randBetween(unint a, unint b) {
  if (b <= a) {
    std::fprintf(stderr, "misuse of randBetween.. exiting\n");
    std::exit(1);
  }
  unint c = b - a, val;
  while (c <= (val = (unint)(std::rand() / (int)(((unsigned)RAND_MAX + 1) / c)))) {
  }
  return val + a;
}

// Permutation of 0..n-1 (Knuth shuffle) seeded from the legacy seed.
void randPerm(unint n, unint *x) {
  std::srand((unsigned)legacy_seed());
  for (unint i = 0; i < n; i++) x[i] = i;
  for (unint i = 0; i + 1 < n; i++) swap(&x[i], &x[randBetween(i + 1, n)]);
}

// First l entries of a random permutation of 0..n-1 (utils.cu:17-37).
void subRandPerm(unint l, unint n, unint *x) {
  std::vector<unint> y(n);
  std::srand((unsigned)legacy_seed());
  for (unint i = 0; i < n; i++) y[i] = i;
  for (unint i = 0; i < MIN(l, n - 1); i++) swap(&y[i], &y[randBetween(i + 1, n)]);
  for (unint i = 0; i < l; i++) x[i] = y[i];
}

void printMat(matrix A) {
  for (unint i = 0; i < A.r; i++) {
    for (unint j = 0; j < A.c; j++) std::printf("%6.4f ", (float)A.mat[IDX(i, j, A.ld)]);
    std::printf("\n");
  }
}

void printMatWithIDs(matrix A, unint *id) {
  for (unint i = 0; i < A.r; i++) {
    for (unint j = 0; j < A.c; j++) std::printf("%6.4f ", (float)A.mat[IDX(i, j, A.ld)]);
    std::printf("%d \n", id[i]);
  }
}

void printCharMat(charMatrix A) {
  for (unint i = 0; i < A.r; i++) {
    for (unint j = 0; j < A.c; j++) std::printf("%d ", (char)A.mat[IDX(i, j, A.ld)]);
    std::printf("\n");
  }
}

void printIntMat(intMatrix A) {
  for (unint i = 0; i < A.r; i++) {
    for (unint j = 0; j < A.c; j++) std::printf("%d ", (unint)A.mat[IDX(i, j, A.ld)]);
    std::printf("\n");
  }
}

void printVector(real *x, unint d) {
  for (unint i = 0; i < d; i++) std::printf("%6.2f ", x[i]);
  std::printf("\n");
}

void copyVector(real *x, real *y, unint d) {
  for (unint i = 0; i < d; i++) x[i] = y[i];
}

// Distance between row k of x and row l of y (utils.cu:183-191; y is read
// with its own leading dimension).
real distVec(matrix x, matrix y, unint k, unint l) {
  return dist_host(&x.mat[IDX(k, 0, x.ld)], &y.mat[IDX(l, 0, y.ld)], x.c);
}

double timeDiff(struct timeval start, struct timeval end) {
  return (double)(end.tv_sec + end.tv_usec / 1e6 - start.tv_sec - start.tv_usec / 1e6);
}

void copyMat(matrix *x, matrix *y) {
  x->r = y->r;
  x->pr = y->pr;
  x->c = y->c;
  x->pc = y->pc;
  x->ld = y->ld;
  for (unint i = 0; i < y->r; i++)
    for (unint j = 0; j < y->c; j++) x->mat[IDX(i, j, x->ld)] = y->mat[IDX(i, j, y->ld)];
}

void initMat(matrix *x, unint r, unint c) {
  x->r = r;
  x->c = c;
  x->pr = PAD(r);
  x->pc = PAD(c);
  x->ld = PAD(c);
}

void initIntMat(intMatrix *x, unint r, unint c) {
  x->r = r;
  x->c = c;
  x->pr = PAD(r);
  x->pc = PAD(c);
  x->ld = PAD(c);
}

size_t sizeOfMatB(matrix x) { return ((size_t)x.pr) * x.pc * sizeof(*x.mat); }
size_t sizeOfIntMatB(intMatrix x) { return ((size_t)x.pr) * x.pc * sizeof(*x.mat); }
size_t sizeOfMat(matrix x) { return ((size_t)x.pr) * x.pc; }
size_t sizeOfIntMat(intMatrix x) { return ((size_t)x.pr) * x.pc; }

// ------------------------------------------------------------------ utilsGPU.h
void copyAndMove(matrix *dx, const matrix *x) {
  *dx = *x;
  size_t b = (size_t)dx->pr * dx->pc * sizeof(real);
  checkErr(cudaMalloc((void **)&dx->mat, b));
  checkErr(cudaMemcpy(dx->mat, x->mat, b, cudaMemcpyHostToDevice));
}

void copyAndMoveI(intMatrix *dx, const intMatrix *x) {
  *dx = *x;
  size_t b = (size_t)dx->pr * dx->pc * sizeof(unint);
  checkErr(cudaMalloc((void **)&dx->mat, b));
  checkErr(cudaMemcpy(dx->mat, x->mat, b, cudaMemcpyHostToDevice));
}

void copyAndMoveC(charMatrix *dx, const charMatrix *x) {
  *dx = *x;
  size_t b = (size_t)dx->pr * dx->pc;
  checkErr(cudaMalloc((void **)&dx->mat, b));
  checkErr(cudaMemcpy(dx->mat, x->mat, b, cudaMemcpyHostToDevice));
}

void checkErr(cudaError_t e) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "GPU-related error:\n\t%s \nexiting ..\n", cudaGetErrorString(e));
    std::exit(1);
  }
}

void checkErr(char *loc, cudaError_t e) {
  std::printf("in %s:\n", loc);
  checkErr(e);
}
