// tune.cu -- the autotuners of the FP32 list search and of the tensor form.
//
// Two knobs shape the plain search: the query tile (16 x TQ queries per CTA,
// TQ rows per thread) and the longest run of list rows a work item covers
// (long lists split into several items so the persistent launch stays
// balanced).  rbc_autotune times every valid pair on sample queries with CUDA
// events and keeps the fastest; a cache file (one line per index shape:
// "n d reps k metric tq item_rows ms") lets later processes skip the timing.
//
// The tensor form has two knobs of its own: how many nearest lists the probe
// round searches (more gives the pruned round a tighter start, at the
// probe round's cost) and from how many rows a probed list goes to the
// tensor cores rather than the FP32 path.  rbc_autotune_tc times a small grid
// of both on sample queries and keeps the fastest.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"
#include "rbc_common.cuh"

using namespace rbc;

namespace {

std::string shape_key(const rbc_index *idx, uint32_t k) {
  char buf[160];
  std::snprintf(buf, sizeof(buf), "%llu %u %u %u %d", (unsigned long long)idx->n, idx->d, idx->nr, k, idx->metric);
  return buf;
}

bool cache_lookup(const char *path, const std::string &key, int *tq, uint32_t *rows) {
  FILE *fp = std::fopen(path, "r");
  if (!fp) return false;
  char line[256];
  bool found = false;
  while (std::fgets(line, sizeof(line), fp)) {
    unsigned long long n;
    unsigned d, nr, k, r;
    int metric, t;
    double ms;
    if (std::sscanf(line, "%llu %u %u %u %d %d %u %lf", &n, &d, &nr, &k, &metric, &t, &r, &ms) != 8) continue;
    char kb[160];
    std::snprintf(kb, sizeof(kb), "%llu %u %u %u %d", n, d, nr, k, metric);
    if (key == kb) {
      *tq = t;
      *rows = r;
      found = true;  // the last entry for a shape wins
    }
  }
  std::fclose(fp);
  return found;
}

}  // namespace

extern "C" {

int rbc_set_tuning(rbc_index *idx, int tq, uint32_t item_rows) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_set_tuning: NULL index");
  if (tq != 0 && tq != 1 && tq != 2 && tq != 4) return fail(RBC_ERR_INVALID, "rbc_set_tuning: tq must be 0, 1, 2 or 4");
  if (item_rows != 0 && item_rows < 32) return fail(RBC_ERR_INVALID, "rbc_set_tuning: item_rows below 32");
  idx->tune_tq = tq;
  idx->item_rows = item_rows ? item_rows : 16384;
  return RBC_OK;
}

int rbc_autotune(rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, const char *cache_path,
                 void *stream) {
  if (!idx || !dQ || m == 0) return fail(RBC_ERR_INVALID, "rbc_autotune: bad argument");
  if (!(idx->flags & RBC_BUILD_PARTITION)) return fail(RBC_ERR_INVALID, "rbc_autotune: index has no partition");
  const std::string key = shape_key(idx, k);
  int tq = 0;
  uint32_t rows = 0;
  if (cache_path && cache_lookup(cache_path, key, &tq, &rows)) return rbc_set_tuning(idx, tq, rows);
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf ids, dists;
  cudaError_t e = ids.alloc(m * k * 4, s);
  if (e == cudaSuccess) e = dists.alloc(m * k * 4, s);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_autotune: buffers");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const bool keep_profile = idx->profile;
  idx->profile = false;
  double best = 1e30;
  int best_tq = 0;
  uint32_t best_rows = 16384;
  int rc = RBC_OK;
  for (int t : {4, 2, 1}) {
    if (search_tq_for(idx->dp, t) != t) continue;
    for (uint32_t r : {4096u, 16384u, 65536u}) {
      idx->tune_tq = t;
      idx->item_rows = r;
      rc = query_index(idx, dQ, m, ldq, k, RBC_QUERY_EXACT, ids.as<uint32_t>(), dists.as<float>(), k, s);
      if (rc != RBC_OK) break;
      double ms_min = 1e30;
      for (int rep = 0; rep < 2 && rc == RBC_OK; rep++) {
        cudaEventRecord(e0, s);
        rc = query_index(idx, dQ, m, ldq, k, RBC_QUERY_EXACT, ids.as<uint32_t>(), dists.as<float>(), k, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms_min = std::min(ms_min, (double)ms);
      }
      if (rc != RBC_OK) break;
      if (ms_min < best) {
        best = ms_min;
        best_tq = t;
        best_rows = r;
      }
    }
    if (rc != RBC_OK) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  idx->profile = keep_profile;
  if (rc != RBC_OK) return rc;
  idx->tune_tq = best_tq;
  idx->item_rows = best_rows;
  if (cache_path) {
    FILE *fp = std::fopen(cache_path, "a");
    if (!fp) return fail(RBC_ERR_IO, std::string("rbc_autotune: cannot write ") + cache_path);
    std::fprintf(fp, "%s %d %u %.4f\n", key.c_str(), best_tq, best_rows, best);
    std::fclose(fp);
  }
  return RBC_OK;
}

int rbc_set_tc_tuning(rbc_index *idx, uint32_t probes, uint64_t probe_rows) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_set_tc_tuning: NULL index");
  if (probes > 16 && probes != RBC_TC_ROUTER_ONLY)
    return fail(RBC_ERR_INVALID, "rbc_set_tc_tuning: probes must be at most 16 (or RBC_TC_ROUTER_ONLY)");
  idx->tc_probes = probes;
  idx->tc_probe_rows = probe_rows;
  idx->tc_plain = false;
  idx->tc_unrouted = false;
  return RBC_OK;
}

int rbc_set_tc_probe_cap(rbc_index *idx, uint64_t rows) {
  if (!idx) return fail(RBC_ERR_INVALID, "rbc_set_tc_probe_cap: NULL index");
  idx->tc_probe_cap = rows;
  return RBC_OK;
}

int rbc_get_tc_tuning(const rbc_index *idx, uint32_t *probes, uint64_t *probe_rows) {
  if (!idx || !probes || !probe_rows) return fail(RBC_ERR_INVALID, "rbc_get_tc_tuning: NULL argument");
  *probes = idx->tc_probes;
  *probe_rows = idx->tc_probe_rows;
  return RBC_OK;
}

int rbc_autotune_tc(rbc_index *idx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
                    void *stream) {
  if (!idx || !dQ || m == 0) return fail(RBC_ERR_INVALID, "rbc_autotune_tc: bad argument");
  if (!(idx->flags & RBC_BUILD_BF16)) return fail(RBC_ERR_INVALID, "rbc_autotune_tc: index has no BF16 lists");
  if ((mode & 0xFFu) != RBC_QUERY_EXACT_TC) return fail(RBC_ERR_INVALID, "rbc_autotune_tc: mode must be RBC_QUERY_EXACT_TC");
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf ids, dists;
  cudaError_t e = ids.alloc(m * k * 4, s);
  if (e == cudaSuccess) e = dists.alloc(m * k * 4, s);
  if (e != cudaSuccess) return cuda_fail(e, "rbc_autotune_tc: buffers");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const bool keep_profile = idx->profile;
  const rbc_query_stats keep_stats = idx->stats;
  idx->profile = false;
  double best = 1e30;
  uint32_t best_p = 0;
  uint64_t best_rows = 0;
  int rc = RBC_OK;
  idx->tc_plain = false;
  idx->tc_probe_cap = 0;
  // the fastest of three calls after a warm-up one
  auto time_calls = [&](uint32_t qmode, double &out) -> int {
    double ms_min = 1e30;
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0, s);
      const int r = query_index(idx, dQ, m, ldq, k, qmode, ids.as<uint32_t>(), dists.as<float>(), k, s);
      if (r != RBC_OK) return r;
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep) ms_min = std::min(ms_min, (double)ms);
    }
    out = ms_min;
    return RBC_OK;
  };
  // routed calls with router picks also try one and two picks, and the
  // nearest lists without the router (picks = kNoRouter below: the call then
  // skips it); a call that plans with the router's distance head (picks = 0)
  // keeps its setting
  const bool routed = (mode & RBC_QUERY_ROUTED) && idx->router;
  const uint32_t user_picks = idx->router_probes;
  constexpr uint32_t kNoRouter = 0xFFFFFFFFu;
  std::vector<uint32_t> picks_set = {user_picks};
  if (routed && user_picks > 0) picks_set = {1u, 2u, kNoRouter};
  uint32_t best_picks = user_picks;
  idx->tc_unrouted = false;
  for (uint32_t picks : picks_set) {
    const bool unrouted = picks == kNoRouter;
    idx->router_probes = unrouted ? user_picks : picks;
    idx->tc_unrouted = unrouted;
    for (uint32_t p : {RBC_TC_ROUTER_ONLY, 1u, 2u, 4u, 8u}) {
      if (p == RBC_TC_ROUTER_ONLY && (!routed || unrouted)) continue;  // the router's picks alone: routed calls only
      for (uint64_t r : {RBC_TC_PREFIX_NONE, 512ull, 2048ull, 8192ull, 32768ull}) {
        idx->tc_probes = p;
        idx->tc_probe_rows = r;
        double ms = 1e30;
        if ((rc = time_calls(mode, ms)) != RBC_OK) break;
        if (ms < best) {
          best = ms;
          best_p = p;
          best_rows = r;
          best_picks = picks;
        }
      }
      if (rc != RBC_OK) break;
    }
    if (rc != RBC_OK) break;
  }
  idx->tc_unrouted = rc == RBC_OK && best_picks == kNoRouter;
  idx->router_probes = rc == RBC_OK && best_picks != kNoRouter ? best_picks : user_picks;
  // the probe cap, on the chosen knobs and with 8 probes (it pays where hub
  // lists hold most of the probed rows)
  uint64_t best_cap = 0;
  const uint64_t prefix = best_rows == RBC_TC_PREFIX_NONE ? 0 : (best_rows ? best_rows : kTcProbeRows);
  std::vector<uint32_t> cap_probes = {best_p};
  if (best_p != 8u) cap_probes.push_back(8u);
  for (uint32_t p : cap_probes) {
    if (rc != RBC_OK) break;
    for (uint64_t c : {32768ull, 65536ull, 131072ull}) {
      if (idx->max_list <= prefix + c) continue;  // the cap would leave every list whole
      idx->tc_probes = p;
      idx->tc_probe_rows = best_rows;
      idx->tc_probe_cap = c;
      double ms = 1e30;
      if ((rc = time_calls(mode, ms)) != RBC_OK) break;
      if (ms < best) {
        best = ms;
        best_p = p;
        best_cap = c;
      }
    }
  }
  idx->tc_probe_cap = 0;
  // the plain FP32 search on the same lists, same routing: when it is the
  // faster of the two, RBC_QUERY_EXACT_TC calls run it
  double plain = 1e30;
  if (rc == RBC_OK) rc = time_calls((mode & ~0xFFu) | RBC_QUERY_EXACT, plain);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  idx->profile = keep_profile;
  idx->stats = keep_stats;
  if (rc != RBC_OK) return rc;
  idx->tc_probes = best_p;
  idx->tc_probe_rows = best_rows;
  idx->tc_probe_cap = best_cap;
  idx->tc_plain = plain < best;
  return RBC_OK;
}

}  // extern "C"
