// tune.cu -- the autotuner of the FP32 list search.
//
// Two knobs shape the plain search: the query tile (16 x TQ queries per CTA,
// TQ rows per thread) and the longest run of list rows a work item covers
// (long lists split into several items so the persistent launch stays
// balanced).  rbc_autotune times every valid pair on sample queries with CUDA
// events and keeps the fastest; a cache file (one line per index shape:
// "n d reps k metric tq item_rows ms") lets later processes skip the timing.
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

}  // extern "C"
