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
