/*
 * rbc_oracle.c -- CPU oracle for the Random Ball Cover engine.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file.  It is used by tests/ as the checker, by
 * __graft_entry__.smoke() as the checker, and by bench.py's CPU-baseline leg.
 *
 * Parity is pinned two ways:
 *   - against the reference's own bruteCPU/distVec compiled from the
 *     reference sources into oracle/_ref (see oracle/Makefile), and
 *   - against golden vectors in tests/golden/ that were produced by this
 *     file and cross-checked against that reference build.
 *
 * Every routine below restates one piece of the reference's algorithm:
 *   distance     : utils.cu:183-191 (distVec) with defs.h:20-21 (DIST):
 *                  a sequential float sum over dims 0..d-1 of (q-x)^2 or |q-x|,
 *                  each multiply and each add rounded separately (this file
 *                  must be compiled with -ffp-contract=off so no FMA forms).
 *   1-NN         : brute.cu:91-112 (bruteCPU): ids scanned in increasing
 *                  order, strict '<', so the lowest id wins a tie.
 *   k-NN         : the k-NN generalisation of bruteCPU with the order
 *                  (distance, id) lexicographic; k=1 reduces to bruteCPU.
 *                  (The reference's bruteKCPU, brute.cu:115-146, is disabled.)
 *   one-shot RBC : rbc.cu:126-208 (buildRBC), with the radius bisection of
 *                  kernels.cu:322-414 replaced by an exact selection of the
 *                  s nearest points of each representative under (dist, id);
 *                  lists are stored in increasing id order as the scatter of
 *                  sKernel.cu:144-153 stores them; queries search the list of
 *                  their nearest representative (rbc.cu:72-123).
 *   range count  : brute.cu:19-40 / kernels.cu:426-471: count of points with
 *                  distance strictly below the query's range.
 *   partition    : the exact-search structure: each point belongs to the list
 *                  of its nearest representative (ties to the lower rep
 *                  index), with the list radius = largest member distance.
 *   double build : the reference compiled with real = double (defs.h:27-31):
 *                  the same loops in double, MAX_REAL = DBL_MAX padding.
 *   synthetic data: the counter-based generator the engine uses on the GPU
 *                  (integer hashing, exactly representable floats, fixed
 *                  summation order) so both sides draw identical bits.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_L2 0
#define ORC_L1 1
#define ORC_DUMMY 0xFFFFFFFFu

/* ------------------------------------------------------------------ */
/* distance (utils.cu:183-191, defs.h:20-21)                           */
/* ------------------------------------------------------------------ */
static inline float orc_dist_l2(const float *a, const float *b, uint32_t d) {
  float acc = 0.0f;
  for (uint32_t i = 0; i < d; i++) {
    float t = a[i] - b[i];
    float sq = t * t;
    acc = acc + sq;
  }
  return acc;
}

static inline float orc_dist_l1(const float *a, const float *b, uint32_t d) {
  float acc = 0.0f;
  for (uint32_t i = 0; i < d; i++) {
    float t = a[i] - b[i];
    acc = acc + fabsf(t);
  }
  return acc;
}

static inline float orc_dist(const float *a, const float *b, uint32_t d, int metric) {
  return metric == ORC_L1 ? orc_dist_l1(a, b, d) : orc_dist_l2(a, b, d);
}

float orc_distance(const float *a, const float *b, uint32_t d, int metric) {
  return orc_dist(a, b, d, metric);
}

/* FP64 distance of the same pair, for error reporting. */
double orc_distance_f64(const float *a, const float *b, uint32_t d, int metric) {
  double acc = 0.0;
  for (uint32_t i = 0; i < d; i++) {
    double t = (double)a[i] - (double)b[i];
    acc += metric == ORC_L1 ? fabs(t) : t * t;
  }
  return acc;
}

/* ------------------------------------------------------------------ */
/* sorted top-k insertion under (dist, id)                             */
/* ------------------------------------------------------------------ */
static inline int orc_less(float da, uint32_t ia, float db, uint32_t ib) {
  return da < db || (da == db && ia < ib);
}

/* Insert (dv, iv) into the sorted list (dk, ik) of length k if it belongs. */
static inline void orc_topk_insert(float *dk, uint32_t *ik, uint32_t k, float dv, uint32_t iv) {
  if (!orc_less(dv, iv, dk[k - 1], ik[k - 1])) return;
  int32_t p = (int32_t)k - 1;
  while (p > 0 && orc_less(dv, iv, dk[p - 1], ik[p - 1])) {
    dk[p] = dk[p - 1];
    ik[p] = ik[p - 1];
    p--;
  }
  dk[p] = dv;
  ik[p] = iv;
}

/* ------------------------------------------------------------------ */
/* brute k-NN, multithreaded over queries                              */
/* ------------------------------------------------------------------ */
typedef struct {
  const float *X; uint64_t n; uint32_t ldx;
  const float *Q; uint64_t m; uint32_t ldq;
  uint32_t d, k; int metric;
  uint32_t *ids; float *dists; uint32_t ldo;
  uint64_t q0, q1;
} orc_knn_job;

static void *orc_knn_worker(void *arg) {
  orc_knn_job *j = (orc_knn_job *)arg;
  for (uint64_t qi = j->q0; qi < j->q1; qi++) {
    float *dk = j->dists + qi * j->ldo;
    uint32_t *ik = j->ids + qi * j->ldo;
    for (uint32_t t = 0; t < j->k; t++) { dk[t] = FLT_MAX; ik[t] = ORC_DUMMY; }
    const float *q = j->Q + qi * j->ldq;
    for (uint64_t xi = 0; xi < j->n; xi++) {
      float dv = orc_dist(q, j->X + xi * j->ldx, j->d, j->metric);
      orc_topk_insert(dk, ik, j->k, dv, (uint32_t)xi);
    }
  }
  return NULL;
}

/* Exact k-NN of every query under (dist, id).  Missing entries (n < k) are
 * FLT_MAX / 0xFFFFFFFF, the padding of kernels.cu:116-119. */
int orc_knn(const float *X, uint64_t n, uint32_t ldx, const float *Q, uint64_t m, uint32_t ldq,
            uint32_t d, uint32_t k, int metric, uint32_t *ids, float *dists, uint32_t ldo,
            int nthreads) {
  if (k == 0 || ldo < k) return -1;
  if (nthreads < 1) nthreads = 1;
  if ((uint64_t)nthreads > m) nthreads = m ? (int)m : 1;
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  orc_knn_job *jobs = (orc_knn_job *)calloc((size_t)nthreads, sizeof(orc_knn_job));
  if (!th || !jobs) { free(th); free(jobs); return -2; }
  for (int t = 0; t < nthreads; t++) {
    orc_knn_job *j = &jobs[t];
    j->X = X; j->n = n; j->ldx = ldx; j->Q = Q; j->m = m; j->ldq = ldq;
    j->d = d; j->k = k; j->metric = metric; j->ids = ids; j->dists = dists; j->ldo = ldo;
    j->q0 = m * (uint64_t)t / (uint64_t)nthreads;
    j->q1 = m * (uint64_t)(t + 1) / (uint64_t)nthreads;
  }
  for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, orc_knn_worker, &jobs[t]);
  orc_knn_worker(&jobs[0]);
  for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
  free(th);
  free(jobs);
  return 0;
}

/* bruteCPU restated (brute.cu:91-112): 1-NN, strict '<', ids ascending. */
void orc_brute_1nn(const float *X, uint64_t n, uint32_t ldx, const float *Q, uint64_t m,
                   uint32_t ldq, uint32_t d, int metric, uint32_t *nns) {
  for (uint64_t i = 0; i < m; i++) {
    float best = FLT_MAX;
    nns[i] = 0;
    for (uint64_t j = 0; j < n; j++) {
      float t = orc_dist(Q + i * ldq, X + j * ldx, d, metric);
      if (t < best) { best = t; nns[i] = (uint32_t)j; }
    }
  }
}

/* bruteRangeCount restated (brute.cu:19-40, kernels.cu:455): dist < range. */
void orc_range_count(const float *X, uint64_t n, uint32_t ldx, const float *Q, uint64_t m,
                     uint32_t ldq, uint32_t d, int metric, const float *ranges, uint32_t *cnts) {
  for (uint64_t i = 0; i < m; i++) {
    uint32_t c = 0;
    for (uint64_t j = 0; j < n; j++)
      c += orc_dist(Q + i * ldq, X + j * ldx, d, metric) < ranges[i];
    cnts[i] = c;
  }
}

/* ------------------------------------------------------------------ */
/* nearest representative (rbc.cu:233-247 computeReps / nnKernel)      */
/* ------------------------------------------------------------------ */
/* For each row of A, the index of the nearest row of R under (dist, index). */
void orc_nearest_rep(const float *A, uint64_t na, uint32_t lda, const float *R, uint32_t nr,
                     uint32_t ldr, uint32_t d, int metric, uint32_t *rep, float *rdist) {
  for (uint64_t i = 0; i < na; i++) {
    float best = FLT_MAX;
    uint32_t b = 0;
    for (uint32_t r = 0; r < nr; r++) {
      float t = orc_dist(A + i * lda, R + (uint64_t)r * ldr, d, metric);
      if (t < best) { best = t; b = r; }
    }
    rep[i] = b;
    if (rdist) rdist[i] = best;
  }
}

/* ------------------------------------------------------------------ */
/* partition lists (exact-search structure)                            */
/* ------------------------------------------------------------------ */
/* owner[i] = nearest rep of X[i]; offsets has nr+1 entries; members holds the
 * ids of each list in increasing order; radius[r] = max member distance. */
void orc_partition(const float *X, uint64_t n, uint32_t ldx, const uint32_t *rep_ids, uint32_t nr,
                   uint32_t d, int metric, uint32_t *owner, float *odist, uint64_t *offsets,
                   uint32_t *members, float *radius) {
  float *R = (float *)malloc((size_t)nr * d * sizeof(float));
  for (uint32_t r = 0; r < nr; r++) memcpy(R + (size_t)r * d, X + (uint64_t)rep_ids[r] * ldx, d * sizeof(float));
  orc_nearest_rep(X, n, ldx, R, nr, d, d, metric, owner, odist);
  for (uint32_t r = 0; r <= nr; r++) offsets[r] = 0;
  for (uint64_t i = 0; i < n; i++) offsets[owner[i] + 1]++;
  for (uint32_t r = 0; r < nr; r++) offsets[r + 1] += offsets[r];
  uint64_t *cur = (uint64_t *)malloc((size_t)nr * sizeof(uint64_t));
  for (uint32_t r = 0; r < nr; r++) { cur[r] = offsets[r]; radius[r] = 0.0f; }
  for (uint64_t i = 0; i < n; i++) {
    uint32_t o = owner[i];
    members[cur[o]++] = (uint32_t)i;
    if (odist[i] > radius[o]) radius[o] = odist[i];
  }
  free(cur);
  free(R);
}

/* ------------------------------------------------------------------ */
/* one-shot lists (rbc.cu:126-208 with exact s-selection)              */
/* ------------------------------------------------------------------ */
typedef struct { float d; uint32_t id; } orc_pair;

static int orc_pair_cmp(const void *a, const void *b) {
  const orc_pair *x = (const orc_pair *)a, *y = (const orc_pair *)b;
  if (x->d < y->d) return -1;
  if (x->d > y->d) return 1;
  return (x->id > y->id) - (x->id < y->id);
}

static int orc_u32_cmp(const void *a, const void *b) {
  uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  return (x > y) - (x < y);
}

/* lists is nr x lds; list r holds the min(s, n) nearest points of rep r under
 * (dist, id), in increasing id order.  counts[r] = min(s, n).  rho[r] is the
 * distance of the last selected point in (dist, id) order. */
void orc_oneshot_build(const float *X, uint64_t n, uint32_t ldx, const uint32_t *rep_ids, uint32_t nr,
                       uint32_t d, int metric, uint32_t s, uint32_t *lists, uint32_t lds,
                       uint32_t *counts, float *rho) {
  orc_pair *row = (orc_pair *)malloc((size_t)n * sizeof(orc_pair));
  uint32_t take = (uint64_t)s < n ? s : (uint32_t)n;
  for (uint32_t r = 0; r < nr; r++) {
    const float *rp = X + (uint64_t)rep_ids[r] * ldx;
    for (uint64_t j = 0; j < n; j++) {
      row[j].d = orc_dist(rp, X + j * ldx, d, metric);
      row[j].id = (uint32_t)j;
    }
    qsort(row, (size_t)n, sizeof(orc_pair), orc_pair_cmp);
    uint32_t *L = lists + (uint64_t)r * lds;
    for (uint32_t t = 0; t < take; t++) L[t] = row[t].id;
    qsort(L, take, sizeof(uint32_t), orc_u32_cmp);
    counts[r] = take;
    rho[r] = take ? row[take - 1].d : 0.0f;
  }
  free(row);
}

/* One-shot k-NN query (rbc.cu:72-123): search the list of the nearest rep. */
void orc_oneshot_query(const float *X, uint32_t ldx, const uint32_t *rep_ids, uint32_t nr,
                       const uint32_t *lists, uint32_t lds, const uint32_t *counts,
                       const float *Q, uint64_t m, uint32_t ldq, uint32_t d, int metric, uint32_t k,
                       uint32_t *ids, float *dists, uint32_t ldo) {
  float *R = (float *)malloc((size_t)nr * d * sizeof(float));
  for (uint32_t r = 0; r < nr; r++) memcpy(R + (size_t)r * d, X + (uint64_t)rep_ids[r] * ldx, d * sizeof(float));
  for (uint64_t i = 0; i < m; i++) {
    uint32_t rq;
    orc_nearest_rep(Q + i * ldq, 1, ldq, R, nr, d, d, metric, &rq, NULL);
    float *dk = dists + i * ldo;
    uint32_t *ik = ids + i * ldo;
    for (uint32_t t = 0; t < k; t++) { dk[t] = FLT_MAX; ik[t] = ORC_DUMMY; }
    const uint32_t *L = lists + (uint64_t)rq * lds;
    for (uint32_t t = 0; t < counts[rq]; t++) {
      float dv = orc_dist(Q + i * ldq, X + (uint64_t)L[t] * ldx, d, metric);
      orc_topk_insert(dk, ik, k, dv, L[t]);
    }
  }
  free(R);
}

/* ------------------------------------------------------------------ */
/* synthetic data: counter-based generator shared with the GPU         */
/* ------------------------------------------------------------------ */
static inline uint64_t orc_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static inline uint64_t orc_rng(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t key = orc_mix64(seed + 0x9E3779B97F4A7C15ull * (stream + 1));
  return orc_mix64(key + idx);
}

/* uniform float in [0,1): 24 random bits, exactly representable. */
static inline float orc_u01(uint64_t seed, uint64_t stream, uint64_t idx) {
  return (float)(orc_rng(seed, stream, idx) >> 40) * 5.9604644775390625e-08f;
}

/* 12-term Irwin-Hall approximate standard normal, fixed summation order. */
static inline float orc_normal(uint64_t seed, uint64_t stream, uint64_t idx) {
  float s = 0.0f;
  for (int j = 0; j < 12; j++) s = s + orc_u01(seed, stream, idx * 12u + (uint64_t)j);
  return s - 6.0f;
}

/* Geometric thresholds: T[v] = floor(2^32 (1-p)^v) for v = 1..255 with
 * 1-p = num/den, computed in 2^56 fixed point by repeated exact integer
 * multiply-divide so every machine builds the same table.  T[0] unused. */
void orc_geometric_table(uint32_t num, uint32_t den, uint32_t *T) {
  uint64_t t = 1ull << 56;
  T[0] = 0xFFFFFFFFu;
  for (int v = 1; v < 256; v++) {
    t = t * num / den;
    T[v] = (uint32_t)(t >> 24);
  }
}

/* Fill rows [r0, r1) of an n x d (ld) matrix.
 * kind 0: uniform [0,1)          (params unused)
 * kind 1: Gaussian mixture       (ncomp components, means U[0,1)^d, sigma
 *                                 sigma_lo + (sigma_hi-sigma_lo)*U per comp)
 * kind 2: geometric integers     (table T from orc_geometric_table)
 * stream selects the independent draw (database vs queries). */
void orc_synth(int kind, uint64_t seed, uint64_t stream, uint64_t r0, uint64_t r1, uint32_t d,
               uint32_t ld, float *out, uint32_t ncomp, float sigma_lo, float sigma_hi,
               const uint32_t *T) {
  for (uint64_t i = r0; i < r1; i++) {
    float *row = out + (i - r0) * ld;
    if (kind == 0) {
      for (uint32_t c = 0; c < d; c++) row[c] = orc_u01(seed, stream, i * d + c);
    } else if (kind == 1) {
      uint32_t comp = (uint32_t)(orc_rng(seed, stream + 100, i) % ncomp);
      float sg = sigma_lo + (sigma_hi - sigma_lo) * orc_u01(seed, 201, comp);
      for (uint32_t c = 0; c < d; c++) {
        float mu = orc_u01(seed, 200, (uint64_t)comp * d + c);
        float z = orc_normal(seed, stream, i * d + c);
        float sz = sg * z;
        row[c] = mu + sz;
      }
    } else {
      for (uint32_t c = 0; c < d; c++) {
        uint32_t u = (uint32_t)(orc_rng(seed, stream, i * d + c) >> 32);
        uint32_t lo = 0, hi = 255; /* largest v in [0,255] with v==0 or u < T[v] */
        while (lo < hi) {
          uint32_t mid = (lo + hi + 1) >> 1;
          if (u < T[mid]) lo = mid; else hi = mid - 1;
        }
        row[c] = (float)lo;
      }
    }
    for (uint32_t c = d; c < ld; c++) row[c] = 0.0f;
  }
}

/* ------------------------------------------------------------------ */
/* double-precision variant: the reference built with real = double    */
/* (defs.h:27-31, readme.txt:134-152): the same sequential sum, every  */
/* subtract, multiply and add rounded to double on its own.            */
/* ------------------------------------------------------------------ */
static inline double orc_dist64(const double *a, const double *b, uint32_t d, int metric) {
  double acc = 0.0;
  for (uint32_t i = 0; i < d; i++) {
    double t = a[i] - b[i];
    double term = metric == ORC_L1 ? fabs(t) : t * t;
    acc = acc + term;
  }
  return acc;
}

double orc_distance64(const double *a, const double *b, uint32_t d, int metric) {
  return orc_dist64(a, b, d, metric);
}

static inline int orc_less64(double da, uint32_t ia, double db, uint32_t ib) {
  return da < db || (da == db && ia < ib);
}

typedef struct {
  const double *X; uint64_t n; uint32_t ldx;
  const double *Q; uint64_t m; uint32_t ldq;
  uint32_t d, k; int metric;
  uint32_t *ids; double *dists; uint32_t ldo;
  uint64_t q0, q1;
} orc_knn64_job;

static void *orc_knn64_worker(void *arg) {
  orc_knn64_job *j = (orc_knn64_job *)arg;
  for (uint64_t qi = j->q0; qi < j->q1; qi++) {
    double *dk = j->dists + qi * j->ldo;
    uint32_t *ik = j->ids + qi * j->ldo;
    for (uint32_t t = 0; t < j->k; t++) { dk[t] = DBL_MAX; ik[t] = ORC_DUMMY; }
    const double *q = j->Q + qi * j->ldq;
    for (uint64_t xi = 0; xi < j->n; xi++) {
      double dv = orc_dist64(q, j->X + xi * j->ldx, j->d, j->metric);
      uint32_t iv = (uint32_t)xi;
      if (!orc_less64(dv, iv, dk[j->k - 1], ik[j->k - 1])) continue;
      int32_t p = (int32_t)j->k - 1;
      while (p > 0 && orc_less64(dv, iv, dk[p - 1], ik[p - 1])) {
        dk[p] = dk[p - 1];
        ik[p] = ik[p - 1];
        p--;
      }
      dk[p] = dv;
      ik[p] = iv;
    }
  }
  return NULL;
}

/* Exact k-NN in double under (dist, id); missing entries are DBL_MAX /
 * 0xFFFFFFFF (MAX_REAL of the double build). */
int orc_knn_f64(const double *X, uint64_t n, uint32_t ldx, const double *Q, uint64_t m, uint32_t ldq,
                uint32_t d, uint32_t k, int metric, uint32_t *ids, double *dists, uint32_t ldo,
                int nthreads) {
  if (k == 0 || ldo < k) return -1;
  if (nthreads < 1) nthreads = 1;
  if ((uint64_t)nthreads > m) nthreads = m ? (int)m : 1;
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  orc_knn64_job *jobs = (orc_knn64_job *)calloc((size_t)nthreads, sizeof(orc_knn64_job));
  if (!th || !jobs) { free(th); free(jobs); return -2; }
  for (int t = 0; t < nthreads; t++) {
    orc_knn64_job *j = &jobs[t];
    j->X = X; j->n = n; j->ldx = ldx; j->Q = Q; j->m = m; j->ldq = ldq;
    j->d = d; j->k = k; j->metric = metric; j->ids = ids; j->dists = dists; j->ldo = ldo;
    j->q0 = m * (uint64_t)t / (uint64_t)nthreads;
    j->q1 = m * (uint64_t)(t + 1) / (uint64_t)nthreads;
  }
  for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, orc_knn64_worker, &jobs[t]);
  orc_knn64_worker(&jobs[0]);
  for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
  free(th);
  free(jobs);
  return 0;
}

/* bruteCPU of the double build (brute.cu:91-112): strict '<' from DBL_MAX. */
void orc_brute_1nn_f64(const double *X, uint64_t n, uint32_t ldx, const double *Q, uint64_t m,
                       uint32_t ldq, uint32_t d, int metric, uint32_t *nns) {
  for (uint64_t i = 0; i < m; i++) {
    double best = DBL_MAX;
    nns[i] = 0;
    for (uint64_t j = 0; j < n; j++) {
      double t = orc_dist64(Q + i * ldq, X + j * ldx, d, metric);
      if (t < best) { best = t; nns[i] = (uint32_t)j; }
    }
  }
}

/* bruteRangeCount of the double build: count of rows with dist < range. */
void orc_range_count_f64(const double *X, uint64_t n, uint32_t ldx, const double *Q, uint64_t m,
                         uint32_t ldq, uint32_t d, int metric, const double *ranges, uint32_t *cnts) {
  for (uint64_t i = 0; i < m; i++) {
    uint32_t c = 0;
    for (uint64_t j = 0; j < n; j++)
      c += orc_dist64(Q + i * ldq, X + j * ldx, d, metric) < ranges[i];
    cnts[i] = c;
  }
}
