// testRBC -- command-line driver with the reference driver's interface
// (driver.cu:22-198): the same flags, file formats and output layout, plus
// options for the engine's query modes and index files.
//
//   testRBC -x db.bin -q queries.bin -n N -m M -d D -r numReps [-o out.bin] [-g gpu] [-b] [-e]
//   text input/output: -X / -Q / -O in place of -x / -q / -o
//   extensions: -k K      neighbours per query written (default 32, at most RBC_K_LIMIT = 128)
//               -M mode   exact (default) | tc (BF16 tensor cores, exact) | oneshot (reference algorithm)
//               -s seed   representative sampling seed
//               -l        L1 distance instead of squared L2
//               -S file   save the built index;  -L file  load an index instead of building
//               -D        the double build (real = double, defs.h:27-31): 8-byte input and
//                         output values, distances in double
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/time.h>
#include <vector>

#include <cuda_runtime.h>

#include "rbc_gb300.h"

namespace {

const char *dbX = nullptr, *dbQ = nullptr, *dbXt = nullptr, *dbQt = nullptr, *outB = nullptr, *outT = nullptr;
const char *saveIdx = nullptr, *loadIdx = nullptr;
bool runBrute = false, runEval = false, useDouble = false;
uint64_t n = 0, m = 0;
uint32_t d = 0, numReps = 0, k = RBC_KMAX;
int device = 0, metric = RBC_L2;
uint32_t mode = RBC_QUERY_EXACT;
unsigned long long seed = 0x5EED;

double now() {
  timeval t;
  gettimeofday(&t, nullptr);
  return t.tv_sec + t.tv_usec / 1e6;
}

void check(int rc, const char *what) {
  if (rc != RBC_OK) {
    std::fprintf(stderr, "%s failed: %s (%s).. exiting\n", what, rbc_status_string(rc), rbc_last_error());
    std::exit(1);
  }
}

void usage() {
  std::printf("\nusage: \n  testRBC -x datafileX -q datafileQ  -n numPts (DB) -m numQueries -d dim -r numReps "
              "[-o outFile] [-g GPU num] [-b] [-e]\n\n");
  std::printf("\tdatafileX    = binary file containing the database\n");
  std::printf("\tdatafileQ    = binary file containing the queries\n");
  std::printf("\tnumPts       = size of database\n");
  std::printf("\tnumQueries   = number of queries\n");
  std::printf("\tdim          = dimensionality\n");
  std::printf("\tnumReps      = number of representatives (must be at least 32)\n");
  std::printf("\toutFile      = binary output file (optional)\n");
  std::printf("\tGPU num      = ID # of the GPU to use (optional) for multi-GPU machines\n");
  std::printf("\n\tuse -b to run brute force in addition the RBC\n");
  std::printf("\tuse -e to run the evaluation routine (implicitly runs brute force)\n");
  std::printf("\n\tTo input/output data in text format (instead of bin), use the \n\t-X and -Q and -O switches in "
              "place of -x and -q and -o (respectively).\n");
  std::printf("\n\textensions: -k K, -M exact|tc|oneshot, -s seed, -l (L1), -S indexfile, -L indexfile,\n"
              "\t            -D (double precision: 8-byte values in and out)\n\n");
  std::exit(0);
}

void parse(int argc, char **argv) {
  if (argc <= 1) usage();
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    auto next = [&]() -> const char * {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "%s needs a value.. exiting\n", a.c_str());
        std::exit(1);
      }
      return argv[++i];
    };
    if (a == "-x") dbX = next();
    else if (a == "-q") dbQ = next();
    else if (a == "-X") dbXt = next();
    else if (a == "-Q") dbQt = next();
    else if (a == "-n") n = std::strtoull(next(), nullptr, 10);
    else if (a == "-m") m = std::strtoull(next(), nullptr, 10);
    else if (a == "-d") d = (uint32_t)std::atoi(next());
    else if (a == "-r") numReps = (uint32_t)std::atoi(next());
    else if (a == "-o") outB = next();
    else if (a == "-O") outT = next();
    else if (a == "-g") device = std::atoi(next());
    else if (a == "-b") runBrute = true;
    else if (a == "-e") runEval = true;
    else if (a == "-k") k = (uint32_t)std::atoi(next());
    else if (a == "-s") seed = std::strtoull(next(), nullptr, 0);
    else if (a == "-l") metric = RBC_L1;
    else if (a == "-D") useDouble = true;
    else if (a == "-S") saveIdx = next();
    else if (a == "-L") loadIdx = next();
    else if (a == "-M") {
      std::string v = next();
      mode = v == "tc" ? RBC_QUERY_EXACT_TC : v == "oneshot" ? RBC_QUERY_ONESHOT : RBC_QUERY_EXACT;
    } else {
      std::fprintf(stderr, "%s : unrecognized option.. exiting\n", argv[i]);
      std::exit(1);
    }
  }
  if (!n || !m || !d || (!numReps && !loadIdx)) {
    std::fprintf(stderr, "more arguments needed.. exiting\n");
    std::exit(1);
  }
  if ((!dbX && !dbXt) || (!dbQ && !dbQt)) {
    std::fprintf(stderr, "more arguments needed.. exiting\n");
    std::exit(1);
  }
  if ((dbX && dbXt) || (dbQ && dbQt)) {
    std::fprintf(stderr, "you can only give one database file and one query file.. exiting\n");
    std::exit(1);
  }
  if (!loadIdx && numReps > n) {
    std::fprintf(stderr, "can't have more representatives than points.. exiting\n");
    std::exit(1);
  }
  if (!loadIdx && numReps < 32) {
    std::fprintf(stderr, "number of representatives must be at least 32\n");
    std::exit(1);
  }
  if (useDouble && mode == RBC_QUERY_ONESHOT) {
    std::fprintf(stderr, "the one-shot lists are not available in double precision.. exiting\n");
    std::exit(1);
  }
  if (k < 1 || k > RBC_K_LIMIT) {
    std::fprintf(stderr, "k must be in [1, %d].. exiting\n", RBC_K_LIMIT);
    std::exit(1);
  }
}

// The library calls of one precision: float (the reference's default build)
// or double (its real = double build).
template <typename R>
struct Api;
template <>
struct Api<float> {
  static int read_bin(const char *p, float *h, uint64_t r, uint32_t c, uint32_t ld) {
    return rbc_read_matrix_bin(p, h, r, c, ld);
  }
  static int read_text(const char *p, float *h, uint64_t r, uint32_t c, uint32_t ld) {
    return rbc_read_matrix_text(p, h, r, c, ld);
  }
  static int build(const float *dX, uint64_t n, uint32_t d, uint32_t ld, const rbc_build_params *p, rbc_index **o) {
    return rbc_build(dX, n, d, ld, p, nullptr, o);
  }
  static int query(rbc_index *i, const float *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode, uint32_t *ids,
                   float *dists, uint32_t ldo) {
    return rbc_query(i, dQ, m, ldq, k, mode, ids, dists, ldo, nullptr);
  }
  static int brute(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t d,
                   uint32_t k, int metric, uint32_t *ids, float *dists, uint32_t ldo) {
    return rbc_brute_knn(dX, n, ldx, dQ, m, ldq, d, k, metric, ids, dists, ldo, nullptr);
  }
  static int range(const float *dX, uint64_t n, uint32_t ldx, const float *dQ, uint64_t m, uint32_t ldq, uint32_t d,
                   int metric, const float *r, uint32_t *c) {
    return rbc_brute_range_count(dX, n, ldx, dQ, m, ldq, d, metric, r, c, nullptr);
  }
  static int write_bin(const char *p, const uint32_t *i, const float *dd, uint64_t m, uint32_t k, uint32_t ld) {
    return rbc_write_neighbors_bin(p, i, dd, m, k, ld);
  }
  static int write_text(const char *p, const uint32_t *i, const float *dd, uint64_t m, uint32_t k, uint32_t ld) {
    return rbc_write_neighbors_text(p, i, dd, m, k, ld);
  }
};
template <>
struct Api<double> {
  static int read_bin(const char *p, double *h, uint64_t r, uint32_t c, uint32_t ld) {
    return rbc_read_matrix_bin_f64(p, h, r, c, ld);
  }
  static int read_text(const char *p, double *h, uint64_t r, uint32_t c, uint32_t ld) {
    return rbc_read_matrix_text_f64(p, h, r, c, ld);
  }
  static int build(const double *dX, uint64_t n, uint32_t d, uint32_t ld, const rbc_build_params *p, rbc_index **o) {
    return rbc_build_f64(dX, n, d, ld, p, nullptr, o);
  }
  static int query(rbc_index *i, const double *dQ, uint64_t m, uint32_t ldq, uint32_t k, uint32_t mode,
                   uint32_t *ids, double *dists, uint32_t ldo) {
    return rbc_query_f64(i, dQ, m, ldq, k, mode, ids, dists, ldo, nullptr);
  }
  static int brute(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m, uint32_t ldq,
                   uint32_t d, uint32_t k, int metric, uint32_t *ids, double *dists, uint32_t ldo) {
    return rbc_brute_knn_f64(dX, n, ldx, dQ, m, ldq, d, k, metric, ids, dists, ldo, nullptr, nullptr);
  }
  static int range(const double *dX, uint64_t n, uint32_t ldx, const double *dQ, uint64_t m, uint32_t ldq,
                   uint32_t d, int metric, const double *r, uint32_t *c) {
    return rbc_brute_range_count_f64(dX, n, ldx, dQ, m, ldq, d, metric, r, c, nullptr);
  }
  static int write_bin(const char *p, const uint32_t *i, const double *dd, uint64_t m, uint32_t k, uint32_t ld) {
    return rbc_write_neighbors_bin_f64(p, i, dd, m, k, ld);
  }
  static int write_text(const char *p, const uint32_t *i, const double *dd, uint64_t m, uint32_t k, uint32_t ld) {
    return rbc_write_neighbors_text_f64(p, i, dd, m, k, ld);
  }
};

// Read, build (or load), query, optionally brute force and evaluate, write.
template <typename R>
int run() {
  using A = Api<R>;
  double t0;
  const uint32_t ld = (d + 15) / 16 * 16;
  std::vector<R> x(n * ld), q(m * ld);
  check(dbXt ? A::read_text(dbXt, x.data(), n, d, ld) : A::read_bin(dbX, x.data(), n, d, ld), "reading the database");
  check(dbQt ? A::read_text(dbQt, q.data(), m, d, ld) : A::read_bin(dbQ, q.data(), m, d, ld), "reading the queries");
  void *dx = nullptr, *dq = nullptr;
  if (cudaMalloc(&dx, x.size() * sizeof(R)) != cudaSuccess || cudaMalloc(&dq, q.size() * sizeof(R)) != cudaSuccess) {
    std::fprintf(stderr, "not enough device memory for the database and queries.. exiting\n");
    return 1;
  }

  rbc_index *idx = nullptr;
  std::printf("building the rbc..\n");
  t0 = now();
  if (loadIdx) {
    check(rbc_load(loadIdx, &idx), "loading the index");
    rbc_index_info info{};
    check(rbc_get_info(idx, &info), "reading the index");
    if (((info.flags & RBC_BUILD_F64) != 0) != (sizeof(R) == 8)) {
      std::fprintf(stderr, "the index file was built in the other precision (-D).. exiting\n");
      return 1;
    }
  } else {
    rbc_build_params p{};
    p.num_reps = numReps;
    p.s = numReps;
    p.metric = metric;
    p.flags = RBC_BUILD_PARTITION | (mode == RBC_QUERY_ONESHOT ? RBC_BUILD_ONESHOT : 0u) |
              (mode == RBC_QUERY_EXACT_TC ? RBC_BUILD_BF16 : 0u);
    p.seed = seed;
    cudaMemcpy(dx, x.data(), x.size() * sizeof(R), cudaMemcpyHostToDevice);
    check(A::build((const R *)dx, n, d, ld, &p, &idx), "buildRBC");
  }
  std::printf("\t.. build time = %6.4f \n", now() - t0);
  if (saveIdx) check(rbc_save(idx, saveIdx), "saving the index");

  // K columns per query: the reference's 32, or k when more are asked for;
  // the evaluation reads the first 32
  const uint32_t K = k > RBC_KMAX ? k : RBC_KMAX;
  std::vector<uint32_t> ids(m * K);
  std::vector<R> dists(m * K);
  void *di = nullptr, *dd = nullptr;
  cudaMalloc(&di, ids.size() * 4);
  cudaMalloc(&dd, dists.size() * sizeof(R));
  t0 = now();
  cudaMemcpy(dq, q.data(), q.size() * sizeof(R), cudaMemcpyHostToDevice);
  check(A::query(idx, (const R *)dq, m, ld, K, mode, (uint32_t *)di, (R *)dd, K), "kqueryRBC");
  cudaMemcpy(ids.data(), di, ids.size() * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(dists.data(), dd, dists.size() * sizeof(R), cudaMemcpyDeviceToHost);
  std::printf("\t.. query time for krbc = %6.4f \n", now() - t0);

  std::vector<uint32_t> bids;
  std::vector<R> bdists;
  if (runBrute || runEval) {
    std::printf("running k-brute force..\n");
    bids.resize(m * K);
    bdists.resize(m * K);
    t0 = now();
    cudaMemcpy(dx, x.data(), x.size() * sizeof(R), cudaMemcpyHostToDevice);
    cudaMemcpy(dq, q.data(), q.size() * sizeof(R), cudaMemcpyHostToDevice);
    check(A::brute((const R *)dx, n, ld, (const R *)dq, m, ld, d, K, metric, (uint32_t *)di, (R *)dd, K), "bruteK");
    cudaMemcpy(bids.data(), di, bids.size() * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(bdists.data(), dd, bdists.size() * sizeof(R), cudaMemcpyDeviceToHost);
    std::printf("\t.. time elapsed = %6.4f \n", now() - t0);
    if (runEval) {
      // overlap of the returned 32 ids with brute force, and the rank of the
      // returned 32nd neighbour (driver.cu:283-349)
      std::printf("\nComputing error rates (this might take a while)\n");
      double sum = 0, sum2 = 0;
      for (uint64_t i = 0; i < m; i++) {
        uint32_t ol = 0;
        for (uint32_t j = 0; j < RBC_KMAX; j++)
          for (uint32_t t = 0; t < RBC_KMAX; t++) ol += ids[i * K + j] == bids[i * K + t];
        sum += ol;
        sum2 += (double)ol * ol;
      }
      double mean = sum / m;
      std::printf("\tavg overlap = %6.4f/%d; std dev = %6.4f \n", mean, RBC_KMAX, std::sqrt(sum2 / m - mean * mean));
      std::vector<R> ranges(m);
      for (uint64_t i = 0; i < m; i++) ranges[i] = dists[i * K + RBC_KMAX - 1];
      void *dr = nullptr, *dc = nullptr;
      cudaMalloc(&dr, m * sizeof(R));
      cudaMalloc(&dc, m * 4);
      cudaMemcpy(dr, ranges.data(), m * sizeof(R), cudaMemcpyHostToDevice);
      check(A::range((const R *)dx, n, ld, (const R *)dq, m, ld, d, metric, (const R *)dr, (uint32_t *)dc),
            "bruteRangeCount");
      std::vector<uint32_t> cnt(m);
      cudaMemcpy(cnt.data(), dc, m * 4, cudaMemcpyDeviceToHost);
      sum = sum2 = 0;
      for (uint64_t i = 0; i < m; i++) {
        sum += cnt[i];
        sum2 += (double)cnt[i] * cnt[i];
      }
      mean = sum / m;
      std::printf("\tavg actual rank of 32nd NN returned by the RBC = %6.4f; std dev = %6.4f \n\n", mean,
                  std::sqrt(std::max(0.0, sum2 / m - mean * mean)));
      cudaFree(dr);
      cudaFree(dc);
    }
  }
  cudaFree(dx);
  cudaFree(dq);
  cudaFree(di);
  cudaFree(dd);
  cudaError_t cE = cudaGetLastError();
  if (cE != cudaSuccess) std::printf("Execution failed; error type: %s \n", cudaGetErrorString(cE));

  if (outB) check(A::write_bin(outB, ids.data(), dists.data(), m, k, K), "writing the output");
  if (outT) check(A::write_text(outT, ids.data(), dists.data(), m, k, K), "writing the output");
  rbc_destroy(idx);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  std::printf("*****************\n");
  std::printf("RANDOM BALL COVER\n");
  std::printf("*****************\n");
  parse(argc, argv);
  double t0 = now();
  std::printf("Using GPU #%d\n", device);
  if (cudaSetDevice(device) != cudaSuccess) {
    std::printf("Unable to select device %d.. exiting. \n", device);
    return 1;
  }
  size_t memFree = 0, memTot = 0;
  cudaMemGetInfo(&memFree, &memTot);
  std::printf("GPU memory free = %lu/%lu (MB) \n", (unsigned long)(memFree >> 20), (unsigned long)(memTot >> 20));
  std::printf(" init time: %6.2f \n", now() - t0);

  return useDouble ? run<double>() : run<float>();
}
