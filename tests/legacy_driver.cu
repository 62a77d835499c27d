// A program written against the reference's C++ API (the calls driver.cu
// makes, in the same order) and linked against librbcgb.so -- or, compiled
// with RBC_REAL_DOUBLE (real = double), against librbcgb_f64.so.  Used by
// tests/test_legacy_api.py.
//
//   legacy_driver db.bin q.bin n m d numReps out_rbc.bin out_brute.bin out_1nn.bin
#include <cstdio>
#include <cstdlib>

#include "rbc_include.h"

// ids block, then distances block (writeNeighbs, driver.cu:352-393), in real
static int write_neighbors(const char *path, intMatrix ids, matrix dists, unint m) {
  FILE *fp = fopen(path, "wb");
  if (!fp) return 1;
  for (unint i = 0; i < m; i++) fwrite(&ids.mat[IDX(i, 0, ids.ld)], sizeof(unint), KMAX, fp);
  for (unint i = 0; i < m; i++) fwrite(&dists.mat[IDX(i, 0, dists.ld)], sizeof(real), KMAX, fp);
  return fclose(fp) != 0;
}

static void read_bin(const char *path, matrix x) {
  FILE *fp = fopen(path, "rb");
  if (!fp) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(1);
  }
  for (unint i = 0; i < x.r; i++)
    if (fread(&x.mat[IDX(i, 0, x.ld)], sizeof(real), x.c, fp) != x.c) {
      fprintf(stderr, "short read\n");
      exit(1);
    }
  fclose(fp);
}

int main(int argc, char **argv) {
  if (argc < 10) {
    fprintf(stderr, "usage: legacy_driver db q n m d numReps out_rbc out_brute out_1nn\n");
    return 2;
  }
  unint n = atoi(argv[3]), m = atoi(argv[4]), d = atoi(argv[5]), numReps = atoi(argv[6]);
  matrix x, q;
  initMat(&x, n, d);
  initMat(&q, m, d);
  x.mat = (real *)calloc(sizeOfMat(x), sizeof(*x.mat));
  q.mat = (real *)calloc(sizeOfMat(q), sizeof(*q.mat));
  read_bin(argv[1], x);
  read_bin(argv[2], q);

  intMatrix nnsRBC;
  matrix distsRBC;
  initIntMat(&nnsRBC, m, KMAX);
  initMat(&distsRBC, m, KMAX);
  nnsRBC.mat = (unint *)calloc(sizeOfIntMat(nnsRBC), sizeof(*nnsRBC.mat));
  distsRBC.mat = (real *)calloc(sizeOfMat(distsRBC), sizeof(*distsRBC.mat));

  rbcStruct rbcS;
  buildRBC(x, &rbcS, numReps, numReps);
  kqueryRBC(q, rbcS, nnsRBC, distsRBC);

  intMatrix nnsB;
  matrix distsB;
  initIntMat(&nnsB, m, KMAX);
  initMat(&distsB, m, KMAX);
  nnsB.mat = (unint *)calloc(sizeOfIntMat(nnsB), sizeof(*nnsB.mat));
  distsB.mat = (real *)calloc(sizeOfMat(distsB), sizeof(*distsB.mat));
  bruteK(x, q, nnsB, distsB);

  unint *nnCPU = (unint *)calloc(m, sizeof(unint));
  unint *nnGPU = (unint *)calloc(m, sizeof(unint));
  unint *nnRBC = (unint *)calloc(m, sizeof(unint));
  real *dRBC = (real *)calloc(m, sizeof(real));
  bruteCPU(x, q, nnCPU);
  bruteSearch(x, q, nnGPU);
  queryRBC(q, rbcS, nnRBC, dRBC);

  cudaError_t cE = cudaGetLastError();
  if (cE != cudaSuccess) {
    printf("Execution failed; error type: %s \n", cudaGetErrorString(cE));
    return 1;
  }
  if (write_neighbors(argv[7], nnsRBC, distsRBC, m)) return 1;
  if (write_neighbors(argv[8], nnsB, distsB, m)) return 1;
  FILE *fp = fopen(argv[9], "wb");
  fwrite(nnCPU, sizeof(unint), m, fp);
  fwrite(nnGPU, sizeof(unint), m, fp);
  fwrite(nnRBC, sizeof(unint), m, fp);
  fwrite(dRBC, sizeof(real), m, fp);
  fclose(fp);

  // the one-shot lists stay observable through rbcStruct as in the reference
  unint total = 0;
  for (unint r = 0; r < numReps; r++) total += rbcS.groupCount[r];
  printf("one-shot list entries: %u\n", total);

  destroyRBC(&rbcS);
  free(nnsRBC.mat);
  free(distsRBC.mat);
  free(nnsB.mat);
  free(distsB.mat);
  free(nnCPU);
  free(nnGPU);
  free(nnRBC);
  free(dRBC);
  free(x.mat);
  free(q.mat);
  return 0;
}
