// A program that runs the reference's query plan step by step, as kqueryRBC
// and queryRBC do inside the reference (rbc.cu:19-123), through the plan
// functions of its rbc.h: computeReps, computeCounts, buildQMap, the
// computation matrix, initCompPlan, computeKNNs / computeNNs, freeCompPlan.
// Linked against librbcgb.so.  Used by tests/test_legacy_api.py.
//
//   legacy_plan_driver db.bin q.bin n m d numReps out.bin
//
// out.bin: the queries' nearest representatives (m), the one-shot lists
// (numReps x numReps ids, rows of dxMap) and their lengths (numReps), then
// three answers, each ids (m x KMAX) and distances (m x KMAX): computeKNNs
// under the identity matrix, computeKNNs under the full matrix, and the
// computeNNs 1-NN (m ids, m distances).
#include <cstdio>
#include <cstdlib>

#include "rbc_include.h"

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

static void plan_knn(const matrix q, const matrix dq, const rbcStruct &rbcS, const unint *repIDsQ, bool full,
                     intMatrix NNs, matrix NNdists, unint *nn1, real *d1) {
  const unint m = q.r, numReps = rbcS.dr.r;
  unint *groupCountQ = (unint *)calloc(PAD(numReps), sizeof(unint));
  computeCounts((unint *)repIDsQ, m, groupCountQ);
  unint compLength = 0;
  unint *qMap = (unint *)calloc(PAD(m + (BLOCK_SIZE - 1) * PAD(numReps)), sizeof(unint));
  buildQMap(q, qMap, (unint *)repIDsQ, numReps, &compLength);
  charMatrix cM;
  cM.r = cM.c = numReps;
  cM.pr = cM.pc = cM.ld = PAD(numReps);
  cM.mat = (char *)calloc((size_t)cM.pr * cM.pc, 1);
  if (full)
    fullIntersection(cM);
  else
    idIntersection(cM);
  compPlan dcP;
  initCompPlan(&dcP, cM, groupCountQ, rbcS.groupCount, numReps);
  unint *dqMap = nullptr;
  checkErr(cudaMalloc((void **)&dqMap, compLength * sizeof(unint)));
  checkErr(cudaMemcpy(dqMap, qMap, compLength * sizeof(unint), cudaMemcpyHostToDevice));
  computeKNNs(rbcS.dx, rbcS.dxMap, dq, dqMap, dcP, NNs, NNdists, compLength);
  if (nn1) computeNNs(rbcS.dx, rbcS.dxMap, dq, dqMap, dcP, nn1, d1, compLength);
  freeCompPlan(&dcP);
  cudaFree(dqMap);
  free(cM.mat);
  free(qMap);
  free(groupCountQ);
}

int main(int argc, char **argv) {
  if (argc < 8) {
    fprintf(stderr, "usage: legacy_plan_driver db q n m d numReps out\n");
    return 2;
  }
  unint n = atoi(argv[3]), m = atoi(argv[4]), d = atoi(argv[5]), numReps = atoi(argv[6]);
  matrix x, q, dq;
  initMat(&x, n, d);
  initMat(&q, m, d);
  x.mat = (real *)calloc(sizeOfMat(x), sizeof(*x.mat));
  q.mat = (real *)calloc(sizeOfMat(q), sizeof(*q.mat));
  read_bin(argv[1], x);
  read_bin(argv[2], q);

  rbcStruct rbcS;
  buildRBC(x, &rbcS, numReps, numReps);
  copyAndMove(&dq, &q);
  unint *repIDsQ = (unint *)calloc(m, sizeof(unint));
  real *distToRepsQ = (real *)calloc(m, sizeof(real));
  computeReps(dq, rbcS.dr, repIDsQ, distToRepsQ);

  intMatrix nnsId, nnsFull;
  matrix dId, dFull;
  initIntMat(&nnsId, m, KMAX);
  initIntMat(&nnsFull, m, KMAX);
  initMat(&dId, m, KMAX);
  initMat(&dFull, m, KMAX);
  nnsId.mat = (unint *)calloc(sizeOfIntMat(nnsId), sizeof(unint));
  nnsFull.mat = (unint *)calloc(sizeOfIntMat(nnsFull), sizeof(unint));
  dId.mat = (real *)calloc(sizeOfMat(dId), sizeof(real));
  dFull.mat = (real *)calloc(sizeOfMat(dFull), sizeof(real));
  unint *nn1 = (unint *)calloc(m, sizeof(unint));
  real *d1 = (real *)calloc(m, sizeof(real));
  plan_knn(q, dq, rbcS, repIDsQ, false, nnsId, dId, nn1, d1);
  plan_knn(q, dq, rbcS, repIDsQ, true, nnsFull, dFull, nullptr, nullptr);

  unint *lists = (unint *)calloc((size_t)numReps * rbcS.dxMap.ld, sizeof(unint));
  checkErr(cudaMemcpy(lists, rbcS.dxMap.mat, (size_t)numReps * rbcS.dxMap.ld * sizeof(unint), cudaMemcpyDeviceToHost));
  FILE *fp = fopen(argv[7], "wb");
  if (!fp) return 1;
  fwrite(repIDsQ, sizeof(unint), m, fp);
  for (unint r = 0; r < numReps; r++) fwrite(&lists[(size_t)r * rbcS.dxMap.ld], sizeof(unint), numReps, fp);
  fwrite(rbcS.groupCount, sizeof(unint), numReps, fp);
  for (intMatrix *I : {&nnsId, &nnsFull}) {
    matrix *D = I == &nnsId ? &dId : &dFull;
    for (unint i = 0; i < m; i++) fwrite(&I->mat[IDX(i, 0, I->ld)], sizeof(unint), KMAX, fp);
    for (unint i = 0; i < m; i++) fwrite(&D->mat[IDX(i, 0, D->ld)], sizeof(real), KMAX, fp);
  }
  fwrite(nn1, sizeof(unint), m, fp);
  fwrite(d1, sizeof(real), m, fp);
  if (fclose(fp) != 0) return 1;

  cudaError_t cE = cudaGetLastError();
  if (cE != cudaSuccess) {
    printf("Execution failed; error type: %s \n", cudaGetErrorString(cE));
    return 1;
  }
  destroyRBC(&rbcS);
  cudaFree(dq.mat);
  printf("plan queries done\n");
  return 0;
}
