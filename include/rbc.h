/*
 * rbc.h -- legacy Random Ball Cover API (C++ linkage, by-value structs).
 *
 * Same declarations as the reference's rbc.h:11-26 so programs written for it
 * (driver.cu, or code that runs the query plan step by step) compile and link
 * unchanged.  buildRBC builds both the
 * reference's one-shot lists (exposed in rbcStruct) and the partition used for
 * exact search; queryRBC / kqueryRBC return EXACT 1 / 32 nearest neighbours by
 * default.  rbc_set_legacy_query_mode(RBC_QUERY_ONESHOT) restores the
 * reference's one-shot search.  Failures print a message and exit(1), the
 * reference's checkErr convention (utilsGPU.cu:52-59).
 */
#ifndef RBC_H
#define RBC_H

#include "defs.h"

void buildRBC(const matrix, rbcStruct *, unint, unint);
void queryRBC(const matrix, const rbcStruct, unint *, real *);
void kqueryRBC(const matrix, const rbcStruct, intMatrix, matrix);
void destroyRBC(rbcStruct *);
void distSubMat(matrix, matrix, matrix, unint, unint);
void computeReps(matrix, matrix, unint *, real *);
void computeRadii(unint *, real *, real *, unint, unint);
void computeCounts(unint *, unint, unint *);
void buildQMap(matrix, unint *, unint *, unint, unint *);
void idIntersection(charMatrix);
void fullIntersection(charMatrix);
void initCompPlan(compPlan *, charMatrix, unint *, unint *, unint);
void freeCompPlan(compPlan *);
void computeNNs(matrix, intMatrix, matrix, unint *, compPlan, unint *, real *, unint);
void computeKNNs(matrix, intMatrix, matrix, unint *, compPlan, intMatrix, matrix, unint);
void setupReps(matrix, rbcStruct *, unint);

#ifdef __cplusplus
extern "C" {
#endif
/* Settings of the legacy layer (no counterpart in the reference, whose
 * metric is a compile-time macro and whose representatives are seeded from
 * the clock). */
void rbc_set_legacy_query_mode(unsigned mode); /* RBC_QUERY_EXACT (default) or _ONESHOT */
void rbc_set_legacy_metric(int metric);        /* RBC_L2 (default) or RBC_L1           */
void rbc_set_legacy_seed(unsigned long long seed);
#ifdef __cplusplus
}
#endif

#endif
