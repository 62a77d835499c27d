/*
 * brute.h -- legacy brute-force API (reference brute.h:10-13).
 * bruteK returns the 32 nearest neighbours sorted by (distance, id);
 * bruteSearch the nearest; bruteRangeCount the number of database points
 * strictly closer than each query's range; bruteCPU is the host 1-NN scan.
 */
#ifndef BRUTE_H
#define BRUTE_H

#include "defs.h"

void bruteRangeCount(matrix, matrix, real *, unint *);
void bruteSearch(matrix, matrix, unint *);
void bruteCPU(matrix, matrix, unint *);
void bruteK(matrix, matrix, intMatrix, matrix);

#endif
