/* utilsGPU.h -- legacy device-copy helpers (reference utilsGPU.h:12-17). */
#ifndef UTILSGPU_H
#define UTILSGPU_H

#include <cuda_runtime.h>
#include "defs.h"

void copyAndMove(matrix *, const matrix *);
void copyAndMoveI(intMatrix *, const intMatrix *);
void copyAndMoveC(charMatrix *, const charMatrix *);

void checkErr(cudaError_t);
void checkErr(char *, cudaError_t);

#endif
