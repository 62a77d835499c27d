/* rbc_include.h -- umbrella header of the legacy API (reference rbc_include.h:4-10). */
#ifndef RBC_INCLUDE_H
#define RBC_INCLUDE_H

#include "defs.h"
#include "utils.h"
#include "utilsGPU.h"
#include "rbc.h"
#include "brute.h"
#include "sKernel.h"
#include "rbc_gb300.h"
#include <cuda_runtime.h>

/* Programs written for the reference call two runtime functions that CUDA
 * has since removed; map them to their successors so they build unchanged. */
#define cudaThreadSynchronize cudaDeviceSynchronize
#define cudaThreadExit cudaDeviceReset

#endif
