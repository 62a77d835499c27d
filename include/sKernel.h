/* sKernel.h -- kept so programs including rbc_include.h compile unchanged.
 * The reference declares its scan kernels here (sKernel.h:8-12); this
 * engine's scan kernels are internal to the library and not declared. */
#ifndef SKERNEL_H
#define SKERNEL_H
#include "defs.h"
#endif
