/*
 * defs.h -- types and macros of the legacy (reference-compatible) API.
 *
 * The struct layouts, names and macro values below must equal those of the
 * reference's defs.h (defs.h:9-100) because user programs allocate these
 * structs themselves and pass them by value to functions whose C++ mangled
 * names include the type names: matrix / intMatrix / charMatrix are
 * {pointer, r, c, pr, pc, ld} with rows and columns padded to multiples of 16
 * (ld == pc), rbcStruct is {dx, dxMap, dr, groupCount}.
 */
#ifndef DEFS_H
#define DEFS_H

#include <float.h>
#include <stdint.h>
#include <limits.h>

#define FLOAT_TOL 1e-7

#define KMAX 32       /* neighbours returned by kqueryRBC / bruteK          */
#define BLOCK_SIZE 16 /* row/column padding granularity                      */
#define MAX_BS 65535
#define SCAN_WIDTH 1024

/* Per-coordinate distance term.  The engine selects the metric at run time
 * (rbc_set_legacy_metric); this macro is the default L2 term. */
#define DIST(i, j) (((i) - (j)) * ((i) - (j)))

/* The reference switches to double by editing these two lines
 * (defs.h:27-31, readme.txt:134-152); here RBC_REAL_DOUBLE selects the double
 * build, whose library is librbcgb_f64.so. */
#ifdef RBC_REAL_DOUBLE
typedef double real;
#define MAX_REAL DBL_MAX
#else
typedef float real;
#define MAX_REAL FLT_MAX
#endif

#define MEM_USABLE .95
#define DUMMY_IDX UINT_MAX

#define IDX(i, j, ld) (((size_t)(i) * (ld)) + (j))
#define PAD(i) (((i) % BLOCK_SIZE) == 0 ? (i) : ((i) / BLOCK_SIZE) * BLOCK_SIZE + BLOCK_SIZE)
#define DPAD(i) (((i) % BLOCK_SIZE) == 0 ? (i) : ((i) / BLOCK_SIZE) * BLOCK_SIZE)

#define MAX(i, j) ((i) > (j) ? (i) : (j))
#define MIN(i, j) ((i) <= (j) ? (i) : (j))

typedef uint32_t unint;

typedef struct {
  real *mat;
  unint r;  /* rows                       */
  unint c;  /* columns                    */
  unint pr; /* padded rows                */
  unint pc; /* padded columns             */
  unint ld; /* leading dimension (== pc)  */
} matrix;

typedef struct {
  char *mat;
  unint r, c, pr, pc, ld;
} charMatrix;

typedef struct {
  unint *mat;
  unint r, c, pr, pc, ld;
} intMatrix;

typedef struct {
  unint *numGroups;
  unint *groupCountX;
  unint *qToQGroup;
  unint *qGroupToXGroup;
  unint ld;
} compPlan;

typedef struct {
  matrix dx;        /* device copy of the database (padded, original order) */
  intMatrix dxMap;  /* device one-shot lists: row r = ids owned by rep r     */
  matrix dr;        /* device representatives                              */
  unint *groupCount;/* host: ids in each one-shot list                      */
} rbcStruct;

#endif
