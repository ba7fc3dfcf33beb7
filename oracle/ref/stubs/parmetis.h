/* Declarations-only stand-in for ParMETIS/METIS used to compile the reference
 * as a single-rank oracle.  Graph partitioning is never called with one rank. */
#ifndef OCPX_ORACLE_PARMETIS_STUB_H
#define OCPX_ORACLE_PARMETIS_STUB_H
#include <stdint.h>
#include "mpi.h"
typedef int64_t idx_t;
typedef float real_t;
#define IDX_T MPI_LONG_LONG_INT
#define REAL_T 4
#define METIS_OK 1
#define METIS_ERROR (-4)
#ifdef __cplusplus
extern "C" {
#endif
int ParMETIS_V3_PartKway(idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*,
                         real_t*, real_t*, idx_t*, idx_t*, idx_t*, MPI_Comm*);
int METIS_PartGraphKway(idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, real_t*,
                        real_t*, idx_t*, idx_t*, idx_t*);
int METIS_PartGraphRecursive(idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, real_t*,
                             real_t*, idx_t*, idx_t*, idx_t*);
#ifdef __cplusplus
}
#endif
#endif
