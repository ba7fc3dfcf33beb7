/*
 * ocpx_oracle.h -- CPU restatement of OpenCAEPoroX's FIM Newton-step path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU path is checked
 * against (tests/, the smoke entry point, and the CPU baseline of the bench);
 * it is never part of the product.  It restates the reference's per-cell and
 * per-connection loops in plain C, in the reference's own array layout
 * (BulkVarSet, include/BulkVarSet.hpp: cell-major, then phase, then
 * component), following the source line by line (citations per function in
 * ocpx_oracle.c).  Its results are pinned against fixtures dumped from the
 * reference itself (tests/golden/, tests/test_oracle.py).
 */
#ifndef OCPX_ORACLE_H
#define OCPX_ORACLE_H

#include <stdint.h>
#include "../include/ocpx.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oc_model oc_model;

/* Bulk state, reference layout; arrays owned by the caller. */
typedef struct oc_bulk {
    int nb, np, nc;
    const double *v, *depth, *poroInit;
    double *P, *T, *Pb, *Ni, *lNi, *Nt, *vf, *vfP, *vfi;
    double *Pj, *Pc, *S;
    uint32_t* phaseExist;
    double *xij, *rho, *xi, *mu, *rhoP, *xiP, *muP, *rhox, *xix, *mux;
    double *kr, *dKrdS, *dPcdS, *dSec_dPri, *poro, *poroP, *rockVp;
    uint32_t* skip_flag;
    double *skip_minEig, *skip_P, *skip_T, *skip_zi;
    int32_t* ftype;  /* out: flash type left by the flash */
    int32_t* iters;  /* out: [nb*5] iteration counters */
} oc_bulk;

/* Connections (reference order) and their CalFlux results. */
typedef struct oc_conn {
    int nconn;
    const uint32_t *bId, *eId;
    const double* trans;
    uint32_t* upblock;  /* [nconn*np] */
    double *dP, *flux_vj, *flux_ni;  /* [nconn*np], [nconn*np], [nconn*nc] */
} oc_conn;

oc_model* oc_create(const ocpx_model_desc* md);
void oc_destroy(oc_model* m);

/* NR.CheckPhysical("BulkNi","BulkP") (src/OCPNRsuite.cpp:304-376):
 * returns 0 on success, 1 negative Ni, 2 negative P. */
int oc_check(const oc_model* m, oc_bulk* b);
/* CalFlash for cells [n0, n1) (src/IsoThermalMethod.cpp:1016-1071). */
void oc_flash(const oc_model* m, oc_bulk* b, int n0, int n1);
/* CalKrPc + CalRock (src/IsoThermalMethod.cpp:1073-1088, 19-30). */
void oc_krpc_rock(const oc_model* m, oc_bulk* b, int n0, int n1);
/* CalRes, bulk part (src/IsoThermalMethod.cpp:1090-1185): res [nb*(nc+1)]
 * negated; norms[0..3] = maxRelRes_V, maxRelRes_N, maxId_V, maxId_N. */
void oc_calres(const oc_model* m, oc_bulk* b, oc_conn* c, double dt, double* res, double* resRelV,
               double* resRelN, double* norms);
/* AssembleMatBulks (src/IsoThermalMethod.cpp:1187-1269): block CSR with the
 * reference's push-back order; rowptr [nb+1], col [nnz], val [nnz*(nc+1)^2];
 * returns nnz (blocks). */
long oc_assemble(const oc_model* m, const oc_bulk* b, const oc_conn* c, double dt, uint32_t* rowptr, uint32_t* col,
                 double* val);
/* GetSolution, bulk part (src/IsoThermalMethod.cpp:1282-1418). */
void oc_newton_update(const oc_model* m, oc_bulk* b, const double* u, double dSmax);

#ifdef __cplusplus
}
#endif
#endif
