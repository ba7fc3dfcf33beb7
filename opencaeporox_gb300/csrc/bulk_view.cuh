// Structure-of-arrays view of the bulk (cell) state on the device.
//
// Reference layout (BulkVarSet, include/BulkVarSet.hpp) is array-of-structs
// per cell: x_ij at xij[(n*np + j)*nc + i].  On the device every per-cell
// quantity is its own array of length nb, so a warp touching 32 consecutive
// cells issues one coalesced load per quantity: value (n, j, i) lives at
// base[((j*nc) + i) * nb + n].  Transposition to and from the reference
// layout happens only at the C-ABI boundary.
#pragma once
#include "ocpx_common.cuh"

namespace ocpx {

struct BulkView {
    int nb;    // cells: interior, then ghost
    int nbI;   // interior cells (rows of the residual and the Jacobian)
    int np;    // phases
    int nc;    // components (incl. water)
    // static
    const double* v;
    const double* depth;
    const double* poroInit;
    // primary and secondary state
    double* P;
    double* T;         // reservoir temperature, input units (C/F)
    double* Pb;        // bubble point (black-oil)
    double* Ni;        // [nc][nb]
    double* lNi;       // [nc][nb] last time step
    double* Nt;
    double* vf;
    double* vfP;
    double* vfi;       // [nc][nb]
    double* Pj;        // [np][nb]
    double* Pc;        // [np][nb]
    double* S;         // [np][nb]
    uint8_t* phaseExist;  // [np][nb]
    double* xij;       // [np*nc][nb]
    double* rho;       // [np][nb]
    double* xi;
    double* mu;
    double* rhoP;
    double* xiP;
    double* muP;
    double* rhox;      // [np*nc][nb]
    double* xix;
    double* mux;
    double* kr;        // [np][nb]
    double* dKrdS;     // [np*np][nb]
    double* dPcdS;     // [np*np][nb]
    double* dSec_dPri; // [np*(nc+1) * (nc+1)][nb], row-major rows (S_j, x_ij) x cols (P, N_k);
                       // NULL when the flash derivatives are recomputed where they are used
    double* njhc;      // [2][nb] mole numbers of the hydrocarbon phases (label order, 0 if absent)
                       // kept by the flash for that recomputation; NULL otherwise
    double* poro;
    double* poroP;
    double* rockVp;
    // skip-stability state (SkipPSAVarset, include/AcceleratePEC.hpp:22-50)
    uint8_t* skip_flag;
    double* skip_minEig;
    double* skip_P;
    double* skip_T;
    double* skip_zi;   // [NC][nb]
    // per-cell diagnostics of the last flash
    uint32_t* status;
    int8_t* ftype;
    int32_t* iters;    // [5][nb]: SSM-stability, NR-stability, SSM-split, NR-split, RR

    OCPX_HD int idx(int k, int n) const { return k * nb + n; }
};

}  // namespace ocpx
