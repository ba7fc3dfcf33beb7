// Connection-level and row-level operations of the FIM step: two-point
// flux with phase upwinding, the residual, and the block-CSR Jacobian.
//
// Reference: IsoT_FIM::CalRes (src/IsoThermalMethod.cpp:1090-1185),
// OCPConvection01::CalFlux / AssembleMatFIM (src/OCPConvection.cpp:22-187),
// BulkAccumuTerm01::CalResFIM / CaldFdXpFIM (src/BulkAccumuModule.cpp:24-71),
// IsoT_FIM::AssembleMatBulks (src/IsoThermalMethod.cpp:1187-1269) with
// DaABpbC (src/DenseMat.cpp:61-85), OCPMatrix::NewDiag/AddDiag/NewOffDiag
// (src/OCPMatrix.cpp:92-138).
//
// Scatter-free design: every row (cell) gathers the connections incident to
// it in increasing connection order, which is the order in which the
// reference's connection loop adds into that row.  No atomics are used, and
// each row's sums are formed in the reference's order.
#pragma once
#include "bulk_view.cuh"

namespace ocpx {

struct ConnView {
    int nconn;
    const uint32_t* bId;
    const uint32_t* eId;
    const double* trans;
    // per connection results of CalFlux, SoA [k][nconn]
    uint32_t* upblock;  // [np][nconn]
    double* dP;         // [np][nconn]
    double* flux_vj;    // [np][nconn]
    double* flux_ni;    // [nc][nconn]
    // row -> incident connections, increasing connection index; entry
    // (c << 1) | side, side 0 when the row is the connection's bId
    const uint32_t* row_ptr;  // [nb+1]
    const uint32_t* row_conn;
};

// OCPConvection01::CalFlux for connection c
OCPX_HD void conn_flux(const Model& M, const BulkView& b, const ConnView& cv, int c)
{
    const int np = b.np, nc = b.nc, nconn = cv.nconn;
    const int bId = (int)cv.bId[c], eId = (int)cv.eId[c];
    const double Akd = cv.trans[c];
    const double G = M.units.gravity_factor;
    double flux[NCT_MAX];
    for (int i = 0; i < nc; i++) flux[i] = 0;
    for (int j = 0; j < np; j++) {
        const bool exb = b.phaseExist[b.idx(j, bId)] != 0;
        const bool exe = b.phaseExist[b.idx(j, eId)] != 0;
        double rho;
        if (exb && exe) rho = (b.rho[b.idx(j, bId)] + b.rho[b.idx(j, eId)]) / 2;
        else if (exb) rho = b.rho[b.idx(j, bId)];
        else if (exe) rho = b.rho[b.idx(j, eId)];
        else {
            cv.upblock[j * nconn + c] = bId;
            cv.dP[j * nconn + c] = 0;
            cv.flux_vj[j * nconn + c] = 0;
            continue;
        }
        const double dP = (b.Pj[b.idx(j, bId)] - G * rho * b.depth[bId]) - (b.Pj[b.idx(j, eId)] - G * rho * b.depth[eId]);
        const int u = dP < 0 ? eId : bId;
        cv.upblock[j * nconn + c] = u;
        cv.dP[j * nconn + c] = dP;
        if (!b.phaseExist[b.idx(j, u)]) {
            cv.flux_vj[j * nconn + c] = 0;
            continue;
        }
        const double vj = Akd * b.kr[b.idx(j, u)] / b.mu[b.idx(j, u)] * dP;
        cv.flux_vj[j * nconn + c] = vj;
        const double xiu = b.xi[b.idx(j, u)];
        for (int i = 0; i < nc; i++) flux[i] += vj * xiu * b.xij[b.idx(j * nc + i, u)];
    }
    for (int i = 0; i < nc; i++) cv.flux_ni[i * nconn + c] = flux[i];
}

// Residual of one cell (accumulation + fluxes in connection order), its
// relative norms and the per-cell maxima used by the global max reduction.
// res is cell-major [n*(nc+1) + i], already negated as the reference does.
struct RowNorm {
    double maxV; int idV;
    double maxN; int idN;
};

OCPX_HD void cell_residual(const BulkView& b, const ConnView& cv, int n, double dt, double* res,
                           double* resRelV, double* resRelN, RowNorm* rn)
{
    const int nc = b.nc, len = nc + 1, nconn = cv.nconn;
    double r[NCT_MAX + 1];
    r[0] = b.rockVp[n] - b.vf[n];
    for (int i = 0; i < nc; i++) r[i + 1] = b.Ni[b.idx(i, n)] - b.lNi[b.idx(i, n)];
    for (uint32_t k = cv.row_ptr[n]; k < cv.row_ptr[n + 1]; k++) {
        const uint32_t e = cv.row_conn[k];
        const int c = (int)(e >> 1);
        if ((e & 1u) == 0) {
            for (int i = 0; i < nc; i++) r[1 + i] += dt * cv.flux_ni[i * nconn + c];
        }
        else {
            for (int i = 0; i < nc; i++) r[1 + i] -= dt * cv.flux_ni[i * nconn + c];
        }
    }
    // relative residuals (IsoT_FIM::CalRes :1147-1167)
    double mv = 0, sv = 0, mN = 0, sN = 0;
    int iv = -1, iN = -1;
    const double vp = b.rockVp[n], Nt = b.Nt[n];
    for (int i = 0; i < len; i++) {
        const double t = fabs(r[i] / vp);
        if (mv < t) { mv = t; iv = n; }
        sv += t * t;
    }
    for (int i = 1; i < len; i++) {
        const double t = fabs(r[i] / Nt);
        if (mN < t) { mN = t; iN = n; }
        sN += t * t;
    }
    resRelV[n] = sqrt(sv);
    resRelN[n] = sqrt(sN);
    rn->maxV = mv; rn->idV = iv;
    rn->maxN = mN; rn->idN = iN;
    for (int i = 0; i < len; i++) res[(size_t)n * len + i] = -1.0 * r[i];
}

// OCPConvection01::AssembleMatFIM for one connection followed by the two
// DaABpbC products: bmat = dt * (dFdXp + dFdXs * dSec_dPri[side cell]).
// Writes bmatB (side 0) and bmatE (side 1), each ncol x ncol row-major.
template <int NCT>
OCPX_HD void conn_jac_blocks(const Model& M, const BulkView& b, const ConnView& cv, int c, double dt,
                             double* bmatB, double* bmatE)
{
    const int np = b.np, nc = b.nc, nconn = cv.nconn;
    const int ncol = nc + 1, ncol2 = np * nc + np;
    constexpr int NCOL = NCT + 1, NCOL2 = NP * NCT + NP;
    double dFdXpB[NCOL], dFdXpE[NCOL];         // column 0 only (rows 0..ncol-1)
    double dFdXsB[NCOL * NCOL2], dFdXsE[NCOL * NCOL2];
    for (int r = 0; r < ncol; r++) { dFdXpB[r] = 0; dFdXpE[r] = 0; }
    for (int k = 0; k < ncol * ncol2; k++) { dFdXsB[k] = 0; dFdXsE[k] = 0; }
    const int bId = (int)cv.bId[c], eId = (int)cv.eId[c];
    const double Akd = cv.trans[c];
    const double dGamma = M.units.gravity_factor * (b.depth[bId] - b.depth[eId]);
    for (int j = 0; j < np; j++) {
        const int u = (int)cv.upblock[j * nconn + c];
        if (!b.phaseExist[b.idx(j, u)]) continue;
        const bool up_is_b = (u == bId);
        const int d = up_is_b ? eId : bId;
        const bool exD = b.phaseExist[b.idx(j, d)] != 0;
        double* dFdXpU = up_is_b ? dFdXpB : dFdXpE;
        double* dFdXpD = up_is_b ? dFdXpE : dFdXpB;
        double* dFdXsU = up_is_b ? dFdXsB : dFdXsE;
        double* dFdXsD = up_is_b ? dFdXsE : dFdXsB;
        const double rhoWghtU = exD ? 0.5 : 1;
        const double rhoWghtD = exD ? 0.5 : 0;
        const double dP = cv.dP[j * nconn + c];
        const double xi = b.xi[b.idx(j, u)];
        const double kr = b.kr[b.idx(j, u)];
        const double mu = b.mu[b.idx(j, u)];
        const double muP = b.muP[b.idx(j, u)];
        const double xiP = b.xiP[b.idx(j, u)];
        const double rhoPu = b.rhoP[b.idx(j, u)];
        const double rhoPd = b.rhoP[b.idx(j, d)];
        const double transJ = Akd * kr / mu;
        for (int i = 0; i < nc; i++) {
            const double xij = b.xij[b.idx(j * nc + i, u)];
            const double transIJ = xij * xi * transJ;
            dFdXpB[i + 1] += transIJ;
            dFdXpE[i + 1] -= transIJ;
            double tmp = transJ * xiP * xij * dP;
            tmp += -transIJ * muP / mu * dP;
            dFdXpU[i + 1] += (tmp - transIJ * rhoWghtU * rhoPu * dGamma);
            dFdXpD[i + 1] += -transIJ * rhoWghtD * rhoPd * dGamma;
            double* rowB = dFdXsB + (i + 1) * ncol2;
            double* rowE = dFdXsE + (i + 1) * ncol2;
            double* rowU = dFdXsU + (i + 1) * ncol2;
            double* rowD = dFdXsD + (i + 1) * ncol2;
            for (int k = 0; k < np; k++) {
                rowB[k] += transIJ * b.dPcdS[b.idx(j * np + k, bId)];
                rowE[k] -= transIJ * b.dPcdS[b.idx(j * np + k, eId)];
                rowU[k] += Akd * b.dKrdS[b.idx(j * np + k, u)] / mu * xi * xij * dP;
            }
            for (int k = 0; k < nc; k++) {
                const double rhox = b.rhox[b.idx(j * nc + k, u)];
                const double xix = b.xix[b.idx(j * nc + k, u)];
                const double mux = b.mux[b.idx(j * nc + k, u)];
                double t2 = -transIJ * rhoWghtU * rhox * dGamma;
                t2 += transJ * xix * xij * dP;
                t2 += -transIJ * mux / mu * dP;
                rowU[np + j * nc + k] += t2;
                rowD[np + j * nc + k] += -transIJ * rhoWghtD * b.rhox[b.idx(j * nc + k, d)] * dGamma;
            }
            rowU[np + j * nc + i] += transJ * xi * dP;
        }
    }
    // bmat = dt * (dFdXs * dSec) + dt * dFdXp.  The reference forms the product
    // with BLAS dgemm (DaABpbC, src/DenseMat.cpp:61-85), whose rounding is
    // that of fused multiply-adds in some order; here: fused multiply-adds in
    // column order.  In the compositional model the rows of dSec_dPri for the
    // water phase's composition are identically zero (the water composition
    // is fixed, CaldXsdXpW), so their columns of dFdXs are skipped.
    const int kend = (M.mixture == 1) ? np + (np - 1) * nc : ncol2;
    for (int side = 0; side < 2; side++) {
        const double* Xs = side == 0 ? dFdXsB : dFdXsE;
        const double* Xp = side == 0 ? dFdXpB : dFdXpE;
        const int cell = side == 0 ? bId : eId;
        double* out = side == 0 ? bmatB : bmatE;
        for (int col = 0; col < ncol; col++) out[col] = dt * 0.0 + dt * (col == 0 ? Xp[0] : 0.0);
        for (int r = 1; r < ncol; r++) {
            double acc[NCOL];
#pragma unroll
            for (int col = 0; col < NCOL; col++) acc[col] = 0;
            for (int k = 0; k < kend; k++) {
                const double x = Xs[r * ncol2 + k];
                const double* ds = b.dSec_dPri + (size_t)(k * ncol) * b.nb + cell;
#pragma unroll
                for (int col = 0; col < NCOL; col++)
                    if (col < ncol) acc[col] = fma(x, ds[(size_t)col * b.nb], acc[col]);
            }
#pragma unroll
            for (int col = 0; col < NCOL; col++) {
                if (col >= ncol) break;
                const double cv0 = (col == 0) ? Xp[r] : 0.0;
                out[r * ncol + col] = dt * acc[col] + dt * cv0;
            }
        }
    }
}

// One block row of the Jacobian: the accumulation diagonal block
// (BulkAccumuTerm01::CaldFdXpFIM) plus the connection blocks, in the
// reference's order: diagonal first, then one off-diagonal block per incident
// connection in increasing connection order.
OCPX_HD void row_assemble(const BulkView& b, const ConnView& cv, int r, const double* bmat, const uint32_t* jac_rowptr,
                          double* jac_val)
{
    const int nc = b.nc, dim = nc + 1, bsize = dim * dim;
    double diag[(NCT_MAX + 1) * (NCT_MAX + 1)];
    for (int k = 0; k < bsize; k++) diag[k] = 0;
    diag[0] = b.v[r] * b.poroP[r] - b.vfP[r];
    for (int i = 0; i < nc; i++) diag[i + 1] = -b.vfi[b.idx(i, r)];
    for (int i = 1; i < dim; i++) diag[i * dim + i] = 1;
    double* out = jac_val + (size_t)jac_rowptr[r] * bsize;
    int slot = 1;
    for (uint32_t k = cv.row_ptr[r]; k < cv.row_ptr[r + 1]; k++, slot++) {
        const uint32_t e = cv.row_conn[k];
        const size_t c = e >> 1;
        const double* bB = bmat + (c * 2 + 0) * bsize;
        const double* bE = bmat + (c * 2 + 1) * bsize;
        double* off = out + (size_t)slot * bsize;
        if ((e & 1u) == 0) {
            // row is bId: AddDiag(bId, bmatB); NewOffDiag(bId, eId, bmatE)
            for (int q = 0; q < bsize; q++) diag[q] += bB[q];
            for (int q = 0; q < bsize; q++) off[q] = bE[q];
        }
        else {
            // row is eId: NewOffDiag(eId, bId, -bmatB); AddDiag(eId, -bmatE)
            for (int q = 0; q < bsize; q++) off[q] = -1.0 * bB[q];
            for (int q = 0; q < bsize; q++) diag[q] += -1.0 * bE[q];
        }
    }
    for (int q = 0; q < bsize; q++) out[q] = diag[q];
}

}  // namespace ocpx
