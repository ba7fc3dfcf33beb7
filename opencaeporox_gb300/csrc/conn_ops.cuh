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
//
// The reference fills the dense ncol x ncol2 matrix dFdXs and multiplies it
// by dSec_dPri with dgemm.  Its rows have a fixed structure: phase j adds
// x_ij * v_j to row i + 1 (component i), where the row vector v_j does not
// depend on i, plus one diagonal entry transJ*xi*dP in the upwind side's
// column of (j, i).  So
//   (dFdXs * dSec)[i+1] = sum_j x_ij * (v_j * dSec) + sum_j e_j * dSec[np+j*nc+i]
// and only np vectors W_j = v_j * dSec of length ncol are formed per side,
// from the np saturation rows and the nc composition rows of phase j.  Each
// entry is the same sum of products as the reference's, grouped by phase
// (rounding differs from dgemm's, as any dgemm blocking does).  Everything
// stays in registers.  Column 0 of dFdXp is accumulated phase by phase with
// the reference's operations.  In the compositional model the rows of
// dSec_dPri for the water phase's composition are identically zero (the
// water composition is fixed, CaldXsdXpW), so they are skipped.
// the per-phase quantities of a connection that both sides' blocks use
struct ConnPhase {
    int bId, eId, jcomp_end;
    double Akd, dGamma;
    int up[NP];
    bool act[NP];
    double transJ[NP], xiU[NP], dPj[NP], muU[NP], wU[NP], wD[NP], muP[NP], xiP[NP], rhoPu[NP], rhoPd[NP];
};

OCPX_HD void conn_phase(const Model& M, const BulkView& b, const ConnView& cv, int c, ConnPhase& q)
{
    const int np = b.np, nconn = cv.nconn;
    q.bId = (int)cv.bId[c];
    q.eId = (int)cv.eId[c];
    const int bId = q.bId, eId = q.eId;
    q.Akd = cv.trans[c];
    q.dGamma = M.units.gravity_factor * (b.depth[bId] - b.depth[eId]);
    q.jcomp_end = (M.mixture == 1) ? np - 1 : np;  // phases whose composition rows of dSec are nonzero
#pragma unroll
    for (int j = 0; j < NP; j++) {
        const int u = j < np ? (int)cv.upblock[j * nconn + c] : bId;
        q.up[j] = u;
        q.act[j] = j < np && b.phaseExist[b.idx(j, u)] != 0;
        q.transJ[j] = 0; q.xiU[j] = 0; q.dPj[j] = 0; q.muU[j] = 1; q.wU[j] = 0; q.wD[j] = 0;
        q.muP[j] = 0; q.xiP[j] = 0; q.rhoPu[j] = 0; q.rhoPd[j] = 0;
        if (!q.act[j]) continue;
        const int d = (u == bId) ? eId : bId;
        const bool exD = b.phaseExist[b.idx(j, d)] != 0;
        q.wU[j] = exD ? 0.5 : 1;
        q.wD[j] = exD ? 0.5 : 0;
        q.dPj[j] = cv.dP[j * nconn + c];
        q.xiU[j] = b.xi[b.idx(j, u)];
        q.muU[j] = b.mu[b.idx(j, u)];
        q.transJ[j] = q.Akd * b.kr[b.idx(j, u)] / q.muU[j];
        q.muP[j] = b.muP[b.idx(j, u)];
        q.xiP[j] = b.xiP[b.idx(j, u)];
        q.rhoPu[j] = b.rhoP[b.idx(j, u)];
        q.rhoPd[j] = b.rhoP[b.idx(j, d)];
    }
}

// The block of one side (0: bId, 1: eId) of a connection, with the side
// cell's dSec_dPri at ds[(k * ncol + col) * stride] (the stored SoA rows, or
// a recomputed copy).
template <int NCT>
OCPX_HD void conn_jac_side(const BulkView& b, const ConnPhase& q, int side, const double* ds, size_t stride,
                           double dt, double* out)
{
    const int np = b.np, nc = b.nc;
    const int ncol = nc + 1;
    constexpr int NCOL = NCT + 1;
    const int cell = side == 0 ? q.bId : q.eId;
    const double sgn = side == 0 ? 1.0 : -1.0;
    const double Akd = q.Akd, dGamma = q.dGamma;
    const int jcomp_end = q.jcomp_end;
    double W[NP][NCOL];
#pragma unroll
    for (int j = 0; j < NP; j++) {
#pragma unroll
        for (int col = 0; col < NCOL; col++) W[j][col] = 0;
        if (!q.act[j]) continue;
        const int u = q.up[j];
        const bool isU = (u == cell);
        const double xt = q.xiU[j] * q.transJ[j];
        // saturation columns: sgn*xi*transJ*dPcdS(side cell) [+ Akd*dKrdS(U)/mu*xi*dP on the upwind side]
        for (int k = 0; k < np; k++) {
            double a = sgn * xt * b.dPcdS[b.idx(j * np + k, cell)];
            if (isU) a += Akd * b.dKrdS[b.idx(j * np + k, u)] / q.muU[j] * q.xiU[j] * q.dPj[j];
#pragma unroll
            for (int col = 0; col < NCOL; col++)
                if (col < ncol) W[j][col] = fma(a, ds[(size_t)(k * ncol + col) * stride], W[j][col]);
        }
        if (j >= jcomp_end) continue;
        // composition columns of phase j
        for (int m = 0; m < nc; m++) {
            double g;
            if (isU) {
                const double rhox = b.rhox[b.idx(j * nc + m, u)];
                const double xix = b.xix[b.idx(j * nc + m, u)];
                const double mux = b.mux[b.idx(j * nc + m, u)];
                g = -xt * q.wU[j] * rhox * dGamma;
                g += q.transJ[j] * xix * q.dPj[j];
                g += -xt * mux / q.muU[j] * q.dPj[j];
            }
            else {
                if (q.wD[j] == 0) continue;
                g = -xt * q.wD[j] * b.rhox[b.idx(j * nc + m, cell)] * dGamma;
            }
            const int k = np + j * nc + m;
#pragma unroll
            for (int col = 0; col < NCOL; col++)
                if (col < ncol) W[j][col] = fma(g, ds[(size_t)(k * ncol + col) * stride], W[j][col]);
        }
    }
    // row 0 has no flux term: dt * 0 + dt * 0
    for (int col = 0; col < ncol; col++) out[col] = dt * 0.0 + dt * 0.0;
    for (int i = 0; i < nc; i++) {
        double acc[NCOL];
#pragma unroll
        for (int col = 0; col < NCOL; col++) acc[col] = 0;
        double xp = 0;  // dFdXp[i + 1][0] of this side
#pragma unroll
        for (int j = 0; j < NP; j++) {
            if (!q.act[j]) continue;
            const double xij = b.xij[b.idx(j * nc + i, q.up[j])];
            const double transIJ = xij * q.xiU[j] * q.transJ[j];
            xp += sgn * transIJ;
            if (q.up[j] == cell) {
                double tmp = q.transJ[j] * q.xiP[j] * xij * q.dPj[j];
                tmp += -transIJ * q.muP[j] / q.muU[j] * q.dPj[j];
                xp += (tmp - transIJ * q.wU[j] * q.rhoPu[j] * dGamma);
            }
            else {
                xp += -transIJ * q.wD[j] * q.rhoPd[j] * dGamma;
            }
#pragma unroll
            for (int col = 0; col < NCOL; col++)
                if (col < ncol) acc[col] = fma(xij, W[j][col], acc[col]);
            if (q.up[j] == cell && j < jcomp_end) {
                const double e = q.transJ[j] * q.xiU[j] * q.dPj[j];
                const int k = np + j * nc + i;
#pragma unroll
                for (int col = 0; col < NCOL; col++)
                    if (col < ncol) acc[col] = fma(e, ds[(size_t)(k * ncol + col) * stride], acc[col]);
            }
        }
#pragma unroll
        for (int col = 0; col < NCOL; col++) {
            if (col >= ncol) break;
            const double cv0 = (col == 0) ? xp : 0.0;
            out[(i + 1) * ncol + col] = dt * acc[col] + dt * cv0;
        }
    }
}

template <int NCT>
OCPX_HD void conn_jac_blocks(const Model& M, const BulkView& b, const ConnView& cv, int c, double dt,
                             double* bmatB, double* bmatE)
{
    ConnPhase q;
    conn_phase(M, b, cv, c, q);
    const size_t nb = (size_t)b.nb;
    conn_jac_side<NCT>(b, q, 0, b.dSec_dPri + q.bId, nb, dt, bmatB);
    conn_jac_side<NCT>(b, q, 1, b.dSec_dPri + q.eId, nb, dt, bmatE);
}

// One block row of the Jacobian: the accumulation diagonal block
// (BulkAccumuTerm01::CaldFdXpFIM) plus the connection blocks, in the
// reference's order: diagonal first, then one off-diagonal block per incident
// connection in increasing connection order.  One warp per row: lane `lane`
// owns the block entries q = lane, lane + 32, ...; each entry's sum is formed
// in the same order as a single thread would, and every load of a
// connection block and store of a row block is contiguous across the warp.
OCPX_HD void row_assemble_warp(const BulkView& b, const ConnView& cv, int r, const double* bmat,
                               const uint32_t* jac_rowptr, double* jac_val, int lane)
{
    constexpr int QPL = ((NCT_MAX + 1) * (NCT_MAX + 1) + 31) / 32;
    const int nc = b.nc, dim = nc + 1, bsize = dim * dim;
    const double d0 = b.v[r] * b.poroP[r] - b.vfP[r];
    double diag[QPL];
#pragma unroll
    for (int t = 0; t < QPL; t++) {
        const int q = lane + 32 * t;
        double x = 0;
        if (q == 0) x = d0;
        else if (q < dim) x = -b.vfi[b.idx(q - 1, r)];
        else if (q < bsize && q % dim == q / dim) x = 1;
        diag[t] = x;
    }
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
#pragma unroll
            for (int t = 0; t < QPL; t++) {
                const int q = lane + 32 * t;
                if (q < bsize) { diag[t] += bB[q]; off[q] = bE[q]; }
            }
        }
        else {
            // row is eId: NewOffDiag(eId, bId, -bmatB); AddDiag(eId, -bmatE)
#pragma unroll
            for (int t = 0; t < QPL; t++) {
                const int q = lane + 32 * t;
                if (q < bsize) { off[q] = -1.0 * bB[q]; diag[t] += -1.0 * bE[q]; }
            }
        }
    }
#pragma unroll
    for (int t = 0; t < QPL; t++) {
        const int q = lane + 32 * t;
        if (q < bsize) out[q] = diag[t];
    }
}

}  // namespace ocpx
