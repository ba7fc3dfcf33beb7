// Adjoint of the FIM bulk residual: vector-Jacobian products with a vector
// lambda of residual size.  The reference has no adjoint; these are the
// transposes of its own residual (IsoT_FIM::CalRes, src/IsoThermalMethod.cpp:
// 1090-1185) and Jacobian (AssembleMatBulks, :1187-1269).
//
//  * J^T lambda from the assembled block-CSR Jacobian: cell n gathers the
//    blocks of column n (its diagonal block and, for each incident
//    connection, the neighbour's off-diagonal block in that connection's
//    slot), with no atomics.
//  * dR/dT_c: the connection flux of OCPConvection01::CalFlux
//    (src/OCPConvection.cpp:22-79) is Akd * kr/mu * dP * xi * x_ij summed over
//    the upwind phases, linear in the transmissibility Akd; the bulk residual
//    is R_b = -(... + dt F), R_e = -(... - dt F), so
//    (dR/dT_c)^T lambda = dt * sum_i F_i(Akd = 1) (lambda_e,i - lambda_b,i).
//  * dR/dporoInit_n: only the volume balance R_n,0 = vf - v poro(P) depends on
//    it, with poro = poroInit (1 + (cp1 + cp2/2 dP) dP)
//    (OCPRockIsoT_Linear::CalPoro, src/OCPRock.cpp:19-24).
#pragma once
#include "conn_ops.cuh"

namespace ocpx {

// out[n*dim + a] = sum over blocks B of column n of sum_r B[r][a] lam[row(B)*dim + r]
OCPX_HD void jt_lambda_entry(const BulkView& b, const ConnView& cv, const uint32_t* rowptr, const double* val,
                             const uint32_t* slot, const double* lam, double* out, int n, int a)
{
    const int dim = b.nc + 1, bsize = dim * dim, nconn = cv.nconn;
    const double* diag = val + (size_t)rowptr[n] * bsize;
    double acc = 0;
    for (int r = 0; r < dim; r++) acc += diag[r * dim + a] * lam[(size_t)n * dim + r];
    for (uint32_t k = cv.row_ptr[n]; k < cv.row_ptr[n + 1]; k++) {
        const uint32_t e = cv.row_conn[k];
        const uint32_t c = e >> 1, side = e & 1u;
        // the neighbour's row holds the block of column n in the slot of connection c
        const uint32_t other = side ? cv.bId[c] : cv.eId[c];
        const uint32_t blk = slot[(size_t)(1u - side) * nconn + c];
        const double* B = val + (size_t)blk * bsize;
        for (int r = 0; r < dim; r++) acc += B[r * dim + a] * lam[(size_t)other * dim + r];
    }
    out[(size_t)n * dim + a] = acc;
}

// (dR/dT_c)^T lambda
OCPX_HD double vjp_trans_conn(const BulkView& b, const ConnView& cv, double dt, const double* lam, int c)
{
    const int np = b.np, nc = b.nc, nconn = cv.nconn, dim = nc + 1;
    const int bId = (int)cv.bId[c], eId = (int)cv.eId[c];
    double acc = 0;
    for (int j = 0; j < np; j++) {
        const bool exb = b.phaseExist[b.idx(j, bId)] != 0;
        const bool exe = b.phaseExist[b.idx(j, eId)] != 0;
        if (!exb && !exe) continue;
        const int u = (int)cv.upblock[j * nconn + c];
        if (!b.phaseExist[b.idx(j, u)]) continue;
        const double dP = cv.dP[j * nconn + c];
        const double v1 = b.kr[b.idx(j, u)] / b.mu[b.idx(j, u)] * dP;  // phase flux per unit transmissibility
        const double xiu = b.xi[b.idx(j, u)];
        for (int i = 0; i < nc; i++)
            acc += v1 * xiu * b.xij[b.idx(j * nc + i, u)] * (lam[(size_t)eId * dim + 1 + i] - lam[(size_t)bId * dim + 1 + i]);
    }
    return dt * acc;
}

// (dR/dporoInit_n)^T lambda
OCPX_HD double vjp_poro_cell(const Model& M, const BulkView& b, const double* lam, int n)
{
    const double dP = b.P[n] - M.rock.Pref;
    const double dporo = 1 + (M.rock.cp1 + M.rock.cp2 / 2 * dP) * dP;
    return -lam[(size_t)n * (b.nc + 1)] * b.v[n] * dporo;
}

}  // namespace ocpx
