// The wells' part of the FIM residual and Jacobian, per perforation, on the
// device.
//
// Reference: PeacemanWell::CalTrans / CalFlux (src/WellPeaceman.cpp:365-466),
// PeacemanWellIsoT::CalResFIM (:1226-1265), AssembleMatInjFIM (:1268-1361),
// AssembleMatProdFIM (:1488-1613).  One thread per perforation: wells are few
// and their perforations fewer than the cells of one block row, so the kernel
// is small next to the bulk step.  Each thread writes its perforation's
// rates, the dQ/dP_well column, the block added to its cell's diagonal and,
// under rate control, the well-to-cell block; the host sums them per well in
// perforation order, as the reference does.  Every expression keeps the
// reference's operation order; the dQ/dXs * dSec_dPri product, which the
// reference hands to BLAS dgemm, is summed in column order here.
#include "ocpx_kernels.h"

namespace ocpx {

namespace {

constexpr int WNCOL = NCT_MAX + 1;        // nc + 1 at most
constexpr int WNCOL2 = 3 * (NCT_MAX + 1);  // np * nc + np at most (np = 3)

__global__ void k_well_perf(BulkView b, const WellPerf* __restrict__ perf, int nperf,
                            const double* __restrict__ inj_zi, const double* __restrict__ factor, double dt,
                            double* __restrict__ out_qi, double* __restrict__ out_dqw,
                            double* __restrict__ out_bb, double* __restrict__ out_wb)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nperf) return;
    const WellPerf f = perf[p];
    const int np = b.np, nc = b.nc, n = f.cell;
    const int ncol = nc + 1, ncol2 = np * nc + np;
    const double* zi = inj_zi + (size_t)f.well * nc;
    const double* fac = factor + (size_t)f.well * nc;
    double dqb[WNCOL], dqw[WNCOL], qi[WNCOL];
    double dqs[WNCOL][WNCOL2];
    for (int r = 0; r < ncol; r++) {
        dqb[r] = 0;
        dqw[r] = 0;
        for (int c = 0; c < ncol2; c++) dqs[r][c] = 0;
    }
    for (int i = 0; i < nc; i++) qi[i] = 0;
    const double Pperf = f.bhp + f.dG;  // CalPerfP
    double transINJ = 0;
    double transj[3] = {0, 0, 0};
    for (int j = 0; j < np; j++) {
        if (!b.phaseExist[b.idx(j, n)]) continue;
        transj[j] = f.WIm * b.kr[b.idx(j, n)] / b.mu[b.idx(j, n)];
        transINJ += transj[j];
    }
    if (f.type == 0) {
        // CalFlux, injector
        const double dPf = b.P[n] - Pperf;
        const double qt = transINJ * dPf;
        for (int i = 0; i < nc; i++) qi[i] = qt * f.xi_inj * zi[i];
        // AssembleMatInjFIM
        for (int j = 0; j < np; j++) {
            if (!b.phaseExist[b.idx(j, n)]) continue;
            const double mu = b.mu[b.idx(j, n)], muP = b.muP[b.idx(j, n)];
            const double dP = b.P[n] - f.bhp - f.dG;
            for (int i = 0; i < nc; i++) {
                const double transIJ = transj[j] * f.xi_inj * zi[i];
                dqb[i + 1] += transIJ * (1 - dP * muP / mu);
                dqw[i + 1] += -transIJ;
                for (int k = 0; k < np; k++)
                    dqs[i + 1][k] += f.WIm * f.xi_inj * zi[i] * b.dKrdS[b.idx(j * np + k, n)] * dP / mu;
                for (int k = 0; k < nc; k++)
                    dqs[i + 1][np + j * nc + k] += -transIJ * dP / mu * b.mux[b.idx(j * nc + k, n)];
            }
        }
    }
    else {
        for (int j = 0; j < np; j++) {
            if (!b.phaseExist[b.idx(j, n)]) continue;
            // CalFlux, producer
            const double dPf = b.Pj[b.idx(j, n)] - Pperf;
            const double qj = transj[j] * dPf;
            const double xi = b.xi[b.idx(j, n)];
            for (int i = 0; i < nc; i++) qi[i] += qj * xi * b.xij[b.idx(j * nc + i, n)];
            // AssembleMatProdFIM
            const double dP = b.Pj[b.idx(j, n)] - f.bhp - f.dG;
            const double mu = b.mu[b.idx(j, n)], muP = b.muP[b.idx(j, n)], xiP = b.xiP[b.idx(j, n)];
            for (int i = 0; i < nc; i++) {
                const double xij = b.xij[b.idx(j * nc + i, n)];
                const double transIJ = transj[j] * xi * xij;
                dqb[i + 1] += transIJ * (1 - dP * muP / mu) + dP * transj[j] * xij * xiP;
                dqw[i + 1] += -transIJ;
                for (int k = 0; k < np; k++) {
                    double tmp = f.WIm * dP / mu * xi * xij * b.dKrdS[b.idx(j * np + k, n)];
                    tmp += transIJ * b.dPcdS[b.idx(j * np + k, n)];
                    dqs[i + 1][k] += tmp;
                }
                for (int k = 0; k < nc; k++) {
                    const double tmp = dP * transj[j] * xij *
                                       (b.xix[b.idx(j * nc + k, n)] - xi / mu * b.mux[b.idx(j * nc + k, n)]);
                    dqs[i + 1][np + j * nc + k] += tmp;
                }
                dqs[i + 1][np + j * nc + i] += transj[j] * xi * dP;
            }
        }
    }
    // dQ/dXs * dSec_dPri: rows 1..nc (row 0 of dQ is zero)
    const size_t bs = (size_t)ncol * ncol;
    double* bb = out_bb + p * bs;
    double* wb = out_wb + p * bs;
    for (size_t e = 0; e < bs; e++) { bb[e] = 0; wb[e] = 0; }
    for (int r = 0; r < ncol; r++)
        for (int c = 0; c < ncol; c++) {
            double s = 0;
            for (int k = 0; k < ncol2; k++) s += dqs[r][k] * b.dSec_dPri[b.idx(k * ncol + c, n)];
            const double q = c == 0 ? dqb[r] : 0.0;
            bb[r * ncol + c] = dt * s + dt * q;
            if (f.mode == 1 && r > 0) wb[c] += fac[r - 1] * (s + q);
        }
    for (int i = 0; i < nc; i++) {
        out_qi[(size_t)p * nc + i] = qi[i];
        out_dqw[(size_t)p * nc + i] = dqw[i + 1];
    }
}

}  // namespace

cudaError_t launch_well_perf(const BulkView& b, const WellPerf* perf, int nperf, const double* inj_zi,
                             const double* factor, double dt, double* qi, double* dqw, double* bb, double* wb,
                             cudaStream_t s)
{
    if (nperf <= 0) return cudaSuccess;
    k_well_perf<<<(nperf + 63) / 64, 64, 0, s>>>(b, perf, nperf, inj_zi, factor, dt, qi, dqw, bb, wb);
    return cudaGetLastError();
}

}  // namespace ocpx
