// The wells' part of the FIM residual and Jacobian on the device.
//
// Reference: PeacemanWell::CalTrans / CalFlux (src/WellPeaceman.cpp:365-466),
// PeacemanWellIsoT::CalResFIM (:1226-1265), AssembleMatInjFIM (:1268-1361),
// AssembleMatProdFIM (:1488-1613), GetSolutionFIM (:1198-1204), called by
// IsoT_FIM::CalRes and AssembleMatWells (src/IsoThermalMethod.cpp:1272-1280)
// after the bulk rows.
//
// Per perforation (one thread each: wells are few and their perforations
// fewer than the cells of one block row) the phase transmissibilities, mole
// rates qi, dQ/dP_bulk (dqb), dQ/dP_well (dqw) and the product
// S = dQ/dXs * dSec_dPri of the perforated cell, which the reference hands to
// BLAS dgemm and which is summed in column order here.  Every other
// expression keeps the reference's operation order.
//
// Inside the Newton step (WellSys), after the bulk rows:
//   residual  each perforated cell adds qi * dt of its perforations, in well
//             then perforation order, to its component rows (on the negated
//             residual: -(R + x) == -R - x exactly), and its relative
//             residual is recomputed; each open well's row is its control
//             equation (bhp - target, or +-target rate + sum qi * factor);
//             maxWellRelRes_mol over the rate-controlled wells in well order;
//   Jacobian  each perforated cell's diagonal block gets dt*S + dt*dQdXp of
//             its perforations in order, and its row one bulk-to-well block
//             per perforation after the connection blocks; each well's row
//             holds its diagonal (the sum over its perforations) then one
//             well-to-bulk block per perforation;
//   update    bhp += u of the well's row (GetSolutionFIM).
// A cell perforated more than once gets its additions in the reference's
// order, by one thread that walks its perforations.
#include "ocpx_kernels.h"

namespace ocpx {

namespace {

constexpr int WNCOL = NCT_MAX + 1;        // nc + 1 at most
constexpr int WNCOL2 = 3 * (NCT_MAX + 1);  // np * nc + np at most (np = 3)

// qi [nc], dqb [ncol] (row 0 zero), dqw [nc], S [ncol * ncol] of one perforation
// (the perforated cell's dSec_dPri at ds[(row * ncol + col) * stride])
__device__ void well_perf_terms(const BulkView& b, const WellPerf& f, double bhp, const double* __restrict__ zi,
                                const double* ds, size_t stride, double* qi, double* dqb, double* dqw, double* S)
{
    const int np = b.np, nc = b.nc, n = f.cell;
    const int ncol = nc + 1, ncol2 = np * nc + np;
    double dqs[WNCOL][WNCOL2];
    for (int r = 0; r < ncol; r++) {
        dqb[r] = 0;
        for (int c = 0; c < ncol2; c++) dqs[r][c] = 0;
    }
    for (int i = 0; i < nc; i++) {
        qi[i] = 0;
        dqw[i] = 0;
    }
    const double Pperf = bhp + f.dG;  // CalPerfP
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
            const double dP = b.P[n] - bhp - f.dG;
            for (int i = 0; i < nc; i++) {
                const double transIJ = transj[j] * f.xi_inj * zi[i];
                dqb[i + 1] += transIJ * (1 - dP * muP / mu);
                dqw[i] += -transIJ;
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
            const double dP = b.Pj[b.idx(j, n)] - bhp - f.dG;
            const double mu = b.mu[b.idx(j, n)], muP = b.muP[b.idx(j, n)], xiP = b.xiP[b.idx(j, n)];
            for (int i = 0; i < nc; i++) {
                const double xij = b.xij[b.idx(j * nc + i, n)];
                const double transIJ = transj[j] * xi * xij;
                dqb[i + 1] += transIJ * (1 - dP * muP / mu) + dP * transj[j] * xij * xiP;
                dqw[i] += -transIJ;
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
    // dQ/dXs * dSec_dPri (row 0 of dQ is zero)
    for (int r = 0; r < ncol; r++)
        for (int c = 0; c < ncol; c++) {
            double s = 0;
            for (int k = 0; k < ncol2; k++) s += dqs[r][k] * ds[(size_t)(k * ncol + c) * stride];
            S[r * ncol + c] = s;
        }
}

// ocpx_wells_eval: the terms of each perforation, with the cell's diagonal
// addition bb = dt*S + dt*dQdXp and, under rate control, the well-to-cell
// block wb (row 0: sum_i factor_i (S + dQdXp)[i + 1])
__global__ void k_well_perf_eval(BulkView b, const WellPerf* __restrict__ perf, int nperf,
                                 const double* __restrict__ inj_zi, const double* __restrict__ factor, double dt,
                                 double* __restrict__ out_qi, double* __restrict__ out_dqw,
                                 double* __restrict__ out_bb, double* __restrict__ out_wb)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nperf) return;
    const WellPerf f = perf[p];
    const int nc = b.nc, ncol = nc + 1;
    const double* fac = factor + (size_t)f.well * nc;
    double qi[WNCOL], dqb[WNCOL], dqw[WNCOL], S[WNCOL * WNCOL];
    well_perf_terms(b, f, f.bhp, inj_zi + (size_t)f.well * nc, b.dSec_dPri + f.cell, (size_t)b.nb, qi, dqb, dqw, S);
    const size_t bs = (size_t)ncol * ncol;
    double* bb = out_bb + p * bs;
    double* wb = out_wb + p * bs;
    for (size_t e = 0; e < bs; e++) { bb[e] = 0; wb[e] = 0; }
    for (int r = 0; r < ncol; r++)
        for (int c = 0; c < ncol; c++) {
            const double s = S[r * ncol + c];
            const double q = c == 0 ? dqb[r] : 0.0;
            bb[r * ncol + c] = dt * s + dt * q;
            if (f.mode == 1 && r > 0) wb[c] += fac[r - 1] * (s + q);
        }
    for (int i = 0; i < nc; i++) {
        out_qi[(size_t)p * nc + i] = qi[i];
        out_dqw[(size_t)p * nc + i] = dqw[i];
    }
}

// ---- inside the step
__global__ void k_well_perf(BulkView b, WellSys w)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= w.nperf) return;
    const WellPerf f = w.perf[p];
    const int nc = b.nc, ncol = nc + 1;
    // the stored dSec_dPri, or the copy recomputed for the perforated cells
    const double* ds = w.dsec ? w.dsec + (size_t)w.perf_pc[p] * 3 * ncol * ncol : b.dSec_dPri + f.cell;
    const size_t stride = w.dsec ? 1 : (size_t)b.nb;
    well_perf_terms(b, f, w.bhp[f.well], w.zi + (size_t)f.well * nc, ds, stride, w.qi + (size_t)p * nc,
                    w.dqb + (size_t)p * ncol, w.dqw + (size_t)p * nc, w.S + (size_t)p * ncol * ncol);
}

// perforated cells' residual rows (before the norms are reduced)
__global__ void k_well_res_cells(BulkView b, WellSys w, double dt, double* __restrict__ res,
                                 double* __restrict__ resRelV, double* __restrict__ resRelN, RowNorm* __restrict__ rn)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= w.npc) return;
    const int n = w.pc_cell[q], nc = b.nc, len = nc + 1;
    double* r = res + (size_t)n * len;
    for (int k = w.pc_start[q]; k < w.pc_start[q + 1]; k++) {
        const int p = w.pc_perf[k];
        for (int i = 0; i < nc; i++) r[1 + i] = r[1 + i] - w.qi[(size_t)p * nc + i] * dt;
    }
    // relative residuals of the row (IsoT_FIM::CalRes :1147-1167): |-x| == |x|
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
    rn[n].maxV = mv; rn[n].idV = iv;
    rn[n].maxN = mN; rn[n].idN = iN;
}

// the wells' rows of the residual (one thread per well) and maxWellRelRes_mol
__global__ void k_well_res_rows(int nc, WellSys w, int nb, double* __restrict__ res)
{
    const int len = nc + 1;
    for (int wi = threadIdx.x; wi < w.nw; wi += blockDim.x) {
        const WellDev W = w.well[wi];
        double r;
        if (W.mode == 0) r = w.bhp[wi] - W.tar_bhp;
        else {
            // qi_lbmol: the perforations' rates summed in order (PeacemanWell::CalFlux)
            double qw[WNCOL];
            for (int i = 0; i < nc; i++) qw[i] = 0;
            for (int p = W.p0; p < W.p1; p++)
                for (int i = 0; i < nc; i++) qw[i] += w.qi[(size_t)p * nc + i];
            r = W.type == 0 ? W.tar_rate : -W.tar_rate;
            for (int i = 0; i < nc; i++) r += qw[i] * w.factor[(size_t)wi * nc + i];
        }
        double* row = res + (size_t)(nb + wi) * len;
        row[0] = -1.0 * r;
        for (int i = 1; i < len; i++) row[i] = -1.0 * 0.0;
        w.wrel[wi] = W.mode == 0 ? 0.0 : fabs(r / W.tar_rate);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0;  // res.maxWellRelRes_mol = max(res.maxWellRelRes_mol, |R_w / target|), in well order
        for (int wi = 0; wi < w.nw; wi++)
            if (w.well[wi].mode != 0) m = m < w.wrel[wi] ? w.wrel[wi] : m;
        *w.maxrel = m;
    }
}

// perforated cells' Jacobian rows: diagonal additions and bulk-to-well blocks
__global__ void k_well_jac_cells(int nc, WellSys w, double dt, const uint32_t* __restrict__ rowptr,
                                 double* __restrict__ val)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= w.npc) return;
    const int n = w.pc_cell[q], ncol = nc + 1, bs = ncol * ncol;
    double* diag = val + (size_t)rowptr[n] * bs;
    for (int k = w.pc_start[q]; k < w.pc_start[q + 1]; k++) {
        const int p = w.pc_perf[k];
        const double* S = w.S + (size_t)p * bs;
        const double* dqb = w.dqb + (size_t)p * ncol;
        // Bulk - Bulk: AddDiag(n, dt * dQ/dXs dSec + dt * dQdXpB)
        for (int r = 0; r < ncol; r++)
            for (int c = 0; c < ncol; c++) {
                const double qv = c == 0 ? dqb[r] : 0.0;
                diag[r * ncol + c] += dt * S[r * ncol + c] + dt * qv;
            }
        // Bulk - Well: NewOffDiag(n, wId, dt * dQdXpW)
        double* bw = val + (size_t)w.slot_bw[p] * bs;
        for (int e = 0; e < bs; e++) bw[e] = 0.0;
        for (int i = 0; i < nc; i++) bw[(i + 1) * ncol] = w.dqw[(size_t)p * nc + i] * dt;
    }
}

// the wells' Jacobian rows (one block per well, a thread per block entry)
__global__ void k_well_jac_rows(int nc, WellSys w, const uint32_t* __restrict__ rowptr, int nb,
                                double* __restrict__ val)
{
    const int wi = blockIdx.x;
    const int ncol = nc + 1, bs = ncol * ncol;
    const WellDev W = w.well[wi];
    double* diag = val + (size_t)rowptr[nb + wi] * bs;
    for (int e = threadIdx.x; e < bs; e += blockDim.x) {
        const int r = e / ncol, c = e % ncol;
        // Well - Well: NewDiag(wId, 0), then AddDiag per perforation
        double d = 0.0;
        for (int p = W.p0; p < W.p1; p++) {
            double add = 0.0;
            if (W.mode == 0) add = r == c ? 1.0 : 0.0;
            else if (e == 0) {
                for (int i = 0; i < nc; i++) add += w.dqw[(size_t)p * nc + i] * w.factor[(size_t)wi * nc + i];
            }
            else add = (r == c) ? 1.0 : 0.0;
            d += add;
        }
        diag[e] = d;
        // Well - Bulk: NewOffDiag(wId, n, row 0 = sum_i factor_i (dQdXpB + dQ/dXs dSec)[i + 1]) per perforation
        for (int p = W.p0; p < W.p1; p++) {
            double v = 0.0;
            if (W.mode == 1 && r == 0) {
                const double* S = w.S + (size_t)p * bs;
                const double* dqb = w.dqb + (size_t)p * ncol;
                for (int i = 0; i < nc; i++) {
                    const double qv = c == 0 ? dqb[i + 1] : 0.0;
                    v += w.factor[(size_t)wi * nc + i] * (S[(i + 1) * ncol + c] + qv);
                }
            }
            val[(size_t)w.slot_wb[p] * bs + e] = v;
        }
    }
}

// GetSolutionFIM: bhp += u of the well's row
__global__ void k_well_update(int nc, WellSys w, int nb, const double* __restrict__ u)
{
    for (int wi = threadIdx.x; wi < w.nw; wi += blockDim.x) w.bhp[wi] += u[(size_t)(nb + wi) * (nc + 1)];
}

// J^T lambda: the wells' blocks.  Perforated cells add, in order, the
// transposed well-to-bulk blocks of their perforations (column n of the well
// rows); each well's entry is its diagonal and its perforations' bulk-to-well
// blocks, transposed.
__global__ void k_well_jt_cells(int nc, WellSys w, const double* __restrict__ val, int nb,
                                const double* __restrict__ lam, double* __restrict__ out)
{
    const int dim = nc + 1, bs = dim * dim;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)w.npc * dim) return;
    const int q = (int)(t / dim), a = (int)(t % dim);
    const int n = w.pc_cell[q];
    double acc = out[(size_t)n * dim + a];
    for (int k = w.pc_start[q]; k < w.pc_start[q + 1]; k++) {
        const int p = w.pc_perf[k];
        const int wi = w.perf[p].well;
        const double* B = val + (size_t)w.slot_wb[p] * bs;
        for (int r = 0; r < dim; r++) acc += B[r * dim + a] * lam[(size_t)(nb + wi) * dim + r];
    }
    out[(size_t)n * dim + a] = acc;
}

__global__ void k_well_jt_rows(int nc, WellSys w, const uint32_t* __restrict__ rowptr, const double* __restrict__ val,
                               int nb, const double* __restrict__ lam, double* __restrict__ out)
{
    const int dim = nc + 1, bs = dim * dim;
    const int wi = blockIdx.x;
    const WellDev W = w.well[wi];
    for (int a = threadIdx.x; a < dim; a += blockDim.x) {
        const double* D = val + (size_t)rowptr[nb + wi] * bs;
        double acc = 0;
        for (int r = 0; r < dim; r++) acc += D[r * dim + a] * lam[(size_t)(nb + wi) * dim + r];
        for (int p = W.p0; p < W.p1; p++) {
            const double* B = val + (size_t)w.slot_bw[p] * bs;
            const int n = w.perf[p].cell;
            for (int r = 0; r < dim; r++) acc += B[r * dim + a] * lam[(size_t)n * dim + r];
        }
        out[(size_t)(nb + wi) * dim + a] = acc;
    }
}

}  // namespace

cudaError_t launch_well_perf(const BulkView& b, const WellPerf* perf, int nperf, const double* inj_zi,
                             const double* factor, double dt, double* qi, double* dqw, double* bb, double* wb,
                             cudaStream_t s)
{
    if (nperf <= 0) return cudaSuccess;
    k_well_perf_eval<<<(nperf + 63) / 64, 64, 0, s>>>(b, perf, nperf, inj_zi, factor, dt, qi, dqw, bb, wb);
    return cudaGetLastError();
}

cudaError_t launch_wells_res(const BulkView& b, const WellSys& w, double dt, double* res, double* resRelV,
                             double* resRelN, RowNorm* rn, cudaStream_t s)
{
    if (w.nw <= 0) return cudaSuccess;
    if (w.nperf > 0) k_well_perf<<<(w.nperf + 63) / 64, 64, 0, s>>>(b, w);
    if (w.npc > 0) k_well_res_cells<<<(w.npc + 63) / 64, 64, 0, s>>>(b, w, dt, res, resRelV, resRelN, rn);
    k_well_res_rows<<<1, 128, 0, s>>>(b.nc, w, b.nb, res);
    return cudaGetLastError();
}

cudaError_t launch_wells_jac(const BulkView& b, const WellSys& w, double dt, const uint32_t* rowptr, double* val,
                             cudaStream_t s)
{
    if (w.nw <= 0) return cudaSuccess;
    if (w.npc > 0) k_well_jac_cells<<<(w.npc + 63) / 64, 64, 0, s>>>(b.nc, w, dt, rowptr, val);
    k_well_jac_rows<<<w.nw, 128, 0, s>>>(b.nc, w, rowptr, b.nb, val);
    return cudaGetLastError();
}

cudaError_t launch_wells_update(const BulkView& b, const WellSys& w, const double* u, cudaStream_t s)
{
    if (w.nw <= 0) return cudaSuccess;
    k_well_update<<<1, 128, 0, s>>>(b.nc, w, b.nb, u);
    return cudaGetLastError();
}

cudaError_t launch_wells_jt(const BulkView& b, const WellSys& w, const uint32_t* rowptr, const double* val,
                            const double* lam, double* out, cudaStream_t s)
{
    if (w.nw <= 0) return cudaSuccess;
    const long long n = (long long)w.npc * (b.nc + 1);
    if (n > 0) k_well_jt_cells<<<(int)((n + 127) / 128), 128, 0, s>>>(b.nc, w, val, b.nb, lam, out);
    k_well_jt_rows<<<w.nw, 32, 0, s>>>(b.nc, w, rowptr, val, b.nb, lam, out);
    return cudaGetLastError();
}

}  // namespace ocpx
