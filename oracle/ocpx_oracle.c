/*
 * ocpx_oracle.c -- CPU restatement of OpenCAEPoroX's FIM Newton-step path.
 *
 * TEST INFRASTRUCTURE ONLY (see ocpx_oracle.h).  Straight C in the
 * reference's data layout and loop structure, including its recomputation of
 * EoS invariants on every call, so it is also a faithful CPU cost baseline.
 * Cell loops run on all host threads with OpenMP (each thread keeps its own
 * flash workspace, as the reference keeps one per mixture object).
 * Build: cc -O2 -ffp-contract=off -fopenmp -shared -fPIC (oracle/build.py).
 */
#include "ocpx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NCX 16        /* max hydrocarbon components */
#define NPH 3         /* phases o, g, w */
#define D1 2.41421356237    /* include/OCPEoS.hpp:111 */
#define D2 (-0.41421356237) /* include/OCPEoS.hpp:112 */
#define PI_ 3.141592653     /* include/OCPConst.hpp:32 */
#define TINY_ 1E-8          /* include/OCPConst.hpp:30 */

typedef struct { int nrow, ncol; double* d; } tab_t; /* column-major like OCPTable::data */

struct oc_model {
    int mixture, nc, NC;
    double G, darcy, R, conv1, conv3, conv4;
    double pref, cp1, cp2;
    tab_t swof, sgof, pvtw, pvco, pvdg;
    double rho_o, rho_g, rho_w, vo, vg, vw;
    double Tc[NCX], Pc[NCX], Vc[NCX], MW[NCX], OA[NCX], OB[NCX], acf[NCX], BIC[NCX * NCX], Vsh[NCX];
    double coef[5], Vcvis[NCX], sqrtMWC[NCX], auxB[NCX];
    /* flash controls (OCPPhaseEquilibrium::Setup, src/OCPPhaseEquilibrium.cpp:45-64) */
    int ssta_it; double ssta_tol2, ssta_eYt, ssta_Ktol, ssta_dYtol;
    int nsta_it; double nsta_tol;
    int ssp_it; double ssp_tol2;
    int nsp_it; double nsp_tol;
    int rr_it; double rr_tol;
    int skip;
};

static double sgn(double d) { return d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0); } /* signD, src/UtilMath.cpp:84 */
static double dlt(int i, int j) { return i == j ? 1.0 : 0.0; }               /* delta, src/UtilMath.cpp:97 */

static tab_t tab_copy(const ocpx_table* t)
{
    tab_t o = {t->nrow, t->ncol, NULL};
    if (t->nrow > 0) {
        o.d = (double*)malloc(sizeof(double) * t->nrow * t->ncol);
        memcpy(o.d, t->data, sizeof(double) * t->nrow * t->ncol);
    }
    return o;
}

/* OCPTable::Eval_All (src/OCPTable.cpp:26-64) -- linear scan from the start. */
static void tab_eval_all(const tab_t* t, int j, double val, double* out, double* slope)
{
    const double* x = t->d + j * t->nrow;
    int r;
    if (val < x[0] || val >= x[t->nrow - 1]) {
        const int e = val < x[0] ? 0 : t->nrow - 1;
        for (int k = 0; k < t->ncol; k++) {
            if (slope) slope[k] = 0;
            out[k] = t->d[k * t->nrow + e];
        }
        return;
    }
    for (r = 0; r + 1 < t->nrow; r++)
        if (val < x[r + 1]) break;
    for (int k = 0; k < t->ncol; k++) {
        const double* c = t->d + k * t->nrow;
        const double s = (c[r + 1] - c[r]) / (x[r + 1] - x[r]);
        if (slope) slope[k] = s;
        out[k] = c[r] + s * (val - x[r]);
    }
}
/* OCPTable::Eval (src/OCPTable.cpp:232-257) */
static double tab_eval(const tab_t* t, int j, double val, int dj)
{
    double out[8];
    tab_eval_all(t, j, val, out, NULL);
    return out[dj];
}
/* OCPTable::GetCloseRow (src/OCPTable.cpp:312-345) */
static int tab_close(const tab_t* t, int j, double val)
{
    const double* x = t->d + j * t->nrow;
    if (val < x[0]) return 0;
    if (val >= x[t->nrow - 1]) return t->nrow - 1;
    int r = 0;
    while (r + 1 < t->nrow && !(val < x[r + 1])) r++;
    return ((val - x[r]) > (x[r + 1] - val)) ? r + 1 : r;
}

oc_model* oc_create(const ocpx_model_desc* md)
{
    oc_model* m = (oc_model*)calloc(1, sizeof(oc_model));
    m->mixture = md->mixture;
    m->nc = md->nc;
    m->NC = md->mixture == 1 ? md->nc - 1 : 0;
    m->G = md->gravity_factor; m->darcy = md->conv_darcy; m->R = md->gas_constant;
    m->conv1 = md->conv1; m->conv3 = md->conv3; m->conv4 = md->conv4;
    m->pref = md->rock_pref; m->cp1 = md->rock_cp1; m->cp2 = md->rock_cp2;
    m->swof = tab_copy(&md->swof); m->sgof = tab_copy(&md->sgof); m->pvtw = tab_copy(&md->pvtw);
    m->pvco = tab_copy(&md->pvco); m->pvdg = tab_copy(&md->pvdg);
    m->rho_o = md->std_rho_o; m->rho_g = md->std_rho_g; m->rho_w = md->std_rho_w;
    m->vo = md->std_vo; m->vg = md->std_vg; m->vw = md->std_vw;
    if (m->mixture == 1) {
        const int NC = m->NC;
        for (int i = 0; i < NC; i++) {
            m->Tc[i] = md->Tc[i]; m->Pc[i] = md->Pc[i]; m->Vc[i] = md->Vc[i]; m->MW[i] = md->MW[i];
            m->OA[i] = md->OmegaA[i]; m->OB[i] = md->OmegaB[i]; m->acf[i] = md->acf[i];
            m->Vsh[i] = md->Vshift[i]; m->Vcvis[i] = md->Vcvis[i];
            for (int k = 0; k < NC; k++) m->BIC[i * NC + k] = md->BIC[i * NC + k];
            /* ViscosityMethod03 constructor (src/OCPFuncPVT.cpp:415-460) */
            m->sqrtMWC[i] = sqrt(m->MW[i]);
            m->auxB[i] = 5.4402 * pow(m->Tc[i], 1.0 / 6) / pow(m->Pc[i], 2.0 / 3);
        }
        for (int k = 0; k < 5; k++) m->coef[k] = md->lbc_coef[k];
        const double* f = md->flash_ctrl;
        m->ssta_it = (int)f[0]; m->ssta_tol2 = f[1] * f[1]; m->ssta_eYt = f[2]; m->ssta_Ktol = f[3];
        m->ssta_dYtol = f[4]; m->nsta_it = (int)f[5]; m->nsta_tol = f[6]; m->ssp_it = (int)f[7];
        m->ssp_tol2 = f[8] * f[8]; m->nsp_it = (int)f[9]; m->nsp_tol = f[10]; m->rr_it = (int)f[11];
        m->rr_tol = f[12]; m->skip = md->skip_psa;
    }
    return m;
}

void oc_destroy(oc_model* m)
{
    if (!m) return;
    free(m->swof.d); free(m->sgof.d); free(m->pvtw.d); free(m->pvco.d); free(m->pvdg.d);
    free(m);
}

/* ===================================================================== EoS */
/* EoS_PR (src/OCPEoS.cpp:19-414) with its per-call scratch */
typedef struct {
    const oc_model* m;
    int nc;
    double Ai[NCX], Bi[NCX], Aj, Bj, Zj, Z[3];
    double Ax[NCX], Bx[NCX], Zx[NCX], An[NCX], Bn[NCX], Zn[NCX], Ap, Bp, Zp;
} eos_t;

/* NTcubicroot (src/UtilMath.cpp:56-80) */
static void nt_cubicroot(double* root, double a, double b, double c)
{
    double e = *root * (*root * (*root + a) + b) + c, df, iter = 0, optroot = *root, opte = fabs(e);
    while (fabs(e) > 1E-8) {
        df = *root * (3 * *root + 2 * a) + b;
        *root = *root - e / df;
        iter++;
        if (iter > 10) break;
        e = *root * (*root * (*root + a) + b) + c;
        if (fabs(e) <= opte) { opte = fabs(e); optroot = *root; }
    }
    *root = optroot;
}

/* CubicRoot (src/UtilMath.cpp:15-53) */
static int cubic_root(double a, double b, double c, double* z)
{
    double Q = (a * a - 3 * b) / 9;
    double R = (2 * a * a * a - 9 * a * b + 27 * c) / 54;
    double Q3 = Q * Q * Q;
    double M = R * R - Q3;
    if (M <= 0) {
        double theta = acos(R / sqrt(Q3));
        z[0] = -2 * sqrt(Q) * cos(theta / 3) - a / 3;
        z[1] = -2 * sqrt(Q) * cos((theta + 2 * PI_) / 3) - a / 3;
        z[2] = -2 * sqrt(Q) * cos((theta - 2 * PI_) / 3) - a / 3;
        nt_cubicroot(&z[0], a, b, c);
        nt_cubicroot(&z[1], a, b, c);
        nt_cubicroot(&z[2], a, b, c);
        for (int i = 0; i < 3; i++)  /* sort(z.begin(), z.end()) */
            for (int j = i + 1; j < 3; j++)
                if (z[j] < z[i]) { double t = z[i]; z[i] = z[j]; z[j] = t; }
        return 3;
    }
    double tmp1 = -R + sqrt(M);
    double tmp2 = R + sqrt(M);
    double S = sgn(tmp1) * pow(fabs(tmp1), 1.0 / 3);
    double T = -sgn(tmp2) * pow(fabs(tmp2), 1.0 / 3);
    z[0] = S + T - a / 3;
    nt_cubicroot(&z[0], a, b, c);
    return 1;
}

/* CalAiBi (:68-84) */
static void eos_aibi(eos_t* e, double P, double T)
{
    const oc_model* m = e->m;
    for (int i = 0; i < e->nc; i++) {
        double mwi;
        if (m->acf[i] <= 0.49) mwi = 0.37464 + 1.54226 * m->acf[i] - 0.26992 * pow(m->acf[i], 2);
        else mwi = 0.379642 + 1.48503 * m->acf[i] - 0.164423 * pow(m->acf[i], 2) + 0.016667 * pow(m->acf[i], 3);
        double Pri = P / m->Pc[i], Tri = T / m->Tc[i];
        e->Ai[i] = m->OA[i] * Pri / pow(Tri, 2) * pow((1 + mwi * (1 - sqrt(Tri))), 2);
        e->Bi[i] = m->OB[i] * Pri / Tri;
    }
}
/* CalAjBj (:87-99) */
static void eos_ajbj(eos_t* e, const double* x)
{
    const int nc = e->nc;
    const double* BIC = e->m->BIC;
    e->Aj = 0;
    e->Bj = 0;
    for (int i1 = 0; i1 < nc; i1++) {
        e->Bj += e->Bi[i1] * x[i1];
        e->Aj += x[i1] * x[i1] * e->Ai[i1] * (1 - BIC[i1 * nc + i1]);
        for (int i2 = 0; i2 < i1; i2++)
            e->Aj += 2 * x[i1] * x[i2] * sqrt(e->Ai[i1] * e->Ai[i2]) * (1 - BIC[i1 * nc + i2]);
    }
}
/* CalZj (:102-124) */
static void eos_zj(eos_t* e)
{
    const double Aj = e->Aj, Bj = e->Bj;
    const double a = (D1 + D2 - 1) * Bj - 1;
    const double b = (Aj + D1 * D2 * Bj * Bj - (D1 + D2) * Bj * (Bj + 1));
    const double c = -(Aj * Bj + D1 * D2 * Bj * Bj * (Bj + 1));
    if (cubic_root(a, b, c, e->Z) == 1) {
        e->Zj = e->Z[0];
    }
    else {
        double zj1 = e->Z[0], zj2 = e->Z[2];
        double dG = (zj2 - zj1) + log((zj1 - Bj) / (zj2 - Bj)) -
                    Aj / (Bj * (D2 - D1)) * log((zj1 + D1 * Bj) * (zj2 + D2 * Bj) / ((zj1 + D2 * Bj) * (zj2 + D1 * Bj)));
        e->Zj = dG > 0 ? zj1 : zj2;
    }
}
static void eos_ajbjzj(eos_t* e, double P, double T, const double* x)
{
    eos_aibi(e, P, T);
    eos_ajbj(e, x);
    eos_zj(e);
}
#define ZNUM(e) ((e->Aj + (D1 * D2) * (3 * e->Bj * e->Bj + 2 * e->Bj)) + ((D1 + D2) * (2 * e->Bj + 1) - 2 * (D1 * D2) * e->Bj) * e->Zj - ((D1 + D2) - 1) * e->Zj * e->Zj)
#define ZDEN(e) (3 * e->Zj * e->Zj + 2 * (((D1 + D2) - 1) * e->Bj - 1) * e->Zj + (e->Aj + (D1 * D2) * e->Bj * e->Bj - (D1 + D2) * e->Bj * (e->Bj + 1)))
/* CalAxBxZx (:127-143) */
static void eos_axbxzx(eos_t* e, const double* x)
{
    const int nc = e->nc;
    const double* BIC = e->m->BIC;
    for (int i = 0; i < nc; i++) e->Bx[i] = e->Bi[i];
    for (int i = 0; i < nc; i++) {
        double tmp = 0;
        for (int k = 0; k < nc; k++) tmp += x[k] * (1 - BIC[i * nc + k]) * sqrt(e->Ai[i] * e->Ai[k]);
        e->Ax[i] = 2 * tmp;
        e->Zx[i] = ((e->Bj - e->Zj) * e->Ax[i] + ZNUM(e) * e->Bx[i]) / ZDEN(e);
    }
}
/* CalAnBnZn (:146-161) */
static void eos_anbnzn(eos_t* e, const double* x, double nt)
{
    const int nc = e->nc;
    const double* BIC = e->m->BIC;
    for (int i = 0; i < nc; i++) {
        double tmp = 0;
        for (int k = 0; k < nc; k++) tmp += (1 - BIC[i * nc + k]) * sqrt(e->Ai[i] * e->Ai[k]) * x[k];
        e->An[i] = 2 / nt * (tmp - e->Aj);
        e->Bn[i] = 1 / nt * (e->Bi[i] - e->Bj);
        e->Zn[i] = ((e->Bj - e->Zj) * e->An[i] + ZNUM(e) * e->Bn[i]) / ZDEN(e);
    }
}
/* CalApBpZp (:164-173) */
static void eos_apbpzp(eos_t* e, double P)
{
    e->Ap = e->Aj / P;
    e->Bp = e->Bj / P;
    e->Zp = ((e->Bj - e->Zj) * e->Ap + ZNUM(e) * e->Bp) / ZDEN(e);
}
/* CalFugPhi (:199-214) / CalFug (:183-196) */
static void eos_fugphi(eos_t* e, double P, double T, const double* x, double* fug, double* phi)
{
    const int nc = e->nc;
    const double* BIC = e->m->BIC;
    eos_ajbjzj(e, P, T, x);
    const double Aj = e->Aj, Bj = e->Bj, Zj = e->Zj;
    for (int i = 0; i < nc; i++) {
        double tmp = 0;
        for (int k = 0; k < nc; k++) tmp += 2 * (1 - BIC[i * nc + k]) * sqrt(e->Ai[i] * e->Ai[k]) * x[k];
        double ph = exp(e->Bi[i] / Bj * (Zj - 1) - log(Zj - Bj) -
                        Aj / (D1 - D2) / Bj * (tmp / Aj - e->Bi[i] / Bj) * log((Zj + D1 * Bj) / (Zj + D2 * Bj)));
        if (phi) phi[i] = ph;
        fug[i] = ph * x[i] * P;
    }
}
/* CalLnFugX (:217-251) */
static void eos_lnfugx(eos_t* e, double P, double T, const double* x, double* out)
{
    const int nc = e->nc;
    const double* BIC = e->m->BIC;
    eos_ajbjzj(e, P, T, x);
    eos_axbxzx(e, x);
    const double Aj = e->Aj, Bj = e->Bj, Zj = e->Zj;
    double G = (Zj + D1 * Bj) / (Zj + D2 * Bj);
    for (int i = 0; i < nc; i++) {
        double C = x[i] * P / (Zj - Bj);
        double E = -Aj / ((D1 - D2) * Bj) * (e->Ax[i] / Aj - e->Bx[i] / Bj);
        for (int k = 0; k < nc; k++) {
            double aik = (1 - BIC[i * nc + k]) * sqrt(e->Ai[i] * e->Ai[k]);
            double Cxk = ((Zj - Bj) * dlt(i, k) - x[i] * (e->Zx[k] - e->Bx[k])) * P / ((Zj - Bj) * (Zj - Bj));
            double Dxk = e->Bx[i] / Bj * (e->Zx[k] - e->Bx[k] * (Zj - 1) / Bj);
            double Exk = (2 * (Aj / Bj * e->Bx[k] * e->Bx[i] + Bj * aik) - e->Ax[i] * e->Bx[k] - e->Ax[k] * e->Bi[i]) / (Bj * Bj);
            Exk /= -(D1 - D2);
            double Gxk = (D1 - D2) / (Zj + D2 * Bj) / (Zj + D2 * Bj) * (Zj * e->Bx[k] - e->Zx[k] * Bj);
            out[i * nc + k] = 1 / C * Cxk + Dxk + Exk * log(G) + E / G * Gxk;
        }
    }
}
/* CalLnFugN (:254-300) when phi == 0, CalLnPhiN (:343-382) when phi == 1 */
static void eos_lnn(eos_t* e, double P, double T, const double* x, double nt, double* out, int phi)
{
    const int nc = e->nc;
    const double* BIC = e->m->BIC;
    eos_ajbjzj(e, P, T, x);
    eos_anbnzn(e, x, nt);
    const double Aj = e->Aj, Bj = e->Bj, Zj = e->Zj;
    double G = (Zj + D1 * Bj) / (Zj + D2 * Bj);
    for (int i = 0; i < nc; i++) {
        double C = phi ? 1 / (Zj - Bj) : x[i] * P / (Zj - Bj);
        double tmp = 0;
        for (int k = 0; k < nc; k++) tmp += (1 - BIC[i * nc + k]) * sqrt(e->Ai[i] * e->Ai[k]) * x[k];
        double E = -Aj / ((D1 - D2) * Bj) * (2 * tmp / Aj - e->Bi[i] / Bj);
        for (int k = 0; k <= i; k++) {
            double aik = (1 - BIC[i * nc + k]) * sqrt(e->Ai[i] * e->Ai[k]);
            double Cnk = phi ? (e->Bn[k] - e->Zn[k]) / ((Zj - Bj) * (Zj - Bj))
                             : P / (Zj - Bj) / (Zj - Bj) * ((Zj - Bj) / nt * (dlt(i, k) - x[i]) - x[i] * (e->Zn[k] - e->Bn[k]));
            double Dnk = e->Bi[i] / Bj * (e->Zn[k] - (e->Bi[k] - Bj) * (Zj - 1) / (nt * Bj));
            double Gnk = (D1 - D2) / ((Zj + D2 * Bj) * (Zj + D2 * Bj)) * (e->Bn[k] * Zj - e->Zn[k] * Bj);
            double Enk = -1 / (D1 - D2) / (Bj * Bj) *
                         (2 * (Bj * aik / nt + e->Bn[k] * (e->Bi[i] * Aj / Bj - tmp)) - e->An[k] * e->Bi[i] - Aj * e->Bi[i] / nt);
            Enk -= E / nt;
            out[i * nc + k] = 1 / C * Cnk + Dnk + Enk * log(G) + E / G * Gnk;
            out[k * nc + i] = out[i * nc + k];
        }
    }
}
/* CalLnFugP (:303-340) */
static void eos_lnfugp(eos_t* e, double P, double T, const double* x, double* out)
{
    const int nc = e->nc;
    const double* BIC = e->m->BIC;
    eos_ajbjzj(e, P, T, x);
    eos_apbpzp(e, P);
    const double Aj = e->Aj, Bj = e->Bj, Zj = e->Zj;
    double G = (Zj + D1 * Bj) / (Zj + D2 * Bj);
    double Gp = (D1 - D2) / ((Zj + D2 * Bj) * (Zj + D2 * Bj)) * (e->Bp * Zj - e->Zp * Bj);
    for (int i = 0; i < nc; i++) {
        double C = P / (Zj - Bj);
        double tmp = 0;
        for (int k = 0; k < nc; k++) tmp += (1 - BIC[i * nc + k]) * sqrt(e->Ai[i] * e->Ai[k]) * x[k];
        double E = -Aj / ((D1 - D2) * Bj) * (2 * tmp / Aj - e->Bi[i] / Bj);
        double Cp = ((Zj - Bj) - P * (e->Zp - e->Bp)) / ((Zj - Bj) * (Zj - Bj));
        double Dp = e->Bi[i] / Bj * e->Zp;
        out[i] = Cp / C + Dp + E / G * Gp;
    }
}
/* CalVmDer (:396-414) */
static double eos_vmder(eos_t* e, double P, double T, const double* x, double* vmP, double* vmx)
{
    eos_ajbjzj(e, P, T, x);
    eos_axbxzx(e, x);
    eos_apbpzp(e, P);
    const double CgTP = e->m->R * T / P;
    double v = e->Zj * CgTP;
    for (int i = 0; i < e->nc; i++) v -= x[i] * e->m->Vsh[i];
    for (int i = 0; i < e->nc; i++) vmx[i] = CgTP * e->Zx[i] - e->m->Vsh[i];
    *vmP = CgTP * (e->Zp - e->Zj / P);
    return v;
}

/* ======================================================== dense solves ==== */
/* Gaussian elimination with partial pivoting and an explicit permutation;
 * A is n x n with leading dimension lda (row r, col c at A[r*lda + c]).
 * Returns 0 on success, 1 if a pivot is exactly zero (b then unchanged). */
static int ge_solve(int n, const double* A0, int lda, double* b, int nrhs, int ldb)
{
    double A[NCX * NCX];
    int perm[NCX];
    for (int r = 0; r < n; r++) {
        perm[r] = r;
        for (int c = 0; c < n; c++) A[r * NCX + c] = A0[r * lda + c];
    }
    for (int k = 0; k < n; k++) {
        int p = k;
        for (int r = k + 1; r < n; r++)
            if (fabs(A[perm[r] * NCX + k]) > fabs(A[perm[p] * NCX + k])) p = r;
        int t = perm[k]; perm[k] = perm[p]; perm[p] = t;
        const double piv = A[perm[k] * NCX + k];
        if (piv == 0.0) return 1;
        for (int r = k + 1; r < n; r++) {
            const double l = A[perm[r] * NCX + k] / piv;
            A[perm[r] * NCX + k] = l;
            for (int c = k + 1; c < n; c++) A[perm[r] * NCX + c] -= l * A[perm[k] * NCX + c];
        }
    }
    for (int q = 0; q < nrhs; q++) {
        double y[NCX], *bb = b + q * ldb;
        for (int r = 0; r < n; r++) {
            double s = bb[perm[r]];
            for (int c = 0; c < r; c++) s -= A[perm[r] * NCX + c] * y[c];
            y[r] = s;
        }
        for (int r = n - 1; r >= 0; r--) {
            double s = y[r];
            for (int c = r + 1; c < n; c++) s -= A[perm[r] * NCX + c] * y[c];
            y[r] = s / A[perm[r] * NCX + r];
        }
        for (int r = 0; r < n; r++) bb[r] = y[r];
    }
    return 0;
}
/* SYSSolve -> dsysv_('U') on the reference's row-major buffer
 * (src/DenseMat.cpp:107-123): the column-major upper triangle it reads is
 * the row-major lower triangle, mirrored. */
static int sys_solve(int n, const double* J, double* b)
{
    double S[NCX * NCX];
    for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) S[r * n + c] = r >= c ? J[r * n + c] : J[c * n + r];
    return ge_solve(n, S, n, b, 1, n);
}
/* LUSolve -> dgesv_ (src/DenseMat.cpp:88-105): column-major A, nrhs columns. */
static int lu_solve(int nrhs, int n, const double* A, double* b)
{
    double At[NCX * NCX];
    for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) At[r * n + c] = A[c * n + r];
    return ge_solve(n, At, n, b, nrhs, n);
}
/* CalEigenSY -> ssyevd_ (src/DenseMat.cpp:126-145): smallest eigenvalue of a
 * symmetric single-precision matrix; Jacobi sweeps in double on the float
 * entries, rounded back to float. */
static float min_eig_sym(int n, const float* Af)
{
    double A[NCX * NCX];
    for (int i = 0; i < n * n; i++) A[i] = Af[i];
    for (int sweep = 0; sweep < 50; sweep++) {
        double off = 0;
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++) off += A[i * n + j] * A[i * n + j];
        if (off < 1e-36) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                if (A[p * n + q] == 0) continue;
                double th = 0.5 * atan2(2 * A[p * n + q], A[q * n + q] - A[p * n + p]);
                double c = cos(th), s = sin(th);
                for (int k = 0; k < n; k++) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
            }
    }
    double mn = A[0];
    for (int i = 1; i < n; i++) if (A[i * n + i] < mn) mn = A[i * n + i];
    return (float)mn;
}

/* ==================================================== phase equilibrium == */
/* OCPPhaseEquilibrium (src/OCPPhaseEquilibrium.cpp) state */
typedef struct {
    const oc_model* m;
    eos_t eos;
    int NC, NP, ftype;
    unsigned lNP;
    double P, T, zi[NCX], nu[2], x[2][NCX], n[2][NCX], ln[2][NCX], phi[2][NCX], fug[2][NCX];
    double Kw[4][NCX], Ks[NCX], lKs[NCX], phiSta[NCX], fugSta[NCX], Y[NCX], Yt, di[NCX];
    double resSTA[NCX], JmatSTA[NCX * NCX], lnfugX[NCX * NCX], resSP[NCX], JmatSP[NCX * NCX];
    double lnfugN[2][NCX * NCX];
    int ssm_sta_conv, nr_sta_conv, ssm_sp_conv, nr_sp_conv;
    int it[5];
} pe_t;

static double dnorm2(int n, const double* x)
{
    double s = 0;
    for (int i = 0; i < n; i++) s += x[i] * x[i];
    return sqrt(s);
}
static void dscal(int n, double a, double* x) { for (int i = 0; i < n; i++) x[i] = a * x[i]; }

/* CalKwilson (:244-252) */
static void pe_kwilson(pe_t* p)
{
    const oc_model* m = p->m;
    for (int i = 0; i < p->NC; i++) {
        p->Kw[0][i] = (m->Pc[i] / p->P) * exp(5.373 * (1 + m->acf[i]) * (1 - m->Tc[i] / p->T));
        p->Kw[1][i] = 1 / p->Kw[0][i];
        p->Kw[2][i] = pow(p->Kw[0][i], 1.0 / 3);
        p->Kw[3][i] = pow(p->Kw[1][i], 1.0 / 3);
    }
}
/* StableSSM01 (:299-395), tested phase 0 */
static int pe_stable_ssm01(pe_t* p)
{
    const oc_model* m = p->m;
    const int NC = p->NC;
    double Se = 0, Sk = 0, dY;
    const double* xj = p->x[0];
    eos_fugphi(&p->eos, p->P, p->T, xj, p->fug[0], NULL);
    for (int k = 0; k < 2; k++) {
        memcpy(p->Ks, p->Kw[k], sizeof(double) * NC);
        int iter = 0, flag = 0;
        for (;;) {
            p->Yt = 0;
            for (int i = 0; i < NC; i++) { p->Y[i] = xj[i] * p->Ks[i]; p->Yt += p->Y[i]; }
            dscal(NC, 1 / p->Yt, p->Y);
            if (iter > 0) {
                dY = 0;
                for (int i = 0; i < NC; i++) dY += pow((p->Y[i] - p->di[i]), 2);
                if (dY < m->ssta_dYtol) { flag = 1; break; }
            }
            eos_fugphi(&p->eos, p->P, p->T, p->Y, p->fugSta, NULL);
            Se = 0;
            Sk = 0;
            for (int i = 0; i < NC; i++) {
                p->di[i] = p->fug[0][i] / (p->fugSta[i] * p->Yt);
                p->Ks[i] *= p->di[i];
                Se += pow(p->di[i] - 1, 2);
                Sk += pow(log(p->Ks[i]), 2);
            }
            iter++;
            if (Se < m->ssta_tol2) { flag = 1; break; }
            if (Sk < m->ssta_Ktol) { flag = 1; break; }
            if (iter > m->ssta_it) break;
            memcpy(p->di, p->Y, sizeof(double) * NC);
        }
        p->it[0] += iter;
        if (flag && p->Yt > 1 - 0.1 && Sk > 1) p->ftype = 2;
        if (flag && p->Yt > 1 + m->ssta_eYt) { p->ssm_sta_conv = 1; return 0; }
    }
    return 1;
}
/* StableNR (:475-521) + AssembleJmatSTA (:523-541) */
static int pe_stable_nr(pe_t* p)
{
    const oc_model* m = p->m;
    const int NC = p->NC;
    for (int i = 0; i < NC; i++) p->resSTA[i] = log(p->fug[0][i] / (p->fugSta[i] * p->Yt));
    double Se = dnorm2(NC, p->resSTA);
    const double alpha = 1;
    int iter = 0;
    while (Se > m->nsta_tol) {
        eos_lnfugx(&p->eos, p->P, p->T, p->Y, p->lnfugX);
        for (int i = 0; i < NC; i++) {
            double tmp = 0;
            for (int k = 0; k < NC; k++) tmp += p->Y[k] * p->lnfugX[i * NC + k];
            for (int j = 0; j < NC; j++) p->JmatSTA[i * NC + j] = (p->lnfugX[i * NC + j] - tmp + 1) / p->Yt;
        }
        sys_solve(NC, p->JmatSTA, p->resSTA);
        double lYt = p->Yt;
        p->Yt = 0;
        for (int i = 0; i < NC; i++) { p->Y[i] = p->Y[i] * lYt + alpha * p->resSTA[i]; p->Yt += p->Y[i]; }
        dscal(NC, 1 / p->Yt, p->Y);
        eos_fugphi(&p->eos, p->P, p->T, p->Y, p->fugSta, NULL);
        for (int i = 0; i < NC; i++) p->resSTA[i] = log(p->fug[0][i] / (p->fugSta[i] * p->Yt));
        Se = dnorm2(NC, p->resSTA);
        iter++;
        if (iter > m->nsta_it) { p->it[1] += iter; p->nr_sta_conv = 0; return 0; }
    }
    p->it[1] += iter;
    p->nr_sta_conv = 1;
    return 1;
}
/* StableSSM (:397-473) */
static int pe_stable_ssm(pe_t* p)
{
    const oc_model* m = p->m;
    const int NC = p->NC;
    const double* xj = p->x[0];
    eos_fugphi(&p->eos, p->P, p->T, xj, p->fug[0], p->phi[0]);
    for (int i = 0; i < NC; i++) p->di[i] = p->phi[0][i] * xj[i];
    double Se;
    int flag;
    for (int k = 0; k < 4; k++) {
        p->Yt = 0;
        for (int i = 0; i < NC; i++) { p->Y[i] = xj[i] / p->Kw[k][i]; p->Yt += p->Y[i]; }
        dscal(NC, 1 / p->Yt, p->Y);
        eos_fugphi(&p->eos, p->P, p->T, p->Y, p->fugSta, p->phiSta);
        Se = 0;
        for (int i = 0; i < NC; i++) Se += pow(log(p->fugSta[i] / p->fug[0][i] * p->Yt), 2);
        flag = 1;
        int iter = 0;
        while (Se > m->ssta_tol2) {
            p->Yt = 0;
            for (int i = 0; i < NC; i++) { p->Y[i] = p->di[i] / p->phiSta[i]; p->Yt += p->Y[i]; }
            dscal(NC, 1 / p->Yt, p->Y);
            eos_fugphi(&p->eos, p->P, p->T, p->Y, p->fugSta, p->phiSta);
            Se = 0;
            for (int i = 0; i < NC; i++) Se += pow(log(p->fugSta[i] / p->fug[0][i] * p->Yt), 2);
            iter++;
            if (iter > m->ssta_it) { flag = 0; break; }
        }
        (void)flag;
        p->it[0] += iter;
        flag = pe_stable_nr(p);
        if (flag && p->Yt > 1 + m->ssta_eYt) { p->ssm_sta_conv = 1; return 0; }
    }
    return 1;
}
/* PhaseStable (:260-297) */
static int pe_phase_stable(pe_t* p)
{
    p->ssm_sta_conv = p->nr_sta_conv = 0;
    unsigned tmpNP = (unsigned)p->NP;
    int flag;
    if (p->lNP == 0) flag = pe_stable_ssm(p);
    else {
        flag = pe_stable_ssm01(p);
        if (!flag) tmpNP++;
        if (tmpNP != p->lNP) { flag = pe_stable_ssm(p); p->ftype = 2; }
    }
    return flag;
}
/* RachfordRice2 (:651-705) */
static void pe_rr2(pe_t* p)
{
    const oc_model* m = p->m;
    const int NC = p->NC;
    double Kmin = p->Ks[0], Kmax = p->Ks[0];
    for (int i = 1; i < NC; i++) { if (p->Ks[i] < Kmin) Kmin = p->Ks[i]; if (p->Ks[i] > Kmax) Kmax = p->Ks[i]; }
    const double numin = 1 / (1 - Kmax), numax = 1 / (1 - Kmin);
    p->nu[0] = 0.5 * (numin + numax);
    int iter = 0;
    const double maxIt = m->rr_it;
    for (;;) {
        double rj = 0, J = 0;
        for (int i = 0; i < NC; i++) {
            double tmp = 1 + p->nu[0] * (p->Ks[i] - 1);
            rj += p->zi[i] * (p->Ks[i] - 1) / tmp;
            J -= p->zi[i] * (p->Ks[i] - 1) * (p->Ks[i] - 1) / (tmp * tmp);
        }
        if (fabs(rj) < m->rr_tol || iter > maxIt) break;
        double dnuj = -rj / J, tmpnu = p->nu[0] + dnuj;
        if (tmpnu < numax && tmpnu > numin) p->nu[0] = tmpnu;
        else if (dnuj > 0) p->nu[0] = (p->nu[0] + numax) / 2;
        else p->nu[0] = (p->nu[0] + numin) / 2;
        iter++;
    }
    p->it[4] += iter;
    p->nu[1] = 1 - p->nu[0];
}
/* SplitSSM2 (:586-647) with UpdateXRR (:778-791) */
static void pe_split_ssm2(pe_t* p, int restart)
{
    const oc_model* m = p->m;
    const int NC = p->NC;
    p->ssm_sp_conv = 1;
    double Se = 1, Stol = m->ssp_tol2;
    int maxIt = m->ssp_it;
    if (!restart) {
        if (p->lNP == 2) memcpy(p->Ks, p->lKs, sizeof(double) * NC);
        else memcpy(p->Ks, p->Kw[0], sizeof(double) * NC);
    }
    else { Stol *= 1E-1; maxIt *= 2; }
    if (p->Yt < 1.1) { Stol *= 1E-1; maxIt *= 2; }
    int iter = 0;
    while (Se > Stol) {
        pe_rr2(p);
        for (int i = 0; i < NC; i++) {
            double tmp = 1;
            tmp += p->nu[0] * (p->Ks[i] - 1);
            p->x[1][i] = p->zi[i] / tmp;
            p->x[0][i] = p->Ks[i] * p->x[1][i];
        }
        eos_fugphi(&p->eos, p->P, p->T, p->x[0], p->fug[0], p->phi[0]);
        eos_fugphi(&p->eos, p->P, p->T, p->x[1], p->fug[1], p->phi[1]);
        Se = 0;
        for (int i = 0; i < NC; i++) {
            Se += pow(p->fug[1][i] / p->fug[0][i] - 1, 2);
            p->Ks[i] = p->phi[1][i] / p->phi[0][i];
        }
        iter++;
        if (iter > maxIt) { p->ssm_sp_conv = 0; break; }
    }
    p->it[2] += iter;
}
/* SplitNR (:805-897), CalResSP (:899-907), AssembleJmatSP (:911-937), CalStepNRsp (:939-957) */
static void pe_split_nr(pe_t* p)
{
    const oc_model* m = p->m;
    const int NC = p->NC;
    p->nr_sp_conv = 0;
    for (int j = 0; j < 2; j++) for (int i = 0; i < NC; i++) p->n[j][i] = p->nu[j] * p->x[j][i];
    for (int i = 0; i < NC; i++) p->resSP[i] = log(p->fug[1][i] / p->fug[0][i]);
    double eNR = dnorm2(NC, p->resSP);
    const double eNR0 = eNR;
    int iter = 0;
    while (eNR > m->nsp_tol) {
        memcpy(p->ln, p->n, sizeof(p->n));
        eos_lnn(&p->eos, p->P, p->T, p->x[0], p->nu[0], p->lnfugN[0], 0);
        eos_lnn(&p->eos, p->P, p->T, p->x[1], p->nu[1], p->lnfugN[1], 0);
        for (int i = 0; i < NC; i++)
            for (int k = 0; k < NC; k++) p->JmatSP[i * NC + k] = p->lnfugN[0][i * NC + k] + p->lnfugN[1][i * NC + k];
        sys_solve(NC, p->JmatSP, p->resSP);
        double alpha = 1;
        for (int i = 0; i < NC; i++) {
            double tmp = p->n[0][i] + alpha * p->resSP[i];
            if (tmp < 0) alpha *= 0.9 * fabs(p->n[0][i] / p->resSP[i]);
        }
        memcpy(p->n[1], p->zi, sizeof(double) * NC);
        p->nu[1] = 1;
        p->nu[0] = 0;
        for (int i = 0; i < NC; i++) {
            p->n[0][i] += alpha * p->resSP[i];
            p->n[1][i] -= p->n[0][i];
            p->nu[0] += p->n[0][i];
        }
        p->nu[1] -= p->nu[0];
        for (int i = 0; i < NC; i++) p->x[0][i] = fabs(p->n[0][i] / p->nu[0]);
        for (int i = 0; i < NC; i++) p->x[1][i] = fabs(p->n[1][i] / p->nu[1]);
        eos_fugphi(&p->eos, p->P, p->T, p->x[0], p->fug[0], NULL);
        eos_fugphi(&p->eos, p->P, p->T, p->x[1], p->fug[1], NULL);
        for (int i = 0; i < NC; i++) p->resSP[i] = log(p->fug[1][i] / p->fug[0][i]);
        eNR = dnorm2(NC, p->resSP);
        iter++;
        if (eNR > eNR0 || iter > m->nsp_it) break;
        double en = 0;
        for (int j = 0; j < 2; j++) for (int i = 0; i < NC; i++) en += (p->ln[j][i] - p->n[j][i]) * (p->ln[j][i] - p->n[j][i]);
        if (en < 1E-16 * (2 * NC) * (2 * NC)) { p->nr_sp_conv = 1; break; }
    }
    if (eNR < m->nsp_tol) p->nr_sp_conv = 1;
    p->it[3] += iter;
}
/* CheckSplit (:960-1010) */
static int pe_check_split(pe_t* p)
{
    if (p->NP == 2) {
        double eX = 0, nuMax = p->nu[0] > p->nu[1] ? p->nu[0] : p->nu[1];
        for (int i = 0; i < p->NC; i++) eX += (p->x[0][i] - p->x[1][i]) * (p->x[0][i] - p->x[1][i]);
        if (nuMax < 1 && p->nr_sp_conv && isfinite(eX)) {
        }
        else if (!isfinite(eX) || 1 - nuMax < 1E-3) {
            p->NP = 1;
            memcpy(p->x[0], p->zi, sizeof(double) * p->NC);
            p->nu[0] = 1;
            p->ssm_sta_conv = p->nr_sta_conv = 0;
            return 0;
        }
    }
    return 1;
}
/* PhaseSplit (:549-573); the restart loop is capped in the oracle as well */
static void pe_phase_split(pe_t* p)
{
    p->ssm_sp_conv = p->nr_sp_conv = 0;
    pe_split_ssm2(p, 0);
    pe_split_nr(p);
    int guard = 0;
    while (!p->nr_sp_conv && guard++ < 64) {
        pe_split_ssm2(p, 1);
        pe_split_nr(p);
        if (!pe_check_split(p)) break;
        if (p->ssm_sp_conv) break;
    }
    pe_check_split(p);
}
/* PhaseEquilibrium (:71-112) + SetInitalValue (:121-138) */
static void pe_run(pe_t* p, double P, double T, const double* zi, int ftype, unsigned lNP, const double* lx, int nc)
{
    p->P = P;
    p->T = T;
    memcpy(p->zi, zi, sizeof(double) * p->NC);
    p->ftype = ftype;
    p->lNP = lNP;
    if (p->lNP == 2)
        for (int i = 0; i < p->NC; i++) p->lKs[i] = lx[i] / lx[i + nc];
    switch (p->ftype) {
    case 0:
        p->NP = 1;
        p->nu[0] = 1;
        memcpy(p->x[0], p->zi, sizeof(double) * p->NC);
        pe_kwilson(p);
        while (!pe_phase_stable(p)) {
            p->NP++;
            pe_phase_split(p);
            if (p->NP == 2 || p->NP == 1) break;
        }
        break;
    case 1:
        p->NP = 1;
        p->nu[0] = 1;
        memcpy(p->x[0], p->zi, sizeof(double) * p->NC);
        break;
    default:
        p->NP = 2;
        p->Yt = 1.01;
        pe_kwilson(p);
        pe_phase_split(p);
        break;
    }
    if (p->NP > 1) p->ftype = 2;
}

/* ============================================ compositional FlashDer ====== */
/* ViscosityMethod03::CalViscosity with derivatives (src/OCPFuncPVT.cpp:462-576) */
static double lbc_mu(const oc_model* m, int nc, double T, const double* x, double xi, double xiP, const double* xix,
                     double* muP, double* mux)
{
    double MW = 0, tmp, Tri, xPc = 0, xTc = 0, xVc = 0, a[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < nc; i++) MW += x[i] * m->MW[i];
    for (int i = 0; i < nc; i++) {
        tmp = m->auxB[i] / sqrt(MW);
        Tri = T / m->Tc[i];
        if (Tri <= 1.5) tmp = 34 * 1E-5 * pow(Tri, 0.94) / tmp;
        else tmp = 17.78 * 1E-5 * pow((4.58 * Tri - 1.67), 0.625) / tmp;
        a[0] += x[i] * m->sqrtMWC[i] * tmp;
        a[1] += x[i] * m->sqrtMWC[i];
        xPc += x[i] * m->Pc[i];
        xTc += x[i] * m->Tc[i];
        xVc += x[i] * m->Vcvis[i];
    }
    a[2] = 5.4402 * pow(xTc, 1.0 / 6) / sqrt(MW) / pow(xPc, 2.0 / 3);
    a[3] = xi * xVc;
    const double* c = m->coef;
    a[4] = a[3] * (a[3] * (a[3] * (c[4] * a[3] + c[3]) + c[2]) + c[1]) + c[0];
    const double mu = a[0] / a[1] + 1E-4 * (pow(a[4], 4) - 1) / a[2];
    double der7J = xVc * xiP;
    double der8J = der7J * (c[1] + a[3] * (2 * c[2] + a[3] * (3 * c[3] + a[3] * 4 * c[4])));
    *muP = (4 * 1E-4) * pow(a[4], 3) * der8J / a[2];
    for (int k = 0; k < nc; k++) {
        double der3J = 0;
        for (int i = 0; i < nc; i++) {
            double val1 = m->auxB[i] / sqrt(MW);
            double der1 = 0; /* -(1 / 2) * ... is integer zero in the reference (:537) */
            Tri = T / m->Tc[i];
            tmp = Tri <= 1.5 ? 34 * 1E-5 * pow(Tri, 0.94) : 17.78 * 1E-5 * pow(4.58 * Tri - 1.67, 0.625);
            double val2 = tmp / val1;
            double der2 = -tmp * der1 / (val1 * val1);
            der3J += x[i] * m->sqrtMWC[i] * der2 + dlt(i, k) * m->sqrtMWC[k] * val2;
        }
        double der4J = m->sqrtMWC[k];
        double der6J = 5.4402 * (1.0 / 6 * pow(xTc, -5.0 / 6) * m->Tc[k] - pow(xTc, 1.0 / 6) * (0.5 / MW * m->MW[k] + 2.0 / 3 / xPc * m->Pc[k])) /
                       (sqrt(MW) * pow(xPc, 2.0 / 3));
        der7J = xix[k] * xVc + xi * m->Vcvis[k];
        der8J = der7J * (c[1] + a[3] * (2 * c[2] + a[3] * (3 * c[3] + a[3] * 4 * c[4])));
        mux[k] = (der3J * a[1] - a[0] * der4J) / (a[1] * a[1]) +
                 1E-4 * (4 * pow(a[4], 3) * der8J * a[2] - (pow(a[4], 4) - 1) * der6J) / (a[2] * a[2]);
    }
    return mu;
}
/* OCP_PVTW::CalRhoXiMuDer (src/OCPFuncPVT.cpp:32-56) */
static void pvtw_der(const oc_model* m, double P, double* rho, double* xi, double* mu, double* rhoP, double* xiP, double* muP)
{
    const tab_t* t = &m->pvtw;
    int r = tab_close(t, 0, P);
    double Pref = t->d[r], bref = t->d[t->nrow + r], Cb = t->d[2 * t->nrow + r], muref = t->d[3 * t->nrow + r],
           Cmu = t->d[4 * t->nrow + r];
    double b = bref * (1 - Cb * (P - Pref)), bp = -Cb * bref;
    *mu = muref * (1 + Cmu * (P - Pref));
    *muP = Cmu * muref;
    *xi = 1 / m->conv1 / (b * m->vw);
    *xiP = -1 / m->conv1 * bp / ((b * b) * m->vw);
    *rho = m->rho_w / b;
    *rhoP = -m->rho_w * bp / (b * b);
}

/* the mixture varset of one cell (OCPMixtureVarSet) */
typedef struct {
    double P, T, Ni[NCX + 1], S[NPH], nj[NPH], vj[NPH], x[NPH][NCX + 1], rho[NPH], xi[NPH], mu[NPH];
    double rhoP[NPH], xiP[NPH], muP[NPH], rhox[NPH][NCX + 1], xix[NPH][NCX + 1], mux[NPH][NCX + 1];
    double vfP, vfi[NCX + 1], vjP[NPH], vji[NPH][NCX + 1], Vf, Nt, dX[NPH * (NCX + 2) * (NCX + 2)];
    int ex[NPH];
} mvs_t;

static void swapd(double* a, double* b, int n) { for (int i = 0; i < n; i++) { double t = a[i]; a[i] = b[i]; b[i] = t; } }

/* One cell: OCPMixtureComp::FlashDer (include/OCPMixture.hpp:85-90) =
 * SetVarSet, SkipPSA CalFtype02, OCPMixtureMethodComp01::FlashDer
 * (src/OCPMixtureMethodComp.cpp:746-755), CalSkipForNextStep; then
 * IsoT_FIM::PassFlashValue (src/IsoThermalMethod.cpp:1027-1071). */
static void comp_cell(const oc_model* m, oc_bulk* b, int n, pe_t* pe, mvs_t* vs)
{
    const int nc = b->nc, NC = m->NC, np = NPH, ncol = nc + 1;
    const int w = 2;
    /* SetVarSet (:671-687) */
    vs->P = b->P[n];
    vs->T = b->T[n] + m->conv4;
    unsigned phaseNum = 0;
    for (int i = 0; i < nc; i++) vs->Ni[i] = b->Ni[n * nc + i];
    for (int j = 0; j < np; j++) {
        vs->S[j] = b->S[n * np + j];
        vs->ex[j] = b->phaseExist[n * np + j] != 0;
        if (vs->ex[j]) phaseNum++;
        for (int i = 0; i < nc; i++) vs->x[j][i] = b->xij[(n * np + j) * nc + i];
    }
    /* SkipPSAMethod01::CalFtype02 (src/AcceleratePEC.cpp:64-124) */
    int ftype = 0;
    const unsigned npPE = phaseNum - 1;
    if (m->skip) {
        int skip = 0;
        if (b->skip_flag[n]) {
            double Nt = 0;
            for (int i = 0; i < NC; i++) Nt += vs->Ni[i];
            const double me = b->skip_minEig[n];
            skip = 1;
            if (fabs(1 - b->skip_P[n] / vs->P) >= me / 10) skip = 0;
            else if (fabs(b->skip_T[n] - vs->T) >= me * 10) skip = 0;
            else for (int i = 0; i < NC; i++) if (fabs(vs->Ni[i] / Nt - b->skip_zi[n * NC + i]) >= me / 10) { skip = 0; break; }
        }
        if (skip) ftype = 1;
        else if (npPE >= 2) {
            unsigned tmp = 0;
            for (int j = 0; j < 2; j++) if (vs->S[j] >= 1E-4) tmp++;
            ftype = tmp == npPE ? (int)npPE : 0;
        }
    }
    /* InitNtZ (:812-818) */
    double Nt = 0, zi[NCX];
    for (int i = 0; i < NC; i++) Nt += vs->Ni[i];
    for (int i = 0; i < NC; i++) zi[i] = vs->Ni[i] / Nt;
    vs->Nt = Nt + vs->Ni[NC];
    /* x as the varset holds it, phase-major with nc entries per phase */
    double lx[NPH * (NCX + 1)];
    for (int j = 0; j < np; j++) for (int i = 0; i < nc; i++) lx[j * nc + i] = vs->x[j][i];
    memset(pe->it, 0, sizeof(pe->it));
    pe_run(pe, vs->P, vs->T, zi, ftype, (unsigned)(double)(phaseNum - 1), lx, nc);
    /* CalPropertyDer (:134-142) */
    const int NP = pe->NP;
    double MW[2], vm[2], vmP[2], vmx[2][NCX];
    for (int j = 0; j < NP; j++) {
        vs->nj[j] = Nt * pe->nu[j];
        for (int i = 0; i < NC; i++) vs->x[j][i] = pe->x[j][i];
    }
    for (int j = 0; j < NP; j++) { MW[j] = 0; for (int i = 0; i < NC; i++) MW[j] += vs->x[j][i] * m->MW[i]; }
    for (int j = 0; j < NP; j++) { vm[j] = eos_vmder(&pe->eos, vs->P, vs->T, vs->x[j], &vmP[j], vmx[j]); vs->vj[j] = vs->nj[j] * vm[j]; }
    for (int j = 0; j < NP; j++) {
        vs->xi[j] = 1 / vm[j];
        vs->xiP[j] = -vs->xi[j] * vs->xi[j] * vmP[j];
        for (int i = 0; i < NC; i++) vs->xix[j][i] = -vs->xi[j] * vs->xi[j] * vmx[j][i];
        vs->rho[j] = MW[j] * vs->xi[j];
        vs->rhoP[j] = MW[j] * vs->xiP[j];
        for (int i = 0; i < NC; i++) vs->rhox[j][i] = vs->xix[j][i] * MW[j] + vs->xi[j] * m->MW[i];
        vs->mu[j] = lbc_mu(m, NC, vs->T, vs->x[j], vs->xi[j], vs->xiP[j], vs->xix[j], &vs->muP[j], vs->mux[j]);
    }
    /* IdentifyPhase (:174-214) */
    int label0_oil;
    vs->ex[0] = vs->ex[1] = 0;
    if (NP == 1) {
        double A = 0, B = 0;
        for (int i = 0; i < NC; i++) { A += zi[i] * m->Vc[i] * m->Tc[i]; B += zi[i] * m->Vc[i]; }
        if (vs->T > A / B) { label0_oil = 0; vs->ex[1] = 1; }
        else { label0_oil = 1; vs->ex[0] = 1; }
    }
    else { label0_oil = MW[0] > MW[1]; vs->ex[0] = vs->ex[1] = 1; }
    /* ReOrderPhaseDer (:235-256) */
    if (!label0_oil) {
        swapd(&vs->nj[0], &vs->nj[1], 1); swapd(vs->x[0], vs->x[1], NC); swapd(&MW[0], &MW[1], 1);
        swapd(&vs->vj[0], &vs->vj[1], 1); swapd(&vm[0], &vm[1], 1); swapd(&vmP[0], &vmP[1], 1);
        swapd(vmx[0], vmx[1], NC); swapd(&vs->xi[0], &vs->xi[1], 1); swapd(&vs->xiP[0], &vs->xiP[1], 1);
        swapd(vs->xix[0], vs->xix[1], NC); swapd(&vs->rho[0], &vs->rho[1], 1); swapd(&vs->rhoP[0], &vs->rhoP[1], 1);
        swapd(vs->rhox[0], vs->rhox[1], NC); swapd(&vs->mu[0], &vs->mu[1], 1); swapd(&vs->muP[0], &vs->muP[1], 1);
        swapd(vs->mux[0], vs->mux[1], NC);
    }
    /* CalPropertyW (:846-860) */
    vs->ex[w] = 1;
    vs->x[w][NC] = 1.0;
    pvtw_der(m, vs->P, &vs->rho[w], &vs->xi[w], &vs->mu[w], &vs->rhoP[w], &vs->xiP[w], &vs->muP[w]);
    vs->nj[w] = vs->Ni[NC];
    vs->vj[w] = vs->nj[w] / vs->xi[w];
    for (int i = 0; i <= NC; i++) vs->vji[w][i] = 0;
    vs->vji[w][NC] = 1 / vs->xi[w];
    vs->vjP[w] = -vs->nj[w] * vs->xiP[w] / (vs->xi[w] * vs->xi[w]);
    /* CalVfS (include/OCPMixtureVarSet.hpp:143-155) */
    vs->Vf = 0;
    for (int j = 0; j < np; j++) if (vs->ex[j]) vs->Vf += vs->vj[j];
    for (int j = 0; j < np; j++) vs->S[j] = vs->ex[j] ? vs->vj[j] / vs->Vf : 0;
    /* CalVfiVfp_full02 (:462-524) + AddVfpVfiW (:896-901) */
    double rhs[NCX * (NCX + 1)];
    vs->vji[0][NC] = vs->vji[1][NC] = 0;
    if (NP == 1) {
        const int j = vs->ex[0] ? 0 : 1;
        vs->vjP[j] = vs->nj[j] * vmP[j];
        vs->vfP = vs->vjP[j];
        for (int i = 0; i < NC; i++) {
            vs->vji[j][i] = vm[j] + vmx[j][i];
            for (int k = 0; k < NC; k++) vs->vji[j][i] -= vmx[j][k] * vs->x[j][k];
            vs->vfi[i] = vs->vji[j][i];
        }
    }
    else {
        double lnP[2][NCX], J[NCX * NCX];
        for (int j = 0; j < 2; j++) {
            eos_lnn(&pe->eos, vs->P, vs->T, vs->x[j], vs->nj[j], pe->lnfugN[j], 0);
            eos_lnfugp(&pe->eos, vs->P, vs->T, vs->x[j], lnP[j]);
        }
        for (int i = 0; i < NC; i++)
            for (int k = 0; k < NC; k++) J[i * NC + k] = pe->lnfugN[0][i * NC + k] + pe->lnfugN[1][i * NC + k];
        for (int i = 0; i < NC; i++) rhs[i] = lnP[1][i] - lnP[0][i];
        for (int k = 0; k < NC; k++) for (int i = 0; i < NC; i++) rhs[(k + 1) * NC + i] = pe->lnfugN[1][k * NC + i];
        lu_solve(NC + 1, NC, J, rhs);
        double tmp0 = 0, tmp1 = 0;
        for (int i = 0; i < NC; i++) { tmp0 -= vmx[0][i] * vs->x[0][i]; tmp1 -= vmx[1][i] * vs->x[1][i]; }
        vs->vjP[0] = vs->nj[0] * vmP[0];
        vs->vjP[1] = vs->nj[1] * vmP[1];
        for (int k = 0; k < NC; k++) {
            vs->vjP[0] += (vm[0] + tmp0 + vmx[0][k]) * rhs[k];
            vs->vjP[1] -= (vm[1] + tmp1 + vmx[1][k]) * rhs[k];
        }
        vs->vfP = vs->vjP[0] + vs->vjP[1];
        for (int i = 0; i < NC; i++) {
            const double* dN = rhs + (i + 1) * NC;
            vs->vji[0][i] = 0;
            vs->vji[1][i] = 0;
            for (int k = 0; k < NC; k++) {
                vs->vji[0][i] += (vm[0] + tmp0 + vmx[0][k]) * dN[k];
                vs->vji[1][i] += (vm[1] + tmp1 + vmx[1][k]) * (dlt(i, k) - dN[k]);
            }
            vs->vfi[i] = vs->vji[0][i] + vs->vji[1][i];
        }
    }
    vs->vfP += vs->vjP[w];
    vs->vfi[NC] = vs->vji[w][NC];
    /* CaldXsdXp02 (:565-642) + CaldXsdXpW (:904-920) */
    double* dX = vs->dX;
    const int nrow = np * nc + np;
    memset(dX, 0, sizeof(double) * nrow * ncol);
    for (int j = 0; j < 2; j++) {
        if (!vs->ex[j]) continue;
        dX[j * ncol] = (vs->vjP[j] - vs->vfP * vs->S[j]) / vs->Vf;
        for (int mm = 0; mm < NC; mm++) dX[j * ncol + 1 + mm] = (vs->vji[j][mm] - vs->vfi[mm] * vs->S[j]) / vs->Vf;
    }
    if (NP == 1) {
        const int j = vs->ex[0] ? 0 : 1;
        for (int i = 0; i < NC; i++)
            for (int mm = 0; mm < NC; mm++)
                dX[(np + j * nc + i) * ncol + 1 + mm] = (dlt(i, mm) * Nt - vs->Ni[i]) / (Nt * Nt);
    }
    else {
        const double* d = rhs;
        double s = 0;
        for (int i = 0; i < NC; i++) s += d[i];
        for (int i = 0; i < NC; i++) {
            dX[(np + i) * ncol] = (d[i] - s * vs->x[0][i]) / vs->nj[0];
            dX[(np + nc + i) * ncol] = (-d[i] + s * vs->x[1][i]) / vs->nj[1];
        }
        for (int mm = 0; mm < NC; mm++) {
            d = rhs + (mm + 1) * NC;
            s = 0;
            for (int i = 0; i < NC; i++) s += d[i];
            for (int i = 0; i < NC; i++) {
                dX[(np + i) * ncol + mm + 1] = (d[i] - s * vs->x[0][i]) / vs->nj[0];
                dX[(np + nc + i) * ncol + mm + 1] = ((dlt(i, mm) - d[i]) - (1 - s) * vs->x[1][i]) / vs->nj[1];
            }
        }
    }
    for (int j = 0; j < 2; j++) if (vs->ex[j]) dX[j * ncol + NC + 1] = (vs->vji[j][NC] - vs->vfi[NC] * vs->S[j]) / vs->Vf;
    dX[w * ncol] = (vs->vjP[w] - vs->vfP * vs->S[w]) / vs->Vf;
    for (int i = 0; i < nc; i++) dX[w * ncol + 1 + i] = (vs->vji[w][i] - vs->vfi[i] * vs->S[w]) / vs->Vf;
    /* SkipPSAMethod01::CalSkipForNextStep (src/AcceleratePEC.cpp:127-170) */
    if (m->skip) {
        if (pe->ftype == 0) {
            double lnphiN[NCX * NCX];
            float A[NCX * NCX];
            eos_lnn(&pe->eos, vs->P, vs->T, zi, Nt, lnphiN, 1);
            for (int i = 0; i < NC; i++)
                for (int j = 0; j <= i; j++) {
                    A[i * NC + j] = (float)(dlt(i, j) + Nt * sqrt(zi[i] * zi[j]) * lnphiN[i * NC + j]);
                    A[j * NC + i] = A[i * NC + j];
                }
            b->skip_flag[n] = 1;
            b->skip_minEig[n] = min_eig_sym(NC, A);
            b->skip_P[n] = vs->P;
            b->skip_T[n] = vs->T;
            for (int i = 0; i < NC; i++) b->skip_zi[n * NC + i] = zi[i];
        }
        else b->skip_flag[n] = pe->ftype == 1 ? 1 : 0;
    }
    /* PassFlashValue */
    b->Nt[n] = vs->Nt;
    b->vf[n] = vs->Vf;
    for (int j = 0; j < np; j++) {
        b->S[n * np + j] = vs->S[j];
        b->phaseExist[n * np + j] = vs->ex[j];
        if (!vs->ex[j]) continue;
        b->rho[n * np + j] = vs->rho[j]; b->xi[n * np + j] = vs->xi[j]; b->mu[n * np + j] = vs->mu[j];
        b->rhoP[n * np + j] = vs->rhoP[j]; b->xiP[n * np + j] = vs->xiP[j]; b->muP[n * np + j] = vs->muP[j];
        for (int i = 0; i < nc; i++) {
            const int hc = j < 2 && i < NC;
            b->xij[(n * np + j) * nc + i] = vs->x[j][i];
            b->rhox[(n * np + j) * nc + i] = hc ? vs->rhox[j][i] : 0;
            b->xix[(n * np + j) * nc + i] = hc ? vs->xix[j][i] : 0;
            b->mux[(n * np + j) * nc + i] = hc ? vs->mux[j][i] : 0;
        }
    }
    b->vfP[n] = vs->vfP;
    for (int i = 0; i < nc; i++) b->vfi[n * nc + i] = vs->vfi[i];
    memcpy(&b->dSec_dPri[(size_t)n * nrow * ncol], dX, sizeof(double) * nrow * ncol);
    if (b->ftype) b->ftype[n] = pe->ftype;
    if (b->iters) for (int k = 0; k < 5; k++) b->iters[n * 5 + k] = pe->it[k];
}

/* ==================================================== black-oil OGW01 ==== */
/* OCPMixtureMethodK_OGW01::FlashDer (src/OCPMixtureMethodK.cpp:521-759) */
static void bo_cell(const oc_model* m, oc_bulk* b, int n)
{
    const int np = 3, nc = 3;
    const double P = b->P[n];
    double Ni[3], S[3], rho[3], xi[3], mu[3], rhoP[3] = {0}, xiP[3] = {0}, muP[3] = {0};
    double rhox[9] = {0}, xix[9] = {0}, mux[9] = {0}, dX[48] = {0};
    double vj[3], vjP[3] = {0}, vji[3][3] = {{0}}, vfi[3], Vf, vfP, xo[3] = {0, 0, 0};
    int ex[3];
    for (int i = 0; i < 3; i++) Ni[i] = b->Ni[n * nc + i];
    const double Nt = Ni[0] + Ni[1] + Ni[2];
    double x = tab_eval(&m->pvco, 0, P, 1) * m->vo / m->vg;
    double d[6], cd[6];
    pvtw_der(m, P, &rho[2], &xi[2], &mu[2], &rhoP[2], &xiP[2], &muP[2]);
    if (Ni[0] < Nt * TINY_) {
        if (Ni[1] <= Ni[0] * x) {
            ex[0] = 0; ex[1] = 0; ex[2] = 1;
            S[0] = 0; S[1] = 0; S[2] = 1;
            vj[0] = 0; vj[1] = 0; vj[2] = Ni[2] / xi[2];
            Vf = vj[2];
            vjP[2] = -Ni[2] * xiP[2] / (xi[2] * xi[2]);
            vfP = vjP[2];
            vji[2][2] = 1 / xi[2];
            vfi[0] = 0; vfi[1] = 0; vfi[2] = vji[2][2];
            dX[1 * 4 + 2] = 1 / (1 / m->conv1 / (tab_eval(&m->pvdg, 0, P, 1) * m->vg)) / Vf;
            dX[2 * 4 + 0] = (vjP[2] - S[2] * vfP) / Vf;
            dX[2 * 4 + 1] = -S[2] * vfi[0] / Vf;
            dX[2 * 4 + 2] = -S[2] * vfi[1] / Vf;
            dX[2 * 4 + 3] = (vji[2][2] - S[2] * vfi[2]) / Vf;
        }
        else {
            ex[0] = 0; ex[1] = 1; ex[2] = 1;
            /* OCP_PVDG::CalRhoXiMuDer (src/OCPFuncPVT.cpp:167-196) */
            tab_eval_all(&m->pvdg, 0, P, d, cd);
            rho[1] = m->conv3 * m->rho_g / d[1]; xi[1] = 1 / m->conv1 / (d[1] * m->vg); mu[1] = d[2];
            rhoP[1] = -m->conv3 * m->rho_g * cd[1] / (d[1] * d[1]); xiP[1] = -1 / m->conv1 * cd[1] / ((d[1] * d[1]) * m->vg); muP[1] = cd[2];
            /* OCP_PVCO::CalRhoXiMuRsDer (:87-114) */
            tab_eval_all(&m->pvco, 0, P, d, cd);
            double rs = d[1], bo = d[2], rsP = cd[1], bP = cd[2];
            mu[0] = d[3]; muP[0] = cd[3];
            double xx = rs * (m->vo / m->vg), xP0 = rsP * (m->vo / m->vg);
            xi[0] = (1 + xx) / (bo * m->conv1 * m->vo);
            xiP[0] = (xP0 * bo - (1 + xx) * bP) / ((bo * bo) * (m->conv1 * m->vo));
            rho[0] = (m->rho_o + m->conv3 * rs * m->rho_g) / bo;
            rhoP[0] = m->conv3 * m->rho_g * rsP / bo - (m->rho_o + m->conv3 * rs * m->rho_g) * bP / (bo * bo);
            x = rs * (m->vo / m->vg);
            const double xP = rsP * (m->vo / m->vg);
            vj[0] = 0; vj[1] = (Ni[1] - x * Ni[0]) / xi[1]; vj[2] = Ni[2] / xi[2];
            Vf = vj[1] + vj[2];
            S[0] = 0; S[1] = vj[1] / Vf; S[2] = vj[2] / Vf;
            vjP[0] = Ni[0] * (xP * xi[0] - (1 + x) * xiP[0]) / (xi[0] * xi[0]);
            vjP[1] = (-xP * Ni[0] * xi[1] - (Ni[1] - x * Ni[0]) * xiP[1]) / (xi[1] * xi[1]);
            vjP[2] = -Ni[2] * xiP[2] / (xi[2] * xi[2]);
            vfP = vjP[0] + vjP[1] + vjP[2];
            vji[0][0] = (1 + x) / xi[0]; vji[1][0] = -x / xi[1]; vji[1][1] = 1 / xi[1]; vji[2][2] = 1 / xi[2];
            vfi[0] = vji[0][0] + vji[1][0]; vfi[1] = vji[1][1]; vfi[2] = vji[2][2];
            dX[1] = vji[0][0] / Vf;
            dX[4] = (vjP[1] - S[1] * vfP) / Vf; dX[5] = (vji[1][0] - S[1] * vfi[0]) / Vf;
            dX[6] = (vji[1][1] - S[1] * vfi[1]) / Vf; dX[7] = -S[1] * vfi[2] / Vf;
            dX[8] = (vjP[2] - S[2] * vfP) / Vf; dX[9] = -S[2] * vfi[0] / Vf;
            dX[10] = -S[2] * vfi[1] / Vf; dX[11] = (vji[2][2] - S[2] * vfi[2]) / Vf;
            dX[12] = -xP / ((1 + x) * (1 + x)); dX[16] = -dX[12];
        }
    }
    else if (Ni[1] <= Ni[0] * x) {
        x = Ni[1] / Ni[0];
        ex[0] = 1; ex[1] = 0; ex[2] = 1;
        xo[0] = 1 / (1 + x); xo[1] = 1 - xo[0];
        const double rs = x * (m->vg / m->vo);
        /* OCP_PVCO::CalRhoXiMuDer (:117-155) */
        tab_eval_all(&m->pvco, 1, rs, d, cd);
        const double Pref = d[0], bref = d[2], muref = d[3], Cb = d[4], Cmu = d[5];
        const double PrefRs = cd[0], brefRs = cd[2], murefRs = cd[3], CbRs = cd[4], CmuRs = cd[5];
        const double bo = bref * (1 - Cb * (P - Pref)), bP = -bref * Cb;
        const double bRs = brefRs * (1 - Cb * (P - Pref)) + bref * (-CbRs * (P - Pref) + Cb * PrefRs);
        mu[0] = muref * (1 + Cmu * (P - Pref)); muP[0] = muref * Cmu;
        const double muRs = murefRs * (1 + Cmu * (P - Pref)) + muref * (CmuRs * (P - Pref) - Cmu * PrefRs);
        const double xx = rs * (m->vo / m->vg), xRs = m->vo / m->vg;
        xi[0] = (1 + xx) / (bo * m->conv1 * m->vo);
        xiP[0] = -(1 + xx) * bP / ((bo * bo) * (m->conv1 * m->vo));
        const double xiRs = (xRs * bo - (1 + xx) * bRs) / ((bo * bo) * m->conv1 * m->vo);
        rho[0] = (m->rho_o + m->conv3 * rs * m->rho_g) / bo;
        rhoP[0] = -(m->rho_o + m->conv3 * rs * m->rho_g) * bP / (bo * bo);
        const double rhoRs = (m->conv3 * m->rho_g * bo - (m->rho_o + m->conv3 * rs * m->rho_g) * bRs) / (bo * bo);
        const double xiox = xiRs * (m->vg / m->vo), rhoox = rhoRs * (m->vg / m->vo), muox = muRs * (m->vg / m->vo);
        vj[0] = (Ni[0] + Ni[1]) / xi[0]; vj[1] = 0; vj[2] = Ni[2] / xi[2];
        Vf = vj[0] + vj[2];
        S[0] = vj[0] / Vf; S[1] = 0; S[2] = vj[2] / Vf;
        vjP[0] = -(Ni[0] + Ni[1]) * xiP[0] / (xi[0] * xi[0]);
        vjP[2] = -Ni[2] * xiP[2] / (xi[2] * xi[2]);
        vfP = vjP[0] + vjP[2];
        vji[0][0] = (xi[0] + x * (1 + x) * xiox) / (xi[0] * xi[0]);
        vji[0][1] = (xi[0] - (1 + x) * xiox) / (xi[0] * xi[0]);
        vji[2][2] = 1 / xi[2];
        vfi[0] = vji[0][0]; vfi[1] = vji[0][1]; vfi[2] = vji[2][2];
        dX[0] = (vjP[0] - S[0] * vfP) / Vf; dX[1] = (vji[0][0] - S[0] * vfi[0]) / Vf;
        dX[2] = (vji[0][1] - S[0] * vfi[1]) / Vf; dX[3] = -S[0] / Vf * vfi[2];
        dX[8] = (vjP[2] - S[2] * vfP) / Vf; dX[9] = -S[2] * vfi[0] / Vf;
        dX[10] = -S[2] * vfi[1] / Vf; dX[11] = (vji[2][2] - S[2] * vfi[2]) / Vf;
        dX[13] = Ni[1] / pow((Ni[0] + Ni[1]), 2); dX[14] = -Ni[0] / pow((Ni[0] + Ni[1]), 2);
        dX[17] = -dX[13]; dX[18] = -dX[14];
        const double t2 = (1 + x) * (1 + x);
        mux[0] = -muox * t2; mux[1] = muox * t2; xix[0] = -xiox * t2; xix[1] = xiox * t2;
        rhox[0] = -rhoox * t2; rhox[1] = rhoox * t2;
    }
    else {
        ex[0] = 1; ex[1] = 1; ex[2] = 1;
        tab_eval_all(&m->pvco, 0, P, d, cd);
        double rs = d[1], bo = d[2], rsP = cd[1], bP = cd[2];
        mu[0] = d[3]; muP[0] = cd[3];
        double xx = rs * (m->vo / m->vg), xP0 = rsP * (m->vo / m->vg);
        xi[0] = (1 + xx) / (bo * m->conv1 * m->vo);
        xiP[0] = (xP0 * bo - (1 + xx) * bP) / ((bo * bo) * (m->conv1 * m->vo));
        rho[0] = (m->rho_o + m->conv3 * rs * m->rho_g) / bo;
        rhoP[0] = m->conv3 * m->rho_g * rsP / bo - (m->rho_o + m->conv3 * rs * m->rho_g) * bP / (bo * bo);
        tab_eval_all(&m->pvdg, 0, P, d, cd);
        rho[1] = m->conv3 * m->rho_g / d[1]; xi[1] = 1 / m->conv1 / (d[1] * m->vg); mu[1] = d[2];
        rhoP[1] = -m->conv3 * m->rho_g * cd[1] / (d[1] * d[1]); xiP[1] = -1 / m->conv1 * cd[1] / ((d[1] * d[1]) * m->vg); muP[1] = cd[2];
        x = rs * (m->vo / m->vg);
        const double xP = rsP * (m->vo / m->vg);
        xo[0] = 1 / (1 + x); xo[1] = 1 - xo[0];
        vj[0] = Ni[0] * (1 + x) / xi[0]; vj[1] = (Ni[1] - x * Ni[0]) / xi[1]; vj[2] = Ni[2] / xi[2];
        Vf = vj[0] + vj[1] + vj[2];
        S[0] = vj[0] / Vf; S[1] = vj[1] / Vf; S[2] = vj[2] / Vf;
        vjP[0] = Ni[0] * (xP * xi[0] - (1 + x) * xiP[0]) / (xi[0] * xi[0]);
        vjP[1] = (-xP * Ni[0] * xi[1] - (Ni[1] - x * Ni[0]) * xiP[1]) / (xi[1] * xi[1]);
        vjP[2] = -Ni[2] * xiP[2] / (xi[2] * xi[2]);
        vfP = vjP[0] + vjP[1] + vjP[2];
        vji[0][0] = (1 + x) / xi[0]; vji[1][0] = -x / xi[1]; vji[1][1] = 1 / xi[1]; vji[2][2] = 1 / xi[2];
        vfi[0] = vji[0][0] + vji[1][0]; vfi[1] = vji[1][1]; vfi[2] = vji[2][2];
        dX[0] = (vjP[0] - S[0] * vfP) / Vf; dX[1] = (vji[0][0] - S[0] * vfi[0]) / Vf;
        dX[2] = -S[0] * vfi[1] / Vf; dX[3] = -S[0] * vfi[2] / Vf;
        dX[4] = (vjP[1] - S[1] * vfP) / Vf; dX[5] = (vji[1][0] - S[1] * vfi[0]) / Vf;
        dX[6] = (vji[1][1] - S[1] * vfi[1]) / Vf; dX[7] = -S[1] * vfi[2] / Vf;
        dX[8] = (vjP[2] - S[2] * vfP) / Vf; dX[9] = -S[2] * vfi[0] / Vf;
        dX[10] = -S[2] * vfi[1] / Vf; dX[11] = (vji[2][2] - S[2] * vfi[2]) / Vf;
        dX[12] = -xP / ((1 + x) * (1 + x)); dX[16] = -dX[12];
    }
    const double xfix[3][3] = {{xo[0], xo[1], 0}, {0, 1, 0}, {0, 0, 1}};
    b->Nt[n] = Nt;
    b->vf[n] = Vf;
    for (int j = 0; j < np; j++) {
        b->S[n * np + j] = S[j];
        b->phaseExist[n * np + j] = ex[j];
        if (!ex[j]) continue;
        b->rho[n * np + j] = rho[j]; b->xi[n * np + j] = xi[j]; b->mu[n * np + j] = mu[j];
        b->rhoP[n * np + j] = rhoP[j]; b->xiP[n * np + j] = xiP[j]; b->muP[n * np + j] = muP[j];
        for (int i = 0; i < nc; i++) {
            b->xij[(n * np + j) * nc + i] = xfix[j][i];
            b->rhox[(n * np + j) * nc + i] = rhox[j * nc + i];
            b->xix[(n * np + j) * nc + i] = xix[j * nc + i];
            b->mux[(n * np + j) * nc + i] = mux[j * nc + i];
        }
    }
    b->vfP[n] = vfP;
    for (int i = 0; i < nc; i++) b->vfi[n * nc + i] = vfi[i];
    memcpy(&b->dSec_dPri[(size_t)n * 48], dX, sizeof(dX));
    if (b->ftype) b->ftype[n] = -1;
}

/* ================================================================ API ==== */
int oc_check(const oc_model* m, oc_bulk* b)
{
    (void)m;
    /* Bulk::CheckNi (src/Bulk.cpp:178-213): stops at the first failure */
    const long len = (long)b->nb * b->nc;
    for (long k = 0; k < len; k++) {
        if (b->Ni[k] < 0) {
            const long n = k / b->nc;
            if ((b->Ni[k] > -1E-5 * b->Nt[n]) || (b->lNi[k] < 1E-3 * b->Nt[n])) b->Ni[k] = 1E-40 * b->Nt[n];
            else return 1;
        }
    }
    /* Bulk::CheckP (:116-131) */
    for (int n = 0; n < b->nb; n++) if (b->P[n] < 0) return 2;
    return 0;
}

void oc_flash(const oc_model* m, oc_bulk* b, int n0, int n1)
{
    if (m->mixture == 1) {
#pragma omp parallel
        {
            pe_t* pe = (pe_t*)calloc(1, sizeof(pe_t));
            mvs_t* vs = (mvs_t*)calloc(1, sizeof(mvs_t));
            pe->m = m;
            pe->NC = m->NC;
            pe->eos.m = m;
            pe->eos.nc = m->NC;
#pragma omp for schedule(dynamic, 16)
            for (int n = n0; n < n1; n++) comp_cell(m, b, n, pe, vs);
            free(pe);
            free(vs);
        }
    }
    else {
#pragma omp parallel for schedule(static)
        for (int n = n0; n < n1; n++) bo_cell(m, b, n);
    }
}

void oc_krpc_rock(const oc_model* m, oc_bulk* b, int n0, int n1)
{
    const int np = 3, o = 0, g = 1, w = 2;
#pragma omp parallel for schedule(static)
    for (int n = n0; n < n1; n++) {
        double kr[3], Pc[3] = {0, 0, 0}, dKr[9] = {0}, dPc[9] = {0}, d[4], cd[4];
        /* OCP_SWOF / OCP_SGOF (include/OCPFuncSAT.hpp:66-76, 168-178) */
        tab_eval_all(&m->swof, 0, b->S[n * np + w], d, cd);
        kr[w] = d[1]; const double krow = d[2]; Pc[w] = -d[3];
        dKr[w * np + w] = cd[1]; const double dKrowdSw = cd[2]; dPc[w * np + w] = -cd[3];
        tab_eval_all(&m->sgof, 0, b->S[n * np + g], d, cd);
        kr[g] = d[1]; const double krog = d[2]; Pc[g] = d[3];
        dKr[g * np + g] = cd[1]; const double dKrogdSg = cd[2]; dPc[g * np + g] = cd[3];
        /* OCP3POilPerMethod01::CalOilPerDer (src/OCPFuncSAT.cpp:162-190); the
         * So-derivatives of krow/krog stay at their initial 0 in the reference */
        const double krocw = m->swof.d[2 * m->swof.nrow];
        const double dKrowdSo = 0, dKrogdSo = 0;
        kr[o] = krocw * ((krow / krocw + kr[w]) * (krog / krocw + kr[g]) - (kr[w] + kr[g]));
        if (kr[o] < 0) { kr[o] = 0; dKr[0] = dKr[1] = dKr[2] = 0; }
        else {
            dKr[o * np + o] = dKrowdSo * (krog / krocw + kr[g]) + dKrogdSo * (krow / krocw + kr[w]);
            dKr[o * np + w] = krocw * ((dKrowdSw / krocw + dKr[w * np + w]) * (krog / krocw + kr[g]) - (dKr[w * np + w]));
            dKr[o * np + g] = krocw * ((krow / krocw + kr[w]) * (dKrogdSg / krocw + dKr[g * np + g]) - (dKr[g * np + g]));
        }
        for (int j = 0; j < np; j++) {
            b->kr[n * np + j] = kr[j];
            b->Pc[n * np + j] = Pc[j];
            b->Pj[n * np + j] = b->P[n] + Pc[j];
        }
        memcpy(&b->dKrdS[n * 9], dKr, sizeof(dKr));
        memcpy(&b->dPcdS[n * 9], dPc, sizeof(dPc));
        /* OCPRockIsoT_Linear::CalPoro (src/OCPRock.cpp:19-24) */
        const double dP = (b->P[n] - m->pref);
        b->poro[n] = b->poroInit[n] * (1 + (m->cp1 + m->cp2 / 2 * dP) * dP);
        b->poroP[n] = b->poroInit[n] * (m->cp1 + m->cp2 * dP);
        b->rockVp[n] = b->v[n] * b->poro[n];
    }
}

void oc_calres(const oc_model* m, oc_bulk* b, oc_conn* c, double dt, double* res, double* resRelV, double* resRelN,
               double* norms)
{
    const int nb = b->nb, np = b->np, nc = b->nc, len = nc + 1;
    memset(res, 0, sizeof(double) * nb * len);
    memset(resRelV, 0, sizeof(double) * nb);
    memset(resRelN, 0, sizeof(double) * nb);
    /* BulkAccumuTerm01::CalResFIM (src/BulkAccumuModule.cpp:24-45) */
    for (int n = 0; n < nb; n++) {
        res[n * len] = b->rockVp[n] - b->vf[n];
        for (int i = 0; i < nc; i++) res[n * len + 1 + i] = b->Ni[n * nc + i] - b->lNi[n * nc + i];
    }
    /* OCPConvection01::CalFlux (src/OCPConvection.cpp:22-79) */
    for (int k = 0; k < c->nconn; k++) {
        const int bId = c->bId[k], eId = c->eId[k];
        const double Akd = c->trans[k];
        double flux[NCX + 1] = {0};
        for (int j = 0; j < np; j++) {
            const int bj = bId * np + j, ej = eId * np + j;
            const int exb = b->phaseExist[bj] != 0, exe = b->phaseExist[ej] != 0;
            double rho;
            if (exb && exe) rho = (b->rho[bj] + b->rho[ej]) / 2;
            else if (exb) rho = b->rho[bj];
            else if (exe) rho = b->rho[ej];
            else { c->upblock[k * np + j] = bId; c->dP[k * np + j] = 0; c->flux_vj[k * np + j] = 0; continue; }
            c->upblock[k * np + j] = bId;
            double dP = (b->Pj[bj] - m->G * rho * b->depth[bId]) - (b->Pj[ej] - m->G * rho * b->depth[eId]);
            c->dP[k * np + j] = dP;
            if (dP < 0) c->upblock[k * np + j] = eId;
            const int uj = c->upblock[k * np + j] * np + j;
            if (!b->phaseExist[uj]) { c->flux_vj[k * np + j] = 0; continue; }
            const double vj = Akd * b->kr[uj] / b->mu[uj] * dP;
            c->flux_vj[k * np + j] = vj;
            for (int i = 0; i < nc; i++) flux[i] += vj * b->xi[uj] * b->xij[uj * nc + i];
        }
        for (int i = 0; i < nc; i++) {
            c->flux_ni[k * nc + i] = flux[i];
            res[bId * len + 1 + i] += dt * flux[i];
            res[eId * len + 1 + i] -= dt * flux[i];
        }
    }
    /* relative residuals (src/IsoThermalMethod.cpp:1147-1167) */
    double mV = 0, mN = 0;
    int iV = 0, iN = 0;
    for (int n = 0; n < nb; n++) {
        for (int i = 0; i < len; i++) {
            double t = fabs(res[n * len + i] / b->rockVp[n]);
            if (mV < t) { mV = t; iV = n; }
            resRelV[n] += t * t;
        }
        resRelV[n] = sqrt(resRelV[n]);
        for (int i = 1; i < len; i++) {
            double t = fabs(res[n * len + i] / b->Nt[n]);
            if (mN < t) { mN = t; iN = n; }
            resRelN[n] += t * t;
        }
        resRelN[n] = sqrt(resRelN[n]);
    }
    for (int k = 0; k < nb * len; k++) res[k] = -1.0 * res[k];
    norms[0] = mV; norms[1] = mN; norms[2] = iV; norms[3] = iN;
}

/* OCPConvection01::AssembleMatFIM (src/OCPConvection.cpp:82-187) for one connection */
static void conn_dfdx(const oc_model* m, const oc_bulk* b, const oc_conn* c, int k, double* pB, double* pE, double* sB,
                      double* sE)
{
    const int np = b->np, nc = b->nc, n1 = nc + 1, n2 = np * nc + np;
    memset(pB, 0, sizeof(double) * n1 * n1); memset(pE, 0, sizeof(double) * n1 * n1);
    memset(sB, 0, sizeof(double) * n1 * n2); memset(sE, 0, sizeof(double) * n1 * n2);
    const int bId = c->bId[k], eId = c->eId[k];
    const double Akd = c->trans[k], dGamma = m->G * (b->depth[bId] - b->depth[eId]);
    for (int j = 0; j < np; j++) {
        const int uj = c->upblock[k * np + j] * np + j;
        if (!b->phaseExist[uj]) continue;
        const int bj = bId * np + j, ej = eId * np + j;
        int dj;
        double *pU, *pD, *sU, *sD;
        if (bj == uj) { dj = ej; pU = pB; pD = pE; sU = sB; sD = sE; }
        else { dj = bj; pU = pE; pD = pB; sU = sE; sD = sB; }
        const double wU = b->phaseExist[dj] ? 0.5 : 1, wD = b->phaseExist[dj] ? 0.5 : 0;
        const double dP = c->dP[k * np + j], xi = b->xi[uj], kr = b->kr[uj], mu = b->mu[uj];
        const double muP = b->muP[uj], xiP = b->xiP[uj], transJ = Akd * kr / mu;
        for (int i = 0; i < nc; i++) {
            const double xij = b->xij[uj * nc + i], transIJ = xij * xi * transJ;
            pB[(i + 1) * n1] += transIJ;
            pE[(i + 1) * n1] -= transIJ;
            double tmp = transJ * xiP * xij * dP;
            tmp += -transIJ * muP / mu * dP;
            pU[(i + 1) * n1] += (tmp - transIJ * wU * b->rhoP[uj] * dGamma);
            pD[(i + 1) * n1] += -transIJ * wD * b->rhoP[dj] * dGamma;
            for (int q = 0; q < np; q++) {
                sB[(i + 1) * n2 + q] += transIJ * b->dPcdS[bj * np + q];
                sE[(i + 1) * n2 + q] -= transIJ * b->dPcdS[ej * np + q];
                sU[(i + 1) * n2 + q] += Akd * b->dKrdS[uj * np + q] / mu * xi * xij * dP;
            }
            for (int q = 0; q < nc; q++) {
                const double rhox = b->rhox[uj * nc + q], xix = b->xix[uj * nc + q], mux = b->mux[uj * nc + q];
                tmp = -transIJ * wU * rhox * dGamma;
                tmp += transJ * xix * xij * dP;
                tmp += -transIJ * mux / mu * dP;
                sU[(i + 1) * n2 + np + j * nc + q] += tmp;
                sD[(i + 1) * n2 + np + j * nc + q] += -transIJ * wD * b->rhox[dj * nc + q] * dGamma;
            }
            sU[(i + 1) * n2 + np + j * nc + i] += transJ * xi * dP;
        }
    }
}

long oc_assemble(const oc_model* m, const oc_bulk* b, const oc_conn* c, double dt, uint32_t* rowptr, uint32_t* col,
                 double* val)
{
    const int nb = b->nb, np = b->np, nc = b->nc, n1 = nc + 1, n2 = np * nc + np, bs = n1 * n1;
    /* the reference's push-back matrix (OCPMatrix::NewDiag/AddDiag/NewOffDiag,
     * src/OCPMatrix.cpp:92-138): rows filled in call order */
    int* cnt = (int*)calloc(nb, sizeof(int));
    for (int k = 0; k < c->nconn; k++) { cnt[c->bId[k]]++; cnt[c->eId[k]]++; }
    rowptr[0] = 0;
    for (int n = 0; n < nb; n++) rowptr[n + 1] = rowptr[n] + 1 + cnt[n];
    int* fill = (int*)calloc(nb, sizeof(int));
    /* BulkAccumuTerm01::CaldFdXpFIM (src/BulkAccumuModule.cpp:47-71) */
    for (int n = 0; n < nb; n++) {
        double* dg = val + (size_t)rowptr[n] * bs;
        memset(dg, 0, sizeof(double) * bs);
        dg[0] = b->v[n] * b->poroP[n] - b->vfP[n];
        for (int i = 0; i < nc; i++) dg[i + 1] = -b->vfi[n * nc + i];
        for (int i = 1; i < n1; i++) dg[i * n1 + i] = 1;
        col[rowptr[n]] = n;
        fill[n] = 1;
    }
    double* pB = (double*)malloc(sizeof(double) * n1 * n1);
    double* pE = (double*)malloc(sizeof(double) * n1 * n1);
    double* sB = (double*)malloc(sizeof(double) * n1 * n2);
    double* sE = (double*)malloc(sizeof(double) * n1 * n2);
    double* bm = (double*)malloc(sizeof(double) * bs);
    const int lend = np * n1 * n1;
    for (int k = 0; k < c->nconn; k++) {
        const int bId = c->bId[k], eId = c->eId[k];
        conn_dfdx(m, b, c, k, pB, pE, sB, sE);
        for (int side = 0; side < 2; side++) {
            const double* s = side ? sE : sB;
            const double* sec = b->dSec_dPri + (size_t)(side ? eId : bId) * lend;
            /* DaABpbC (src/DenseMat.cpp:61-85): bmat = dt*dFdXs*dSec + dt*dFdXp.
             * Each element sums its products in t order.  Rows go four at a
             * time, so that each row of dSec is read once per four rows, and
             * the inner loop runs over the contiguous columns q. */
            for (int q = 0; q < bs; q++) bm[q] = 0;
            int r = 0;
            for (; r + 4 <= n1; r += 4) {
                double *a0 = bm + r * n1, *a1 = a0 + n1, *a2 = a1 + n1, *a3 = a2 + n1;
                const double *s0 = s + r * n2, *s1 = s0 + n2, *s2 = s1 + n2, *s3 = s2 + n2;
                for (int t = 0; t < n2; t++) {
                    const double* srow = sec + t * n1;
                    const double f0 = s0[t], f1 = s1[t], f2 = s2[t], f3 = s3[t];
                    for (int q = 0; q < n1; q++) {
                        const double x = srow[q];
                        a0[q] += f0 * x; a1[q] += f1 * x; a2[q] += f2 * x; a3[q] += f3 * x;
                    }
                }
            }
            for (; r < n1; r++) {
                double* acc = bm + r * n1;
                for (int t = 0; t < n2; t++) {
                    const double a = s[r * n2 + t];
                    const double* srow = sec + t * n1;
                    for (int q = 0; q < n1; q++) acc[q] += a * srow[q];
                }
            }
            {
                const double* pp = side ? pE : pB;
                for (int q = 0; q < bs; q++) bm[q] = dt * bm[q] + dt * pp[q];
            }
            if (side == 0) {
                double* dg = val + (size_t)rowptr[bId] * bs;
                for (int q = 0; q < bs; q++) dg[q] += bm[q];                    /* AddDiag(bId) */
                double* off = val + (size_t)(rowptr[eId] + fill[eId]) * bs;    /* NewOffDiag(eId, bId) */
                for (int q = 0; q < bs; q++) off[q] = -1.0 * bm[q];
                col[rowptr[eId] + fill[eId]++] = bId;
            }
            else {
                double* off = val + (size_t)(rowptr[bId] + fill[bId]) * bs;    /* NewOffDiag(bId, eId) */
                for (int q = 0; q < bs; q++) off[q] = bm[q];
                col[rowptr[bId] + fill[bId]++] = eId;
                double* dg = val + (size_t)rowptr[eId] * bs;
                for (int q = 0; q < bs; q++) dg[q] += -1.0 * bm[q];             /* AddDiag(eId) */
            }
        }
    }
    free(pB); free(pE); free(sB); free(sE); free(bm); free(cnt); free(fill);
    return rowptr[nb];
}

void oc_newton_update(const oc_model* m, oc_bulk* b, const double* u, double dSmax)
{
    (void)m;
    const int np = b->np, nc = b->nc, row = np * (nc + 1), col = nc + 1;
#pragma omp parallel for schedule(static)
    for (int n = 0; n < b->nb; n++) {
        double dtmp[NPH * (NCX + 2)];
        const double* A = b->dSec_dPri + (size_t)n * b->np * (nc + 1) * (nc + 1);
        /* OCP_aAxpby (include/DenseMat.hpp:211-219) */
        for (int i = 0; i < row; i++) {
            dtmp[i] = 1.0 * 0.0;
            for (int j = 0; j < col; j++) dtmp[i] += 1.0 * A[i * col + j] * u[n * col + j];
        }
        double chopmin = 1;
        for (int j = 0; j < np; j++) {
            double choptmp = 1;
            if (fabs(dtmp[j]) > dSmax) choptmp = dSmax / fabs(dtmp[j]);
            else if (b->S[n * np + j] + dtmp[j] < 0.0) choptmp = 0.9 * b->S[n * np + j] / fabs(dtmp[j]);
            chopmin = choptmp < chopmin ? choptmp : chopmin;
        }
        for (int j = 0; j < np; j++) b->S[n * np + j] += chopmin * dtmp[j];
        int js = np;
        for (int j = 0; j < np; j++)
            for (int i = 0; i < nc; i++) b->xij[(n * np + j) * nc + i] += chopmin * dtmp[js++];
        b->P[n] += u[n * col];
        for (int i = 0; i < nc; i++) b->Ni[n * nc + i] += chopmin * u[n * col + 1 + i];
    }
}
