// Peng-Robinson EoS for one cell at fixed (P, T), following EoS_PR
// (src/OCPEoS.cpp:19-414) and CubicRoot/NTcubicroot (src/UtilMath.cpp:15-80).
//
// GB300 layout decisions:
//  * Ai, Bi and the mixing factors sqrt(Ai*Ak) depend only on (P, T); the
//    reference recomputes them (NC pow + NC^2 sqrt) on every EoS call.  They
//    are computed once per flash here; every arithmetic expression is kept in
//    the reference's evaluation order, so the hoisting changes no bits.
//  * Loop-invariant logarithms and denominators are computed once per call.
//  * All arrays are per-thread (registers / local memory), sized by the
//    template capacity NCM; the runtime component count is nc <= NCM.
#pragma once
#include "ocpx_common.cuh"

namespace ocpx {

template <int NCM>
struct EosPR {
    int nc;
    double P, T;
    const CompModel* m;
    double Ai[NCM], Bi[NCM];
    double s[NCM * NCM];  // sqrt(Ai[i] * Ai[k])
    double s2[NCM * NCM]; // 2 * (1 - BIC_ik) * sqrt(Ai[i] * Ai[k]), the factor of CalFug/CalFugPhi's sum
    // per-call scratch
    double Aj, Bj, Zj;
    double Ax[NCM], Zx[NCM], An[NCM], Bn[NCM], Zn[NCM];
    double Ap, Bp, Zp;

    // EoS_PR::CalAiBi (src/OCPEoS.cpp:68-84) + the sqrt table
    OCPX_HD void setup(const CompModel* model, double gas_constant, double Pin, double Tin)
    {
        m = model;
        m_gas = gas_constant;
        nc = model->nc;
        P = Pin;
        T = Tin;
        for (int i = 0; i < nc; i++) {
            const double mwi = m->mwi[i];
            const double Pri = P / m->Pc[i];
            const double Tri = T / m->Tc[i];
            const double q = 1 + mwi * (1 - sqrt(Tri));
            Ai[i] = m->OmegaA[i] * Pri / (Tri * Tri) * (q * q);
            Bi[i] = m->OmegaB[i] * Pri / Tri;
        }
        for (int i = 0; i < nc; i++)
            for (int k = 0; k <= i; k++) {
                const double v = sqrt(Ai[i] * Ai[k]);
                s[i * NCM + k] = v;
                s[k * NCM + i] = v;
            }
        for (int i = 0; i < nc; i++)
            for (int k = 0; k < nc; k++) s2[i * NCM + k] = 2 * omb(i, k) * s[i * NCM + k];
    }

    OCPX_HD double omb(int i, int k) const { return m->omb[i * NC_MAX + k]; }

    // EoS_PR::CalAjBj (:87-99)
    OCPX_HD void cal_AjBj(const double* x)
    {
        Aj = 0;
        Bj = 0;
        for (int i1 = 0; i1 < nc; i1++) {
            Bj += Bi[i1] * x[i1];
            Aj += x[i1] * x[i1] * Ai[i1] * omb(i1, i1);
            for (int i2 = 0; i2 < i1; i2++) {
                Aj += 2 * x[i1] * x[i2] * s[i1 * NCM + i2] * omb(i1, i2);
            }
        }
    }

    // NTcubicroot (src/UtilMath.cpp:56-80)
    OCPX_HD static void nt_cubic(double& root, double a, double b, double c)
    {
        double e = root * (root * (root + a) + b) + c;
        double df;
        double iter = 0;
        double optroot = root;
        double opte = fabs(e);
        while (fabs(e) > 1E-8) {
            df = root * (3 * root + 2 * a) + b;
            root = root - e / df;
            iter++;
            if (iter > 10) break;
            e = root * (root * (root + a) + b) + c;
            if (fabs(e) <= opte) {
                opte = fabs(e);
                optroot = root;
            }
        }
        root = optroot;
    }

    // CubicRoot (src/UtilMath.cpp:15-53) with Newton refinement, roots sorted
    OCPX_HD_NOINLINE static int cubic_root(double a, double b, double c, double* z)
    {
        const double Q = (a * a - 3 * b) / 9;
        const double R = (2 * a * a * a - 9 * a * b + 27 * c) / 54;
        const double Q3 = Q * Q * Q;
        const double M = R * R - Q3;
        if (M <= 0) {
            const double theta = acos(R / sqrt(Q3));
            z[0] = -2 * sqrt(Q) * cos(theta / 3) - a / 3;
            z[1] = -2 * sqrt(Q) * cos((theta + 2 * PI_REF) / 3) - a / 3;
            z[2] = -2 * sqrt(Q) * cos((theta - 2 * PI_REF) / 3) - a / 3;
            nt_cubic(z[0], a, b, c);
            nt_cubic(z[1], a, b, c);
            nt_cubic(z[2], a, b, c);
            // sort ascending (std::sort on three values)
            double t;
            if (z[1] < z[0]) { t = z[0]; z[0] = z[1]; z[1] = t; }
            if (z[2] < z[1]) { t = z[1]; z[1] = z[2]; z[2] = t; }
            if (z[1] < z[0]) { t = z[0]; z[0] = z[1]; z[1] = t; }
            return 3;
        }
        const double tmp1 = -R + sqrt(M);
        const double tmp2 = R + sqrt(M);
        const double S = sign_d(tmp1) * pow_third(fabs(tmp1));
        const double Tt = -sign_d(tmp2) * pow_third(fabs(tmp2));
        z[0] = S + Tt - a / 3;
        nt_cubic(z[0], a, b, c);
        return 1;
    }

    // EoS_PR::CalZj (:102-124): the root of smaller Gibbs energy
    OCPX_HD static double zj_of(double Aj, double Bj)
    {
        const double a = (DELTA1 + DELTA2 - 1) * Bj - 1;
        const double b = (Aj + DELTA1 * DELTA2 * Bj * Bj - (DELTA1 + DELTA2) * Bj * (Bj + 1));
        const double c = -(Aj * Bj + DELTA1 * DELTA2 * Bj * Bj * (Bj + 1));
        double z[3];
        const int flag = cubic_root(a, b, c, z);
        if (flag == 1) return z[0];
        const double zj1 = z[0];
        const double zj2 = z[2];
        const double dG = (zj2 - zj1) + log((zj1 - Bj) / (zj2 - Bj)) -
                          Aj / (Bj * (DELTA2 - DELTA1)) *
                              log((zj1 + DELTA1 * Bj) * (zj2 + DELTA2 * Bj) /
                                  ((zj1 + DELTA2 * Bj) * (zj2 + DELTA1 * Bj)));
        return dG > 0 ? zj1 : zj2;
    }
    OCPX_HD void cal_Zj() { Zj = zj_of(Aj, Bj); }

    OCPX_HD void cal_AjBjZj(const double* x)
    {
        cal_AjBj(x);
        cal_Zj();
    }

    // numerator factor and denominator shared by Zx, Zn, Zp (:127-180)
    OCPX_HD static double dz_num_of(double Aj, double Bj, double Zj)
    {
        return (Aj + (DELTA1 * DELTA2) * (3 * Bj * Bj + 2 * Bj)) +
               ((DELTA1 + DELTA2) * (2 * Bj + 1) - 2 * (DELTA1 * DELTA2) * Bj) * Zj -
               ((DELTA1 + DELTA2) - 1) * Zj * Zj;
    }
    OCPX_HD static double dz_den_of(double Aj, double Bj, double Zj)
    {
        return (3 * Zj * Zj + 2 * (((DELTA1 + DELTA2) - 1) * Bj - 1) * Zj +
                (Aj + (DELTA1 * DELTA2) * Bj * Bj - (DELTA1 + DELTA2) * Bj * (Bj + 1)));
    }
    OCPX_HD double dz_num() const { return dz_num_of(Aj, Bj, Zj); }
    OCPX_HD double dz_den() const { return dz_den_of(Aj, Bj, Zj); }

    // EoS_PR::CalAxBxZx (:127-143); Bx == Bi
    OCPX_HD_NOINLINE void cal_AxZx(const double* x)
    {
        const double num = dz_num(), den = dz_den();
        for (int i = 0; i < nc; i++) {
            double tmp = 0;
            for (int k = 0; k < nc; k++) tmp += x[k] * omb(i, k) * s[i * NCM + k];
            Ax[i] = 2 * tmp;
            Zx[i] = ((Bj - Zj) * Ax[i] + num * Bi[i]) / den;
        }
    }

    // EoS_PR::CalAnBnZn (:146-161)
    OCPX_HD_NOINLINE void cal_AnBnZn(const double* x, double nt)
    {
        const double num = dz_num(), den = dz_den();
        for (int i = 0; i < nc; i++) {
            double tmp = 0;
            for (int mm = 0; mm < nc; mm++) tmp += omb(i, mm) * s[i * NCM + mm] * x[mm];
            An[i] = 2 / nt * (tmp - Aj);
            Bn[i] = 1 / nt * (Bi[i] - Bj);
            Zn[i] = ((Bj - Zj) * An[i] + num * Bn[i]) / den;
        }
    }

    // EoS_PR::CalApBpZp (:164-173)
    OCPX_HD void cal_ApBpZp()
    {
        Ap = Aj / P;
        Bp = Bj / P;
        Zp = ((Bj - Zj) * Ap + dz_num() * Bp) / dz_den();
    }

    // sum_k 2 (1-BIC_ik) sqrt(Ai Ak) x_k, as CalFug/CalFugPhi form it
    OCPX_HD double mix2(int i, const double* x) const
    {
        double tmp = 0;
        for (int k = 0; k < nc; k++) tmp += s2[i * NCM + k] * x[k];  // (2 * omb * s) * x
        return tmp;
    }
    // sum_k (1-BIC_ik) sqrt(Ai Ak) x_k, as CalLnFugN/P/PhiN form it
    OCPX_HD double mix1(int i, const double* x) const
    {
        double tmp = 0;
        for (int k = 0; k < nc; k++) tmp += omb(i, k) * s[i * NCM + k] * x[k];
        return tmp;
    }

    // EoS_PR::CalFugPhi (:199-214); phi may be null (CalFug, :183-196)
    OCPX_HD_NOINLINE void cal_fug_phi(const double* x, double* fug, double* phi)
    {
        cal_AjBjZj(x);
        const double l1 = log(Zj - Bj);
        const double lg = log((Zj + DELTA1 * Bj) / (Zj + DELTA2 * Bj));
        const double c1 = Aj / (DELTA1 - DELTA2) / Bj;
        for (int i = 0; i < nc; i++) {
            const double tmp = mix2(i, x);
            const double ph = exp(Bi[i] / Bj * (Zj - 1) - l1 - c1 * (tmp / Aj - Bi[i] / Bj) * lg);
            if (phi) phi[i] = ph;
            fug[i] = ph * x[i] * P;
        }
    }

    // EoS_PR::CalLnFugX (:217-251), result row-major [i*nc + k]
    OCPX_HD_NOINLINE void cal_lnfugX(const double* x, double* lnfugx)
    {
        cal_AjBjZj(x);
        cal_AxZx(x);
        const double G = (Zj + DELTA1 * Bj) / (Zj + DELTA2 * Bj);
        const double lG = log(G);
        const double zb = Zj - Bj;
        const double gden = (DELTA1 - DELTA2) / (Zj + DELTA2 * Bj) / (Zj + DELTA2 * Bj);
        for (int i = 0; i < nc; i++) {
            const double C = x[i] * P / zb;
            const double E = -Aj / ((DELTA1 - DELTA2) * Bj) * (Ax[i] / Aj - Bi[i] / Bj);
            for (int k = 0; k < nc; k++) {
                const double aik = omb(i, k) * s[i * NCM + k];
                const double Cxk = (zb * (i == k ? 1.0 : 0.0) - x[i] * (Zx[k] - Bi[k])) * P / (zb * zb);
                const double Dxk = Bi[i] / Bj * (Zx[k] - Bi[k] * (Zj - 1) / Bj);
                double Exk = (2 * (Aj / Bj * Bi[k] * Bi[i] + Bj * aik) - Ax[i] * Bi[k] - Ax[k] * Bi[i]) / (Bj * Bj);
                Exk /= -(DELTA1 - DELTA2);
                const double Gxk = gden * (Zj * Bi[k] - Zx[k] * Bj);
                lnfugx[i * nc + k] = 1 / C * Cxk + Dxk + Exk * lG + E / G * Gxk;
            }
        }
    }

    // EoS_PR::CalLnFugN (:254-300) and CalLnPhiN (:343-382) share the Enk/Dnk/Gnk terms
    template <bool PHI>
    OCPX_HD_NOINLINE void cal_lnN(const double* x, double nt, double* out)
    {
        cal_AjBjZj(x);
        cal_AnBnZn(x, nt);
        const double G = (Zj + DELTA1 * Bj) / (Zj + DELTA2 * Bj);
        const double lG = log(G);
        const double zb = Zj - Bj;
        const double gden = (DELTA1 - DELTA2) / ((Zj + DELTA2 * Bj) * (Zj + DELTA2 * Bj));
        const double eden = -1 / (DELTA1 - DELTA2) / (Bj * Bj);
        for (int i = 0; i < nc; i++) {
            const double C = PHI ? 1 / zb : x[i] * P / zb;
            const double tmp = mix1(i, x);
            const double E = -Aj / ((DELTA1 - DELTA2) * Bj) * (2 * tmp / Aj - Bi[i] / Bj);
            for (int k = 0; k <= i; k++) {
                const double aik = omb(i, k) * s[i * NCM + k];
                double Cnk;
                if (PHI)
                    Cnk = (Bn[k] - Zn[k]) / (zb * zb);
                else
                    Cnk = P / zb / zb * (zb / nt * ((i == k ? 1.0 : 0.0) - x[i]) - x[i] * (Zn[k] - Bn[k]));
                const double Dnk = Bi[i] / Bj * (Zn[k] - (Bi[k] - Bj) * (Zj - 1) / (nt * Bj));
                const double Gnk = gden * (Bn[k] * Zj - Zn[k] * Bj);
                double Enk = eden * (2 * (Bj * aik / nt + Bn[k] * (Bi[i] * Aj / Bj - tmp)) - An[k] * Bi[i] - Aj * Bi[i] / nt);
                Enk -= E / nt;
                const double v = 1 / C * Cnk + Dnk + Enk * lG + E / G * Gnk;
                out[i * nc + k] = v;
                out[k * nc + i] = v;
            }
        }
    }
    OCPX_HD void cal_lnfugN(const double* x, double nt, double* out) { cal_lnN<false>(x, nt, out); }
    OCPX_HD void cal_lnphiN(const double* x, double nt, double* out) { cal_lnN<true>(x, nt, out); }

    // EoS_PR::CalLnFugP (:303-340)
    OCPX_HD_NOINLINE void cal_lnfugP(const double* x, double* lnfugP)
    {
        cal_AjBjZj(x);
        cal_ApBpZp();
        const double G = (Zj + DELTA1 * Bj) / (Zj + DELTA2 * Bj);
        const double Gp = (DELTA1 - DELTA2) / ((Zj + DELTA2 * Bj) * (Zj + DELTA2 * Bj)) * (Bp * Zj - Zp * Bj);
        const double C = P / (Zj - Bj);
        const double Cp = ((Zj - Bj) - P * (Zp - Bp)) / ((Zj - Bj) * (Zj - Bj));
        for (int i = 0; i < nc; i++) {
            const double tmp = mix1(i, x);
            const double E = -Aj / ((DELTA1 - DELTA2) * Bj) * (2 * tmp / Aj - Bi[i] / Bj);
            const double Dp = Bi[i] / Bj * Zp;
            lnfugP[i] = Cp / C + Dp + E / G * Gp;
        }
    }

    // EoS_PR::CalVmDer (:396-414)
    OCPX_HD_NOINLINE double cal_vm_der(const double* x, double& vmP, double* vmx)
    {
        cal_AjBjZj(x);
        cal_AxZx(x);
        cal_ApBpZp();
        const double CgTP = m_gas * T / P;
        double v = Zj * CgTP;
        for (int i = 0; i < nc; i++) v -= x[i] * m->Vshift[i];
        for (int i = 0; i < nc; i++) vmx[i] = CgTP * Zx[i] - m->Vshift[i];
        vmP = CgTP * (Zp - Zj / P);
        return v;
    }
    double m_gas;
};

}  // namespace ocpx
