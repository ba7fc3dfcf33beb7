// Phase equilibrium of one cell on a whole warp, for the cells whose
// equilibrium ran over the work budget of the one-thread-per-cell kernel.
//
// Why: on GB300 an FP64 warp instruction costs the same 64 issue cycles of
// an SM sub-partition whether it carries 1 active lane or 32, so a cell that
// needs thousands of serial SSM iterations sets the time of the whole flash.
// Spreading that cell over a warp shortens its instruction stream:
//   * lane i of each half-warp owns EoS component i (NC <= 16);
//   * in the phase split the two half-warps evaluate the two phases at once;
//   * in the stability test the two half-warps run two Wilson starts at once
//     (speculatively), and the results are merged in the reference's order,
//     so iteration counts, flags and the deciding trial are the ones the
//     sequential algorithm produces.
// Every sum over components keeps the reference's sequential order (terms are
// formed in parallel, then added one by one), and every expression is the one
// in CompFlash / EosPR, so the result is bit-identical to the thread version
// (OCPPhaseEquilibrium, src/OCPPhaseEquilibrium.cpp:71-1010; EoS_PR,
// src/OCPEoS.cpp:68-414).  The small Newton systems are solved by one lane
// per half with the thread version's solver, in shared memory.
//
// Synchronisation: every __syncwarp and shuffle below is reached by all 32
// lanes; loops whose trip count differs between the halves run while any
// half is active and commit state only in the active half.
#pragma once
#include "flash_comp.cuh"

namespace ocpx {

constexpr unsigned FULL_MASK = 0xffffffffu;
constexpr int COOP_WARPS = 2;  // warps (cells in flight) per block
constexpr int EXCL_WARPS = 4;  // warps per block of the SM-exclusive form: one per SM sub-partition
constexpr int FUSED_WARPS = 4; // warps per block of the fused batched flash

template <int NCM>
struct CoopSh {
    double Ai[NCM], Bi[NCM];
    double s[NCM * NCM], omb[NCM * NCM];
    double s2[NCM * NCM];         // 2 (1 - BIC) sqrt(Ai Ak), the factor of CalFugPhi's sum
    double xs[2][NCM];            // EoS input composition of each half
    double tA[2][NCM * NCM];      // Aj terms
    double tB[2][NCM];            // Bj terms
    double v1[2][NCM], v2[2][NCM];  // ordered-sum terms
    double K[2][NCM];             // K values for the Rachford-Rice bracket
    double fg[2][NCM], ph[2][NCM];  // fugacity / phi exchange between the halves
    double d1[2][NCM], d2[2][NCM], d3[2][NCM];  // An/Ax, Bn, Zn/Zx
    double lnf[2][NCM * NCM];
    double J[2][NCM * NCM];
    double W[2][NCM * NCM];
    double r[2][NCM];
};

template <int NCM>
struct CoopPE {
    CoopSh<NCM>& sh;
    const CompModel& m;
    const int NC;
    const int lane, h, i, ic;
    const bool act;
    double P, T;
    // own component
    double z, Ai, Bi;
    double Kw0, Kw1, Kw2, Kw3;
    double Ks, lKs;
    double x0, x1;   // compositions of the two phases, own component
    // cell state (uniform across the warp)
    int ftype;
    unsigned lNP;
    int NP;
    double nu0, nu1, Yt;
    bool ssm_sta_conv, nr_sta_conv, ssm_sp_conv, nr_sp_conv;
    int it_ssm_sta, it_nr_sta, it_ssm_sp, it_nr_sp, it_rr;
    uint32_t status;
    // EoS scalars of the half's last evaluation
    double Aj, Bj, Zj;

    __device__ CoopPE(CoopSh<NCM>& shm, const CompModel& model)
        : sh(shm), m(model), NC(model.nc), lane(threadIdx.x & 31), h((threadIdx.x & 31) >> 4),
          i(threadIdx.x & 15), ic((threadIdx.x & 15) < model.nc ? (threadIdx.x & 15) : 0),
          act((threadIdx.x & 15) < model.nc)
    {
    }

    __device__ double kw(int k) const { return k == 0 ? Kw0 : (k == 1 ? Kw1 : (k == 2 ? Kw2 : Kw3)); }
    __device__ double omb(int a, int c) const { return sh.omb[a * NCM + c]; }

    // sum of one term per component, added in component order (per half)
    __device__ double osum(double term)
    {
        double* v = sh.v1[h];
        if (act) v[i] = term;
        __syncwarp();
        double acc = 0;
#pragma unroll
        for (int k = 0; k < NCM; k++)
            if (k < NC) acc += v[k];
        __syncwarp();
        return acc;
    }

    __device__ void set_x(double xv)
    {
        if (act) sh.xs[h][i] = xv;
        __syncwarp();
    }

    // ------------------------------------------------------------ EoS ----
    // EoS_PR::CalAiBi + the sqrt(Ai Ak) table (EosPR::setup)
    __device__ void setup(double gas_constant)
    {
        (void)gas_constant;
        if (act) {
            const double mwi = m.mwi[i];
            const double Pri = P / m.Pc[i];
            const double Tri = T / m.Tc[i];
            const double q = 1 + mwi * (1 - sqrt(Tri));
            Ai = m.OmegaA[i] * Pri / (Tri * Tri) * (q * q);
            Bi = m.OmegaB[i] * Pri / Tri;
            if (h == 0) {
                sh.Ai[i] = Ai;
                sh.Bi[i] = Bi;
                for (int k = 0; k < NC; k++) sh.omb[i * NCM + k] = m.omb[i * NC_MAX + k];
            }
        }
        else {
            Ai = 0;
            Bi = 0;
        }
        __syncwarp();
        if (act && h == 0)
            for (int k = 0; k <= i; k++) {
                const double v = sqrt(sh.Ai[i] * sh.Ai[k]);
                sh.s[i * NCM + k] = v;
                sh.s[k * NCM + i] = v;
            }
        __syncwarp();
        if (act && h == 0)
            for (int k = 0; k < NC; k++) sh.s2[i * NCM + k] = 2 * omb(i, k) * sh.s[i * NCM + k];
        __syncwarp();
    }

    // EoS_PR::CalAjBj for the half's composition
    __device__ void AjBj()
    {
        const double* x = sh.xs[h];
        double* tA = sh.tA[h];
        double* tB = sh.tB[h];
        if (act) {
            const double xi = x[i];
            tB[i] = Bi * xi;
            tA[i * NCM + i] = xi * xi * Ai * omb(i, i);
            for (int k = 0; k < i; k++) tA[i * NCM + k] = 2 * xi * x[k] * sh.s[i * NCM + k] * omb(i, k);
        }
        __syncwarp();
        double a = 0, bsum = 0;
#pragma unroll
        for (int i1 = 0; i1 < NCM; i1++) {
            if (i1 < NC) {
                bsum += tB[i1];
                a += tA[i1 * NCM + i1];
#pragma unroll
                for (int i2 = 0; i2 < i1; i2++) a += tA[i1 * NCM + i2];
            }
        }
        Aj = a;
        Bj = bsum;
        __syncwarp();
    }

    // EoS_PR::CalZj with CubicRoot, the independent operations spread over
    // lanes of the half so that one warp instruction sequence serves several
    // of them: the two divisions of Q and R (lanes 0-1), the square roots
    // (lanes 0-1), the three trigonometric roots and their Newton refinements
    // (lanes 0-2) or the two Cardano cube roots (lanes 0-1), and the two
    // logarithms of the Gibbs-energy test (lanes 0-1).  The expressions are
    // those of EosPR::zj_of / cubic_root / nt_cubic, so the bits are the same.
    // Every shuffle is made by the whole warp, outside the branches (the two
    // halves may be in different root cases).
    __device__ double zj_lanes() const
    {
        const int hb = h * 16;
        const double a = (DELTA1 + DELTA2 - 1) * Bj - 1;
        const double b = (Aj + DELTA1 * DELTA2 * Bj * Bj - (DELTA1 + DELTA2) * Bj * (Bj + 1));
        const double c = -(Aj * Bj + DELTA1 * DELTA2 * Bj * Bj * (Bj + 1));
        // lane 1: R = (2a^3 - 9ab + 27c) / 54, the others Q = (a^2 - 3b) / 9 (one division)
        const double qr = ((i == 1) ? (2 * a * a * a - 9 * a * b + 27 * c) : (a * a - 3 * b)) / ((i == 1) ? 54.0 : 9.0);
        const double Q = __shfl_sync(FULL_MASK, qr, hb);
        const double R = __shfl_sync(FULL_MASK, qr, hb + 1);
        const double Q3 = Q * Q * Q;
        const double M = R * R - Q3;
        const bool three = M <= 0;
        const double sv = sqrt(three ? (i == 1 ? Q : Q3) : M);
        const double s0 = __shfl_sync(FULL_MASK, sv, hb);
        const double s1 = __shfl_sync(FULL_MASK, sv, hb + 1);
        double zl;
        if (three) {
            const double theta = acos(R / s0);
            const double t = (i == 1) ? (theta + 2 * PI_REF) : (i == 2 ? (theta - 2 * PI_REF) : theta);
            zl = -2 * s1 * cos(t / 3) - a / 3;
        }
        else {
            const double tmp1 = -R + s0;
            const double tmp2 = R + s0;
            zl = pow_third(fabs(i == 1 ? tmp2 : tmp1));
        }
        const double c0 = __shfl_sync(FULL_MASK, zl, hb);
        const double c1 = __shfl_sync(FULL_MASK, zl, hb + 1);
        if (!three) {
            const double tmp1 = -R + s0;
            const double tmp2 = R + s0;
            const double S = sign_d(tmp1) * c0;
            const double Tt = -sign_d(tmp2) * c1;
            zl = S + Tt - a / 3;
        }
        EosPR<NCM>::nt_cubic(zl, a, b, c);
        const double r0 = __shfl_sync(FULL_MASK, zl, hb);
        const double r1 = __shfl_sync(FULL_MASK, zl, hb + 1);
        const double r2 = __shfl_sync(FULL_MASK, zl, hb + 2);
        double zj1 = r0, zj2 = r0, lv = 0;
        if (three) {
            double z0 = r0, z1 = r1, z2 = r2, t;
            if (z1 < z0) { t = z0; z0 = z1; z1 = t; }
            if (z2 < z1) { t = z1; z1 = z2; z2 = t; }
            if (z1 < z0) { t = z0; z0 = z1; z1 = t; }
            zj1 = z0;
            zj2 = z2;
            const double num = (i == 1) ? (zj1 + DELTA1 * Bj) * (zj2 + DELTA2 * Bj) : zj1 - Bj;
            const double den = (i == 1) ? ((zj1 + DELTA2 * Bj) * (zj2 + DELTA1 * Bj)) : zj2 - Bj;
            lv = log(num / den);
        }
        const double lA = __shfl_sync(FULL_MASK, lv, hb);
        const double lB = __shfl_sync(FULL_MASK, lv, hb + 1);
        if (!three) return r0;
        const double dG = (zj2 - zj1) + lA - Aj / (Bj * (DELTA2 - DELTA1)) * lB;
        return dG > 0 ? zj1 : zj2;
    }

    // EoS_PR::CalFugPhi: fugacity and phi of the own component.  Divisions
    // share instruction sequences across lanes: the logarithm arguments and
    // Aj/(d1-d2) in one, then Bi/Bj, tmp/Aj and c1 (secondary lanes i+8 when
    // NC <= 8, otherwise in sequence).
    __device__ void fug_phi(double& fug, double& phi)
    {
        AjBj();
        Zj = zj_lanes();
        const int hb = h * 16;
        const double num1 = (i == 1) ? Zj + DELTA1 * Bj : (i == 2 ? Aj : Zj - Bj);
        const double den1 = (i == 1) ? Zj + DELTA2 * Bj : (i == 2 ? (DELTA1 - DELTA2) : 1.0);
        const double q1 = num1 / den1;
        const double lv = log(q1);
        const double l1 = __shfl_sync(FULL_MASK, lv, hb);
        const double lg = __shfl_sync(FULL_MASK, lv, hb + 1);
        const double c1a = __shfl_sync(FULL_MASK, q1, hb + 2);
        const double* x = sh.xs[h];
        const bool paired = NC <= 8;
        const int comp = (paired && i >= 8) ? i - 8 : ic;
        const int cc = comp < NC ? comp : 0;
        double tmp = 0;
        // (2 * omb * s) * x in the reference's association; the factor is precomputed
        for (int k = 0; k < NC; k++) tmp += sh.s2[cc * NCM + k] * x[k];
        double BiBj, tA, c1;
        if (paired) {
            // lane i: Bi/Bj; lane i+8: tmp/Aj of component i; lane 15 (free when NC <= 7): c1
            const bool second = i >= 8;
            const double num = second ? (i == 15 && NC <= 7 ? c1a : tmp) : Bi;
            const double den = second ? (i == 15 && NC <= 7 ? Bj : Aj) : Bj;
            const double q = num / den;
            const double qo = __shfl_xor_sync(FULL_MASK, q, 8);
            BiBj = q;
            tA = qo;
            c1 = (NC <= 7) ? __shfl_sync(FULL_MASK, q, hb + 15) : c1a / Bj;
        }
        else {
            BiBj = Bi / Bj;
            tA = tmp / Aj;
            c1 = c1a / Bj;
        }
        const double ph = exp(BiBj * (Zj - 1) - l1 - c1 * (tA - BiBj) * lg);
        phi = ph;
        fug = ph * x[ic] * P;
    }

    // EoS_PR::CalLnFugX into sh.lnf[h] (row-major, leading dimension NC)
    __device__ void lnfugX()
    {
        AjBj();
        Zj = zj_lanes();
        const double* x = sh.xs[h];
        const double num = EosPR<NCM>::dz_num_of(Aj, Bj, Zj), den = EosPR<NCM>::dz_den_of(Aj, Bj, Zj);
        double tmp = 0;
        for (int k = 0; k < NC; k++) tmp += x[k] * omb(ic, k) * sh.s[ic * NCM + k];
        const double Axi = 2 * tmp;
        const double Zxi = ((Bj - Zj) * Axi + num * Bi) / den;
        if (act) {
            sh.d1[h][i] = Axi;
            sh.d3[h][i] = Zxi;
        }
        __syncwarp();
        const double G = (Zj + DELTA1 * Bj) / (Zj + DELTA2 * Bj);
        const double lG = log(G);
        const double zb = Zj - Bj;
        const double gden = (DELTA1 - DELTA2) / (Zj + DELTA2 * Bj) / (Zj + DELTA2 * Bj);
        const double* Ax = sh.d1[h];
        const double* Zx = sh.d3[h];
        if (act) {
            const double xi = x[i];
            const double C = xi * P / zb;
            const double E = -Aj / ((DELTA1 - DELTA2) * Bj) * (Axi / Aj - Bi / Bj);
            for (int k = 0; k < NC; k++) {
                const double aik = omb(i, k) * sh.s[i * NCM + k];
                const double Bik = sh.Bi[k];
                const double Cxk = (zb * (i == k ? 1.0 : 0.0) - xi * (Zx[k] - Bik)) * P / (zb * zb);
                const double Dxk = Bi / Bj * (Zx[k] - Bik * (Zj - 1) / Bj);
                double Exk = (2 * (Aj / Bj * Bik * Bi + Bj * aik) - Axi * Bik - Ax[k] * Bi) / (Bj * Bj);
                Exk /= -(DELTA1 - DELTA2);
                const double Gxk = gden * (Zj * Bik - Zx[k] * Bj);
                sh.lnf[h][i * NC + k] = 1 / C * Cxk + Dxk + Exk * lG + E / G * Gxk;
            }
        }
        __syncwarp();
    }

    // EoS_PR::CalLnFugN into sh.lnf[h] (symmetric, leading dimension NC)
    __device__ void lnfugN(double nt)
    {
        AjBj();
        Zj = zj_lanes();
        const double* x = sh.xs[h];
        const double num = EosPR<NCM>::dz_num_of(Aj, Bj, Zj), den = EosPR<NCM>::dz_den_of(Aj, Bj, Zj);
        double tmp = 0;
        for (int k = 0; k < NC; k++) tmp += omb(ic, k) * sh.s[ic * NCM + k] * x[k];
        const double Ani = 2 / nt * (tmp - Aj);
        const double Bni = 1 / nt * (Bi - Bj);
        const double Zni = ((Bj - Zj) * Ani + num * Bni) / den;
        if (act) {
            sh.d1[h][i] = Ani;
            sh.d2[h][i] = Bni;
            sh.d3[h][i] = Zni;
        }
        __syncwarp();
        const double G = (Zj + DELTA1 * Bj) / (Zj + DELTA2 * Bj);
        const double lG = log(G);
        const double zb = Zj - Bj;
        const double gden = (DELTA1 - DELTA2) / ((Zj + DELTA2 * Bj) * (Zj + DELTA2 * Bj));
        const double eden = -1 / (DELTA1 - DELTA2) / (Bj * Bj);
        const double* An = sh.d1[h];
        const double* Bn = sh.d2[h];
        const double* Zn = sh.d3[h];
        double* out = sh.lnf[h];
        if (act) {
            const double xi = x[i];
            const double C = xi * P / zb;
            const double E = -Aj / ((DELTA1 - DELTA2) * Bj) * (2 * tmp / Aj - Bi / Bj);
            for (int k = 0; k <= i; k++) {
                const double aik = omb(i, k) * sh.s[i * NCM + k];
                const double Cnk = P / zb / zb * (zb / nt * ((i == k ? 1.0 : 0.0) - xi) - xi * (Zn[k] - Bn[k]));
                const double Dnk = Bi / Bj * (Zn[k] - (sh.Bi[k] - Bj) * (Zj - 1) / (nt * Bj));
                const double Gnk = gden * (Bn[k] * Zj - Zn[k] * Bj);
                double Enk = eden * (2 * (Bj * aik / nt + Bn[k] * (Bi * Aj / Bj - tmp)) - An[k] * Bi - Aj * Bi / nt);
                Enk -= E / nt;
                const double v = 1 / C * Cnk + Dnk + Enk * lG + E / G * Gnk;
                out[i * NC + k] = v;
                out[k * NC + i] = v;
            }
        }
        __syncwarp();
    }

    // ------------------------------------------------------ stability ----
    // CalKwilson, own component
    __device__ void cal_kwilson()
    {
        if (act) {
            Kw0 = (m.Pc[i] / P) * exp(5.373 * (1 + m.acf[i]) * (1 - m.Tc[i] / T));
            Kw1 = 1 / Kw0;
            Kw2 = pow_third(Kw0);
            Kw3 = pow_third(Kw1);
        }
        else {
            Kw0 = Kw1 = Kw2 = Kw3 = 1;
        }
    }

    // StableNR from the half's state; returns the half's flag, iterations and
    // status bits.  Y, yt, fS are updated in place (the half's trial).
    __device__ void stable_nr_half(double& Y, double& yt, double& fS, double fug0, bool& flag, int& iters,
                                   uint32_t& st)
    {
        double res = log(fug0 / (fS * yt));
        double Se = sqrt(osum(res * res));
        const int maxIt = m.nr_sta_maxit;
        const double Stol = m.nr_sta_tol;
        const double alpha = 1;
        int iter = 0;
        bool active = Se > Stol;
        flag = true;
        st = 0;
        while (__any_sync(FULL_MASK, active)) {
            set_x(Y);
            lnfugX();
            // AssembleJmatSTA
            if (act) {
                const double* fx = sh.lnf[h];
                const double* Yv = sh.xs[h];
                double tmp = 0;
                for (int k = 0; k < NC; k++) tmp += Yv[k] * fx[i * NC + k];
                for (int j = 0; j < NC; j++) sh.J[h][i * NC + j] = (fx[i * NC + j] - tmp + 1) / yt;
                sh.r[h][i] = res;
            }
            __syncwarp();
            int sing = 0;
            if (i == 0) sing = sym_lower_solve<NCM>(NC, sh.J[h], sh.r[h], sh.W[h]) ? 0 : 1;
            sing = __shfl_sync(FULL_MASK, sing, h * 16);
            __syncwarp();
            const double rs = sh.r[h][ic];
            __syncwarp();
            const double lYt = yt;
            double Yn = Y * lYt + alpha * rs;
            const double ytn = osum(Yn);
            const double a = 1 / ytn;
            Yn = a * Yn;
            set_x(Yn);
            double fSn, pn;
            fug_phi(fSn, pn);
            const double resn = log(fug0 / (fSn * ytn));
            const double Sen = sqrt(osum(resn * resn));
            if (active) {
                if (sing) st |= ST_SINGULAR;
                Y = Yn;
                yt = ytn;
                fS = fSn;
                res = resn;
                Se = Sen;
                iter++;
                if (iter > maxIt) {
                    flag = false;
                    st |= ST_STAB_NONCONV;
                    active = false;
                }
                else if (!(Se > Stol)) active = false;
            }
        }
        iters = iter;
    }

    // StableSSM01: Wilson starts 0 and 1 on halves 0 and 1
    __device__ bool stable_ssm01()
    {
        const double Stol = m.ssm_sta_tol2;
        const int maxIt = m.ssm_sta_maxit;
        const double eYt = m.ssm_sta_eYt;
        const double Ktol = m.ssm_sta_Ktol;
        const double dYtol = m.ssm_sta_dYtol;
        set_x(x0);
        double fug0, phi0;
        fug_phi(fug0, phi0);
        __syncwarp();
        double K = kw(h), di = 0;
        double ytH = 0, Sk = 0;
        int iter = 0;
        bool flag = false, active = true;
        while (__any_sync(FULL_MASK, active)) {
            double Yv = x0 * K;
            const double yt = osum(Yv);
            const double a = 1 / yt;
            Yv = a * Yv;
            const double dY = osum(sq(Yv - di));
            bool brk = false;
            if (active) {
                ytH = yt;
                if (iter > 0 && dY < dYtol) {
                    flag = true;
                    brk = true;
                }
            }
            set_x(Yv);
            double fS, pS;
            fug_phi(fS, pS);
            const double dn = fug0 / (fS * yt);
            const double Kn = K * dn;
            const double Se = osum(sq(dn - 1));
            const double Skn = osum(sq(log(Kn)));
            if (active && !brk) {
                K = Kn;
                Sk = Skn;
                iter++;
                if (Se < Stol) { flag = true; brk = true; }
                else if (Sk < Ktol) { flag = true; brk = true; }
                else if (iter > maxIt) brk = true;
                else di = Yv;
            }
            if (brk) active = false;
        }
        // merge the two starts in order
        for (int k = 0; k < 2; k++) {
            const int itk = __shfl_sync(FULL_MASK, iter, k * 16);
            const bool fk = __shfl_sync(FULL_MASK, flag ? 1 : 0, k * 16) != 0;
            const double ytk = __shfl_sync(FULL_MASK, ytH, k * 16);
            const double skk = __shfl_sync(FULL_MASK, Sk, k * 16);
            it_ssm_sta += itk;
            Yt = ytk;
            if (fk && ytk > 1 - 0.1 && skk > 1) ftype = 2;
            if (fk && ytk > 1 + eYt) {
                ssm_sta_conv = true;
                return false;
            }
        }
        return true;
    }

    // StableSSM: Wilson starts (0, 1) then (2, 3) on the two halves, each
    // followed by StableNR
    __device__ bool stable_ssm()
    {
        set_x(x0);
        double fug0, phi0;
        fug_phi(fug0, phi0);
        __syncwarp();
        const double d0 = phi0 * x0;
        const double Stol = m.ssm_sta_tol2;
        const int maxIt = m.ssm_sta_maxit;
        const double eYt = m.ssm_sta_eYt;
        for (int p = 0; p < 2; p++) {
            const int k = 2 * p + h;
            double Y = x0 / kw(k);
            double yt = osum(Y);
            {
                const double a = 1 / yt;
                Y = a * Y;
            }
            set_x(Y);
            double fS, pS;
            fug_phi(fS, pS);
            double Se = osum(sq(log(fS / fug0 * yt)));
            int iter = 0;
            bool active = Se > Stol;
            while (__any_sync(FULL_MASK, active)) {
                double Yn = d0 / pS;
                const double ytn = osum(Yn);
                const double a = 1 / ytn;
                Yn = a * Yn;
                set_x(Yn);
                double fSn, pSn;
                fug_phi(fSn, pSn);
                const double Sen = osum(sq(log(fSn / fug0 * ytn)));
                if (active) {
                    Y = Yn;
                    yt = ytn;
                    fS = fSn;
                    pS = pSn;
                    Se = Sen;
                    iter++;
                    if (iter > maxIt) active = false;
                    else if (!(Se > Stol)) active = false;
                }
            }
            bool nflag;
            int nit;
            uint32_t nst;
            stable_nr_half(Y, yt, fS, fug0, nflag, nit, nst);
            for (int hh = 0; hh < 2; hh++) {
                it_ssm_sta += __shfl_sync(FULL_MASK, iter, hh * 16);
                it_nr_sta += __shfl_sync(FULL_MASK, nit, hh * 16);
                status |= __shfl_sync(FULL_MASK, nst, hh * 16);
                const bool fk = __shfl_sync(FULL_MASK, nflag ? 1 : 0, hh * 16) != 0;
                const double ytk = __shfl_sync(FULL_MASK, yt, hh * 16);
                nr_sta_conv = fk;
                Yt = ytk;
                if (fk && ytk > 1 + eYt) {
                    ssm_sta_conv = true;
                    return false;
                }
            }
        }
        return true;
    }

    // PhaseStable, called with NP == 1
    __device__ bool phase_stable()
    {
        ssm_sta_conv = false;
        nr_sta_conv = false;
        bool flag;
        unsigned tmpNP = (unsigned)NP;
        if (lNP == 0) {
            flag = stable_ssm();
        }
        else {
            flag = stable_ssm01();
            if (!flag) tmpNP++;
            if (tmpNP != lNP) {
                flag = stable_ssm();
                ftype = 2;
            }
        }
        return flag;
    }

    // ---------------------------------------------------------- split ----
    // RachfordRice2.  Both halves hold the same K and z; they split the work
    // of each iteration: half 0 forms the terms of the function, half 1 those
    // of its derivative (one division sequence for both), and each half adds
    // up its own terms in component order (one addition chain for both).
    __device__ void rachford_rice2()
    {
        double* Kv = sh.K[h];
        if (act) Kv[i] = Ks;
        __syncwarp();
        double Kmin = Kv[0], Kmax = Kv[0];
        for (int k = 1; k < NC; k++) {
            if (Kv[k] < Kmin) Kmin = Kv[k];
            if (Kv[k] > Kmax) Kmax = Kv[k];
        }
        __syncwarp();
        const double qb = 1 / ((i == 1) ? (1 - Kmin) : (1 - Kmax));
        const double numin = __shfl_sync(FULL_MASK, qb, h * 16);
        const double numax = __shfl_sync(FULL_MASK, qb, h * 16 + 1);
        nu0 = 0.5 * (numin + numax);
        int iter = 0;
        const double tol = m.rr_tol;
        const double maxIt = m.rr_maxit;
        double* tv = sh.v1[h];
        while (true) {
            const double tmp = 1 + nu0 * (Ks - 1);
            const double zk = z * (Ks - 1);
            // half 0: z (K-1) / t; half 1: z (K-1) (K-1) / (t t)
            const double q = (h ? zk * (Ks - 1) : zk) / (h ? tmp * tmp : tmp);
            if (act) tv[i] = q;
            __syncwarp();
            // half 0: rj += term; half 1: Jr -= term
            double acc = 0;
#pragma unroll
            for (int k = 0; k < NCM; k++)
                if (k < NC) acc += h ? -tv[k] : tv[k];
            __syncwarp();
            const double rj = __shfl_sync(FULL_MASK, acc, 0);
            const double Jr = __shfl_sync(FULL_MASK, acc, 16);
            if (fabs(rj) < tol || iter > maxIt) break;
            const double dnuj = -rj / Jr;
            const double tmpnu = nu0 + dnuj;
            if (tmpnu < numax && tmpnu > numin) nu0 = tmpnu;
            else if (dnuj > 0) nu0 = (nu0 + numax) / 2;
            else nu0 = (nu0 + numin) / 2;
            iter++;
        }
        it_rr += iter;
        nu1 = 1 - nu0;
    }

    // UpdateXRR
    __device__ void update_x_rr()
    {
        double tmp = 1;
        tmp += nu0 * (Ks - 1);
        x1 = z / tmp;
        x0 = Ks * x1;
    }

    // fugacities (and phi) of both phases: half h evaluates phase h
    __device__ void fug_both(double& f0, double& f1, double& p0, double& p1)
    {
        set_x(h ? x1 : x0);
        double f, p;
        fug_phi(f, p);
        if (act) {
            sh.fg[h][i] = f;
            sh.ph[h][i] = p;
        }
        __syncwarp();
        f0 = sh.fg[0][ic];
        f1 = sh.fg[1][ic];
        p0 = sh.ph[0][ic];
        p1 = sh.ph[1][ic];
        __syncwarp();
    }

    // SplitSSM2
    __device__ void split_ssm2(bool restart, double& f0, double& f1)
    {
        ssm_sp_conv = true;
        double Se = 1;
        double Stol = m.ssm_sp_tol2;
        int maxIt = m.ssm_sp_maxit;
        if (!restart) Ks = (lNP == 2) ? lKs : Kw0;
        else {
            Stol *= 1E-1;
            maxIt *= 2;
        }
        if (Yt < 1.1) {
            Stol *= 1E-1;
            maxIt *= 2;
        }
        int iter = 0;
        while (Se > Stol) {
            rachford_rice2();
            update_x_rr();
            double p0, p1;
            fug_both(f0, f1, p0, p1);
            // half 0: f1/f0 for Se; half 1: phi1/phi0, the new K (one division sequence)
            const double q = (h ? p1 : f1) / (h ? p0 : f0);
            const double qo = __shfl_xor_sync(FULL_MASK, q, 16);
            Ks = h ? q : qo;
            Se = osum(sq((h ? qo : q) - 1));
            iter++;
            if (iter > maxIt) {
                ssm_sp_conv = false;
                break;
            }
        }
        it_ssm_sp += iter;
    }

    // SplitNR (NP = 2); f0, f1: fugacities of the current compositions
    __device__ void split_nr(double& f0, double& f1)
    {
        nr_sp_conv = false;
        double n0 = nu0 * x0, n1 = nu1 * x1;
        double res = log(f1 / f0);
        double eNR = sqrt(osum(res * res));
        const double NRtol = m.nr_sp_tol;
        int iter = 0;
        const double eNR0 = eNR;
        while (eNR > NRtol) {
            const double ln0 = n0, ln1 = n1;
            set_x(h ? x1 : x0);
            lnfugN(h ? nu1 : nu0);
            if (h == 0 && act) {
                for (int k = 0; k < NC; k++) sh.J[0][i * NC + k] = sh.lnf[0][i * NC + k] + sh.lnf[1][i * NC + k];
                sh.r[0][i] = res;
            }
            __syncwarp();
            int sing = 0;
            if (lane == 0) sing = sym_lower_solve<NCM>(NC, sh.J[0], sh.r[0], sh.W[0]) ? 0 : 1;
            sing = __shfl_sync(FULL_MASK, sing, 0);
            __syncwarp();
            if (sing) status |= ST_SINGULAR;
            res = sh.r[0][ic];
            // CalStepNRsp
            if (act) {
                sh.v2[h][i] = n0;
                sh.d2[h][i] = res;
            }
            __syncwarp();
            double alpha = 1;
            for (int k = 0; k < NC; k++) {
                const double tmp = sh.v2[h][k] + alpha * sh.d2[h][k];
                if (tmp < 0) alpha *= 0.9 * fabs(sh.v2[h][k] / sh.d2[h][k]);
            }
            __syncwarp();
            n1 = z;
            n0 += alpha * res;
            n1 -= n0;
            nu0 = osum(n0);
            nu1 = 1;
            nu1 -= nu0;
            // half 0: n0 / nu0, half 1: n1 / nu1 (one division sequence)
            const double qx = (h ? n1 : n0) / (h ? nu1 : nu0);
            const double qxo = __shfl_xor_sync(FULL_MASK, qx, 16);
            x0 = fabs(h ? qxo : qx);
            x1 = fabs(h ? qx : qxo);
            double p0, p1;
            fug_both(f0, f1, p0, p1);
            res = log(f1 / f0);
            eNR = sqrt(osum(res * res));
            iter++;
            if (eNR > eNR0 || iter > m.nr_sp_maxit) break;
            // en: phase 0 terms, then phase 1 terms, in component order
            const double e0 = osum((ln0 - n0) * (ln0 - n0));
            double en = e0;
            {
                double* v = sh.v1[h];
                if (act) v[i] = (ln1 - n1) * (ln1 - n1);
                __syncwarp();
#pragma unroll
                for (int k = 0; k < NCM; k++)
                    if (k < NC) en += v[k];
                __syncwarp();
            }
            if (en < 1E-16 * (2 * NC) * (2 * NC)) {
                nr_sp_conv = true;
                break;
            }
        }
        if (eNR < NRtol) nr_sp_conv = true;
        it_nr_sp += iter;
    }

    // CheckSplit (NP = 2)
    __device__ bool check_split()
    {
        if (NP != 2) return true;
        const double nuMax = nu0 > nu1 ? nu0 : nu1;
        const double eX = osum((x0 - x1) * (x0 - x1));
        if (nuMax < 1 && nr_sp_conv && finite_d(eX)) {
        }
        else if (!finite_d(eX) || 1 - nuMax < 1E-3) {
            NP = 1;
            x0 = z;
            nu0 = 1;
            ssm_sta_conv = false;
            nr_sta_conv = false;
            return false;
        }
        return true;
    }

    // PhaseSplit
    __device__ void phase_split()
    {
        ssm_sp_conv = false;
        nr_sp_conv = false;
        double f0, f1;
        split_ssm2(false, f0, f1);
        split_nr(f0, f1);
        int restarts = 0;
        while (!nr_sp_conv) {
            if (++restarts > SPLIT_RESTART_CAP) {
                status |= ST_ITER_CAP;
                break;
            }
            split_ssm2(true, f0, f1);
            split_nr(f0, f1);
            if (!check_split()) break;
            if (ssm_sp_conv) break;
        }
        check_split();
        if (!nr_sp_conv && NP == 2) status |= ST_SPLIT_NONCONV;
    }

    // PhaseEquilibrium + SetInitalValue for one cell; fills `out` (lanes of
    // half 0 write the compositions)
    __device__ void run(const Model& M, const BulkView& b, const DeferRec& rec, PERes& out)
    {
        const int cell = rec.cell;
        status = 0;
        it_ssm_sta = it_nr_sta = it_ssm_sp = it_nr_sp = it_rr = 0;
        P = b.P[cell];
        T = b.T[cell] + M.units.conv4;
        const double Ni_i = b.Ni[b.idx(ic, cell)];
        // InitNtZ: Nt in component order, then z = Ni / Nt
        const double Nt = osum(Ni_i);
        z = act ? Ni_i / Nt : 0.0;
        setup(M.units.gas_constant);
        ftype = rec.ftype_in;
        lNP = rec.lNP;
        const int nct = NC + 1;
        const double lx0 = b.xij[b.idx(0 * nct + ic, cell)];
        const double lx1 = b.xij[b.idx(1 * nct + ic, cell)];
        lKs = (lNP == 2) ? lx0 / lx1 : 0.0;
        Yt = 0;
        nu0 = 1;
        nu1 = 0;
        x1 = 0;
        switch (ftype) {
        case 0:
            NP = 1;
            nu0 = 1;
            x0 = z;
            cal_kwilson();
            while (!phase_stable()) {
                NP++;
                phase_split();
                if (NP == 2 || NP == 1) break;
            }
            break;
        case 1:
            NP = 1;
            nu0 = 1;
            x0 = z;
            break;
        default:
            NP = 2;
            Yt = 1.01;
            cal_kwilson();
            phase_split();
            break;
        }
        if (NP > 1) ftype = 2;
        if (lane == 0) {
            out.NP = NP;
            out.ftype = ftype;
            out.status = status;
            out.it[0] = it_ssm_sta;
            out.it[1] = it_nr_sta;
            out.it[2] = it_ssm_sp;
            out.it[3] = it_nr_sp;
            out.it[4] = it_rr;
            out.nu[0] = nu0;
            out.nu[1] = nu1;
        }
        if (h == 0 && act) {
            out.x[0][i] = x0;
            out.x[1][i] = x1;
        }
        __syncwarp();
    }
};

}  // namespace ocpx
