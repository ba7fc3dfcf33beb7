// Compositional FIM property update for one cell: skip test, phase
// equilibrium (stability + split), phase properties with derivatives, water,
// volume derivatives and the secondary-variable Jacobian dSec/dPri, and the
// skip state for the next Newton iteration.
//
// Reference path (called per cell by IsoT_FIM::CalFlash,
// src/IsoThermalMethod.cpp:1016-1025):
//   OCPMixtureComp::FlashDer            include/OCPMixture.hpp:85-90
//   OCPMixtureMethodComp01::SetVarSet   src/OCPMixtureMethodComp.cpp:671-687
//   SkipPSAMethod01::CalFtype02/IfSkip  src/AcceleratePEC.cpp:64-124
//   OCPMixtureMethodComp01::FlashDer    src/OCPMixtureMethodComp.cpp:746-755
//   OCPPhaseEquilibrium                 src/OCPPhaseEquilibrium.cpp:71-1010
//   CalPropertyDer / IdentifyPhase      src/OCPMixtureMethodComp.cpp:134-256
//   ViscosityMethod03 (LBC)             src/OCPFuncPVT.cpp:415-576
//   CalPropertyW / OCP_PVTW             src/OCPMixtureMethodComp.cpp:846-860
//   CalVfiVfp_full02 / CaldXsdXp02      src/OCPMixtureMethodComp.cpp:462-642, 896-920
//   SkipPSAMethod01::CalSkipForNextStep src/AcceleratePEC.cpp:127-170
//   IsoT_FIM::PassFlashValue            src/IsoThermalMethod.cpp:1027-1071
//
// The per-cell arithmetic follows the reference operation by operation (same
// evaluation order, no FMA contraction in parity builds) so that phase labels
// and branch decisions match; only LAPACK calls and libm differ in rounding.
#pragma once
#include "bulk_view.cuh"
#include "eos_pr.cuh"
#include "linalg_small.cuh"

namespace ocpx {

// Upper bound on the restarts of the split SSM/NR loop
// (OCPPhaseEquilibrium::PhaseSplit, src/OCPPhaseEquilibrium.cpp:549-573):
// the reference loops until NR converges, which need not terminate; the
// device version stops here and flags the cell.
constexpr int SPLIT_RESTART_CAP = 64;

// Phase-equilibrium outcome handed from the cooperative kernel (flash_coop.cuh)
// to the thread that finishes the cell's properties and derivatives.
struct PERes {
    int NP;
    int ftype;
    uint32_t status;
    int it[5];  // SSM-stability, NR-stability, SSM-split, NR-split, RR
    double nu[2];
    double x[2][NC_MAX];
};

// The state a cell's phase split leaves after its first successive-
// substitution loop (split_ssm2 without restart), for the rest of the split
// to resume from: what the loop writes and what comes after it reads.
struct SplitState {
    double Ks[NC_MAX], nu[2], x[2][NC_MAX], fug[2][NC_MAX], phi[2][NC_MAX];
    int it_ssm_sp, it_rr, work;
    uint32_t status;
    uint8_t conv;   // ssm_sp_conv
    uint8_t skip;   // 1: not a split cell, or left to the cooperative kernel
};

// A cell whose phase equilibrium ran over its work budget, with the inputs
// the equilibrium needs besides the cell state.
struct DeferRec {
    int cell;
    int ftype_in;
    unsigned lNP;
    unsigned seq;  // nonzero once the record is complete (lists read while they fill)
};

// Append-only list of deferred cells (one atomic per deferred cell).  With
// `seq` nonzero the record is published: its fields are written, then, after
// a fence, its seq, so a reader in the same launch that sees the seq sees the
// fields (the fused flash consumes the list while it fills).
struct DeferSink {
    DeferRec* rec;
    unsigned* count;
    int cap;
    unsigned seq = 0;
    OCPX_HD bool push(int cell, int ftype_in, unsigned lNP) const
    {
#ifdef __CUDA_ARCH__
        const unsigned slot = atomicAdd(count, 1u);
        if (slot >= (unsigned)cap) return false;
        rec[slot].cell = cell;
        rec[slot].ftype_in = ftype_in;
        rec[slot].lNP = lNP;
        if (seq) {
            __threadfence();
            atomicExch(&rec[slot].seq, seq);
        }
        return true;
#else
        (void)cell; (void)ftype_in; (void)lNP;
        return false;
#endif
    }
};

// Work units charged against the budget: one EoS fugacity evaluation = 1.
constexpr int WORK_SSM_STA = 1, WORK_NR_STA = 4, WORK_SSM_SP = 2, WORK_NR_SP = 6;

// Work units the last flash of a cell used, from its iteration counters
// (Rachford-Rice iterations at a fifth), plus a constant for the rest.
OCPX_HD long long predicted_work(const BulkView& b, int cell)
{
    const int32_t* it = b.iters;
    return 3LL + WORK_SSM_STA * (long long)it[b.idx(0, cell)] + WORK_NR_STA * (long long)it[b.idx(1, cell)] +
           WORK_SSM_SP * (long long)it[b.idx(2, cell)] + WORK_NR_SP * (long long)it[b.idx(3, cell)] +
           it[b.idx(4, cell)] / 5;
}

// SkipPSAMethod01::CalFtype02 / IfSkip (src/AcceleratePEC.cpp:64-124): the
// flash type the phase equilibrium starts from (0 full test, 1 skip, 2 split).
// Ni: the cell's moles (NC hydrocarbons first), Nt their hydrocarbon sum,
// T in K, Sin the saturations entering the flash, npPE = phaseNum - 1.
OCPX_HD int flash_type_in(const CompModel& m, const BulkView& b, int cell, const double* Ni, double Nt, double P,
                          double T, const double* Sin, unsigned npPE)
{
    const int NC = m.nc;
    int ftype_in = 0;
    bool skip = false;
    if (m.skip_psa && b.skip_flag[cell]) {
        const double me = b.skip_minEig[cell];
        skip = true;
        if (fabs(1 - b.skip_P[cell] / P) >= me / 10) skip = false;
        else if (fabs(b.skip_T[cell] - T) >= me * 10) skip = false;
        else {
            for (int i = 0; i < NC; i++)
                if (fabs(Ni[i] / Nt - b.skip_zi[b.idx(i, cell)]) >= me / 10) { skip = false; break; }
        }
    }
    if (skip) ftype_in = 1;
    else if (m.skip_psa && npPE >= 2) {
        unsigned tmp = 0;
        for (int j = 0; j < 2; j++)
            if (Sin[j] >= 1E-4) tmp++;
        ftype_in = (tmp == npPE) ? (int)npPE : 0;
    }
    return ftype_in;
}

template <int NCM>
struct CompFlash {
    EosPR<NCM> eos;
    const CompModel* m;
    int NC;             // hydrocarbon components
    double P, T;        // T in K
    double zi[NCM];
    double Nt;          // hydrocarbon moles
    // phase equilibrium state (OCPPhaseEquilibrium members)
    int ftype;
    unsigned lNP;
    int NP;
    double nu[2];
    double x[2][NCM], n[2][NCM], ln_[2][NCM];
    double phi[2][NCM], fug[2][NCM];
    double Kw[4][NCM], Ks[NCM], lKs[NCM];
    double phiSta[NCM], fugSta[NCM], Y[NCM], di[NCM], res[NCM];
    double Yt;
    double J[NCM * NCM], W[NCM * NCM];
    double lnf[2][NCM * NCM];
    bool ssm_sta_conv, nr_sta_conv, ssm_sp_conv, nr_sp_conv;
    int it_ssm_sta, it_nr_sta, it_ssm_sp, it_nr_sp, it_rr;
    uint32_t status;
    // work budget: once `work` exceeds `budget` the equilibrium is abandoned
    // (deferred) and its partial state is discarded by the caller
    int work, budget;
    bool deferred;

    OCPX_HD bool charge(int units)
    {
        work += units;
        if (work > budget) deferred = true;
        return deferred;
    }

    OCPX_HD static double dnrm2(int n, const double* v)
    {
        double s = 0;
        for (int i = 0; i < n; i++) s += v[i] * v[i];
        return sqrt(s);
    }
    OCPX_HD void scale_Y()
    {
        const double a = 1 / Yt;
        for (int i = 0; i < NC; i++) Y[i] = a * Y[i];
    }

    // OCPPhaseEquilibrium::CalKwilson (:244-252)
    OCPX_HD void cal_kwilson()
    {
        for (int i = 0; i < NC; i++) {
            Kw[0][i] = (m->Pc[i] / P) * exp(5.373 * (1 + m->acf[i]) * (1 - m->Tc[i] / T));
            Kw[1][i] = 1 / Kw[0][i];
            Kw[2][i] = pow_third(Kw[0][i]);
            Kw[3][i] = pow_third(Kw[1][i]);
        }
    }

    // ------------------------------------------------------ stability ----
    // OCPPhaseEquilibrium::StableSSM01 (:299-395); the tested phase is 0
    OCPX_HD_NOINLINE bool stable_ssm01()
    {
        const double Stol = m->ssm_sta_tol2;
        const int maxIt = m->ssm_sta_maxit;
        const double eYt = m->ssm_sta_eYt;
        const double Ktol = m->ssm_sta_Ktol;
        const double dYtol = m->ssm_sta_dYtol;
        double Se = 0, Sk = 0, dY;
        const double* xj = x[0];
        eos.cal_fug_phi(xj, fug[0], nullptr);
        for (int k = 0; k < 2; k++) {
            for (int i = 0; i < NC; i++) Ks[i] = Kw[k][i];
            int iter = 0;
            bool flag = false;
            while (true) {
                if (charge(WORK_SSM_STA)) return true;
                Yt = 0;
                for (int i = 0; i < NC; i++) {
                    Y[i] = xj[i] * Ks[i];
                    Yt += Y[i];
                }
                scale_Y();
                if (iter > 0) {
                    dY = 0;
                    for (int i = 0; i < NC; i++) dY += sq(Y[i] - di[i]);
                    if (dY < dYtol) { flag = true; break; }
                }
                eos.cal_fug_phi(Y, fugSta, nullptr);
                Se = 0;
                Sk = 0;
                for (int i = 0; i < NC; i++) {
                    di[i] = fug[0][i] / (fugSta[i] * Yt);
                    Ks[i] *= di[i];
                    Se += sq(di[i] - 1);
                    Sk += sq(log(Ks[i]));
                }
                iter++;
                if (Se < Stol) { flag = true; break; }
                if (Sk < Ktol) { flag = true; break; }
                if (iter > maxIt) break;
                for (int i = 0; i < NC; i++) di[i] = Y[i];
            }
            it_ssm_sta += iter;
            if (flag && Yt > 1 - 0.1 && Sk > 1) ftype = 2;
            if (flag && Yt > 1 + eYt) { ssm_sta_conv = true; return false; }
        }
        return true;
    }

    // OCPPhaseEquilibrium::AssembleJmatSTA (:523-541)
    OCPX_HD void assemble_jmat_sta()
    {
        const double* fx = lnf[0];
        for (int i = 0; i < NC; i++) {
            double tmp = 0;
            for (int k = 0; k < NC; k++) tmp += Y[k] * fx[i * NC + k];
            for (int j = 0; j < NC; j++) J[i * NC + j] = (fx[i * NC + j] - tmp + 1) / Yt;
        }
    }

    // OCPPhaseEquilibrium::StableNR (:475-521)
    OCPX_HD_NOINLINE bool stable_nr()
    {
        for (int i = 0; i < NC; i++) res[i] = log(fug[0][i] / (fugSta[i] * Yt));
        const int maxIt = m->nr_sta_maxit;
        const double Stol = m->nr_sta_tol;
        double Se = dnrm2(NC, res);
        const double alpha = 1;
        int iter = 0;
        while (Se > Stol) {
            if (charge(WORK_NR_STA)) return true;
            eos.cal_lnfugX(Y, lnf[0]);
            assemble_jmat_sta();
            if (!sym_lower_solve<NCM>(NC, J, res, W)) status |= ST_SINGULAR;
            const double lYt = Yt;
            Yt = 0;
            for (int i = 0; i < NC; i++) {
                Y[i] = Y[i] * lYt + alpha * res[i];
                Yt += Y[i];
            }
            scale_Y();
            eos.cal_fug_phi(Y, fugSta, nullptr);
            for (int i = 0; i < NC; i++) res[i] = log(fug[0][i] / (fugSta[i] * Yt));
            Se = dnrm2(NC, res);
            iter++;
            if (iter > maxIt) {
                it_nr_sta += iter;
                nr_sta_conv = false;
                status |= ST_STAB_NONCONV;
                return false;
            }
        }
        it_nr_sta += iter;
        nr_sta_conv = true;
        return true;
    }

    // OCPPhaseEquilibrium::StableSSM (:397-473)
    OCPX_HD_NOINLINE bool stable_ssm()
    {
        const double* xj = x[0];
        eos.cal_fug_phi(xj, fug[0], phi[0]);
        for (int i = 0; i < NC; i++) di[i] = phi[0][i] * xj[i];
        const double Stol = m->ssm_sta_tol2;
        const int maxIt = m->ssm_sta_maxit;
        const double eYt = m->ssm_sta_eYt;
        double Se;
        bool flag;
        for (int k = 0; k < 4; k++) {
            Yt = 0;
            for (int i = 0; i < NC; i++) {
                Y[i] = xj[i] / Kw[k][i];
                Yt += Y[i];
            }
            scale_Y();
            eos.cal_fug_phi(Y, fugSta, phiSta);
            Se = 0;
            for (int i = 0; i < NC; i++) Se += sq(log(fugSta[i] / fug[0][i] * Yt));
            flag = true;
            int iter = 0;
            while (Se > Stol) {
                if (charge(WORK_SSM_STA)) return true;
                Yt = 0;
                for (int i = 0; i < NC; i++) {
                    Y[i] = di[i] / phiSta[i];
                    Yt += Y[i];
                }
                scale_Y();
                eos.cal_fug_phi(Y, fugSta, phiSta);
                Se = 0;
                for (int i = 0; i < NC; i++) Se += sq(log(fugSta[i] / fug[0][i] * Yt));
                iter++;
                if (iter > maxIt) { flag = false; break; }
            }
            it_ssm_sta += iter;
            flag = stable_nr();
            if (deferred) return true;
            if (flag && Yt > 1 + eYt) { ssm_sta_conv = true; return false; }
        }
        return true;
    }

    // OCPPhaseEquilibrium::PhaseStable (:260-297); called with NP == 1
    OCPX_HD bool phase_stable()
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
            if (deferred) return true;
            if (!flag) tmpNP++;
            if (tmpNP != lNP) {
                flag = stable_ssm();
                ftype = 2;
            }
        }
        return flag;
    }

    // ---------------------------------------------------------- split ----
    // OCPPhaseEquilibrium::RachfordRice2 (:651-705)
    OCPX_HD_NOINLINE void rachford_rice2()
    {
        double Kmin = Ks[0], Kmax = Ks[0];
        for (int i = 1; i < NC; i++) {
            if (Ks[i] < Kmin) Kmin = Ks[i];
            if (Ks[i] > Kmax) Kmax = Ks[i];
        }
        const double numin = 1 / (1 - Kmax);
        const double numax = 1 / (1 - Kmin);
        nu[0] = 0.5 * (numin + numax);
        int iter = 0;
        const double tol = m->rr_tol;
        const double maxIt = m->rr_maxit;
        while (true) {
            double rj = 0, Jr = 0;
            for (int i = 0; i < NC; i++) {
                const double tmp = 1 + nu[0] * (Ks[i] - 1);
                rj += zi[i] * (Ks[i] - 1) / tmp;
                Jr -= zi[i] * (Ks[i] - 1) * (Ks[i] - 1) / (tmp * tmp);
            }
            if (fabs(rj) < tol || iter > maxIt) break;
            const double dnuj = -rj / Jr;
            const double tmpnu = nu[0] + dnuj;
            if (tmpnu < numax && tmpnu > numin) nu[0] = tmpnu;
            else if (dnuj > 0) nu[0] = (nu[0] + numax) / 2;
            else nu[0] = (nu[0] + numin) / 2;
            iter++;
        }
        it_rr += iter;
        nu[1] = 1 - nu[0];
    }

    // OCPPhaseEquilibrium::UpdateXRR (:778-791), NP = 2
    OCPX_HD void update_x_rr()
    {
        for (int i = 0; i < NC; i++) {
            double tmp = 1;
            tmp += nu[0] * (Ks[i] - 1);
            x[1][i] = zi[i] / tmp;
            x[0][i] = Ks[i] * x[1][i];
        }
    }

    // OCPPhaseEquilibrium::SplitSSM2 (:586-647)
    // the loop's controls: residual, tolerance, iteration cap and count
    struct SsmLoop {
        double Se, Stol;
        int maxIt, iter;
    };
    OCPX_HD void split_ssm_init(bool restart, SsmLoop& L)
    {
        ssm_sp_conv = true;
        L.Se = 1;
        L.Stol = m->ssm_sp_tol2;
        L.maxIt = m->ssm_sp_maxit;
        if (!restart) {
            if (lNP == 2) for (int i = 0; i < NC; i++) Ks[i] = lKs[i];
            else          for (int i = 0; i < NC; i++) Ks[i] = Kw[0][i];
        }
        else {
            L.Stol *= 1E-1;
            L.maxIt *= 2;
        }
        if (Yt < 1.1) {
            L.Stol *= 1E-1;
            L.maxIt *= 2;
        }
        L.iter = 0;
    }
    // one pass of the loop (its test first); true when the loop is over,
    // with it_ssm_sp updated, or when the cell went over its budget (deferred)
    OCPX_HD_NOINLINE bool split_ssm_step(SsmLoop& L)
    {
        if (!(L.Se > L.Stol)) {
            it_ssm_sp += L.iter;
            return true;
        }
        if (charge(WORK_SSM_SP)) return true;
        rachford_rice2();
        update_x_rr();
        eos.cal_fug_phi(x[0], fug[0], phi[0]);
        eos.cal_fug_phi(x[1], fug[1], phi[1]);
        L.Se = 0;
        for (int i = 0; i < NC; i++) {
            L.Se += sq(fug[1][i] / fug[0][i] - 1);
            Ks[i] = phi[1][i] / phi[0][i];
        }
        L.iter++;
        if (L.iter > L.maxIt) {
            ssm_sp_conv = false;
            it_ssm_sp += L.iter;
            return true;
        }
        return false;
    }
    OCPX_HD void split_ssm2(bool restart)
    {
        SsmLoop L;
        split_ssm_init(restart, L);
        while (!split_ssm_step(L)) {
        }
    }

    OCPX_HD void split_save(SplitState& st) const
    {
        for (int i = 0; i < NC; i++) {
            st.Ks[i] = Ks[i];
            for (int j = 0; j < 2; j++) {
                st.x[j][i] = x[j][i];
                st.fug[j][i] = fug[j][i];
                st.phi[j][i] = phi[j][i];
            }
        }
        st.nu[0] = nu[0];
        st.nu[1] = nu[1];
        st.it_ssm_sp = it_ssm_sp;
        st.it_rr = it_rr;
        st.work = work;
        st.status = status;
        st.conv = ssm_sp_conv ? 1 : 0;
    }
    OCPX_HD void split_load(const SplitState& st)
    {
        for (int i = 0; i < NC; i++) {
            Ks[i] = st.Ks[i];
            for (int j = 0; j < 2; j++) {
                x[j][i] = st.x[j][i];
                fug[j][i] = st.fug[j][i];
                phi[j][i] = st.phi[j][i];
            }
        }
        nu[0] = st.nu[0];
        nu[1] = st.nu[1];
        it_ssm_sp = st.it_ssm_sp;
        it_rr = st.it_rr;
        work = st.work;
        status = st.status;
        ssm_sp_conv = st.conv != 0;
    }

    // OCPPhaseEquilibrium::CalResSP (:899-907)
    OCPX_HD void cal_res_sp()
    {
        for (int i = 0; i < NC; i++) res[i] = log(fug[1][i] / fug[0][i]);
    }

    // OCPPhaseEquilibrium::SplitNR (:805-897), NP = 2
    OCPX_HD_NOINLINE void split_nr()
    {
        nr_sp_conv = false;
        for (int j = 0; j < 2; j++)
            for (int i = 0; i < NC; i++) n[j][i] = nu[j] * x[j][i];
        cal_res_sp();
        double eNR = dnrm2(NC, res);
        const double NRtol = m->nr_sp_tol;
        int iter = 0;
        const double eNR0 = eNR;
        while (eNR > NRtol) {
            if (charge(WORK_NR_SP)) return;
            for (int j = 0; j < 2; j++)
                for (int i = 0; i < NC; i++) ln_[j][i] = n[j][i];
            eos.cal_lnfugN(x[0], nu[0], lnf[0]);
            eos.cal_lnfugN(x[1], nu[1], lnf[1]);
            for (int i = 0; i < NC; i++)
                for (int k = 0; k < NC; k++) J[i * NC + k] = lnf[0][i * NC + k] + lnf[1][i * NC + k];
            if (!sym_lower_solve<NCM>(NC, J, res, W)) status |= ST_SINGULAR;
            // OCPPhaseEquilibrium::CalStepNRsp (:939-957)
            double alpha = 1;
            for (int i = 0; i < NC; i++) {
                const double tmp = n[0][i] + alpha * res[i];
                if (tmp < 0) alpha *= 0.9 * fabs(n[0][i] / res[i]);
            }
            for (int i = 0; i < NC; i++) n[1][i] = zi[i];
            nu[1] = 1;
            nu[0] = 0;
            for (int i = 0; i < NC; i++) {
                n[0][i] += alpha * res[i];
                n[1][i] -= n[0][i];
                nu[0] += n[0][i];
            }
            nu[1] -= nu[0];
            for (int i = 0; i < NC; i++) x[0][i] = fabs(n[0][i] / nu[0]);
            for (int i = 0; i < NC; i++) x[1][i] = fabs(n[1][i] / nu[1]);
            eos.cal_fug_phi(x[0], fug[0], nullptr);
            eos.cal_fug_phi(x[1], fug[1], nullptr);
            cal_res_sp();
            eNR = dnrm2(NC, res);
            iter++;
            if (eNR > eNR0 || iter > m->nr_sp_maxit) break;
            double en = 0;
            for (int j = 0; j < 2; j++)
                for (int i = 0; i < NC; i++) en += (ln_[j][i] - n[j][i]) * (ln_[j][i] - n[j][i]);
            if (en < 1E-16 * (2 * NC) * (2 * NC)) {
                nr_sp_conv = true;
                break;
            }
        }
        if (eNR < NRtol) nr_sp_conv = true;
        it_nr_sp += iter;
    }

    // OCPPhaseEquilibrium::CheckSplit (:960-1010), NP = 2
    OCPX_HD bool check_split()
    {
        if (NP != 2) return true;
        double eX = 0;
        const double nuMax = nu[0] > nu[1] ? nu[0] : nu[1];
        for (int i = 0; i < NC; i++) eX += (x[0][i] - x[1][i]) * (x[0][i] - x[1][i]);
        if (nuMax < 1 && nr_sp_conv && finite_d(eX)) {
            // accepted
        }
        else if (!finite_d(eX) || 1 - nuMax < 1E-3) {
            NP = 1;
            for (int i = 0; i < NC; i++) x[0][i] = zi[i];
            nu[0] = 1;
            ssm_sta_conv = false;
            nr_sta_conv = false;
            return false;
        }
        return true;
    }

    // OCPPhaseEquilibrium::PhaseSplit (:549-573)
    OCPX_HD_NOINLINE void phase_split(const SplitState* resume = nullptr)
    {
        ssm_sp_conv = false;
        nr_sp_conv = false;
        // the first successive-substitution loop, or its result computed elsewhere
        if (resume) split_load(*resume);
        else split_ssm2(false);
        if (deferred) return;
        split_nr();
        if (deferred) return;
        int restarts = 0;
        while (!nr_sp_conv) {
            if (++restarts > SPLIT_RESTART_CAP) {
                status |= ST_ITER_CAP;
                break;
            }
            split_ssm2(true);
            if (deferred) return;
            split_nr();
            if (deferred) return;
            if (!check_split()) break;
            if (ssm_sp_conv) break;
        }
        check_split();
        if (!nr_sp_conv && NP == 2) status |= ST_SPLIT_NONCONV;
    }

    // OCPPhaseEquilibrium::PhaseEquilibrium (:71-112) + SetInitalValue (:121-138).
    // lx points to the cell's previous oil composition; lx[i + lx_stride] is gas.
    // split_begin: the prologue of flash type 2 up to the split's first loop
    OCPX_HD void split_prologue(unsigned lNP_in, const double* lx0, const double* lx1)
    {
        ftype = 2;
        lNP = lNP_in;
        if (lNP == 2)
            for (int i = 0; i < NC; i++) lKs[i] = lx0[i] / lx1[i];
        NP = 2;
        Yt = 1.01;
        cal_kwilson();
        ssm_sp_conv = false;
        nr_sp_conv = false;
    }

    // resume (flash type 2 only): the split's first loop was run elsewhere
    OCPX_HD_NOINLINE void phase_equilibrium(int ftype_in, unsigned lNP_in, const double* lx0, const double* lx1,
                                            const SplitState* resume = nullptr)
    {
        ftype = ftype_in;
        lNP = lNP_in;
        if (lNP == 2)
            for (int i = 0; i < NC; i++) lKs[i] = lx0[i] / lx1[i];
        switch (ftype) {
        case 0:
            NP = 1;
            nu[0] = 1;
            for (int i = 0; i < NC; i++) x[0][i] = zi[i];
            cal_kwilson();
            while (!phase_stable()) {
                if (deferred) return;
                NP++;
                phase_split();
                if (NP == 2 || NP == 1) break;
            }
            break;
        case 1:
            NP = 1;
            nu[0] = 1;
            for (int i = 0; i < NC; i++) x[0][i] = zi[i];
            break;
        default:  // 2
            NP = 2;
            Yt = 1.01;
            cal_kwilson();
            phase_split(resume);
            break;
        }
        if (deferred) return;
        if (NP > 1) ftype = 2;
    }
};

// ---------------------------------------------------------------------------
// LBC viscosity with derivatives, ViscosityMethod03 (src/OCPFuncPVT.cpp:462-576).
// tT[i] is the temperature factor 34e-5 Tr^0.94 (Tr <= 1.5) or
// 17.78e-5 (4.58 Tr - 1.67)^0.625, which depends on the cell temperature only
// and is evaluated once per cell instead of once per phase and component.
// The reference's der1IJ is -(1/2)*... = 0 in integer arithmetic, so the
// component-derivative sum reduces exactly to its diagonal term.
template <int NCM>
OCPX_HD_NOINLINE double lbc_viscosity_der(const CompModel& m, int NC, const double* tT, const double* x, double xi,
                                 double xiP, const double* xix, double& muP, double* mux)
{
    double MW = 0;
    for (int i = 0; i < NC; i++) MW += x[i] * m.MW[i];
    double xPc = 0, xTc = 0, xVc = 0;
    double a0 = 0, a1 = 0;
    const double sqMW = sqrt(MW);
    for (int i = 0; i < NC; i++) {
        double tmp = m.auxB[i] / sqMW;
        tmp = tT[i] / tmp;
        a0 += x[i] * m.sqrtMW[i] * tmp;
        a1 += x[i] * m.sqrtMW[i];
        xPc += x[i] * m.Pc[i];
        xTc += x[i] * m.Tc[i];
        xVc += x[i] * m.Vcvis[i];
    }
    const double pTc16 = pow(xTc, 1.0 / 6);
    const double pPc23 = pow(xPc, 2.0 / 3);
    const double a2 = 5.4402 * pTc16 / sqMW / pPc23;
    const double a3 = xi * xVc;
    const double* c = m.lbc;
    const double a4 = a3 * (a3 * (a3 * (c[4] * a3 + c[3]) + c[2]) + c[1]) + c[0];
    const double a4p3 = pow(a4, 3);
    const double a4p4 = pow(a4, 4);
    const double mu = a0 / a1 + 1E-4 * (a4p4 - 1) / a2;
    const double poly = (c[1] + a3 * (2 * c[2] + a3 * (3 * c[3] + a3 * 4 * c[4])));
    {
        const double der7J = xVc * xiP;
        const double der8J = der7J * poly;
        muP = (4 * 1E-4) * a4p3 * der8J / a2;
    }
    const double pTcm56 = pow(xTc, -5.0 / 6);
    const double den6 = (sqMW * pPc23);
    for (int k = 0; k < NC; k++) {
        const double val1 = m.auxB[k] / sqMW;
        const double der3J = m.sqrtMW[k] * (tT[k] / val1);
        const double der4J = m.sqrtMW[k];
        const double der6J = 5.4402 *
                             (1.0 / 6 * pTcm56 * m.Tc[k] -
                              pTc16 * (0.5 / MW * m.MW[k] + 2.0 / 3 / xPc * m.Pc[k])) /
                             den6;
        const double der7J = xix[k] * xVc + xi * m.Vcvis[k];
        const double der8J = der7J * poly;
        mux[k] = (der3J * a1 - a0 * der4J) / (a1 * a1) +
                 1E-4 * (4 * a4p3 * der8J * a2 - (a4p4 - 1) * der6J) / (a2 * a2);
    }
    return mu;
}

// OCP_PVTW::CalRhoXiMuDer (src/OCPFuncPVT.cpp:32-56)
OCPX_HD void pvtw_rho_xi_mu_der(const WaterModel& w, double conv1, double P, double& rho, double& xi,
                                double& mu, double& rhoP, double& xiP, double& muP)
{
    const Table& t = w.pvtw;
    const int r = table_close_row(t, 0, P);
    const double Pref = t.data[0 * t.nrow + r];
    const double bref = t.data[1 * t.nrow + r];
    const double Cbref = t.data[2 * t.nrow + r];
    const double muref = t.data[3 * t.nrow + r];
    const double Cmuref = t.data[4 * t.nrow + r];
    const double b = bref * (1 - Cbref * (P - Pref));
    const double bp = -Cbref * bref;
    mu = muref * (1 + Cmuref * (P - Pref));
    muP = Cmuref * muref;
    xi = 1 / conv1 / (b * w.std_vw);
    xiP = -1 / conv1 * bp / ((b * b) * w.std_vw);
    rho = w.std_rho_w / b;
    rhoP = -w.std_rho_w * bp / (b * b);
}

// ---------------------------------------------------------------------------
// One cell of the compositional FlashDer + PassFlashValue.
template <int NCM>
struct CompCellUpdate {
    CompFlash<NCM> f;
    // phase-level results (indices 0 oil, 1 gas after reordering; 2 water)
    double MW[2], vm[2], vmP[2], vmx[2][NCM];
    double nj[3], vj[3], xiv[3], rho[3], mu[3], xiPv[3], rhoPv[3], muPv[3];
    double xix[2][NCM], rhox[2][NCM], mux[2][NCM];
    double xx[3][NCM + 1];  // compositions, nc entries per phase
    double vjP[3], vji[3][NCM + 1];
    double vfi[NCM + 1];
    double S[3];
    bool ex[3];
    double Vf, vfP;
    double rhs[NCM * (NCM + 1)];
    double tT[NCM];

    // budget: work units the phase equilibrium may use before the cell is
    // handed to `sink` (the plain kernel passes INT_MAX and no sink);
    // injected: a phase-equilibrium result computed elsewhere for this cell.
    // Returns false when the cell was deferred (nothing of it was written).
    // resume: the state of the split's first loop, run elsewhere (flash type 2)
    OCPX_HD bool run(const Model& M, const BulkView& b, int cell, int budget = 0x7fffffff,
                     const DeferSink* sink = nullptr, const PERes* injected = nullptr,
                     const SplitState* resume = nullptr)
    {
        const CompModel& m = M.comp;
        const int NC = m.nc;
        const int nct = NC + 1;   // components incl. water
        const int np = 3;
        const int ncol = nct + 1;
        f.m = &m;
        f.NC = NC;
        f.status = 0;
        f.it_ssm_sta = f.it_nr_sta = f.it_ssm_sp = f.it_nr_sp = f.it_rr = 0;
        f.work = 0;
        f.budget = budget;
        f.deferred = false;

        // ---- SetVarSet (src/OCPMixtureMethodComp.cpp:671-687)
        const double P = b.P[cell];
        const double T = b.T[cell] + M.units.conv4;
        double Ni[NCM + 1];
        for (int i = 0; i < nct; i++) Ni[i] = b.Ni[b.idx(i, cell)];
        double Sin[3];
        unsigned phaseNum = 0;
        for (int j = 0; j < np; j++) {
            Sin[j] = b.S[b.idx(j, cell)];
            ex[j] = b.phaseExist[b.idx(j, cell)] != 0;
            if (ex[j]) phaseNum++;
        }
        for (int j = 0; j < np; j++)
            for (int i = 0; i < nct; i++) xx[j][i] = b.xij[b.idx(j * nct + i, cell)];

        // ---- InitNtZ (:812-818)
        double Nt = 0;
        for (int i = 0; i < NC; i++) Nt += Ni[i];
        for (int i = 0; i < NC; i++) f.zi[i] = Ni[i] / Nt;
        const double NtAll = Nt + Ni[NC];
        f.Nt = Nt;
        f.P = P;
        f.T = T;

        // ---- SkipPSAMethod01::CalFtype02 / IfSkip (src/AcceleratePEC.cpp:64-124)
        const unsigned npPE = phaseNum - 1u;
        const int ftype_in = flash_type_in(m, b, cell, Ni, Nt, P, T, Sin, npPE);

        // ---- phase equilibrium (lNP = phaseNum - 1 passed through double -> USI)
        f.eos.setup(&m, M.units.gas_constant, P, T);
        if (injected) {
            f.NP = injected->NP;
            f.ftype = injected->ftype;
            f.status = injected->status;
            f.it_ssm_sta = injected->it[0];
            f.it_nr_sta = injected->it[1];
            f.it_ssm_sp = injected->it[2];
            f.it_nr_sp = injected->it[3];
            f.it_rr = injected->it[4];
            for (int j = 0; j < 2; j++) {
                f.nu[j] = injected->nu[j];
                for (int i = 0; i < NC; i++) f.x[j][i] = injected->x[j][i];
            }
        }
        else {
            f.phase_equilibrium(ftype_in, npPE, xx[0], xx[1],
                                resume && !resume->skip && ftype_in == 2 ? resume : nullptr);
            if (f.deferred) {
                if (sink && sink->push(cell, ftype_in, npPE)) return false;
                // no room in the list: finish the equilibrium here from the start
                f.status = 0;
                f.it_ssm_sta = f.it_nr_sta = f.it_ssm_sp = f.it_nr_sp = f.it_rr = 0;
                f.work = 0;
                f.budget = 0x7fffffff;
                f.deferred = false;
                f.phase_equilibrium(ftype_in, npPE, xx[0], xx[1]);
            }
        }

        // ---- CalPropertyDer (:134-142): CopyPhaseFromPE, CalMW, CalVmVj, CalXiRhoMuDer
        const int NPh = f.NP;
        {
            const double Tc_ = T;
            for (int i = 0; i < NC; i++) {
                const double Tri = Tc_ / m.Tc[i];
                tT[i] = (Tri <= 1.5) ? 34 * 1E-5 * pow(Tri, 0.94)
                                     : 17.78 * 1E-5 * pow((4.58 * Tri - 1.67), 0.625);
            }
        }
        for (int j = 0; j < NPh; j++) {
            nj[j] = Nt * f.nu[j];
            for (int i = 0; i < NC; i++) xx[j][i] = f.x[j][i];
            MW[j] = 0;
            for (int i = 0; i < NC; i++) MW[j] += xx[j][i] * m.MW[i];
        }
        for (int j = 0; j < NPh; j++) {
            vm[j] = f.eos.cal_vm_der(xx[j], vmP[j], vmx[j]);
            vj[j] = nj[j] * vm[j];
        }
        for (int j = 0; j < NPh; j++) {
            xiv[j] = 1 / vm[j];
            xiPv[j] = -xiv[j] * xiv[j] * vmP[j];
            for (int i = 0; i < NC; i++) xix[j][i] = -xiv[j] * xiv[j] * vmx[j][i];
            rho[j] = MW[j] * xiv[j];
            rhoPv[j] = MW[j] * xiPv[j];
            for (int i = 0; i < NC; i++) rhox[j][i] = xix[j][i] * MW[j] + xiv[j] * m.MW[i];
            mu[j] = lbc_viscosity_der<NCM>(m, NC, tT, xx[j], xiv[j], xiPv[j], xix[j], muPv[j], mux[j]);
        }

        // ---- IdentifyPhase (:174-214) + ReOrderPhaseDer (:235-256)
        ex[0] = false;
        ex[1] = false;
        bool label0_oil;
        if (NPh == 1) {
            double A = 0, B = 0;
            for (int i = 0; i < NC; i++) {
                A += f.zi[i] * m.Vc[i] * m.Tc[i];
                B += f.zi[i] * m.Vc[i];
            }
            const double Tcm = A / B;
            if (T > Tcm) { label0_oil = false; ex[1] = true; }
            else         { label0_oil = true;  ex[0] = true; }
        }
        else {
            label0_oil = MW[0] > MW[1];
            ex[0] = true;
            ex[1] = true;
        }
        if (!label0_oil) swap_phases(NC);

        water_and_saturations(M, P, Ni[NC], NC);
        volume_derivatives(NC, NPh);

        // ---- CaldXsdXp02 + CaldXsdXpW (:565-642, 904-920), written straight to the SoA rows;
        // when the flash derivatives are recomputed where they are used, the
        // phase mole numbers are kept instead
        if (b.dSec_dPri) {
            dsec_rows(NC, NPh, Nt, Ni, [&](int r, int col) -> double& {
                return b.dSec_dPri[b.idx(r * ncol + col, cell)];
            });
        }
        if (b.njhc) {
            b.njhc[b.idx(0, cell)] = ex[0] ? nj[0] : 0.0;
            b.njhc[b.idx(1, cell)] = ex[1] ? nj[1] : 0.0;
        }

        // ---- SkipPSAMethod01::CalSkipForNextStep (src/AcceleratePEC.cpp:127-170)
        if (m.skip_psa) {
            if (f.ftype == 0) {
                double* lnphiN = f.lnf[0];
                f.eos.cal_lnphiN(f.zi, Nt, lnphiN);
                float Af[NCM * NCM];
                for (int i = 0; i < NC; i++)
                    for (int j = 0; j <= i; j++) {
                        const float v = (float)((i == j ? 1.0 : 0.0) + Nt * sqrt(f.zi[i] * f.zi[j]) * lnphiN[i * NC + j]);
                        Af[i * NC + j] = v;
                        Af[j * NC + i] = v;
                    }
                float Wf[NCM * NCM];
                const float eig = sym_min_eig_f32<NCM>(NC, Af, Wf);
                b.skip_flag[cell] = 1;
                b.skip_minEig[cell] = (double)eig;
                b.skip_P[cell] = P;
                b.skip_T[cell] = T;
                for (int i = 0; i < NC; i++) b.skip_zi[b.idx(i, cell)] = f.zi[i];
            }
            else if (f.ftype == 1) b.skip_flag[cell] = 1;
            else b.skip_flag[cell] = 0;
        }

        // ---- IsoT_FIM::PassFlashValue (src/IsoThermalMethod.cpp:1027-1071)
        b.Nt[cell] = NtAll;
        b.vf[cell] = Vf;
        bool finite = finite_d(Vf) && finite_d(vfP);
        for (int j = 0; j < np; j++) {
            b.S[b.idx(j, cell)] = S[j];
            b.phaseExist[b.idx(j, cell)] = ex[j] ? 1 : 0;
            if (!ex[j]) continue;
            b.rho[b.idx(j, cell)] = rho[j];
            b.xi[b.idx(j, cell)] = xiv[j];
            b.mu[b.idx(j, cell)] = mu[j];
            b.rhoP[b.idx(j, cell)] = rhoPv[j];
            b.xiP[b.idx(j, cell)] = xiPv[j];
            b.muP[b.idx(j, cell)] = muPv[j];
            finite = finite && finite_d(rho[j]) && finite_d(mu[j]);
            for (int i = 0; i < nct; i++) {
                b.xij[b.idx(j * nct + i, cell)] = xx[j][i];
                const bool hc = (j < 2) && (i < NC);
                b.rhox[b.idx(j * nct + i, cell)] = hc ? rhox[j][i] : 0.0;
                b.xix[b.idx(j * nct + i, cell)] = hc ? xix[j][i] : 0.0;
                b.mux[b.idx(j * nct + i, cell)] = hc ? mux[j][i] : 0.0;
            }
        }
        b.vfP[cell] = vfP;
        for (int i = 0; i < nct; i++) b.vfi[b.idx(i, cell)] = vfi[i];
        if (!finite) f.status |= ST_NONFINITE;
        b.status[cell] = f.status;
        b.ftype[cell] = (int8_t)f.ftype;
        b.iters[b.idx(0, cell)] = f.it_ssm_sta;
        b.iters[b.idx(1, cell)] = f.it_nr_sta;
        b.iters[b.idx(2, cell)] = f.it_ssm_sp;
        b.iters[b.idx(3, cell)] = f.it_nr_sp;
        b.iters[b.idx(4, cell)] = f.it_rr;
        return true;
    }

    // ---- CalPropertyW (src/OCPMixtureMethodComp.cpp:846-860): water always
    // present; then OCPMixtureVarSet::CalVfS (include/OCPMixtureVarSet.hpp:143-155)
    OCPX_HD void water_and_saturations(const Model& M, double P, double NiW, int NC)
    {
        const int np = 3, nct = NC + 1;
        ex[2] = true;
        xx[2][NC] = 1.0;
        pvtw_rho_xi_mu_der(M.water, M.units.conv1, P, rho[2], xiv[2], mu[2], rhoPv[2], xiPv[2], muPv[2]);
        nj[2] = NiW;
        vj[2] = nj[2] / xiv[2];
        for (int i = 0; i < nct; i++) vji[2][i] = 0;
        vji[2][NC] = 1 / xiv[2];
        vjP[2] = -nj[2] * xiPv[2] / (xiv[2] * xiv[2]);
        Vf = 0;
        for (int j = 0; j < np; j++)
            if (ex[j]) Vf += vj[j];
        for (int j = 0; j < np; j++) S[j] = ex[j] ? vj[j] / Vf : 0;
    }

    // ---- CalVfiVfp_full02 + AddVfpVfiW (src/OCPMixtureMethodComp.cpp:462-524, 896-901),
    // phases in label order; leaves the derivative solve's solution in rhs
    OCPX_HD void volume_derivatives(int NC, int NPh)
    {
        for (int j = 0; j < 2; j++) vji[j][NC] = 0;
        if (NPh == 1) {
            const int j = ex[0] ? 0 : 1;
            vjP[j] = nj[j] * vmP[j];
            vfP = vjP[j];
            for (int i = 0; i < NC; i++) {
                vji[j][i] = vm[j] + vmx[j][i];
                for (int k = 0; k < NC; k++) vji[j][i] -= vmx[j][k] * xx[j][k];
                vfi[i] = vji[j][i];
            }
        }
        else {
            double* lnN0 = f.lnf[0];
            double* lnN1 = f.lnf[1];
            double lnP0[NCM], lnP1[NCM];
            f.eos.cal_lnfugN(xx[0], nj[0], lnN0);
            f.eos.cal_lnfugP(xx[0], lnP0);
            f.eos.cal_lnfugN(xx[1], nj[1], lnN1);
            f.eos.cal_lnfugP(xx[1], lnP1);
            double* Jd = f.J;
            for (int i = 0; i < NC; i++)
                for (int mm = 0; mm < NC; mm++) Jd[i * NC + mm] = lnN0[i * NC + mm] + lnN1[i * NC + mm];
            for (int i = 0; i < NC; i++) rhs[i] = lnP1[i] - lnP0[i];
            for (int k = 0; k < NC; k++)
                for (int i = 0; i < NC; i++) rhs[(k + 1) * NC + i] = lnN1[k * NC + i];
            if (!gen_solve_colmajor<NCM>(NC, Jd, rhs, NC + 1, f.W)) f.status |= ST_SINGULAR;
            double tmp0 = 0, tmp1 = 0;
            for (int i = 0; i < NC; i++) {
                tmp0 -= vmx[0][i] * xx[0][i];
                tmp1 -= vmx[1][i] * xx[1][i];
            }
            const double* dP = rhs;
            vjP[0] = nj[0] * vmP[0];
            vjP[1] = nj[1] * vmP[1];
            for (int k = 0; k < NC; k++) {
                vjP[0] += (vm[0] + tmp0 + vmx[0][k]) * dP[k];
                vjP[1] -= (vm[1] + tmp1 + vmx[1][k]) * dP[k];
            }
            vfP = vjP[0] + vjP[1];
            for (int i = 0; i < NC; i++) {
                const double* dN = rhs + (i + 1) * NC;
                vji[0][i] = 0;
                vji[1][i] = 0;
                for (int k = 0; k < NC; k++) {
                    vji[0][i] += (vm[0] + tmp0 + vmx[0][k]) * dN[k];
                    vji[1][i] += (vm[1] + tmp1 + vmx[1][k]) * ((i == k ? 1.0 : 0.0) - dN[k]);
                }
                vfi[i] = vji[0][i] + vji[1][i];
            }
        }
        vfP += vjP[2];
        vfi[NC] = vji[2][NC];
    }

    // ---- CaldXsdXp02 + CaldXsdXpW (src/OCPMixtureMethodComp.cpp:565-642, 904-920):
    // dSec_dPri row by row through dX(row, column)
    template <class F>
    OCPX_HD void dsec_rows(int NC, int NPh, double Nt, const double* Ni, F dX)
    {
        const int np = 3, nct = NC + 1, ncol = nct + 1;
        const int nrow = np * nct + np;
        for (int r = 0; r < nrow; r++)
            for (int col = 0; col < ncol; col++) dX(r, col) = 0;
        for (int j = 0; j < 2; j++) {
            if (!ex[j]) continue;
            dX(j, 0) = (vjP[j] - vfP * S[j]) / Vf;
            for (int mm = 0; mm < NC; mm++) dX(j, 1 + mm) = (vji[j][mm] - vfi[mm] * S[j]) / Vf;
        }
        if (NPh == 1) {
            const int j = ex[0] ? 0 : 1;
            for (int i = 0; i < NC; i++)
                for (int mm = 0; mm < NC; mm++)
                    dX(np + j * nct + i, 1 + mm) = ((i == mm ? 1.0 : 0.0) * Nt - Ni[i]) / (Nt * Nt);
        }
        else {
            double njDerSum = 0;
            for (int i = 0; i < NC; i++) njDerSum += rhs[i];
            for (int i = 0; i < NC; i++) {
                dX(np + 0 * nct + i, 0) = (rhs[i] - njDerSum * xx[0][i]) / nj[0];
                dX(np + 1 * nct + i, 0) = (-rhs[i] + njDerSum * xx[1][i]) / nj[1];
            }
            for (int mm = 0; mm < NC; mm++) {
                const double* dN = rhs + (mm + 1) * NC;
                njDerSum = 0;
                for (int i = 0; i < NC; i++) njDerSum += dN[i];
                for (int i = 0; i < NC; i++) {
                    dX(np + 0 * nct + i, mm + 1) = (dN[i] - njDerSum * xx[0][i]) / nj[0];
                    dX(np + 1 * nct + i, mm + 1) =
                        (((i == mm ? 1.0 : 0.0) - dN[i]) - (1 - njDerSum) * xx[1][i]) / nj[1];
                }
            }
        }
        for (int j = 0; j < 2; j++)
            if (ex[j]) dX(j, NC + 1) = (vji[j][NC] - vfi[NC] * S[j]) / Vf;
        dX(2, 0) = (vjP[2] - vfP * S[2]) / Vf;
        for (int i = 0; i < nct; i++) dX(2, 1 + i) = (vji[2][i] - vfi[i] * S[2]) / Vf;
    }

    // The prologue of run() for a cell whose flash starts with the phase split
    // (flash type 2), up to the split's first successive-substitution loop,
    // which L then drives one pass at a time (CompFlash::split_ssm_step).
    // False, with nothing set up, for a cell of another flash type.
    OCPX_HD bool split_begin(const Model& M, const BulkView& b, int cell, typename CompFlash<NCM>::SsmLoop& L)
    {
        const CompModel& m = M.comp;
        const int NC = m.nc, nct = NC + 1, np = 3;
        f.m = &m;
        f.NC = NC;
        f.status = 0;
        f.it_ssm_sta = f.it_nr_sta = f.it_ssm_sp = f.it_nr_sp = f.it_rr = 0;
        f.work = 0;
        f.budget = 0x7fffffff;
        f.deferred = false;
        const double P = b.P[cell];
        const double T = b.T[cell] + M.units.conv4;
        double Ni[NCM + 1];
        for (int i = 0; i < nct; i++) Ni[i] = b.Ni[b.idx(i, cell)];
        double Sin[3];
        unsigned phaseNum = 0;
        for (int j = 0; j < np; j++) {
            Sin[j] = b.S[b.idx(j, cell)];
            if (b.phaseExist[b.idx(j, cell)] != 0) phaseNum++;
        }
        for (int j = 0; j < 2; j++)
            for (int i = 0; i < nct; i++) xx[j][i] = b.xij[b.idx(j * nct + i, cell)];
        double Nt = 0;
        for (int i = 0; i < NC; i++) Nt += Ni[i];
        for (int i = 0; i < NC; i++) f.zi[i] = Ni[i] / Nt;
        f.Nt = Nt;
        f.P = P;
        f.T = T;
        const unsigned npPE = phaseNum - 1u;
        if (flash_type_in(m, b, cell, Ni, Nt, P, T, Sin, npPE) != 2) return false;
        f.eos.setup(&m, M.units.gas_constant, P, T);
        f.split_prologue(npPE, xx[0], xx[1]);
        f.split_ssm_init(false, L);
        return true;
    }

    // dSec_dPri of a cell recomputed from the state its flash left (P, T, Ni,
    // phase labels, x_ij and the hydrocarbon phases' mole numbers), with the
    // flash's own statements in the same order, so the values are the ones
    // the flash would have stored: out[(row * (nc + 1) + column) * stride].
    OCPX_HD void recompute_dsec(const Model& M, const BulkView& b, int cell, double* out, size_t stride)
    {
        const CompModel& m = M.comp;
        const int NC = m.nc, nct = NC + 1, ncol = nct + 1;
        f.m = &m;
        f.NC = NC;
        f.status = 0;
        const double P = b.P[cell];
        const double T = b.T[cell] + M.units.conv4;
        double Ni[NCM + 1];
        for (int i = 0; i < nct; i++) Ni[i] = b.Ni[b.idx(i, cell)];
        double Nt = 0;
        for (int i = 0; i < NC; i++) Nt += Ni[i];
        f.eos.setup(&m, M.units.gas_constant, P, T);
        int NPh = 0;
        for (int j = 0; j < 2; j++) {
            ex[j] = b.phaseExist[b.idx(j, cell)] != 0;
            if (!ex[j]) continue;
            NPh++;
            nj[j] = b.njhc[b.idx(j, cell)];
            for (int i = 0; i < NC; i++) xx[j][i] = b.xij[b.idx(j * nct + i, cell)];
            vm[j] = f.eos.cal_vm_der(xx[j], vmP[j], vmx[j]);
            vj[j] = nj[j] * vm[j];
        }
        water_and_saturations(M, P, Ni[NC], NC);
        volume_derivatives(NC, NPh);
        dsec_rows(NC, NPh, Nt, Ni, [&](int r, int col) -> double& { return out[(size_t)(r * ncol + col) * stride]; });
    }

    OCPX_HD void swap_phases(int NC)
    {
        auto sw = [](double& a, double& c) { const double t = a; a = c; c = t; };
        sw(nj[0], nj[1]);
        for (int i = 0; i < NC; i++) sw(xx[0][i], xx[1][i]);
        sw(MW[0], MW[1]);
        sw(vj[0], vj[1]);
        sw(vm[0], vm[1]);
        sw(vmP[0], vmP[1]);
        for (int i = 0; i < NC; i++) sw(vmx[0][i], vmx[1][i]);
        sw(xiv[0], xiv[1]);
        sw(xiPv[0], xiPv[1]);
        for (int i = 0; i < NC; i++) sw(xix[0][i], xix[1][i]);
        sw(rho[0], rho[1]);
        sw(rhoPv[0], rhoPv[1]);
        for (int i = 0; i < NC; i++) sw(rhox[0][i], rhox[1][i]);
        sw(mu[0], mu[1]);
        sw(muPv[0], muPv[1]);
        for (int i = 0; i < NC; i++) sw(mux[0][i], mux[1][i]);
    }
};

}  // namespace ocpx
