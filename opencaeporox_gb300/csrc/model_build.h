// Host-side construction of the device model block from the C-ABI model
// description (no CUDA calls; shared by the library and host-side tools).
#pragma once
#include <cmath>
#include <cstring>
#include <string>
#include "ocpx.h"
#include "ocpx_common.cuh"

namespace ocpx {

inline bool copy_table(Table& t, const ocpx_table& src, int ncol_expected, std::string& err, const char* name)
{
    if (src.nrow <= 0 || src.nrow > TAB_ROWS_MAX || src.ncol != ncol_expected || !src.data) {
        err = std::string("table ") + name + ": need 1.." + std::to_string(TAB_ROWS_MAX) + " rows and " +
              std::to_string(ncol_expected) + " columns";
        return false;
    }
    t.nrow = src.nrow;
    t.ncol = src.ncol;
    std::memcpy(t.data, src.data, sizeof(double) * src.nrow * src.ncol);
    return true;
}

// ParamReservoir -> device model; the PR kappa(omega) and the LBC helper
// constants are evaluated here with the host libm exactly as the reference's
// constructors evaluate them (src/OCPEoS.cpp:68-84, src/OCPFuncPVT.cpp:415-460).
inline ocpx_status fail_msg(std::string& out, const char* m)
{
    out = m;
    return OCPX_INVALID_ARG;
}

inline ocpx_status build_model(const ocpx_model_desc* md, Model& m, std::string& err_out)
{
    std::memset(&m, 0, sizeof(Model));
    std::string err;
    m.mixture = md->mixture;
    m.np = 3;
    m.nc = md->nc;
    m.units = {md->gravity_factor, md->conv_darcy, md->gas_constant, md->conv1, md->conv3, md->conv4};
    m.rock = {md->rock_pref, md->rock_cp1, md->rock_cp2};
    if (!copy_table(m.sat.swof, md->swof, 4, err, "SWOF")) { err_out = err; return OCPX_INVALID_ARG; }
    if (!copy_table(m.sat.sgof, md->sgof, 4, err, "SGOF")) { err_out = err; return OCPX_INVALID_ARG; }
    m.sat.krocw = md->swof.data[2 * md->swof.nrow + 0];  // OCP_SWOF::GetKrocw: krow at the first row
    if (!copy_table(m.water.pvtw, md->pvtw, 5, err, "PVTW")) { err_out = err; return OCPX_INVALID_ARG; }
    m.water.std_rho_w = md->std_rho_w;
    m.water.std_vw = md->std_vw;
    if (md->mixture == 0) {
        if (md->nc != 3) return fail_msg(err_out, "black-oil model needs nc = 3");
        if (!copy_table(m.bo.pvco, md->pvco, 6, err, "PVCO")) { err_out = err; return OCPX_INVALID_ARG; }
        if (!copy_table(m.bo.pvdg, md->pvdg, 3, err, "PVDG")) { err_out = err; return OCPX_INVALID_ARG; }
        m.bo.std_rho_o = md->std_rho_o;
        m.bo.std_rho_g = md->std_rho_g;
        m.bo.std_vo = md->std_vo;
        m.bo.std_vg = md->std_vg;
    }
    else if (md->mixture == 1) {
        const int NC = md->nc - 1;
        if (NC < 1 || NC > NC_MAX) return fail_msg(err_out, "compositional model needs 1..12 components");
        if (!md->Tc || !md->Pc || !md->Vc || !md->MW || !md->OmegaA || !md->OmegaB || !md->acf || !md->BIC ||
            !md->Vshift || !md->Vcvis || !md->lbc_coef || !md->flash_ctrl)
            return fail_msg(err_out, "compositional model arrays missing");
        CompModel& c = m.comp;
        c.nc = NC;
        for (int i = 0; i < NC; i++) {
            c.Tc[i] = md->Tc[i];
            c.Pc[i] = md->Pc[i];
            c.Vc[i] = md->Vc[i];
            c.MW[i] = md->MW[i];
            c.OmegaA[i] = md->OmegaA[i];
            c.OmegaB[i] = md->OmegaB[i];
            c.acf[i] = md->acf[i];
            c.Vshift[i] = md->Vshift[i];
            c.Vcvis[i] = md->Vcvis[i];
            const double a = c.acf[i];
            c.mwi[i] = (a <= 0.49) ? 0.37464 + 1.54226 * a - 0.26992 * std::pow(a, 2)
                                   : 0.379642 + 1.48503 * a - 0.164423 * std::pow(a, 2) + 0.016667 * std::pow(a, 3);
            c.sqrtMW[i] = std::sqrt(c.MW[i]);
            c.auxB[i] = 5.4402 * std::pow(c.Tc[i], 1.0 / 6) / std::pow(c.Pc[i], 2.0 / 3);
            for (int k = 0; k < NC; k++) c.omb[i * NC_MAX + k] = 1 - md->BIC[i * NC + k];
        }
        for (int k = 0; k < 5; k++) c.lbc[k] = md->lbc_coef[k];
        const double* f = md->flash_ctrl;
        c.ssm_sta_maxit = (int)f[0];
        c.ssm_sta_tol = f[1];
        c.ssm_sta_tol2 = f[1] * f[1];
        c.ssm_sta_eYt = f[2];
        c.ssm_sta_Ktol = f[3];
        c.ssm_sta_dYtol = f[4];
        c.nr_sta_maxit = (int)f[5];
        c.nr_sta_tol = f[6];
        c.ssm_sp_maxit = (int)f[7];
        c.ssm_sp_tol2 = f[8] * f[8];
        c.nr_sp_maxit = (int)f[9];
        c.nr_sp_tol = f[10];
        c.rr_maxit = (int)f[11];
        c.rr_tol = f[12];
        c.skip_psa = md->skip_psa;
    }
    else {
        return fail_msg(err_out, "mixture must be 0 (black-oil) or 1 (compositional)");
    }
    return OCPX_OK;
}


}  // namespace ocpx
