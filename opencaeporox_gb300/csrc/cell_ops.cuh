// Per-cell operations of the FIM step other than the compositional flash:
// black-oil FlashDer, relative permeability / capillary pressure, rock,
// the Newton update of the primary variables and the physical checks.
#pragma once
#include "bulk_view.cuh"
#include "flash_comp.cuh"

namespace ocpx {

// ---------------------------------------------------------------------------
// Black-oil OGW (live oil, dry gas, water), OCPMixtureMethodK_OGW01::FlashDer
// (src/OCPMixtureMethodK.cpp:521-759) with OCP_PVCO / OCP_PVDG / OCP_PVTW
// (src/OCPFuncPVT.cpp:22-196).  Components: 0 oil, 1 gas, 2 water.
// Pure rational arithmetic: with FMA contraction disabled the result is
// bit-identical to the reference.
struct BoPVT {
    const BlackOilModel& bo;
    const Units& u;
    // OCP_PVCO::CalRs via OCPTable::Eval(0, P, 1)
    OCPX_HD double rs_of_p(double P) const { return table_eval(bo.pvco, 0, P, 1); }
    // OCP_PVCO::CalRhoXiMuRsDer (:87-99) with CalRsBoMuoDer (:102-114)
    OCPX_HD void oil_sat(double P, double& rho, double& xi, double& mu, double& rs, double& rhoP, double& xiP,
                         double& muP, double& rsP) const
    {
        double d[6], cd[6];
        table_eval_all(bo.pvco, 0, P, d, cd);
        rs = d[1];
        const double b = d[2];
        mu = d[3];
        rsP = cd[1];
        const double bP = cd[2];
        muP = cd[3];
        const double x = rs * (bo.std_vo / bo.std_vg);
        const double xP = rsP * (bo.std_vo / bo.std_vg);
        xi = (1 + x) / (b * u.conv1 * bo.std_vo);
        xiP = (xP * b - (1 + x) * bP) / ((b * b) * (u.conv1 * bo.std_vo));
        rho = (bo.std_rho_o + u.conv3 * rs * bo.std_rho_g) / b;
        rhoP = u.conv3 * bo.std_rho_g * rsP / b - (bo.std_rho_o + u.conv3 * rs * bo.std_rho_g) * bP / (b * b);
    }
    // OCP_PVCO::CalRhoXiMuDer (:117-133) with CalBoMuoDer (:136-155): undersaturated
    OCPX_HD void oil_unsat(double rs, double P, double& rho, double& xi, double& mu, double& rhoP, double& xiP,
                           double& muP, double& rhoRs, double& xiRs, double& muRs) const
    {
        double d[6], cd[6];
        table_eval_all(bo.pvco, 1, rs, d, cd);
        const double Pref = d[0], bref = d[2], muref = d[3], Cbref = d[4], Cmuref = d[5];
        const double PrefRs = cd[0], brefRs = cd[2], murefRs = cd[3], CbrefRs = cd[4], CmurefRs = cd[5];
        const double b = bref * (1 - Cbref * (P - Pref));
        const double bP = -bref * Cbref;
        const double bRs = brefRs * (1 - Cbref * (P - Pref)) + bref * (-CbrefRs * (P - Pref) + Cbref * PrefRs);
        mu = muref * (1 + Cmuref * (P - Pref));
        muP = muref * Cmuref;
        muRs = murefRs * (1 + Cmuref * (P - Pref)) + muref * (CmurefRs * (P - Pref) - Cmuref * PrefRs);
        const double x = rs * (bo.std_vo / bo.std_vg);
        const double xRs = bo.std_vo / bo.std_vg;
        xi = (1 + x) / (b * u.conv1 * bo.std_vo);
        xiP = -(1 + x) * bP / ((b * b) * (u.conv1 * bo.std_vo));
        xiRs = (xRs * b - (1 + x) * bRs) / ((b * b) * u.conv1 * bo.std_vo);
        rho = (bo.std_rho_o + u.conv3 * rs * bo.std_rho_g) / b;
        rhoP = -(bo.std_rho_o + u.conv3 * rs * bo.std_rho_g) * bP / (b * b);
        rhoRs = (u.conv3 * bo.std_rho_g * b - (bo.std_rho_o + u.conv3 * rs * bo.std_rho_g) * bRs) / (b * b);
    }
    // OCP_PVDG::CalRhoXiMuDer (:167-196)
    OCPX_HD void gas(double P, double& rho, double& xi, double& mu, double& rhoP, double& xiP, double& muP) const
    {
        double d[3], cd[3];
        table_eval_all(bo.pvdg, 0, P, d, cd);
        const double b = d[1];
        mu = d[2];
        const double bp = cd[1];
        muP = cd[2];
        xi = 1 / u.conv1 / (b * bo.std_vg);
        xiP = -1 / u.conv1 * bp / ((b * b) * bo.std_vg);
        rho = u.conv3 * bo.std_rho_g / b;
        rhoP = -u.conv3 * bo.std_rho_g * bp / (b * b);
    }
    OCPX_HD double xi_gas(double P) const
    {
        return 1 / u.conv1 / (table_eval(bo.pvdg, 0, P, 1) * bo.std_vg);
    }
};

OCPX_HD void bo_flash_der_cell(const Model& M, const BulkView& b, int cell)
{
    const int np = 3, nc = 3, ncol = 4;
    BoPVT pvt{M.bo, M.units};
    const double P = b.P[cell];
    double Ni[3];
    for (int i = 0; i < nc; i++) Ni[i] = b.Ni[b.idx(i, cell)];
    double S[3], rho[3], xi[3], mu[3], rhoP[3] = {0, 0, 0}, xiP[3] = {0, 0, 0}, muP[3] = {0, 0, 0};
    double rhox[9] = {0}, xix[9] = {0}, mux[9] = {0};
    double dX[20] = {0};
    double vj[3], vjP[3] = {0, 0, 0}, vji[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, vfi[3];
    bool ex[3];
    double xo0 = 0, xo1 = 0;  // oil-phase composition (only set where the reference sets it)
    bool set_xo = false;
    double Vf, vfP;
    // load the previous values the reference leaves in place for absent phases
    for (int j = 0; j < np; j++) {
        rho[j] = b.rho[b.idx(j, cell)];
        xi[j] = b.xi[b.idx(j, cell)];
        mu[j] = b.mu[b.idx(j, cell)];
    }
    const double Nt = Ni[0] + Ni[1] + Ni[2];
    double x = pvt.rs_of_p(P) * M.bo.std_vo / M.bo.std_vg;
    pvtw_rho_xi_mu_der(M.water, M.units.conv1, P, rho[2], xi[2], mu[2], rhoP[2], xiP[2], muP[2]);

    if (Ni[0] < Nt * TINY) {
        if (Ni[1] <= Ni[0] * x) {
            // water only
            ex[0] = false; ex[1] = false; ex[2] = true;
            S[0] = 0; S[1] = 0; S[2] = 1;
            vj[0] = 0; vj[1] = 0; vj[2] = Ni[2] / xi[2];
            Vf = vj[2];
            vjP[2] = -Ni[2] * xiP[2] / (xi[2] * xi[2]);
            vfP = vjP[2];
            vji[2][2] = 1 / xi[2];
            vfi[0] = 0; vfi[1] = 0; vfi[2] = vji[2][2];
            dX[1 * 4 + 2] = 1 / pvt.xi_gas(P) / Vf;
            dX[2 * 4 + 0] = (vjP[2] - S[2] * vfP) / Vf;
            dX[2 * 4 + 1] = -S[2] * vfi[0] / Vf;
            dX[2 * 4 + 2] = -S[2] * vfi[1] / Vf;
            dX[2 * 4 + 3] = (vji[2][2] - S[2] * vfi[2]) / Vf;
        }
        else {
            // dry gas and water
            ex[0] = false; ex[1] = true; ex[2] = true;
            pvt.gas(P, rho[1], xi[1], mu[1], rhoP[1], xiP[1], muP[1]);
            double rs, rsP;
            pvt.oil_sat(P, rho[0], xi[0], mu[0], rs, rhoP[0], xiP[0], muP[0], rsP);
            x = rs * (M.bo.std_vo / M.bo.std_vg);
            const double xP = rsP * (M.bo.std_vo / M.bo.std_vg);
            vj[0] = 0;
            vj[1] = (Ni[1] - x * Ni[0]) / xi[1];
            vj[2] = Ni[2] / xi[2];
            Vf = vj[1] + vj[2];
            S[0] = 0;
            S[1] = vj[1] / Vf;
            S[2] = vj[2] / Vf;
            vjP[0] = Ni[0] * (xP * xi[0] - (1 + x) * xiP[0]) / (xi[0] * xi[0]);
            vjP[1] = (-xP * Ni[0] * xi[1] - (Ni[1] - x * Ni[0]) * xiP[1]) / (xi[1] * xi[1]);
            vjP[2] = -Ni[2] * xiP[2] / (xi[2] * xi[2]);
            vfP = vjP[0] + vjP[1] + vjP[2];
            vji[0][0] = (1 + x) / xi[0];
            vji[1][0] = -x / xi[1];
            vji[1][1] = 1 / xi[1];
            vji[2][2] = 1 / xi[2];
            vfi[0] = vji[0][0] + vji[1][0];
            vfi[1] = vji[1][1];
            vfi[2] = vji[2][2];
            dX[1] = vji[0][0] / Vf;
            dX[1 * 4 + 0] = (vjP[1] - S[1] * vfP) / Vf;
            dX[1 * 4 + 1] = (vji[1][0] - S[1] * vfi[0]) / Vf;
            dX[1 * 4 + 2] = (vji[1][1] - S[1] * vfi[1]) / Vf;
            dX[1 * 4 + 3] = -S[1] * vfi[2] / Vf;
            dX[2 * 4 + 0] = (vjP[2] - S[2] * vfP) / Vf;
            dX[2 * 4 + 1] = -S[2] * vfi[0] / Vf;
            dX[2 * 4 + 2] = -S[2] * vfi[1] / Vf;
            dX[2 * 4 + 3] = (vji[2][2] - S[2] * vfi[2]) / Vf;
            dX[3 * 4 + 0] = -xP / ((1 + x) * (1 + x));
            dX[4 * 4 + 0] = -dX[3 * 4 + 0];
        }
    }
    else if (Ni[1] <= Ni[0] * x) {
        // undersaturated oil and water
        x = Ni[1] / Ni[0];
        ex[0] = true; ex[1] = false; ex[2] = true;
        xo0 = 1 / (1 + x);
        xo1 = 1 - xo0;
        set_xo = true;
        const double rs = x * (M.bo.std_vg / M.bo.std_vo);
        double rhooRs, xioRs, muoRs;
        pvt.oil_unsat(rs, P, rho[0], xi[0], mu[0], rhoP[0], xiP[0], muP[0], rhooRs, xioRs, muoRs);
        const double xiox = xioRs * (M.bo.std_vg / M.bo.std_vo);
        const double rhoox = rhooRs * (M.bo.std_vg / M.bo.std_vo);
        const double muox = muoRs * (M.bo.std_vg / M.bo.std_vo);
        vj[0] = (Ni[0] + Ni[1]) / xi[0];
        vj[1] = 0;
        vj[2] = Ni[2] / xi[2];
        Vf = vj[0] + vj[2];
        S[0] = vj[0] / Vf;
        S[1] = 0;
        S[2] = vj[2] / Vf;
        vjP[0] = -(Ni[0] + Ni[1]) * xiP[0] / (xi[0] * xi[0]);
        vjP[2] = -Ni[2] * xiP[2] / (xi[2] * xi[2]);
        vfP = vjP[0] + vjP[2];
        vji[0][0] = (xi[0] + x * (1 + x) * xiox) / (xi[0] * xi[0]);
        vji[0][1] = (xi[0] - (1 + x) * xiox) / (xi[0] * xi[0]);
        vji[2][2] = 1 / xi[2];
        vfi[0] = vji[0][0];
        vfi[1] = vji[0][1];
        vfi[2] = vji[2][2];
        dX[0] = (vjP[0] - S[0] * vfP) / Vf;
        dX[1] = (vji[0][0] - S[0] * vfi[0]) / Vf;
        dX[2] = (vji[0][1] - S[0] * vfi[1]) / Vf;
        dX[3] = -S[0] / Vf * vfi[2];
        dX[2 * 4 + 0] = (vjP[2] - S[2] * vfP) / Vf;
        dX[2 * 4 + 1] = -S[2] * vfi[0] / Vf;
        dX[2 * 4 + 2] = -S[2] * vfi[1] / Vf;
        dX[2 * 4 + 3] = (vji[2][2] - S[2] * vfi[2]) / Vf;
        dX[3 * 4 + 1] = Ni[1] / pow((Ni[0] + Ni[1]), 2);
        dX[3 * 4 + 2] = -Ni[0] / pow((Ni[0] + Ni[1]), 2);
        dX[4 * 4 + 1] = -dX[3 * 4 + 1];
        dX[4 * 4 + 2] = -dX[3 * 4 + 2];
        const double tmp_new = (1 + x) * (1 + x);
        mux[0] = -muox * tmp_new;
        mux[1] = muox * tmp_new;
        xix[0] = -xiox * tmp_new;
        xix[1] = xiox * tmp_new;
        rhox[0] = -rhoox * tmp_new;
        rhox[1] = rhoox * tmp_new;
    }
    else {
        // saturated oil, gas and water
        ex[0] = true; ex[1] = true; ex[2] = true;
        double rs, rsP;
        pvt.oil_sat(P, rho[0], xi[0], mu[0], rs, rhoP[0], xiP[0], muP[0], rsP);
        pvt.gas(P, rho[1], xi[1], mu[1], rhoP[1], xiP[1], muP[1]);
        x = rs * (M.bo.std_vo / M.bo.std_vg);
        const double xP = rsP * (M.bo.std_vo / M.bo.std_vg);
        xo0 = 1 / (1 + x);
        xo1 = 1 - xo0;
        set_xo = true;
        vj[0] = Ni[0] * (1 + x) / xi[0];
        vj[1] = (Ni[1] - x * Ni[0]) / xi[1];
        vj[2] = Ni[2] / xi[2];
        Vf = vj[0] + vj[1] + vj[2];
        S[0] = vj[0] / Vf;
        S[1] = vj[1] / Vf;
        S[2] = vj[2] / Vf;
        vjP[0] = Ni[0] * (xP * xi[0] - (1 + x) * xiP[0]) / (xi[0] * xi[0]);
        vjP[1] = (-xP * Ni[0] * xi[1] - (Ni[1] - x * Ni[0]) * xiP[1]) / (xi[1] * xi[1]);
        vjP[2] = -Ni[2] * xiP[2] / (xi[2] * xi[2]);
        vfP = vjP[0] + vjP[1] + vjP[2];
        vji[0][0] = (1 + x) / xi[0];
        vji[1][0] = -x / xi[1];
        vji[1][1] = 1 / xi[1];
        vji[2][2] = 1 / xi[2];
        vfi[0] = vji[0][0] + vji[1][0];
        vfi[1] = vji[1][1];
        vfi[2] = vji[2][2];
        dX[0 * 4 + 0] = (vjP[0] - S[0] * vfP) / Vf;
        dX[0 * 4 + 1] = (vji[0][0] - S[0] * vfi[0]) / Vf;
        dX[0 * 4 + 2] = -S[0] * vfi[1] / Vf;
        dX[0 * 4 + 3] = -S[0] * vfi[2] / Vf;
        dX[1 * 4 + 0] = (vjP[1] - S[1] * vfP) / Vf;
        dX[1 * 4 + 1] = (vji[1][0] - S[1] * vfi[0]) / Vf;
        dX[1 * 4 + 2] = (vji[1][1] - S[1] * vfi[1]) / Vf;
        dX[1 * 4 + 3] = -S[1] * vfi[2] / Vf;
        dX[2 * 4 + 0] = (vjP[2] - S[2] * vfP) / Vf;
        dX[2 * 4 + 1] = -S[2] * vfi[0] / Vf;
        dX[2 * 4 + 2] = -S[2] * vfi[1] / Vf;
        dX[2 * 4 + 3] = (vji[2][2] - S[2] * vfi[2]) / Vf;
        dX[3 * 4 + 0] = -xP / ((1 + x) * (1 + x));
        dX[4 * 4 + 0] = -dX[3 * 4 + 0];
    }

    // PassFlashValue (src/IsoThermalMethod.cpp:1027-1071).  The black-oil
    // mixture keeps x_g = (0,1,0) and x_w = (0,0,1) fixed and only writes the
    // oil composition in the oil-present branches; the varset it reads from is
    // shared by all cells, so an oil phase flagged present carries the values
    // of this branch.
    b.Nt[cell] = Nt;
    b.vf[cell] = Vf;
    const double xfix[3][3] = {{xo0, xo1, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int j = 0; j < np; j++) {
        b.S[b.idx(j, cell)] = S[j];
        b.phaseExist[b.idx(j, cell)] = ex[j] ? 1 : 0;
        if (!ex[j]) continue;
        b.rho[b.idx(j, cell)] = rho[j];
        b.xi[b.idx(j, cell)] = xi[j];
        b.mu[b.idx(j, cell)] = mu[j];
        b.rhoP[b.idx(j, cell)] = rhoP[j];
        b.xiP[b.idx(j, cell)] = xiP[j];
        b.muP[b.idx(j, cell)] = muP[j];
        for (int i = 0; i < nc; i++) {
            if (j != 0 || set_xo) b.xij[b.idx(j * nc + i, cell)] = xfix[j][i];
            b.rhox[b.idx(j * nc + i, cell)] = rhox[j * nc + i];
            b.xix[b.idx(j * nc + i, cell)] = xix[j * nc + i];
            b.mux[b.idx(j * nc + i, cell)] = mux[j * nc + i];
        }
    }
    b.vfP[cell] = vfP;
    for (int i = 0; i < nc; i++) b.vfi[b.idx(i, cell)] = vfi[i];
    for (int k = 0; k < np * (nc + 1) * ncol; k++) b.dSec_dPri[b.idx(k, cell)] = dX[k < 20 ? k : 0] * (k < 20 ? 1.0 : 0.0);
    b.status[cell] = finite_d(Vf) ? ST_OK : ST_NONFINITE;
    b.ftype[cell] = -1;
}

// ---------------------------------------------------------------------------
// IsoT_FIM::CalKrPc (src/IsoThermalMethod.cpp:1073-1088) through
// OCPFlowMethod_OGW01::CalKrPcDer (src/OCPFlowMethod.cpp:63-70): SWOF and
// SGOF interpolation, Stone II oil relative permeability
// (OCP3POilPerMethod01::CalOilPerDer, src/OCPFuncSAT.cpp:162-190), then
// Pj = P + Pc; followed by IsothermalMethod::CalRock (:19-30).
OCPX_HD void krpc_rock_cell(const Model& M, const BulkView& b, int cell)
{
    const int np = 3;
    const int o = 0, g = 1, w = 2;
    const double So = b.S[b.idx(o, cell)];
    const double Sg = b.S[b.idx(g, cell)];
    const double Sw = b.S[b.idx(w, cell)];
    (void)So;
    double kr[3], Pc[3] = {0, 0, 0}, dKrdS[9] = {0}, dPcdS[9] = {0};
    double d[4], cd[4];
    table_eval_all(M.sat.swof, 0, Sw, d, cd);
    kr[w] = d[1];
    const double krow = d[2];
    Pc[w] = -d[3];
    dKrdS[w * np + w] = cd[1];
    const double dKrowdSw = cd[2];
    dPcdS[w * np + w] = -cd[3];
    table_eval_all(M.sat.sgof, 0, Sg, d, cd);
    kr[g] = d[1];
    const double krog = d[2];
    Pc[g] = d[3];
    dKrdS[g * np + g] = cd[1];
    const double dKrogdSg = cd[2];
    dPcdS[g * np + g] = cd[3];
    // Stone II; dKrowdSo and dKrogdSo are never assigned in the reference
    // (OCPFlowVarSet::Init0 sets them to 0), so dkro/dSo is identically 0.
    const double krocw = M.sat.krocw;
    const double dKrowdSo = 0, dKrogdSo = 0;
    kr[o] = krocw * ((krow / krocw + kr[w]) * (krog / krocw + kr[g]) - (kr[w] + kr[g]));
    if (kr[o] < 0) {
        kr[o] = 0;
        dKrdS[o * np + o] = 0;
        dKrdS[o * np + g] = 0;
        dKrdS[o * np + w] = 0;
    }
    else {
        dKrdS[o * np + o] = dKrowdSo * (krog / krocw + kr[g]) + dKrogdSo * (krow / krocw + kr[w]);
        dKrdS[o * np + w] = krocw * ((dKrowdSw / krocw + dKrdS[w * np + w]) * (krog / krocw + kr[g]) - (dKrdS[w * np + w]));
        dKrdS[o * np + g] = krocw * ((krow / krocw + kr[w]) * (dKrogdSg / krocw + dKrdS[g * np + g]) - (dKrdS[g * np + g]));
    }
    const double P = b.P[cell];
    for (int j = 0; j < np; j++) {
        b.kr[b.idx(j, cell)] = kr[j];
        b.Pc[b.idx(j, cell)] = Pc[j];
        b.Pj[b.idx(j, cell)] = P + Pc[j];
    }
    for (int k = 0; k < np * np; k++) {
        b.dKrdS[b.idx(k, cell)] = dKrdS[k];
        b.dPcdS[b.idx(k, cell)] = dPcdS[k];
    }
    // OCPRockIsoT_Linear::CalPoro (src/OCPRock.cpp:19-24)
    const double dP = (P - M.rock.Pref);
    const double pi = b.poroInit[cell];
    const double poro = pi * (1 + (M.rock.cp1 + M.rock.cp2 / 2 * dP) * dP);
    b.poro[cell] = poro;
    b.poroP[cell] = pi * (M.rock.cp1 + M.rock.cp2 * dP);
    b.rockVp[cell] = b.v[cell] * poro;
}

// ---------------------------------------------------------------------------
// IsoT_FIM::GetSolution (src/IsoThermalMethod.cpp:1282-1418), one cell:
// secondary update dtmp = dSec_dPri * u with the saturation chop, then S,
// x_ij, P (unchopped) and Ni (chopped).  u holds (dP, dN_0..dN_nc-1) per cell.
// The cell's dSec_dPri is at ds[(row * (nc + 1) + col) * stride]: the stored
// SoA rows, or a copy recomputed before the update.
OCPX_HD void newton_update_cell(const BulkView& b, int cell, const double* u, double dSmax, const double* ds,
                                size_t stride)
{
    const int np = b.np, nc = b.nc, col = nc + 1, row = np * (nc + 1);
    double uc[NCT_MAX + 1];
    for (int k = 0; k < col; k++) uc[k] = u[(size_t)cell * col + k];
    double chopmin = 1;
    double dS[NP];
    for (int j = 0; j < np; j++) {
        double dtmp = 0;
        for (int k = 0; k < col; k++) dtmp += 1.0 * ds[(size_t)(j * col + k) * stride] * uc[k];
        dS[j] = dtmp;
        double choptmp = 1;
        const double Sj = b.S[b.idx(j, cell)];
        if (fabs(dtmp) > dSmax) choptmp = dSmax / fabs(dtmp);
        else if (Sj + dtmp < 0.0) choptmp = 0.9 * Sj / fabs(dtmp);
        chopmin = chopmin < choptmp ? chopmin : choptmp;
    }
    for (int j = 0; j < np; j++) b.S[b.idx(j, cell)] += chopmin * dS[j];
    for (int r = np; r < row; r++) {
        double dtmp = 0;
        for (int k = 0; k < col; k++) dtmp += 1.0 * ds[(size_t)(r * col + k) * stride] * uc[k];
        b.xij[b.idx(r - np, cell)] += chopmin * dtmp;
    }
    b.P[cell] += uc[0];
    for (int i = 0; i < nc; i++) b.Ni[b.idx(i, cell)] += chopmin * uc[1 + i];
}
OCPX_HD void newton_update_cell(const BulkView& b, int cell, const double* u, double dSmax)
{
    newton_update_cell(b, cell, u, dSmax, b.dSec_dPri + cell, (size_t)b.nb);
}

// Bulk::CheckNi (src/Bulk.cpp:178-213) and Bulk::CheckP (:116-131) for one
// cell: small negative moles are reset to 1e-40 Nt; anything else is a
// failure that makes the reference cut the time step.
OCPX_HD uint32_t check_cell(const BulkView& b, int cell)
{
    uint32_t st = 0;
    const double Nt = b.Nt[cell];
    for (int i = 0; i < b.nc; i++) {
        const double v = b.Ni[b.idx(i, cell)];
        if (v < 0) {
            if ((v > -1E-5 * Nt) || (b.lNi[b.idx(i, cell)] < 1E-3 * Nt)) b.Ni[b.idx(i, cell)] = 1E-40 * Nt;
            else st |= ST_NEG_NI;
        }
    }
    if (b.P[cell] < 0) st |= ST_NEG_P;
    return st;
}

}  // namespace ocpx
