// Dump harness around the reference simulator (compiled from its own sources).
//
//   ocp_ref_dump fim   <deck.data> <outdir> <max_newton_iters>
//       Runs the deck with the FIM method exactly as the reference's driver
//       does (main/Main.cpp, src/OCP.cpp:88-142, src/IsoThermalSolver.cpp:70-101),
//       with a dense LU in place of the external linear solver, and writes
//       .npy dumps of the model description, the initial state and, for every
//       Newton iteration, the state entering UpdateProperty, the state and
//       residual leaving it, and the bulk block-CSR Jacobian.
//
//   ocp_ref_dump flash <deck.data> <cells.f64> <ncell> <outdir>
//       Builds the deck's compositional mixture and runs
//       OCPMixtureMethodComp01::FlashDer (src/OCPMixtureMethodComp.cpp:746-755)
//       from flash type 0 with no phase history for every (P, T, Ni) row of
//       cells.f64, writing the per-cell outputs.
//
// Harness code: it only drives and reads the reference; it computes nothing
// of the hot path itself.
#include "OCP.hpp"
#include "PreProcess.hpp"
#include "npy.hpp"
#include "ptn_moles.hpp"

#include <chrono>
#include <sys/stat.h>

using std::string;
using std::vector;

namespace {

string g_out;

void mkdir_p(const string& d) { ::mkdir(d.c_str(), 0755); }

template <typename T>
void put(const string& dir, const string& name, const vector<T>& v)
{
    npy::save(dir + "/" + name + ".npy", v);
}
template <typename T>
void put(const string& dir, const string& name, const T* p, size_t n)
{
    npy::save(dir + "/" + name + ".npy", p, {n});
}
void put1(const string& dir, const string& name, double x) { npy::save(dir + "/" + name + ".npy", &x, {1}); }
void puti(const string& dir, const string& name, int64_t x) { npy::save(dir + "/" + name + ".npy", &x, {1}); }

vector<double> flat(const vector<vector<OCP_DBL>>& cols)
{
    vector<double> out;
    for (auto& c : cols) out.insert(out.end(), c.begin(), c.end());
    return out;
}

// ---------------------------------------------------------------- model ----
void dump_model(const string& dir, Reservoir& rs)
{
    mkdir_p(dir);
    Bulk&       bk  = rs.bulk;
    BulkVarSet& bvs = bk.vs;
    puti(dir, "nb", bvs.nb);
    puti(dir, "nbI", bvs.nbI);
    puti(dir, "np", bvs.np);
    puti(dir, "nc", bvs.nc);
    puti(dir, "numConn", rs.conn.numConn);
    puti(dir, "numWell", rs.GetNumOpenWell());
    put1(dir, "GRAVITY_FACTOR", GRAVITY_FACTOR);
    put1(dir, "CONV_DARCY", CONV_DARCY);
    put1(dir, "GAS_CONSTANT", GAS_CONSTANT);
    put1(dir, "CONV1", CONV1);
    put1(dir, "CONV3", CONV3);
    put1(dir, "CONV4", CONV4);

    vector<uint32_t> b, e, dirn;
    vector<double>   tr, aB, aE;
    for (auto& c : rs.conn.iteratorConn) {
        b.push_back(c.bId);
        e.push_back(c.eId);
        tr.push_back(c.trans);
        dirn.push_back(static_cast<uint32_t>(c.direction));
        aB.push_back(c.areaB);
        aE.push_back(c.areaE);
    }
    put(dir, "conn_bId", b);
    put(dir, "conn_eId", e);
    put(dir, "conn_trans", tr);
    put(dir, "conn_dir", dirn);
    put(dir, "conn_areaB", aB);
    put(dir, "conn_areaE", aE);

    put(dir, "v", bvs.v);
    put(dir, "depth", bvs.depth);
    put(dir, "poroInit", bvs.poroInit);
    put(dir, "ntg", bvs.ntg);
    put(dir, "rockKx", bvs.rockKx);
    put(dir, "rockKy", bvs.rockKy);
    put(dir, "rockKz", bvs.rockKz);
    put(dir, "dx", bvs.dx);
    put(dir, "dy", bvs.dy);
    put(dir, "dz", bvs.dz);

    auto* rock = dynamic_cast<OCPRockIsoT_Linear*>(bk.ROCKm.ROCKs[0]);
    put1(dir, "rock_Pref", rock->Pref);
    put1(dir, "rock_cp1", rock->cp1);
    put1(dir, "rock_cp2", rock->cp2);

    // saturation functions (SWOF/SGOF + Stone II)
    const FlowUnit* fu   = bk.SATm.GetSAT(0);
    auto*           ogw  = dynamic_cast<OCPFlowMethod_OGW01*>(fu->flow->pfMethod);
    if (ogw) {
        put(dir, "SWOF", flat(ogw->SWOF.table.data));
        puti(dir, "SWOF_nrow", ogw->SWOF.table.nRow);
        put(dir, "SGOF", flat(ogw->SGOF.table.data));
        puti(dir, "SGOF_nrow", ogw->SGOF.table.nRow);
    }

    const MixtureUnit* mu  = bk.PVTm.GetPVT(0);
    OCPMixture*        mix = mu->mix;
    if (auto* mc = dynamic_cast<OCPMixtureComp*>(mix)) {
        puti(dir, "mixture_comp", 1);
        auto* pm  = dynamic_cast<OCPMixtureMethodComp01*>(mc->pmMethod);
        auto* eos = dynamic_cast<EoS_PR*>(pm->eos.eos);
        puti(dir, "NC", pm->NC);
        put(dir, "Tc", pm->Tc);
        put(dir, "Pc", pm->Pc);
        put(dir, "Vc", pm->Vc);
        put(dir, "MWC", pm->MWC);
        put(dir, "OmegaA", eos->OmegaA);
        put(dir, "OmegaB", eos->OmegaB);
        put(dir, "acf", eos->acf);
        put(dir, "BIC", eos->BIC);
        put(dir, "Vshift", eos->Vshift);
        auto* lbc = dynamic_cast<ViscosityMethod03*>(pm->visCal.vM);
        put(dir, "LBCcoef", lbc->coef);
        put(dir, "Vcvis", lbc->Vcvis);
        const FlashCtrl& fc = pm->PE.flashCtrl;
        vector<double> ctrl = {double(fc.SSMsta.maxIt), fc.SSMsta.tol, fc.SSMsta.eYt, fc.SSMsta.Ktol,
                               fc.SSMsta.dYtol,        double(fc.NRsta.maxIt), fc.NRsta.tol,
                               double(fc.SSMsp.maxIt), fc.SSMsp.tol,  double(fc.NRsp.maxIt),
                               fc.NRsp.tol,            double(fc.RR.maxIt), fc.RR.tol};
        put(dir, "flash_ctrl", ctrl);
        put(dir, "PVTW", flat(pm->PVTW.table.data));
        puti(dir, "PVTW_nrow", pm->PVTW.table.nRow);
        put1(dir, "stdRhoW", pm->PVTW.stdRhoW);
        put1(dir, "stdVw", pm->PVTW.stdVw);
        puti(dir, "skipPSA", bk.optMs.skipPSA.ifUse);
    }
    else if (auto* mk = dynamic_cast<OCPMixtureK*>(mix)) {
        puti(dir, "mixture_comp", 0);
        auto* pm = dynamic_cast<OCPMixtureMethodK_OGW01*>(mk->pmMethod);
        if (!pm) { std::cerr << "only OGW01 black-oil is dumped\n"; std::exit(4); }
        put(dir, "PVCO", flat(pm->PVCO.table.data));
        puti(dir, "PVCO_nrow", pm->PVCO.table.nRow);
        put(dir, "PVDG", flat(pm->PVDG.table.data));
        puti(dir, "PVDG_nrow", pm->PVDG.table.nRow);
        put(dir, "PVTW", flat(pm->PVTW.table.data));
        puti(dir, "PVTW_nrow", pm->PVTW.table.nRow);
        put1(dir, "stdRhoO", pm->PVCO.stdRhoO);
        put1(dir, "stdRhoG", pm->PVCO.stdRhoG);
        put1(dir, "stdRhoW", pm->PVTW.stdRhoW);
        put1(dir, "stdVo", pm->stdVo);
        put1(dir, "stdVg", pm->stdVg);
        put1(dir, "stdVw", pm->stdVw);
    }
}

// ---------------------------------------------------------------- state ----
void dump_state(const string& dir, Reservoir& rs)
{
    mkdir_p(dir);
    BulkVarSet& s = rs.bulk.vs;
    put(dir, "P", s.P);            put(dir, "T", s.T);          put(dir, "Pb", s.Pb);
    put(dir, "Ni", s.Ni);          put(dir, "Nt", s.Nt);        put(dir, "vf", s.vf);
    put(dir, "Pj", s.Pj);          put(dir, "Pc", s.Pc);        put(dir, "S", s.S);
    put(dir, "phaseExist", s.phaseExist);
    put(dir, "xij", s.xij);        put(dir, "rho", s.rho);      put(dir, "xi", s.xi);
    put(dir, "mu", s.mu);          put(dir, "kr", s.kr);
    put(dir, "rhoP", s.rhoP);      put(dir, "xiP", s.xiP);      put(dir, "muP", s.muP);
    put(dir, "rhox", s.rhox);      put(dir, "xix", s.xix);      put(dir, "mux", s.mux);
    put(dir, "vfP", s.vfP);        put(dir, "vfi", s.vfi);
    put(dir, "dKrdS", s.dKrdS);    put(dir, "dPcdS", s.dPcdS);
    put(dir, "dSec_dPri", s.dSec_dPri);
    put(dir, "poro", s.poro);      put(dir, "poroP", s.poroP);  put(dir, "rockVp", s.rockVp);
    put(dir, "lNi", s.lNi);        put(dir, "lP", s.lP);        put(dir, "lS", s.lS);
    put(dir, "lphaseExist", s.lphaseExist);
    put(dir, "lxij", s.lxij);

    const SkipPSA& sk = rs.bulk.optMs.skipPSA;
    if (sk.ifUse && sk.vs.ifSetup) {
        put(dir, "skip_flag", sk.vs.flag);
        put(dir, "skip_minEigen", sk.vs.minEigen);
        put(dir, "skip_P", sk.vs.P);
        put(dir, "skip_T", sk.vs.T);
        put(dir, "skip_zi", sk.vs.zi);
        put(dir, "skip_lflag", sk.vs.lflag);
        put(dir, "skip_lminEigen", sk.vs.lminEigen);
        put(dir, "skip_lP", sk.vs.lP);
        put(dir, "skip_lT", sk.vs.lT);
        put(dir, "skip_lzi", sk.vs.lzi);
    }
}

// Open wells in AllWells order and their perforations, as the residual just
// computed used them (WellPeaceman.cpp: CalTrans, CalFlux, CalFactor,
// CalResFIM): well arrays per well, perforation arrays concatenated.
void dump_wells(const string& dir, Reservoir& rs)
{
    vector<int32_t> type, mode, nperf, loc, pdir;
    vector<double>  bhp, tar_bhp, tar_rate, factor, inj_zi, qi, WI, mult, dG, P, transj, trans_inj, xi, pqi;
    vector<double>  kh, radius, skin, cdx, cdy, cdz, cntg, ckx, cky, ckz;
    const BulkVarSet& bvs = rs.bulk.vs;
    for (Well* w0 : rs.allWells.wells) {
        PeacemanWell* w = dynamic_cast<PeacemanWell*>(w0);
        if (!w || w->opt.state != WellState::open) continue;
        type.push_back(w->opt.type == WellType::injector ? 0 : 1);
        mode.push_back(w->opt.mode == WellOptMode::bhp ? 0 : 1);
        nperf.push_back((int32_t)w->numPerf);
        bhp.push_back(w->bhp);
        tar_bhp.push_back(w->opt.tarBHP);
        tar_rate.push_back(w->opt.tarRate);
        for (USI i = 0; i < w->nc; i++) {
            factor.push_back(w->factor.size() > i ? w->factor[i] : 0.0);
            inj_zi.push_back(w->opt.injZi.size() > i ? w->opt.injZi[i] : 0.0);
            qi.push_back(w->qi_lbmol[i]);
        }
        for (USI p = 0; p < w->numPerf; p++) {
            const Perforation& f = w->perf[p];
            loc.push_back((int32_t)f.location);
            WI.push_back(f.WI);
            mult.push_back(f.multiplier);
            dG.push_back(w->dG[p]);
            P.push_back(f.P);
            for (USI j = 0; j < w->np; j++) transj.push_back(f.transj[j]);
            trans_inj.push_back(f.transINJ);
            xi.push_back(f.xi);
            for (USI i = 0; i < w->nc; i++) pqi.push_back(f.qi_lbmol[i]);
            pdir.push_back((int32_t)f.direction);
            kh.push_back(f.kh);
            radius.push_back(f.radius);
            skin.push_back(f.skinFactor);
            cdx.push_back(bvs.dx[f.location]);
            cdy.push_back(bvs.dy[f.location]);
            cdz.push_back(bvs.dz[f.location]);
            cntg.push_back(bvs.ntg[f.location]);
            ckx.push_back(bvs.rockKx[f.location]);
            cky.push_back(bvs.rockKy[f.location]);
            ckz.push_back(bvs.rockKz[f.location]);
        }
    }
    put(dir, "perf_dir", pdir);
    put(dir, "perf_kh", kh);
    put(dir, "perf_radius", radius);
    put(dir, "perf_skin", skin);
    put(dir, "perf_cell_dx", cdx);
    put(dir, "perf_cell_dy", cdy);
    put(dir, "perf_cell_dz", cdz);
    put(dir, "perf_cell_ntg", cntg);
    put(dir, "perf_cell_kx", ckx);
    put(dir, "perf_cell_ky", cky);
    put(dir, "perf_cell_kz", ckz);
    put1(dir, "conv_darcy", CONV_DARCY);
    put(dir, "well_type", type);
    put(dir, "well_mode", mode);
    put(dir, "well_nperf", nperf);
    put(dir, "well_bhp", bhp);
    put(dir, "well_tar_bhp", tar_bhp);
    put(dir, "well_tar_rate", tar_rate);
    put(dir, "well_factor", factor);
    put(dir, "well_inj_zi", inj_zi);
    put(dir, "well_qi", qi);
    put(dir, "perf_loc", loc);
    put(dir, "perf_WI", WI);
    put(dir, "perf_mult", mult);
    put(dir, "perf_dG", dG);
    put(dir, "perf_P", P);
    put(dir, "perf_transj", transj);
    put(dir, "perf_trans_inj", trans_inj);
    put(dir, "perf_xi", xi);
    put(dir, "perf_qi", pqi);
}

void dump_conn_res(const string& dir, Reservoir& rs, IsoT_FIM& fim, OCP_DBL dt)
{
    // bulk-only residual: the same CalRes with the well list detached, then the
    // full residual restored for the reference's own control flow.
    BulkConnVarSet& c = rs.conn.vs;
    put(dir, "upblock", c.upblock);
    put(dir, "dP", c.dP);
    put(dir, "flux_vj", c.flux_vj);
    put(dir, "flux_ni", c.flux_ni);
    vector<Well*> wells;
    wells.swap(rs.allWells.wells);
    fim.CalRes(rs, dt, OCP_FALSE);
    const OCP_USI nbI = rs.bulk.vs.nbI, len = rs.bulk.vs.nc + 1;
    put(dir, "res_bulk", fim.NR.res.resAbs.data(), nbI * len);
    put(dir, "resRelV", fim.NR.res.resRelV.data(), nbI);
    put(dir, "resRelN", fim.NR.res.resRelN.data(), nbI);
    put1(dir, "maxRelRes_V", fim.NR.res.maxRelRes_V);
    put1(dir, "maxRelRes_N", fim.NR.res.maxRelRes_N);
    puti(dir, "maxId_V", fim.NR.res.maxId_V);
    puti(dir, "maxId_N", fim.NR.res.maxId_N);
    wells.swap(rs.allWells.wells);
    fim.CalRes(rs, dt, OCP_FALSE);
    put(dir, "res_full", fim.NR.res.resAbs);
    put1(dir, "maxWellRelRes_mol", fim.NR.res.maxWellRelRes_mol);
    dump_wells(dir, rs);
}

void dump_jac(const string& dir, LinearSystem& ls, OCP_USI nbI)
{
    vector<uint32_t> rowptr(1, 0), col;
    vector<double>   val;
    for (OCP_USI r = 0; r < nbI; r++) {
        rowptr.push_back(rowptr.back() + ls.mat.colId[r].size());
        col.insert(col.end(), ls.mat.colId[r].begin(), ls.mat.colId[r].end());
        val.insert(val.end(), ls.mat.val[r].begin(), ls.mat.val[r].end());
    }
    put(dir, "jac_rowptr", rowptr);
    put(dir, "jac_col", col);
    put(dir, "jac_val", val);
}

// every row of the assembled system after the wells' assembly: bulk rows
// (with their well columns) and well rows
void dump_jac_all(const string& dir, LinearSystem& ls)
{
    vector<uint32_t> rowptr(1, 0), col;
    vector<double>   val;
    for (OCP_USI r = 0; r < ls.mat.colId.size() && r < ls.mat.dim; r++) {
        rowptr.push_back(rowptr.back() + ls.mat.colId[r].size());
        col.insert(col.end(), ls.mat.colId[r].begin(), ls.mat.colId[r].end());
        val.insert(val.end(), ls.mat.val[r].begin(), ls.mat.val[r].end());
    }
    put(dir, "jacw_rowptr", rowptr);
    put(dir, "jacw_col", col);
    put(dir, "jacw_val", val);
}

double now()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// The property update of IsoT_FIM::UpdateProperty (src/IsoThermalMethod.cpp:811-836),
// with the per-cell flash loop of IsoT_FIM::CalFlash (:1016-1025) unrolled
// here so per-cell flash iteration counters and flash types can be recorded.
OCP_BOOL update_property(IsoT_FIM& fim, Reservoir& rs, OCPControl& ctrl, const string& dir,
                         double& t_update)
{
    if (!fim.NR.CheckPhysical(rs, {"BulkNi", "BulkP"}, ctrl.time.GetCurrentDt())) {
        ctrl.time.CutDt(fim.NR);
        fim.ResetToLastTimeStep(rs, ctrl);
        return OCP_FALSE;
    }
    mkdir_p(dir);
    Bulk&       bk  = rs.bulk;
    BulkVarSet& bvs = bk.vs;
    vector<int32_t> ftype(bvs.nb, -1), iters(bvs.nb * 5, 0);
    double t0 = now();
    for (OCP_USI n = 0; n < bvs.nb; n++) {
        const MixtureUnit* mu = bk.PVTm.GetPVT(n);
        OCPMixtureComp*    mc = dynamic_cast<OCPMixtureComp*>(mu->mix);
        OCPPhaseEquilibrium* pe = mc ? &dynamic_cast<OCPMixtureMethodComp01*>(mc->pmMethod)->PE : nullptr;
        OCP_ULL c0[5] = {0, 0, 0, 0, 0};
        if (pe) { c0[0] = pe->itersSSMSTA; c0[1] = pe->itersNRSTA; c0[2] = pe->itersSSMSP; c0[3] = pe->itersNRSP; c0[4] = pe->itersRR; }
        mu->FlashFIM(n, bvs);
        fim.PassFlashValue(bk, n);
        if (pe) {
            ftype[n] = pe->ftype;
            iters[n * 5 + 0] = pe->itersSSMSTA - c0[0];
            iters[n * 5 + 1] = pe->itersNRSTA - c0[1];
            iters[n * 5 + 2] = pe->itersSSMSP - c0[2];
            iters[n * 5 + 3] = pe->itersNRSP - c0[3];
            iters[n * 5 + 4] = pe->itersRR - c0[4];
        }
    }
    fim.CalKrPc(bk);
    fim.CalRock(bk);
    rs.allWells.CalFlux(bk);
    fim.CalRes(rs, ctrl.time.GetCurrentDt());
    t_update = now() - t0;
    put(dir, "flash_ftype", ftype);
    put(dir, "flash_iters", iters);
    return OCP_TRUE;
}

// IsothermalSolver::FinishNR for a FIM-only run (src/IsoThermalSolver.cpp:220-250
// with IsoT_FIM::FinishNR, src/IsoThermalMethod.cpp:838-864), unrolled so the
// Newton statistics can be recorded before a reset clears them: the maximum
// changes of CalMaxChangeNR, the residual norms and control parameters that
// CheckConverge reads, and the state it returns as the integer value of
// OCPNRStateC (0 converge, 1 continue iterating, 2 not converged).
OCP_BOOL finish_nr(IsothermalSolver& S, IsoT_FIM& fim, Reservoir& rs, OCPControl& ctrl, const string& dir)
{
    if (S.curMethod != OCPNLMethod::FIM || S.mainMethod != OCPNLMethod::FIM) return S.FinishNR(rs, ctrl);
    OCPNRsuite& NR = fim.NR;
    NR.CalMaxChangeNR(rs);
    put1(dir, "nr_dPBmax", NR.dPBmaxNR.back());
    put1(dir, "nr_dPWmax", NR.dPWmaxNR.back());
    put1(dir, "nr_dTmax", NR.dTmaxNR.back());
    put1(dir, "nr_dNmax", NR.dNmaxNR.back());
    put1(dir, "nr_dSmax", NR.dSmaxNR.back());
    put1(dir, "nr_eVmax", NR.eVmaxNR.back());
    put1(dir, "nr_maxRelRes_V", NR.res.maxRelRes_V);
    put1(dir, "nr_maxRelRes0_V", NR.res.maxRelRes0_V);
    put1(dir, "nr_maxRelRes_N", NR.res.maxRelRes_N);
    put1(dir, "nr_maxWellRelRes_mol", NR.res.maxWellRelRes_mol);
    puti(dir, "nr_iter", static_cast<int>(NR.GetIterNR()));
    put1(dir, "nr_tol", ctrl.NR.wp->tol);
    put1(dir, "nr_dPmin", ctrl.NR.wp->dPmin);
    put1(dir, "nr_dSmin", ctrl.NR.wp->dSmin);
    puti(dir, "nr_maxIter", static_cast<int>(ctrl.NR.wp->maxIter));
    const OCPNRStateC st = ctrl.CheckConverge(NR, {"res", "d"});
    puti(dir, "nr_state", static_cast<int>(st));
    OCP_BOOL conv = OCP_FALSE;
    if (st == OCPNRStateC::converge) {
        if (!NR.CheckPhysical(rs, {"WellP"}, ctrl.time.GetCurrentDt())) {
            ctrl.time.CutDt(NR);
            fim.ResetToLastTimeStep(rs, ctrl);
        }
        else {
            conv = OCP_TRUE;
        }
    }
    else if (st == OCPNRStateC::not_converge) {
        ctrl.time.CutDt();
        fim.ResetToLastTimeStep(rs, ctrl);
    }
    puti(dir, "nr_finish", conv ? 1 : 0);
    return conv;
}

// After IsothermalSolver::FinishStep: CalMaxChangeTime's maxima and the next
// time step of CalNextTimeStep, with the control parameters it read.
void dump_finish_step(IsoT_FIM& fim, OCPControl& ctrl, const string& dir, double time_before)
{
    put1(dir, "ts_time_before", time_before);
    const OCPNRsuite& NR = fim.NR;
    put1(dir, "ts_dPmax", NR.dPmaxT);
    put1(dir, "ts_dPBmax", NR.dPBmaxT);
    put1(dir, "ts_dPWmax", NR.dPWmaxT);
    put1(dir, "ts_dTmax", NR.dTmaxT);
    put1(dir, "ts_dNmax", NR.dNmaxT);
    put1(dir, "ts_dSmax", NR.dSmaxT);
    put1(dir, "ts_eVmax", NR.eVmaxT);
    puti(dir, "ts_iter", static_cast<int>(NR.GetIterNR()));
    const ControlTime& t = ctrl.time;
    put1(dir, "ts_last_dt", t.last_dt);
    put1(dir, "ts_current_time", t.current_time);
    put1(dir, "ts_next_dt", t.current_dt);
    put1(dir, "ts_predict_dt", t.predict_dt);
    put1(dir, "ts_maxIncreFac", t.wp->maxIncreFac);
    put1(dir, "ts_minChopFac", t.wp->minChopFac);
    put1(dir, "ts_dPlim", t.wp->dPlim);
    put1(dir, "ts_dSlim", t.wp->dSlim);
    put1(dir, "ts_timeMax", t.wp->timeMax);
    put1(dir, "ts_timeMin", t.wp->timeMin);
    put1(dir, "ts_end_time", t.wp->end_time);
}

int run_fim(const string& deck, int max_iters)
{
    const char* argv_[] = {"ocp_ref_dump", deck.c_str()};
    OpenCAEPoroX sim;
    {
        PreProcess pre(deck);
        sim.SetupDistParam(2, argv_, pre);
    }
    inject_ptn_moles(sim.reservoir, deck);
    sim.SetupSolver();
    sim.InitReservoir();

    Reservoir&        rs   = sim.reservoir;
    OCPControl&       ctrl = sim.control;
    IsothermalSolver& S    = sim.solver.IsoTSolver;
    IsoT_FIM&         fim  = S.fim;
    LinearSystem&     ls   = S.LSolver;
    const OCP_USI     nbI  = rs.bulk.vs.nbI;

    dump_model(g_out + "/model", rs);
    dump_state(g_out + "/init", rs);
    if (max_iters <= 0) return 0;

    vector<double> log_rows; // step, iter, dt, event, t_update, t_assemble
    int  it = 0, step = 0;
    bool stop = false;
    string last_post;
    ctrl.simTime.Initialize();
    while (!stop) {
        INT d = ctrl.ApplyControl();
        if (d < 0) break;
        rs.ApplyControl(d);
        ctrl.time.CalInitTimeStep4TSTEP(rs.GetWellOptChange());
        while (!ctrl.time.IfEndTSTEP() && !stop) {
            S.Prepare(rs, ctrl);
            int nr = 0;
            while (true) {
                const OCP_DBL dt = ctrl.time.GetCurrentDt();
                if (dt < MIN_TIME_CURSTEP || it >= max_iters) { stop = true; break; }
                char name[64];
                std::snprintf(name, sizeof name, "%s/it%03d", g_out.c_str(), it);
                const string dir = name;
                mkdir_p(dir);
                // jacobian at this iteration, from the current state
                dump_state(dir + "/jac_state", rs);
                dump_conn_res(dir + "/jac_state", rs, fim, dt);
                put1(dir + "/jac_state", "dt", dt);
                ls.SetWorkLS(fim.GetWorkLS());
                double t0 = now();
                fim.AssembleMatBulks(ls, rs, dt);
                double t_asm = now() - t0;
                dump_jac(dir + "/jac_state", ls, nbI);
                fim.AssembleMatWells(ls, rs, dt);
                dump_jac_all(dir + "/jac_state", ls);
                dump_wells(dir + "/jac_state", rs);
                ls.CopyRhs(fim.NR.res.resAbs);
                rs.domain.SetNumActWellLocal(rs.GetNumOpenWell());

                if (!S.SolveLinearSystem(rs, ctrl)) {
                    log_rows.insert(log_rows.end(), {double(step), double(nr), dt, 1.0, 0.0, t_asm});
                    it++; nr++;
                    continue;
                }
                dump_state(dir + "/pre", rs);
                put(dir + "/pre", "u", ls.mat.u);
                put1(dir + "/pre", "dt", dt);
                put1(dir + "/pre", "dSmax", ctrl.NR.DSmax());
                double t_upd = 0;
                if (!update_property(fim, rs, ctrl, dir + "/post", t_upd)) {
                    log_rows.insert(log_rows.end(), {double(step), double(nr), dt, 2.0, 0.0, t_asm});
                    it++; nr++;
                    continue;
                }
                dump_state(dir + "/post", rs);
                dump_conn_res(dir + "/post", rs, fim, dt);
                log_rows.insert(log_rows.end(), {double(step), double(nr), dt, 0.0, t_upd, t_asm});
                it++; nr++;
                const bool conv = finish_nr(S, fim, rs, ctrl, dir + "/post");
                last_post = dir + "/post";
                if (it >= max_iters) { stop = true; break; }
                if (conv) break;
            }
            if (stop) break;
            const double time_before = ctrl.time.GetCurrentTime();
            S.FinishStep(rs, ctrl);
            if (!last_post.empty()) dump_finish_step(fim, ctrl, last_post, time_before);
            step++;
        }
    }
    npy::save(g_out + "/log.npy", log_rows.data(), {log_rows.size() / 6, 6});
    return 0;
}

// ---------------------------------------------------------------- flash ----
int run_flash(const string& deck, const string& cells, size_t ncell)
{
    const char* argv_[] = {"ocp_ref_dump", deck.c_str()};
    OpenCAEPoroX sim;
    {
        PreProcess pre(deck);
        sim.SetupDistParam(2, argv_, pre);
    }
    Reservoir& rs = sim.reservoir;
    dump_model(g_out + "/model", rs);

    const MixtureUnit* mu = rs.bulk.PVTm.GetPVT(0);
    auto* mc = dynamic_cast<OCPMixtureComp*>(mu->mix);
    auto* pm = dynamic_cast<OCPMixtureMethodComp01*>(mc->pmMethod);
    OCPMixtureVarSet& vs = mc->vs;
    const USI nc = vs.nc, np = vs.np;

    vector<double> in(ncell * (2 + nc));
    FILE* f = std::fopen(cells.c_str(), "rb");
    if (!f || std::fread(in.data(), sizeof(double), in.size(), f) != in.size()) { std::cerr << "bad cells file\n"; return 5; }
    std::fclose(f);

    vector<double> S(ncell * np), x(ncell * np * nc), rho(ncell * np), xi(ncell * np), mu_(ncell * np);
    vector<double> rhoP(ncell * np), xiP(ncell * np), muP(ncell * np);
    vector<double> rhox(ncell * np * nc), xix(ncell * np * nc), mux(ncell * np * nc);
    vector<double> vf(ncell), Nt(ncell), vfP(ncell), vfi(ncell * nc), nj(ncell * np);
    vector<double> dX(ncell * vs.dXsdXp.size());
    vector<uint32_t> pex(ncell * np);
    vector<int32_t> ftype(ncell), iters(ncell * 5);
    OCPPhaseEquilibrium& pe = pm->PE;
    double t0 = now();
    for (size_t n = 0; n < ncell; n++) {
        const double* c = &in[n * (2 + nc)];
        pm->SetVarSet(c[0], c[1], c + 2, vs);
        // no phase history: phaseNum = 1 gives lNP = 0 (strict stability test)
        std::fill(vs.x.begin(), vs.x.end(), 0.0);
        std::fill(vs.phaseExist.begin(), vs.phaseExist.end(), OCP_FALSE);
        vs.phaseNum = 1;
        OCP_ULL c0[5] = {pe.itersSSMSTA, pe.itersNRSTA, pe.itersSSMSP, pe.itersNRSP, pe.itersRR};
        pm->FlashDer(vs, 0);
        ftype[n] = pe.ftype;
        iters[n * 5 + 0] = pe.itersSSMSTA - c0[0];
        iters[n * 5 + 1] = pe.itersNRSTA - c0[1];
        iters[n * 5 + 2] = pe.itersSSMSP - c0[2];
        iters[n * 5 + 3] = pe.itersNRSP - c0[3];
        iters[n * 5 + 4] = pe.itersRR - c0[4];
        for (USI j = 0; j < np; j++) {
            pex[n * np + j] = vs.phaseExist[j];
            S[n * np + j]   = vs.S[j];
            nj[n * np + j]  = vs.nj[j];
            if (!vs.phaseExist[j]) continue;  // absent phases keep stale values
            rho[n * np + j] = vs.rho[j];  xi[n * np + j]  = vs.xi[j];  mu_[n * np + j] = vs.mu[j];
            rhoP[n * np + j] = vs.rhoP[j]; xiP[n * np + j] = vs.xiP[j]; muP[n * np + j] = vs.muP[j];
            for (USI i = 0; i < nc; i++) {
                x[(n * np + j) * nc + i]    = vs.x[j * nc + i];
                rhox[(n * np + j) * nc + i] = vs.rhox[j * nc + i];
                xix[(n * np + j) * nc + i]  = vs.xix[j * nc + i];
                mux[(n * np + j) * nc + i]  = vs.mux[j * nc + i];
            }
        }
        vf[n] = vs.Vf; Nt[n] = vs.Nt; vfP[n] = vs.vfP;
        for (USI i = 0; i < nc; i++) vfi[n * nc + i] = vs.vfi[i];
        std::copy(vs.dXsdXp.begin(), vs.dXsdXp.end(), &dX[n * vs.dXsdXp.size()]);
    }
    double t_flash = now() - t0;
    const string d = g_out + "/flash";
    mkdir_p(d);
    put(d, "phaseExist", pex); put(d, "S", S); put(d, "xij", x); put(d, "nj", nj);
    put(d, "rho", rho); put(d, "xi", xi); put(d, "mu", mu_);
    put(d, "rhoP", rhoP); put(d, "xiP", xiP); put(d, "muP", muP);
    put(d, "rhox", rhox); put(d, "xix", xix); put(d, "mux", mux);
    put(d, "vf", vf); put(d, "Nt", Nt); put(d, "vfP", vfP); put(d, "vfi", vfi);
    put(d, "dSec_dPri", dX); put(d, "ftype", ftype); put(d, "iters", iters);
    put1(d, "seconds", t_flash);
    return 0;
}

/// The reference's overlap area of two faces on a vertical plane
/// (CalAreaNotQuadr, src/UtilMesh.cpp) for n pairs read from a raw float64
/// file: per pair face 1 then face 2, each four points (x, depth), the upper
/// edge first; writes <outdir>/area.npy.
int run_overlap(const string& pairs_file, size_t n)
{
    std::ifstream in(pairs_file, std::ios::binary);
    vector<double> buf(n * 16);
    in.read(reinterpret_cast<char*>(buf.data()), buf.size() * sizeof(double));
    if (!in) { std::cerr << "short pairs file\n"; return 2; }
    vector<double> area(n);
    for (size_t m = 0; m < n; m++) {
        HexahedronFace f[2];
        for (int s = 0; s < 2; s++) {
            const double* q = &buf[m * 16 + s * 8];
            f[s].p0 = Point3D(q[0], q[1], 0);
            f[s].p1 = Point3D(q[2], q[3], 0);
            f[s].p2 = Point3D(q[4], q[5], 0);
            f[s].p3 = Point3D(q[6], q[7], 0);
        }
        area[m] = CalAreaNotQuadr(f[0], f[1]);
    }
    put(g_out, "area", area);
    return 0;
}

} // namespace

int main(int argc, char* argv[])
{
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &CURRENT_RANK);
    if (argc < 5) {
        std::cerr << "usage: ocp_ref_dump fim <deck> <outdir> <max_iters>\n"
                     "       ocp_ref_dump flash <deck> <cells.f64> <ncell> <outdir>\n"
                     "       ocp_ref_dump overlap <pairs.f64> <npairs> <outdir>\n";
        return 1;
    }
    const string mode = argv[1];
    int rc = 1;
    if (mode == "fim") {
        g_out = argv[3];
        mkdir_p(g_out);
        rc = run_fim(argv[2], std::atoi(argv[4]));
    }
    else if (mode == "overlap") {
        g_out = argv[4];
        mkdir_p(g_out);
        rc = run_overlap(argv[2], std::strtoull(argv[3], nullptr, 10));
    }
    else if (mode == "flash" && argc >= 6) {
        g_out = argv[5];
        mkdir_p(g_out);
        rc = run_flash(argv[2], argv[3], std::strtoull(argv[4], nullptr, 10));
    }
    MPI_Finalize();
    return rc;
}
