// IsoT_FIM_GPU: the reference-side binding of the GB300 FIM Newton-step
// library (include/ocpx.h) for OpenCAEPoroX.
//
// A maintainer adds this header to the reference's sources, selects the class
// in IsothermalSolver::SetupMethod (src/IsoThermalSolver.cpp:15-43) and makes
// the replaced IsoT_FIM methods virtual (include/IsoThermalMethod.hpp:127-129
// already is for CalRes); the class reads the reference's internal state the
// way IsoT_FIM does, so it is declared a friend where IsoT_FIM is
// (include/Bulk.hpp:82-87, include/BulkConn.hpp:28-35 and the mixture and
// flow method classes).  Define OCPX_OVERRIDE as `override` there.  The
// library replaces the reference's per-cell and per-connection loops:
//
//   UpdateProperty  NR.CheckPhysical + CalFlash + CalKrPc + CalRock
//                   (src/IsoThermalMethod.cpp:811-831)  -> ocpx_update_properties
//   CalRes          (:1090-1185), wells added after      -> ocpx_calres (+ ocpx_set_wells)
//   AssembleMat     AssembleMatBulks + AssembleMatWells  -> ocpx_assemble, rows copied
//                   (:742-752, 1187-1280)                   into the LinearSystem
//   GetSolution     (:1282-1418)                         -> ocpx_newton_update
//   UpdateLastTimeStep / ResetToLastTimeStep (:1473-1517, :1420-1471)
//                                                        -> ocpx_update_last_step,
//                                                           ocpx_checkpoint
// Errors: the library never aborts; a status other than OCPX_OK becomes a
// GpuError (what() carries the library's message), which the host may catch
// to fall back on its own path.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "IsoThermalMethod.hpp"
#include "ocpx.h"

#ifndef OCPX_OVERRIDE
#define OCPX_OVERRIDE
#endif

struct GpuError : std::runtime_error {
    ocpx_status status;
    GpuError(ocpx_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline const char* ocpx_status_name(ocpx_status s)
{
    static const char* names[] = {"OCPX_OK", "OCPX_NONCONVERGED", "OCPX_SINGULAR", "OCPX_NONFINITE",
                                  "OCPX_WATCHDOG", "OCPX_INVALID_ARG", "OCPX_CUDA_ERROR", "OCPX_NEGATIVE_P",
                                  "OCPX_NEGATIVE_NI", "OCPX_NO_DEVICE"};
    return (s >= 0 && s <= OCPX_NO_DEVICE) ? names[s] : "OCPX_?";
}

inline void ocpx_check(ocpx_status s, const char* what)
{
    if (s != OCPX_OK)
        throw GpuError(s, std::string(what) + ": " + ocpx_status_name(s) + ": " + ocpx_last_error());
}

// The reference's model, grid and state in the library's descriptions.  The
// vectors keep the arrays the descriptions point to.
struct OcpxDescription {
    ocpx_model_desc model{};
    ocpx_grid_desc grid{};
    std::vector<std::vector<OCP_DBL>> keep;
    std::vector<uint32_t> conn_b, conn_e;
    std::vector<OCP_DBL> conn_trans;

    const OCP_DBL* hold(std::vector<OCP_DBL> v)
    {
        keep.push_back(std::move(v));
        return keep.back().data();
    }
    // an OCPTable (columns stored one after another) as an ocpx_table
    ocpx_table table(const OCPTable& t)
    {
        std::vector<OCP_DBL> flat;
        for (const auto& col : t.data) flat.insert(flat.end(), col.begin(), col.end());
        return ocpx_table{(int)t.nRow, (int)t.data.size(), hold(std::move(flat))};
    }

    void describe(const Reservoir& rs)
    {
        const Bulk& bk = rs.bulk;
        const BulkVarSet& bvs = bk.vs;
        model.nc = (int)bvs.nc;
        model.gravity_factor = GRAVITY_FACTOR;
        model.conv_darcy = CONV_DARCY;
        model.gas_constant = GAS_CONSTANT;
        model.conv1 = CONV1;
        model.conv3 = CONV3;
        model.conv4 = CONV4;
        const auto* rock = dynamic_cast<const OCPRockIsoT_Linear*>(bk.ROCKm.ROCKs[0]);
        if (!rock) throw GpuError(OCPX_INVALID_ARG, "only the linear isothermal rock is supported");
        model.rock_pref = rock->Pref;
        model.rock_cp1 = rock->cp1;
        model.rock_cp2 = rock->cp2;
        const auto* ogw = dynamic_cast<const OCPFlowMethod_OGW01*>(bk.SATm.GetSAT(0)->flow->pfMethod);
        if (!ogw) throw GpuError(OCPX_INVALID_ARG, "only SWOF/SGOF with Stone II oil is supported");
        model.swof = table(ogw->SWOF.table);
        model.sgof = table(ogw->SGOF.table);
        const OCPMixture* mix = bk.PVTm.GetPVT(0)->mix;
        if (const auto* mc = dynamic_cast<const OCPMixtureComp*>(mix)) {
            const auto* pm = dynamic_cast<const OCPMixtureMethodComp01*>(mc->pmMethod);
            const auto* eos = pm ? dynamic_cast<const EoS_PR*>(pm->eos.eos) : nullptr;
            const auto* lbc = pm ? dynamic_cast<const ViscosityMethod03*>(pm->visCal.vM) : nullptr;
            if (!pm || !eos || !lbc) throw GpuError(OCPX_INVALID_ARG, "only PR-EoS with LBC viscosity is supported");
            model.mixture = 1;
            model.Tc = hold(pm->Tc);
            model.Pc = hold(pm->Pc);
            model.Vc = hold(pm->Vc);
            model.MW = hold(pm->MWC);
            model.OmegaA = hold(eos->OmegaA);
            model.OmegaB = hold(eos->OmegaB);
            model.acf = hold(eos->acf);
            model.BIC = hold(eos->BIC);
            model.Vshift = hold(eos->Vshift);
            model.Vcvis = hold(lbc->Vcvis);
            model.lbc_coef = hold(lbc->coef);
            const FlashCtrl& fc = pm->PE.flashCtrl;
            model.flash_ctrl = hold({OCP_DBL(fc.SSMsta.maxIt), fc.SSMsta.tol, fc.SSMsta.eYt, fc.SSMsta.Ktol,
                                     fc.SSMsta.dYtol, OCP_DBL(fc.NRsta.maxIt), fc.NRsta.tol,
                                     OCP_DBL(fc.SSMsp.maxIt), fc.SSMsp.tol, OCP_DBL(fc.NRsp.maxIt), fc.NRsp.tol,
                                     OCP_DBL(fc.RR.maxIt), fc.RR.tol});
            model.pvtw = table(pm->PVTW.table);
            model.std_rho_w = pm->PVTW.stdRhoW;
            model.std_vw = pm->PVTW.stdVw;
            model.skip_psa = bk.optMs.skipPSA.ifUse ? 1 : 0;
        }
        else if (const auto* mk = dynamic_cast<const OCPMixtureK*>(mix)) {
            const auto* pm = dynamic_cast<const OCPMixtureMethodK_OGW01*>(mk->pmMethod);
            if (!pm) throw GpuError(OCPX_INVALID_ARG, "only the OGW black-oil model is supported");
            model.mixture = 0;
            model.pvco = table(pm->PVCO.table);
            model.pvdg = table(pm->PVDG.table);
            model.pvtw = table(pm->PVTW.table);
            model.std_rho_o = pm->PVCO.stdRhoO;
            model.std_rho_g = pm->PVCO.stdRhoG;
            model.std_rho_w = pm->PVTW.stdRhoW;
            model.std_vo = pm->stdVo;
            model.std_vg = pm->stdVg;
            model.std_vw = pm->stdVw;
        }
        else throw GpuError(OCPX_INVALID_ARG, "unsupported mixture");
        for (const auto& c : rs.conn.iteratorConn) {
            conn_b.push_back(c.BId());
            conn_e.push_back(c.EId());
            conn_trans.push_back(c.Trans());
        }
        grid.nb = (int)bvs.nb;
        grid.nconn = (int)conn_b.size();
        grid.v = bvs.v.data();
        grid.depth = bvs.depth.data();
        grid.poro_init = bvs.poroInit.data();
        grid.conn_b = conn_b.data();
        grid.conn_e = conn_e.data();
        grid.conn_trans = conn_trans.data();
        grid.nb_interior = (int)bvs.nbI;
    }
};

class IsoT_FIM_GPU : public IsoT_FIM {
public:
    ~IsoT_FIM_GPU() { ocpx_destroy(ctx); }

    // IsoT_FIM::Setup, then the library's context for the reservoir's model and grid
    void Setup(Reservoir& rs, const OCPControl& ctrl) OCPX_OVERRIDE
    {
        IsoT_FIM::Setup(rs, ctrl);
        CreateContext(rs);
    }
    void CreateContext(const Reservoir& rs, int device = -1)
    {
        desc.describe(rs);
        ocpx_options opt{};
        opt.struct_size = sizeof(opt);
        opt.recompute_flash_der = recompute_flash_der ? 1 : 0;
        ocpx_check(ocpx_create_ex(&desc.model, &desc.grid, device, &opt, &ctx), "ocpx_create_ex");
    }
    // before Setup: keep no dSec_dPri on the device, recompute it where it is
    // used (compositional models; bit-identical results, less device memory)
    void SetRecomputeFlashDer(bool on) { recompute_flash_der = on; }
    // the host's bulk state to the device (after InitReservoir, or whenever
    // the host changed it)
    void Upload(const BulkVarSet& b)
    {
        set(OCPX_F_P, b.P);
        set(OCPX_F_T, b.T);
        set(OCPX_F_PB, b.Pb);
        set(OCPX_F_NI, b.Ni);
        set(OCPX_F_LNI, b.lNi);
        set(OCPX_F_NT, b.Nt);
        set(OCPX_F_S, b.S);
        set(OCPX_F_XIJ, b.xij);
        set(OCPX_F_PJ, b.Pj);
        std::vector<uint8_t> pe(b.phaseExist.begin(), b.phaseExist.end());
        ocpx_check(ocpx_set_field(ctx, OCPX_F_PHASE_EXIST, pe.data(), pe.size()), "ocpx_set_field");
    }
    OCP_BOOL UpdateProperty(Reservoir& rs, OCPControl& ctrl) OCPX_OVERRIDE
    {
        ocpx_report rep{};
        const ocpx_status st = ocpx_update_properties(ctx, &rep);
        if (st == OCPX_NEGATIVE_NI || st == OCPX_NEGATIVE_P) {  // NR.CheckPhysical failed: cut the step
            ctrl.time.CutDt(NR);
            ResetToLastTimeStep(rs, ctrl);
            return OCP_FALSE;
        }
        ocpx_check(st, "ocpx_update_properties");
        CalRes(rs, ctrl.time.GetCurrentDt());
        return OCP_TRUE;
    }
    void CalRes(Reservoir& rs, const OCP_DBL& dt, const OCP_BOOL& resetRes0 = OCP_FALSE) OCPX_OVERRIDE
    {
        (void)resetRes0;
        ocpx_norms nm{};
        ocpx_check(ocpx_calres(ctx, dt, &nm), "ocpx_calres");
        const size_t nrow = rs.bulk.vs.nbI;
        NR.res.SetZero();
        ocpx_check(ocpx_get_field_range(ctx, OCPX_F_RES, 0, nrow, NR.res.resAbs.data()), "ocpx_get_field_range");
        NR.res.maxRelRes_V = nm.maxRelRes_V;
        NR.res.maxId_V = nm.maxId_V;
        NR.res.maxRelRes_N = nm.maxRelRes_N;
        NR.res.maxId_N = nm.maxId_N;
    }
    // the library's block rows into the LinearSystem in its push-back order
    void AssembleMat(LinearSystem& ls, const Reservoir& rs, const OCP_DBL& dt) const OCPX_OVERRIDE
    {
        (void)rs;
        ocpx_check(ocpx_assemble(ctx, dt), "ocpx_assemble");
        size_t nrow = 0, nnz = 0;
        int bd = 0;
        ocpx_check(ocpx_jacobian_dims(ctx, &nrow, &nnz, &bd), "ocpx_jacobian_dims");
        std::vector<uint32_t> rp(nrow + 1), col(nnz);
        std::vector<OCP_DBL> val(nnz * bd * bd);
        ocpx_check(ocpx_get_jacobian(ctx, rp.data(), col.data(), val.data()), "ocpx_get_jacobian");
        ls.AddDim(nrow);
        for (size_t r = 0; r < nrow; r++)
            for (uint32_t k = rp[r]; k < rp[r + 1]; k++) {
                std::vector<OCP_DBL> blk(val.begin() + (size_t)k * bd * bd, val.begin() + (size_t)(k + 1) * bd * bd);
                if (k == rp[r]) ls.NewDiag(r, blk);
                else ls.NewOffDiag(r, col[k], blk);
            }
        ls.CopyRhs(NR.res.resAbs);
    }
    void GetSolution(Reservoir& rs, std::vector<OCP_DBL>& u, const ControlNR& ctrlNR) OCPX_OVERRIDE
    {
        (void)rs;
        ocpx_check(ocpx_newton_update(ctx, u.data(), ctrlNR.DSmax()), "ocpx_newton_update");
    }
    void UpdateLastTimeStep(Reservoir& rs) const OCPX_OVERRIDE
    {
        IsoT_FIM::UpdateLastTimeStep(rs);
        ocpx_check(ocpx_update_last_step(ctx), "ocpx_update_last_step");
        ocpx_check(ocpx_checkpoint(ctx, 0, 0), "ocpx_checkpoint");
    }
    void ResetToLastTimeStep(Reservoir& rs, OCPControl& ctrl) OCPX_OVERRIDE
    {
        ocpx_check(ocpx_checkpoint(ctx, 0, 1), "ocpx_checkpoint");
        IsoT_FIM::ResetToLastTimeStep(rs, ctrl);
    }

    ocpx_ctx* Context() const { return ctx; }
    const OcpxDescription& Description() const { return desc; }

private:
    void set(ocpx_field f, const std::vector<OCP_DBL>& v)
    {
        ocpx_check(ocpx_set_field(ctx, f, v.data(), v.size()), "ocpx_set_field");
    }
    OcpxDescription desc;
    ocpx_ctx* ctx = nullptr;
    bool recompute_flash_der = false;
};
