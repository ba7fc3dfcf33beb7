// Builds the reference-side binding (opencaeporox_gb300/binding/
// IsoThermalMethodGPU.hpp) against the reference's own headers and drives it
// on a deck set up by the reference's IsothermalSolver (test infrastructure:
// compiled by oracle/ref/Makefile, target gpu_binding).  The binding
// describes the reference's model and grid to the library and creates a
// context.  Without a CUDA device the library validates the descriptions
// and then reports OCPX_NO_DEVICE; with one, the binding uploads the state,
// runs one property update and residual on the device and compares the
// residual with the reference's own CalRes on the same state.
//
//   ocp_gpu_binding <deck> [--recompute]   exit 0: context created or OCPX_NO_DEVICE; 2: other status
//   (PTN moles from "<deck>.ptn_ni" when present; --recompute: a context that
//   recomputes the flash derivatives instead of storing them)
#include "IsoThermalMethodGPU.hpp"

#include "OCP.hpp"
#include "PreProcess.hpp"
#include "ptn_moles.hpp"

int main(int argc, char* argv[])
{
    MPI_Init(&argc, &argv);
    if (argc < 2) {
        std::cerr << "usage: ocp_gpu_binding <deck>\n";
        return 1;
    }
    const char* argv_[] = {"ocp_gpu_binding", argv[1]};
    OpenCAEPoroX sim;
    {
        PreProcess pre(argv[1]);
        sim.SetupDistParam(2, argv_, pre);
    }
    inject_ptn_moles(sim.reservoir, argv[1]);  // "<deck>.ptn_ni" when the deck starts from PTN moles
    sim.SetupSolver();
    sim.InitReservoir();
    Reservoir& rs = sim.reservoir;
    IsoT_FIM& fim = sim.solver.IsoTSolver.fim;
    IsoT_FIM_GPU gpu;
    if (argc > 2 && std::string(argv[2]) == "--recompute") gpu.SetRecomputeFlashDer(true);
    int rc = 0;
    try {
        gpu.CreateContext(rs);
    }
    catch (const GpuError& e) {
        rc = e.status == OCPX_NO_DEVICE ? 0 : 2;
        std::cout << "status " << ocpx_status_name(e.status) << " (" << e.what() << ")\n";
    }
    const OcpxDescription& d = gpu.Description();
    std::cout << "description nb " << d.grid.nb << " nbI " << d.grid.nb_interior << " nconn " << d.grid.nconn
              << " nc " << d.model.nc << " mixture " << d.model.mixture << "\n";
    if (gpu.Context()) {
        std::cout << "status OCPX_OK\n";
        const OCP_DBL dt = sim.control.time.GetCurrentDt();
        gpu.Upload(rs.bulk.vs);
        fim.CalRes(rs, dt, OCP_FALSE);  // the reference's residual of its initialised state
        const std::vector<OCP_DBL> ref = fim.NR.res.resAbs;
        ocpx_check(ocpx_update_properties(gpu.Context(), nullptr), "ocpx_update_properties");
        gpu.CalRes(rs, dt);
        double err = 0, scale = 0;
        const size_t n = (size_t)rs.bulk.vs.nbI * (rs.bulk.vs.nc + 1);
        for (size_t k = 0; k < n; k++) {
            err = std::max(err, std::fabs(fim.NR.res.resAbs[k] - ref[k]));
            scale = std::max(scale, std::fabs(ref[k]));
        }
        std::cout << "residual max difference " << err << " of " << scale << "\n";
    }
    MPI_Finalize();
    return rc;
}
