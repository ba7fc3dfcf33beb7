// Host-side launcher declarations shared by the C-ABI translation unit and
// the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include "bulk_view.cuh"
#include "conn_ops.cuh"
#include "flash_comp.cuh"
#include "ocpx.h"

namespace ocpx {

// capacities the compositional kernels are compiled for (EoS components)
constexpr int kNcmCaps[] = {4, 6, 8, 10, 12};
// capacities of the Jacobian connection kernel (components incl. water)
constexpr int kNctCaps[] = {3, 5, 7, 9, 11, 13};

// Compositional FlashDer for cells [0, nb): one thread per cell.
cudaError_t launch_flash_comp(int ncm, const Model* dm, const BulkView& b, int block, cudaStream_t s);
// Batched form: cost-ordered thread-per-cell flash with a work budget, the
// deferred cells' phase equilibrium on whole warps, then their properties.
struct FlashBatch {
    int budget;        // work units before a cell is deferred
    int block;         // threads per block of the thread-per-cell step
    int coop_blocks;   // blocks of the cooperative step (COOP_WARPS warps each)
    int cap;           // capacity of the deferral list
    DeferRec* rec;
    unsigned* count;   // deferred cells (may exceed cap: the excess finish in place)
    PERes* pe;
    const uint8_t* pre;  // cells pre-deferred to another list (skipped by part 0), may be NULL
    const int* level;    // adaptive work level: the budget is at least its work units, may be NULL
    int prio;            // launch priority of parts 1 and 2 (CUDA stream-priority scale), 0 = the stream's
    int excl_blocks;     // > 0: part 1 runs as this many SM-exclusive blocks (EXCL_WARPS warps each)
    int excl_smem;       // dynamic shared memory of an SM-exclusive block (from setup_flash_batched)
    int cell_blocks;     // > 0: part 0 runs as this many persistent blocks taking 32 cells per warp
    unsigned* cell_next; // their position counter (zero before the launch); part 3's too
    unsigned* coop_next; // slot counter of part 1 (zero before the launch)
    const DeferRec* rin;        // part 3: input list and its count; part 4: the pre-deferred list
    const unsigned* rin_count;
    long long mult;             // part 3: budget multiplier of the round
    PERes* pe_pre;              // part 4: results of the pre-deferred list
    int excl_smem_fused;        // part 4: dynamic shared memory that makes a fused block SM-exclusive
    int coop_only_blocks;       // part 4: leading blocks that run only cooperative work (0: none)
    uint32_t* watchdog;         // part 4: status word for a wait that ran out (ST_ITER_CAP)
    int post_block;             // part 2: threads per block (0: 128)
    const DeferRec* rec2;       // part 2: a second list finished in the same launch
    const unsigned* count2;     //   (its count, capacity cap, and equilibria), NULL: none
    const PERes* pe2;
};
// once per device: configure the SM-exclusive kernels of capacity ncm;
// excl_smem[0]: the cooperative kernel's dynamic shared memory, [1]: the fused kernel's,
// [2]: fused blocks resident per SM without it
cudaError_t setup_flash_batched(int ncm, int* excl_smem);
// part 0: budgeted thread-per-cell flash, 1: cooperative equilibrium, 2: finish deferred cells,
// 3: re-budgeting round over a deferral list (thread per cell), 4: the fused kernel (pre list
// rin / pe_pre, cost order, late list rec / pe; cell_blocks blocks; counters cell_next[0..2];
// SM-exclusive blocks when excl_blocks is nonzero)
cudaError_t launch_flash_batched(int ncm, const Model* dm, const BulkView& b, const int* order,
                                 const FlashBatch& fb, int part, cudaStream_t s);
// Flash derivatives recomputed where they are used (k_flash_comp.cu, part 7):
// dSec_dPri of a list of cells (list NULL: first .. first + n - 1) into
// out[t][np*(nc+1)^2] (soa = 0) or out[k * soa + t]; GetSolution.
cudaError_t launch_dsec_cells(int ncm, const Model* dm, const BulkView& b, const int* list, int first, int n,
                              double* out, size_t soa, cudaStream_t s);
// The connection blocks of the sides whose cell lies in [c0, c1) (incidence
// entries [e0, e1) = [row_ptr[c0], row_ptr[c1])), from those cells'
// dSec_dPri at ds[k * soa + (cell - c0)] (k_fim.cu)
cudaError_t launch_jac_side(int nct, const Model* dm, const BulkView& b, const ConnView& cv, double dt, int c0,
                            uint32_t e0, uint32_t e1, const double* ds, size_t soa, double* bmat, int block,
                            cudaStream_t s);
cudaError_t launch_newton_update_recompute(int ncm, const Model* dm, const BulkView& b, const double* u,
                                           double dSmax, cudaStream_t s);
// dSec_dPri of the cells [first, first + n) into out[k * soa + (cell - first)],
// two-phase cells first within each tile
cudaError_t launch_dsec_slab(int ncm, const Model* dm, const BulkView& b, int first, int n, double* out, size_t soa,
                             cudaStream_t s);
// The cells at positions [0, *n_split) of the cost order (flash type 2):
// the split's first loop with lane refill into st[position], then the rest
// of their flash resumed from it (k_flash_comp.cu, part 8); next: position
// counters, zero before the launch.
cudaError_t launch_split_refill(int ncm, const Model* dm, const BulkView& b, const int* order, const unsigned* n_split,
                                const uint8_t* pre, SplitState* st, unsigned* next, int blocks, cudaStream_t s);
// fb: the fused form's batch (budget, adaptive level, late list)
cudaError_t launch_split_resume(int ncm, const Model* dm, const BulkView& b, const int* order, const unsigned* n_split,
                                const uint8_t* pre, const SplitState* st, unsigned* next, int blocks,
                                const FlashBatch& fb, cudaStream_t s);
// Cells grouped by the flash type they start from (split, stability test,
// skip) and, within a group, in descending order of their predicted work, by
// a counting sort over COST_BUCKETS buckets.
constexpr int COST_BUCKETS = 256;
// level[0] receives the adaptive work level (see k_cost_scan); wt is the
// deferral threshold in work units
cudaError_t launch_cost_order(const Model* dm, const BulkView& b, unsigned* hist, int* order, unsigned coop_cells,
                              long long wt, int* level, cudaStream_t s);
// hand the cells predicted to need more than `threshold` work units (the work
// their last flash used on the segments this flash's type runs), at or above
// the adaptive level, to the cooperative kernel up front (pre[cell] = 1),
// visiting cells in `order`
// bucket_end: launch_cost_order's bucket counts after it ran (the end of each
// bucket in the order)
cudaError_t launch_predefer(const Model* dm, const BulkView& b, const int* order, const unsigned* bucket_end,
                            long long threshold, const int* level, const DeferSink& sink, uint8_t* pre,
                            cudaStream_t s);

// Newton and time-step control (k_nrctl.cu).  mode 0: CalMaxChangeNR against
// the last Newton iterate (lP, lT, lN, lS; replaced by the current state),
// mode 1: CalMaxChangeTime against the last time step (lP, lT, lS, b.lNi).
// out5 receives dP, dT, dN, dS, eV; partial holds MAX_CHANGE_BLOCKS x 5
// candidates of 16 bytes.
using NRControl = ocpx_nr_control;
constexpr int MAX_CHANGE_BLOCKS = 1216;
int max_change_blocks(int nb);
cudaError_t launch_max_change(int mode, const BulkView& b, double* lP, double* lT, double* lN, double* lS,
                              void* partial, double* out5, cudaStream_t s);
cudaError_t launch_nr_converge(const NRControl& c, const double* nr5, const RowNorm* norm, const double* res0,
                               const double* wellrel, int* state, cudaStream_t s);
cudaError_t launch_next_dt(const NRControl& c, const double* ts5, double* out2, cudaStream_t s);

// one perforation of a Peaceman well (k_wells.cu)
struct WellPerf {
    int cell, well, type, mode;
    double bhp, WIm, dG, xi_inj;
};
// per perforation: qi [nc], dQ/dP_well [nc], the cell's diagonal addition and
// the well-to-cell block (rate control) [(nc+1)^2 each] (ocpx_wells_eval)
cudaError_t launch_well_perf(const BulkView& b, const WellPerf* perf, int nperf, const double* inj_zi,
                             const double* factor, double dt, double* qi, double* dqw, double* bb, double* wb,
                             cudaStream_t s);

// The wells inside the Newton step (k_wells.cu).  Well w's row and column are
// nb + w; perforations are listed well by well in perforation order.
struct WellDev {
    int type, mode;          // 0 injector / 1 producer; 0 BHP / 1 rate control
    int p0, p1;              // its perforations [p0, p1)
    double tar_bhp, tar_rate;
};
struct WellSys {
    int nw = 0, nperf = 0, npc = 0;
    const WellDev* well = nullptr;
    double* bhp = nullptr;           // [nw] bottom-hole pressures (state), then two checkpoint slots of nw
    const double* zi = nullptr;      // [nw*nc] injected composition
    const double* factor = nullptr;  // [nw*nc] rate factors
    const WellPerf* perf = nullptr;  // [nperf] (bhp unused: bhp[well])
    const uint32_t* slot_bw = nullptr;  // [nperf] bulk-to-well block index (in the perforated cell's row)
    const uint32_t* slot_wb = nullptr;  // [nperf] well-to-bulk block index (in the well's row)
    const int* pc_cell = nullptr;    // [npc] perforated cells
    const int* pc_start = nullptr;   // [npc+1] their perforations in pc_perf
    const int* pc_perf = nullptr;    // [nperf] perforation indices grouped by cell, in well then perforation order
    double* qi = nullptr;            // [nperf*nc] mole rates
    double* dqb = nullptr;           // [nperf*(nc+1)] dQ/dP of the perforated cell (row 0 zero)
    double* dqw = nullptr;           // [nperf*nc] dQ/dP_well
    double* S = nullptr;             // [nperf*(nc+1)^2] dQ/dXs * dSec_dPri
    double* wrel = nullptr;          // [nw] |R_w / target rate|
    double* maxrel = nullptr;        // [1] maxWellRelRes_mol
    const int* perf_pc = nullptr;    // [nperf] the perforated cell's index in pc_cell
    double* dsec = nullptr;          // [npc][np*(nc+1)^2] the perforated cells' recomputed dSec_dPri
                                     // (NULL: the stored one)
};
// after the bulk residual (before its norms are reduced): the perforations'
// terms, the perforated rows and their relative residuals, the wells' rows
cudaError_t launch_wells_res(const BulkView& b, const WellSys& w, double dt, double* res, double* resRelV,
                             double* resRelN, RowNorm* rn, cudaStream_t s);
// after the bulk Jacobian rows: perforated rows' additions, the wells' rows
cudaError_t launch_wells_jac(const BulkView& b, const WellSys& w, double dt, const uint32_t* rowptr, double* val,
                             cudaStream_t s);
// GetSolutionFIM of every well
cudaError_t launch_wells_update(const BulkView& b, const WellSys& w, const double* u, cudaStream_t s);
// J^T lambda: the wells' blocks added to the perforated cells' entries, and the wells' entries
cudaError_t launch_wells_jt(const BulkView& b, const WellSys& w, const uint32_t* rowptr, const double* val,
                            const double* lam, double* out, cudaStream_t s);

// Linear solve of J u = rhs on the device (k_linsolve.cu): BiCGStab with right
// block-Jacobi preconditioning, x from zero; scratch holds
// linsolve_scratch_doubles(nb, dim) doubles.  The residual norm is tested on
// the device every check_every iterations.  linsolve waits for each test and
// returns the result; linsolve_async enqueues the whole solve without waiting
// (capturable in a graph), and linsolve_read waits for the stream and reads
// the result of the last solve in `scratch`.
struct LinsolveResult {
    int iterations;
    double relres;   // |rhs - J x| / |rhs| of the recursively updated residual
    int converged;
    int breakdown;   // 1: BiCGStab breakdown, 2: singular diagonal block
};
size_t linsolve_scratch_doubles(int nb, int dim);
cudaError_t linsolve(const uint32_t* rowptr, const uint32_t* col, const double* val, int nb, int dim,
                     const double* rhs, double* x, double* scratch, double tol, int maxit, int check_every,
                     LinsolveResult* res, uint64_t* launches, cudaStream_t s);
cudaError_t linsolve_async(const uint32_t* rowptr, const uint32_t* col, const double* val, int nb, int dim,
                           const double* rhs, double* x, double* scratch, double tol, int maxit, int check_every,
                           uint64_t* launches, cudaStream_t s);
cudaError_t linsolve_read(const double* scratch, int nb, int dim, LinsolveResult* res, cudaStream_t s);

cudaError_t launch_flash_bo(const Model* dm, const BulkView& b, int block, cudaStream_t s);
cudaError_t launch_krpc_rock(const Model* dm, const BulkView& b, int block, cudaStream_t s);
cudaError_t launch_check(const BulkView& b, uint32_t* flags, int block, cudaStream_t s);
cudaError_t launch_newton_update(const BulkView& b, const double* u, double dSmax, int block, cudaStream_t s);
cudaError_t launch_conn_flux(const Model* dm, const BulkView& b, const ConnView& cv, int block, cudaStream_t s);
cudaError_t launch_residual(const BulkView& b, const ConnView& cv, double dt, double* res, double* resRelV,
                            double* resRelN, RowNorm* rn, RowNorm* rn_out, RowNorm* part, int block, cudaStream_t s);
// the norm reduction of launch_residual alone (launch_residual with rn_out NULL
// leaves it out, so that the wells' rows can be added first); part: NORM_PARTS
// partial maxima
constexpr int NORM_PARTS = 1024;
cudaError_t launch_norm_reduce(const RowNorm* rn, int nbI, RowNorm* rn_out, RowNorm* part, cudaStream_t s);
cudaError_t launch_jac_conn(int nct, const Model* dm, const BulkView& b, const ConnView& cv, double dt,
                            double* bmat, int block, cudaStream_t s);
cudaError_t launch_jac_rows(const BulkView& b, const ConnView& cv, const double* bmat, const uint32_t* rowptr,
                            double* val, int block, cudaStream_t s);
cudaError_t launch_report(const BulkView& b, uint32_t* out3, int block, cudaStream_t s);
// adjoint vector-Jacobian products (adjoint.cuh)
cudaError_t launch_jt_lambda(const BulkView& b, const ConnView& cv, const uint32_t* rowptr, const double* val,
                             const uint32_t* slot, const double* lam, double* out, int block, cudaStream_t s);
cudaError_t launch_vjp_trans(const BulkView& b, const ConnView& cv, double dt, const double* lam, double* out,
                             int block, cudaStream_t s);
cudaError_t launch_vjp_poro(const Model* dm, const BulkView& b, const double* lam, double* out, int block,
                            cudaStream_t s);

// layout conversion between the reference's cell-major arrays and the
// device structure-of-arrays, for the n entities starting at `first` of an
// SoA array of N entities (N = 0: N = n, first = 0):
// dst[k*N + first + i] = src[i*width + k] (to_soa) and back
cudaError_t launch_transpose(void* dst, const void* src, int n, int width, int elem_bytes, bool to_soa,
                             cudaStream_t s, size_t N = 0, size_t first = 0);

}  // namespace ocpx
