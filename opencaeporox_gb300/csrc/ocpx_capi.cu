// C ABI (include/ocpx.h): context, device memory, layout conversion and the
// launch sequence of one FIM Newton step.
#include "ocpx.h"
#include "ocpx_kernels.h"
#include "model_build.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace ocpx {
cudaError_t launch_flash_comp_4(const Model*, const BulkView&, int, cudaStream_t);
cudaError_t launch_flash_comp_6(const Model*, const BulkView&, int, cudaStream_t);
cudaError_t launch_flash_comp_8(const Model*, const BulkView&, int, cudaStream_t);
cudaError_t launch_flash_comp_10(const Model*, const BulkView&, int, cudaStream_t);
cudaError_t launch_flash_comp_12(const Model*, const BulkView&, int, cudaStream_t);
cudaError_t launch_flash_batched_4(const Model*, const BulkView&, const int*, const FlashBatch&, int, cudaStream_t);
cudaError_t launch_flash_batched_6(const Model*, const BulkView&, const int*, const FlashBatch&, int, cudaStream_t);
cudaError_t launch_flash_batched_8(const Model*, const BulkView&, const int*, const FlashBatch&, int, cudaStream_t);
cudaError_t launch_flash_batched_10(const Model*, const BulkView&, const int*, const FlashBatch&, int, cudaStream_t);
cudaError_t launch_flash_batched_12(const Model*, const BulkView&, const int*, const FlashBatch&, int, cudaStream_t);
cudaError_t setup_flash_batched_4(int*);
cudaError_t setup_flash_batched_6(int*);
cudaError_t setup_flash_batched_8(int*);
cudaError_t setup_flash_batched_10(int*);
cudaError_t setup_flash_batched_12(int*);

cudaError_t launch_flash_comp(int ncm, const Model* dm, const BulkView& b, int block, cudaStream_t s)
{
    switch (ncm) {
    case 4: return launch_flash_comp_4(dm, b, block, s);
    case 6: return launch_flash_comp_6(dm, b, block, s);
    case 8: return launch_flash_comp_8(dm, b, block, s);
    case 10: return launch_flash_comp_10(dm, b, block, s);
    case 12: return launch_flash_comp_12(dm, b, block, s);
    default: return cudaErrorInvalidValue;
    }
}
cudaError_t launch_flash_batched(int ncm, const Model* dm, const BulkView& b, const int* order,
                                 const FlashBatch& fb, int part, cudaStream_t s)
{
    switch (ncm) {
    case 4: return launch_flash_batched_4(dm, b, order, fb, part, s);
    case 6: return launch_flash_batched_6(dm, b, order, fb, part, s);
    case 8: return launch_flash_batched_8(dm, b, order, fb, part, s);
    case 10: return launch_flash_batched_10(dm, b, order, fb, part, s);
    case 12: return launch_flash_batched_12(dm, b, order, fb, part, s);
    default: return cudaErrorInvalidValue;
    }
}
cudaError_t setup_flash_batched(int ncm, int* excl_smem)
{
    switch (ncm) {
    case 4: return setup_flash_batched_4(excl_smem);
    case 6: return setup_flash_batched_6(excl_smem);
    case 8: return setup_flash_batched_8(excl_smem);
    case 10: return setup_flash_batched_10(excl_smem);
    case 12: return setup_flash_batched_12(excl_smem);
    default: return cudaErrorInvalidValue;
    }
}

// the consumers of recomputed flash derivatives, one set per NCM
#define OCPX_RECOMPUTE_DECL(N)                                                                                     \
    cudaError_t launch_dsec_cells_##N(const Model*, const BulkView&, const int*, int, int, double*, size_t,          \
                                      cudaStream_t);                                                                 \
    cudaError_t launch_newton_update_recompute_##N(const Model*, const BulkView&, const double*, double, cudaStream_t); \
    cudaError_t launch_dsec_slab_##N(const Model*, const BulkView&, int, int, double*, size_t, cudaStream_t);
#define OCPX_SPLIT_DECL(N)                                                                                         \
    cudaError_t launch_split_refill_##N(const Model*, const BulkView&, const int*, const unsigned*, const uint8_t*,   \
                                        SplitState*, unsigned*, int, cudaStream_t);                                   \
    cudaError_t launch_split_resume_##N(const Model*, const BulkView&, const int*, const unsigned*, const uint8_t*,   \
                                        const SplitState*, unsigned*, int, const FlashBatch&, cudaStream_t);
OCPX_SPLIT_DECL(4)
OCPX_SPLIT_DECL(6)
OCPX_SPLIT_DECL(8)
OCPX_SPLIT_DECL(10)
OCPX_SPLIT_DECL(12)
#undef OCPX_SPLIT_DECL
OCPX_RECOMPUTE_DECL(4)
OCPX_RECOMPUTE_DECL(6)
OCPX_RECOMPUTE_DECL(8)
OCPX_RECOMPUTE_DECL(10)
OCPX_RECOMPUTE_DECL(12)
#undef OCPX_RECOMPUTE_DECL
#define OCPX_NCM_SWITCH(fn, ...)                      \
    switch (ncm) {                                    \
    case 4: return fn##4(__VA_ARGS__);                \
    case 6: return fn##6(__VA_ARGS__);                \
    case 8: return fn##8(__VA_ARGS__);                \
    case 10: return fn##10(__VA_ARGS__);              \
    case 12: return fn##12(__VA_ARGS__);              \
    default: return cudaErrorInvalidValue;            \
    }
cudaError_t launch_dsec_cells(int ncm, const Model* dm, const BulkView& b, const int* list, int first, int n,
                              double* out, size_t soa, cudaStream_t s)
{
    OCPX_NCM_SWITCH(launch_dsec_cells_, dm, b, list, first, n, out, soa, s)
}
cudaError_t launch_newton_update_recompute(int ncm, const Model* dm, const BulkView& b, const double* u,
                                           double dSmax, cudaStream_t s)
{
    OCPX_NCM_SWITCH(launch_newton_update_recompute_, dm, b, u, dSmax, s)
}
cudaError_t launch_dsec_slab(int ncm, const Model* dm, const BulkView& b, int first, int n, double* out, size_t soa,
                             cudaStream_t s)
{
    OCPX_NCM_SWITCH(launch_dsec_slab_, dm, b, first, n, out, soa, s)
}
cudaError_t launch_split_refill(int ncm, const Model* dm, const BulkView& b, const int* order, const unsigned* n_split,
                                const uint8_t* pre, SplitState* st, unsigned* next, int blocks, cudaStream_t s)
{
    OCPX_NCM_SWITCH(launch_split_refill_, dm, b, order, n_split, pre, st, next, blocks, s)
}
cudaError_t launch_split_resume(int ncm, const Model* dm, const BulkView& b, const int* order, const unsigned* n_split,
                                const uint8_t* pre, const SplitState* st, unsigned* next, int blocks,
                                const FlashBatch& fb, cudaStream_t s)
{
    OCPX_NCM_SWITCH(launch_split_resume_, dm, b, order, n_split, pre, st, next, blocks, fb, s)
}
#undef OCPX_NCM_SWITCH
}  // namespace ocpx

using namespace ocpx;

namespace {

thread_local std::string g_err;

ocpx_status fail(ocpx_status st, const std::string& msg)
{
    g_err = msg;
    return st;
}

#define OCPX_CUDA(call)                                                                                 \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return fail(OCPX_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int cap_ncm(int NC)
{
    for (int c : kNcmCaps)
        if (NC <= c) return c;
    return -1;
}
int cap_nct(int nct)
{
    for (int c : kNctCaps)
        if (nct <= c) return c;
    return -1;
}

// cells per slab when dSec_dPri is recomputed for the Jacobian: 524,288 cells
// hold 1.5 GB of it at nc = 10 (the whole grid's would be 11.6 GB at
// 4,000,000 cells), eight slabs on that grid
constexpr int RECOMPUTE_SLAB_CELLS = 1 << 19;

struct FieldInfo {
    void* dev;       // device SoA base (or cell-major for AoS-native fields)
    int n;           // entities (cells or connections)
    int width;       // values per entity
    int elem;        // bytes per value
    bool soa;        // device layout is [k][n]
    bool writable;
};

}  // namespace

struct ocpx_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    Model host_model{};
    Model* d_model = nullptr;
    int nb = 0, nbI = 0, np = 3, nc = 0, nconn = 0, NC = 0, ncm = 0, nct_cap = 0;
    int variant = 0;
    // dSec_dPri recomputed where it is used instead of stored (ocpx_options):
    // the Jacobian recomputes it slab by slab, dsec_slab cells at a time
    bool recompute = false;
    int dsec_slab = 0;
    double* dsec_scratch = nullptr;
    // the split cells' first loop with lane refill (OCPX_PARAM_SPLIT_REFILL)
    int split_refill = 0;
    SplitState* split_state = nullptr;  // [nb], allocated when the option is first set
    // one arena for everything
    char* arena = nullptr;
    size_t arena_bytes = 0;
    size_t sys_bytes = 0;           // the linear system's buffer (sys)
    size_t wbuf_bytes = 0;          // the wells' buffer (wbuf)
    BulkView b{};
    ConnView cv{};
    double* res = nullptr;
    double* resRelV = nullptr;
    double* resRelN = nullptr;
    RowNorm* rownorm = nullptr;
    RowNorm* norm_out = nullptr;
    RowNorm* norm_part = nullptr;   // partial maxima of the two-pass norm reduction
    uint32_t* flags = nullptr;      // [4]: check OR, report (OR, two-phase, flagged)
    // batched flash: cost order, deferral list, cooperative results
    int* order = nullptr;
    unsigned* cost_hist = nullptr;
    DeferRec* defer_rec = nullptr;     // cells deferred by the per-cell kernel
    unsigned* defer_count = nullptr;   // [32]: [0] deferred by the per-cell kernel, [1] pre-deferred, others counters
    DeferRec* defer_rec2 = nullptr;    // second late list (re-budgeting rounds alternate between the two)
    int rounds = 0;                    // re-budgeting rounds before the late cooperative pass (0..8)
    int round_growth = 4;              // budget factor per round
    int late_count = 0;                // index in defer_count of the list the late cooperative pass takes
    PERes* pe_res = nullptr;
    DeferRec* pre_rec = nullptr;       // cells pre-deferred from their last flash's work
    PERes* pre_res = nullptr;
    uint8_t* pre_flag = nullptr;       // [nb]
    int defer_cap = 0;
    int flash_budget = 48;
    int coop_blocks = 0;
    long long predefer = 192;          // pre-deferral threshold in work units (0: off)
    long long coop_cells = 1216;       // target cells per cooperative pass (adaptive level; 0: off)
    int* adapt_level = nullptr;        // device: adaptive work level of the last cost order
    cudaStream_t stream2 = nullptr;    // high-priority stream of the pre-deferred cooperative kernel
    int prio_hi = 0;                   // greatest stream priority of the device
    int pre_blocks = 0;                // SM-exclusive blocks of the pre-deferred pass (0: shared-SM blocks)
    int excl_smem[3] = {0, 0, 0};      // SM-exclusive blocks' dynamic shared memory (cooperative, fused),
                                       // fused blocks resident per SM without it
    int fused_blocks = 0;              // > 0: the fused batched flash with this many blocks
    int fused_coop_blocks = -1;        // leading fused blocks that run only cooperative work (-1: automatic)
    int fused_excl = 0;                // fused blocks at most the SM count reserve an SM each
    int post_block = 32;               // threads per block of the deferred cells' finishing kernel
    int sms = 0;                       // SMs of the device
    int cell_blocks = 0;               // persistent blocks of the per-cell kernel (0: one thread per cell)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    double* u = nullptr;            // Newton update staging
    double *nr_lP = nullptr, *nr_lT = nullptr, *nr_lN = nullptr, *nr_lS = nullptr;  // last Newton iterate
    double *ts_lP = nullptr, *ts_lT = nullptr, *ts_lS = nullptr;                    // last time step
    void* maxch_partial = nullptr;  // per-block candidates of the max-change reductions
    double* nr_stats = nullptr;     // [5] CalMaxChangeNR: dP, dT, dN, dS, eV
    double* ts_stats = nullptr;     // [5] CalMaxChangeTime
    double* nr_res0 = nullptr;      // initial relative residual of the time step
    int* nr_state = nullptr;        // last CheckConverge state
    double* nr_dt = nullptr;        // [2] next dt, predicted dt
    double* ls_scratch = nullptr;   // linear solver work space (allocated by the first ocpx_linsolve)
    double* bmat = nullptr;         // per-connection Jacobian blocks (2 per connection)
    uint32_t* jac_rowptr = nullptr;
    uint32_t* jac_slot = nullptr;   // [2][nconn]: block index of connection c in row bId / row eId
    double* adj = nullptr;          // adjoint workspace: lambda, J^T lambda [nb*(nc+1)] each
    double* adj_conn = nullptr;     // [nconn]
    // adjoint products inside the step (ocpx_set_adjoint_seed): one allocation
    // holding the seed lambda and J^T lambda [nb*(nc+1)] each, (dR/dporoInit)^T
    // lambda [nb] and (dR/dT)^T lambda [nconn]
    double* step_adj = nullptr;
    bool adj_in_step = false;
    // the linear system's storage (build_system): block-CSR pattern and values
    // of the interior rows and the wells' rows, the residual and the Newton
    // update of the cells and the wells, the adjoint's vectors
    char* sys = nullptr;
    int nrow = 0;                   // system rows: interior cells, then open wells
    std::vector<uint32_t> h_row_ptr, h_row_conn, h_conn_b, h_conn_e;  // connectivity, kept for rebuilds
    // wells inside the step (ocpx_set_wells)
    char* wbuf = nullptr;
    WellSys ws{};
    std::vector<int> well_cells;    // perforated cells, well by well, in perforation order
    std::vector<int> well_nperf;    // perforations per well
    std::vector<uint32_t> h_slot_bw, h_slot_wb;  // their blocks in the system (build_system)
    size_t nv() const { return (size_t)(nb + ws.nw) * (nc + 1); }
    // ocpx_wells_eval's device buffer (grows as needed) and the state
    // generation the last residual was computed at
    char* weval = nullptr;
    size_t weval_bytes = 0;
    uint64_t state_gen = 1, res_gen = 0;
    double last_dt = 0;             // dt of the last residual / Jacobian
    uint32_t* jac_col = nullptr;
    double* jac_val = nullptr;
    size_t jac_nnz = 0;
    void* staging = nullptr;        // host-layout staging for field transfers
    size_t staging_bytes = 0;
    uint32_t* h_flags = nullptr;    // pinned
    RowNorm* h_norm = nullptr;      // pinned
    uint64_t launches = 0;
    int block_cell = 128, block_conn = 128;
    // per-stage event timing
    bool prof = false;
    struct Mark { int stage; cudaEvent_t a, b; cudaStream_t st; };
    std::vector<Mark> marks;
    std::vector<cudaEvent_t> free_events;
    double prof_ms[OCPX_STAGE_COUNT] = {0};
    uint64_t prof_n[OCPX_STAGE_COUNT] = {0};
    cudaEvent_t take_event()
    {
        if (free_events.empty()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            return e;
        }
        cudaEvent_t e = free_events.back();
        free_events.pop_back();
        return e;
    }
    int stage_begin(int s, cudaStream_t on = nullptr)
    {
        if (!prof) return -1;
        Mark m{s, take_event(), take_event(), on ? on : stream};
        cudaEventRecord(m.a, m.st);
        marks.push_back(m);
        return (int)marks.size() - 1;
    }
    void stage_end(int idx)
    {
        if (idx < 0) return;
        cudaEventRecord(marks[idx].b, marks[idx].st);
    }
    // device-side checkpoints of the mutable bulk state
    char* ckpt[2] = {nullptr, nullptr};
    size_t state_off = 0, state_bytes = 0;
    // CUDA graph of one Newton iteration (properties, residual, Jacobian) of
    // the batched variant, captured for one dt and launch configuration
    cudaGraphExec_t graph_exec = nullptr;
    double graph_dt = -1;
    uint64_t graph_launches = 0;    // kernels in the graph
    void drop_graph()
    {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
        graph_dt = -1;
    }

    FieldInfo field(ocpx_field f) const;
};

FieldInfo ocpx_ctx::field(ocpx_field f) const
{
    const int nct = nc, npc = np * nc, lend = np * (nc + 1) * (nc + 1);
    switch (f) {
    case OCPX_F_P: return {b.P, nb, 1, 8, true, true};
    case OCPX_F_T: return {b.T, nb, 1, 8, true, true};
    case OCPX_F_PB: return {b.Pb, nb, 1, 8, true, true};
    case OCPX_F_NI: return {b.Ni, nb, nct, 8, true, true};
    case OCPX_F_LNI: return {b.lNi, nb, nct, 8, true, true};
    case OCPX_F_NT: return {b.Nt, nb, 1, 8, true, true};
    case OCPX_F_VF: return {b.vf, nb, 1, 8, true, true};
    case OCPX_F_VFP: return {b.vfP, nb, 1, 8, true, true};
    case OCPX_F_VFI: return {b.vfi, nb, nct, 8, true, true};
    case OCPX_F_PJ: return {b.Pj, nb, np, 8, true, true};
    case OCPX_F_PC: return {b.Pc, nb, np, 8, true, true};
    case OCPX_F_S: return {b.S, nb, np, 8, true, true};
    case OCPX_F_PHASE_EXIST: return {b.phaseExist, nb, np, 1, true, true};
    case OCPX_F_XIJ: return {b.xij, nb, npc, 8, true, true};
    case OCPX_F_RHO: return {b.rho, nb, np, 8, true, true};
    case OCPX_F_XI: return {b.xi, nb, np, 8, true, true};
    case OCPX_F_MU: return {b.mu, nb, np, 8, true, true};
    case OCPX_F_RHOP: return {b.rhoP, nb, np, 8, true, true};
    case OCPX_F_XIP: return {b.xiP, nb, np, 8, true, true};
    case OCPX_F_MUP: return {b.muP, nb, np, 8, true, true};
    case OCPX_F_RHOX: return {b.rhox, nb, npc, 8, true, true};
    case OCPX_F_XIX: return {b.xix, nb, npc, 8, true, true};
    case OCPX_F_MUX: return {b.mux, nb, npc, 8, true, true};
    case OCPX_F_KR: return {b.kr, nb, np, 8, true, true};
    case OCPX_F_DKRDS: return {b.dKrdS, nb, np * np, 8, true, true};
    case OCPX_F_DPCDS: return {b.dPcdS, nb, np * np, 8, true, true};
    // recomputed on reads when not stored (field_transfer); dev then only marks the field as known
    case OCPX_F_DSEC_DPRI: return {recompute ? (void*)b.njhc : (void*)b.dSec_dPri, nb, lend, 8, true, !recompute};
    case OCPX_F_PORO: return {b.poro, nb, 1, 8, true, true};
    case OCPX_F_POROP: return {b.poroP, nb, 1, 8, true, true};
    case OCPX_F_ROCKVP: return {b.rockVp, nb, 1, 8, true, true};
    case OCPX_F_SKIP_FLAG: return {b.skip_flag, nb, 1, 1, true, true};
    case OCPX_F_SKIP_MINEIG: return {b.skip_minEig, nb, 1, 8, true, true};
    case OCPX_F_SKIP_P: return {b.skip_P, nb, 1, 8, true, true};
    case OCPX_F_SKIP_T: return {b.skip_T, nb, 1, 8, true, true};
    case OCPX_F_SKIP_ZI: return {b.skip_zi, nb, NC > 0 ? NC : 1, 8, true, true};
    case OCPX_F_STATUS: return {b.status, nb, 1, 4, true, false};
    case OCPX_F_FTYPE: return {b.ftype, nb, 1, 1, true, false};
    case OCPX_F_FLASH_ITERS: return {b.iters, nb, 5, 4, true, false};
    case OCPX_F_UPBLOCK: return {cv.upblock, nconn, np, 4, true, false};
    case OCPX_F_CONN_DP: return {cv.dP, nconn, np, 8, true, false};
    case OCPX_F_FLUX_VJ: return {cv.flux_vj, nconn, np, 8, true, false};
    case OCPX_F_FLUX_NI: return {cv.flux_ni, nconn, nc, 8, true, false};
    case OCPX_F_RES: return {res, nb + ws.nw, nc + 1, 8, false, false};
    case OCPX_F_RES_REL_V: return {resRelV, nb, 1, 8, true, false};
    case OCPX_F_RES_REL_N: return {resRelN, nb, 1, 8, true, false};
    case OCPX_F_TRANS: return {(void*)cv.trans, nconn, 1, 8, true, true};
    case OCPX_F_PORO_INIT: return {(void*)b.poroInit, nb, 1, 8, true, true};
    default: return {nullptr, 0, 0, 0, true, false};
    }
}

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// FUSED_COOP_BLOCKS in effect.  Automatic: on small grids half of the fused
// blocks run only the cooperative work when the fused blocks hold one SM each,
// so the longest chains never share an SM with per-lane work (36,000 cells:
// 12.3 ms per step with 76 of 152 blocks and budget 32, 12.9 ms with 57 and
// budget 48, 13.3 ms with none); none on large grids, where four blocks per
// SM cannot all be resident.
int fused_coop_blocks(const ocpx_ctx* ctx)
{
    if (ctx->fused_coop_blocks >= 0) return ctx->fused_coop_blocks;
    return ctx->nb < 131072 && ctx->fused_blocks <= ctx->sms ? ctx->fused_blocks / 2 : 0;
}

// The system's storage and block-CSR pattern: per interior row the diagonal
// block, one block per incident connection in connection order
// (AssembleMatBulks), then one bulk-to-well block per perforation of the cell
// in well then perforation order (AssembleMatWells); per open well its
// diagonal block, then one well-to-bulk block per perforation.  Rebuilt when
// the wells' structure changes; slot_bw / slot_wb receive each perforation's
// block indices.  The contents (residual, update, values) start at zero.
ocpx_status build_system(ocpx_ctx* ctx, std::vector<uint32_t>* slot_bw, std::vector<uint32_t>* slot_wb)
{
    const int nbI = ctx->nbI, nb = ctx->nb, nconn = ctx->nconn, dim = ctx->nc + 1;
    const int nw = (int)ctx->well_nperf.size();
    const size_t bsize = (size_t)dim * dim;
    const std::vector<uint32_t>& rp = ctx->h_row_ptr;
    const std::vector<uint32_t>& rc = ctx->h_row_conn;
    std::vector<uint32_t> pcount(nbI, 0);
    for (int c : ctx->well_cells) pcount[c]++;
    std::vector<uint32_t> jrow((size_t)nbI + nw + 1, 0);
    for (int n = 0; n < nbI; n++) jrow[n + 1] = jrow[n] + 1 + (rp[n + 1] - rp[n]) + pcount[n];
    for (int w = 0; w < nw; w++) jrow[nbI + w + 1] = jrow[nbI + w] + 1 + ctx->well_nperf[w];
    const size_t nnz = jrow.back();
    std::vector<uint32_t> jcol(nnz);
    for (int n = 0; n < nbI; n++) {
        size_t pos = jrow[n];
        jcol[pos++] = n;
        for (uint32_t k = rp[n]; k < rp[n + 1]; k++) {
            const uint32_t c = rc[k] >> 1;
            jcol[pos++] = (rc[k] & 1u) ? ctx->h_conn_b[c] : ctx->h_conn_e[c];
        }
    }
    std::vector<uint32_t> placed(nbI, 0);
    if (slot_bw) slot_bw->assign(ctx->well_cells.size(), 0);
    if (slot_wb) slot_wb->assign(ctx->well_cells.size(), 0);
    size_t p = 0;
    for (int w = 0; w < nw; w++) {
        const uint32_t wrow = nbI + w;
        jcol[jrow[wrow]] = wrow;
        for (int q = 0; q < ctx->well_nperf[w]; q++, p++) {
            const int c = ctx->well_cells[p];
            const size_t bw = jrow[c] + 1 + (rp[c + 1] - rp[c]) + placed[c]++;
            jcol[bw] = wrow;
            const size_t wb = jrow[wrow] + 1 + q;
            jcol[wb] = (uint32_t)c;
            if (slot_bw) (*slot_bw)[p] = (uint32_t)bw;
            if (slot_wb) (*slot_wb)[p] = (uint32_t)wb;
        }
    }
    // block index of each connection in the rows of its two cells (adjoint
    // transpose; a ghost cell's side has none)
    std::vector<uint32_t> jslot(2 * (size_t)(nconn > 0 ? nconn : 1), 0xffffffffu);
    for (int n = 0; n < nbI; n++)
        for (uint32_t k = rp[n]; k < rp[n + 1]; k++) {
            const uint32_t c = rc[k] >> 1, side = rc[k] & 1u;
            jslot[(size_t)side * nconn + c] = jrow[n] + 1 + (k - rp[n]);
        }
    const size_t nv = (size_t)(nb + nw) * dim;
    const size_t o_row = 0, o_col = o_row + align256(sizeof(uint32_t) * jrow.size());
    const size_t o_slot = o_col + align256(sizeof(uint32_t) * nnz);
    const size_t o_res = o_slot + align256(sizeof(uint32_t) * jslot.size());
    const size_t o_u = o_res + align256(sizeof(double) * nv), o_adj = o_u + align256(sizeof(double) * nv);
    const size_t o_val = o_adj + align256(sizeof(double) * 2 * nv);
    const size_t total = o_val + align256(sizeof(double) * nnz * bsize);
    ctx->drop_graph();
    if (ctx->stream) OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->sys) cudaFree(ctx->sys);
    ctx->sys = nullptr;
    ctx->jac_rowptr = nullptr;
    ctx->jac_col = nullptr;
    ctx->jac_slot = nullptr;
    ctx->jac_val = nullptr;
    ctx->res = ctx->u = ctx->adj = nullptr;
    ctx->sys_bytes = 0;
    if (cudaMalloc(&ctx->sys, total) != cudaSuccess)
        return fail(OCPX_CUDA_ERROR, "cudaMalloc of " + std::to_string(total) + " bytes (the linear system) failed");
    ctx->sys_bytes = total;
    ctx->jac_rowptr = (uint32_t*)(ctx->sys + o_row);
    ctx->jac_col = (uint32_t*)(ctx->sys + o_col);
    ctx->jac_slot = (uint32_t*)(ctx->sys + o_slot);
    ctx->res = (double*)(ctx->sys + o_res);
    ctx->u = (double*)(ctx->sys + o_u);
    ctx->adj = (double*)(ctx->sys + o_adj);
    ctx->jac_val = (double*)(ctx->sys + o_val);
    ctx->jac_nnz = nnz;
    ctx->nrow = nbI + nw;
    // on the context's stream, which does not wait for the legacy stream
    OCPX_CUDA(cudaMemsetAsync(ctx->sys, 0, o_val, ctx->stream));
    OCPX_CUDA(cudaMemcpyAsync(ctx->jac_rowptr, jrow.data(), sizeof(uint32_t) * jrow.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
    OCPX_CUDA(cudaMemcpyAsync(ctx->jac_col, jcol.data(), sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, ctx->stream));
    OCPX_CUDA(cudaMemcpyAsync(ctx->jac_slot, jslot.data(), sizeof(uint32_t) * jslot.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->ls_scratch) {  // the solver's work space is sized by the rows
        cudaFree(ctx->ls_scratch);
        ctx->ls_scratch = nullptr;
    }
    return OCPX_OK;
}

}  // namespace

extern "C" {

int ocpx_abi_version(void) { return OCPX_ABI_VERSION; }
const char* ocpx_last_error(void) { return g_err.c_str(); }

ocpx_status ocpx_create(const ocpx_model_desc* md, const ocpx_grid_desc* gd, int device, ocpx_ctx** out)
{
    return ocpx_create_ex(md, gd, device, nullptr, out);
}

ocpx_status ocpx_create_ex(const ocpx_model_desc* md, const ocpx_grid_desc* gd, int device, const ocpx_options* opt,
                           ocpx_ctx** out)
{
    if (!md || !gd || !out) return fail(OCPX_INVALID_ARG, "null argument");
    *out = nullptr;
    if (opt && opt->struct_size != sizeof(ocpx_options))
        return fail(OCPX_INVALID_ARG, "ocpx_options.struct_size must be sizeof(ocpx_options)");
    const bool recompute = opt && opt->recompute_flash_der != 0;
    if (recompute && md->mixture != 1)
        return fail(OCPX_INVALID_ARG, "recompute_flash_der needs the compositional mixture");
    if (gd->nb <= 0 || gd->nconn < 0 || !gd->v || !gd->depth || !gd->poro_init ||
        (gd->nconn > 0 && (!gd->conn_b || !gd->conn_e || !gd->conn_trans)))
        return fail(OCPX_INVALID_ARG, "grid description incomplete");
    if (gd->nb_interior < 0 || gd->nb_interior > gd->nb)
        return fail(OCPX_INVALID_ARG, "nb_interior must lie in [0, nb]");
    const uint32_t nbI_ = gd->nb_interior > 0 ? (uint32_t)gd->nb_interior : (uint32_t)gd->nb;
    // the descriptions are checked before the device, so a host without one
    // can still validate them (OCPX_INVALID_ARG before OCPX_NO_DEVICE)
    for (int c = 0; c < gd->nconn; c++) {
        if (gd->conn_b[c] >= (uint32_t)gd->nb || gd->conn_e[c] >= (uint32_t)gd->nb || gd->conn_b[c] == gd->conn_e[c])
            return fail(OCPX_INVALID_ARG, "connection endpoint out of range at " + std::to_string(c));
        if (gd->conn_b[c] >= nbI_ && gd->conn_e[c] >= nbI_)
            return fail(OCPX_INVALID_ARG, "connection " + std::to_string(c) + " joins two ghost cells");
    }

    ocpx_ctx* ctx = new ocpx_ctx();
    std::string merr;
    ocpx_status st = build_model(md, ctx->host_model, merr);
    if (st != OCPX_OK) { delete ctx; return fail(st, merr); }
    if (md->mixture == 1 && cap_ncm(md->nc - 1) < 0) { delete ctx; return fail(OCPX_INVALID_ARG, "too many components"); }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { delete ctx; return fail(OCPX_NO_DEVICE, "no CUDA device"); }
    if (device >= 0) {
        if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return fail(OCPX_NO_DEVICE, "cudaSetDevice failed"); }
        ctx->device = device;
    }
    else {
        cudaGetDevice(&ctx->device);
    }
    ctx->nb = gd->nb;
    ctx->nbI = (int)nbI_;
    ctx->recompute = recompute;
    ctx->nc = md->nc;
    ctx->np = 3;
    ctx->nconn = gd->nconn;
    ctx->NC = md->mixture == 1 ? md->nc - 1 : 0;
    ctx->ncm = md->mixture == 1 ? cap_ncm(ctx->NC) : 0;
    ctx->nct_cap = cap_nct(md->nc);
    if (ctx->nct_cap < 0 || (md->mixture == 1 && ctx->ncm < 0)) { delete ctx; return fail(OCPX_INVALID_ARG, "too many components"); }

    const int nb = ctx->nb, nbI = ctx->nbI, np = ctx->np, nc = ctx->nc, nconn = ctx->nconn;
    const int lend = np * (nc + 1) * (nc + 1), bsize = (nc + 1) * (nc + 1);

    // row -> incident connections (increasing connection index) and the
    // block-CSR pattern of the interior rows: diagonal first, then one block
    // per incident connection
    std::vector<uint32_t> deg(nb + 1, 0);
    for (int c = 0; c < nconn; c++) { deg[gd->conn_b[c]]++; deg[gd->conn_e[c]]++; }
    std::vector<uint32_t> row_ptr(nb + 1, 0);
    for (int n = 0; n < nb; n++) row_ptr[n + 1] = row_ptr[n] + deg[n];
    std::vector<uint32_t> row_conn(row_ptr[nb]);
    std::vector<uint32_t> fill(row_ptr.begin(), row_ptr.end() - 1);
    for (int c = 0; c < nconn; c++) {
        row_conn[fill[gd->conn_b[c]]++] = ((uint32_t)c << 1) | 0u;
        row_conn[fill[gd->conn_e[c]]++] = ((uint32_t)c << 1) | 1u;
    }

    // arena layout
    struct Slot { void** p; size_t bytes; };
    std::vector<Slot> slots;
    auto add = [&](void* pp, size_t bytes) { slots.push_back({(void**)pp, bytes}); };
    BulkView& b = ctx->b;
    b.nb = nb; b.nbI = nbI; b.np = np; b.nc = nc;
    const size_t D = sizeof(double) * (size_t)nb;
    add(&b.v, D); add(&b.depth, D); add(&b.poroInit, D);
    add(&b.P, D); add(&b.T, D); add(&b.Pb, D);
    add(&b.Ni, D * nc); add(&b.lNi, D * nc);
    add(&b.Nt, D); add(&b.vf, D); add(&b.vfP, D); add(&b.vfi, D * nc);
    add(&b.Pj, D * np); add(&b.Pc, D * np); add(&b.S, D * np);
    add(&b.phaseExist, (size_t)nb * np);
    add(&b.xij, D * np * nc);
    add(&b.rho, D * np); add(&b.xi, D * np); add(&b.mu, D * np);
    add(&b.rhoP, D * np); add(&b.xiP, D * np); add(&b.muP, D * np);
    add(&b.rhox, D * np * nc); add(&b.xix, D * np * nc); add(&b.mux, D * np * nc);
    add(&b.kr, D * np); add(&b.dKrdS, D * np * np); add(&b.dPcdS, D * np * np);
    // dSec_dPri, or what recomputing it needs beyond the other fields: the
    // hydrocarbon phases' mole numbers (both inside the state range, so the
    // checkpoints keep them)
    if (recompute) add(&b.njhc, D * 2);
    else add(&b.dSec_dPri, D * lend);
    add(&b.poro, D); add(&b.poroP, D); add(&b.rockVp, D);
    add(&b.skip_flag, (size_t)nb); add(&b.skip_minEig, D); add(&b.skip_P, D); add(&b.skip_T, D);
    add(&b.skip_zi, D * (ctx->NC > 0 ? ctx->NC : 1));
    add(&b.status, sizeof(uint32_t) * (size_t)nb); add(&b.ftype, (size_t)nb);
    add(&b.iters, sizeof(int32_t) * (size_t)nb * 5);
    ConnView& cv = ctx->cv;
    cv.nconn = nconn;
    const size_t C = (size_t)(nconn > 0 ? nconn : 1);
    add(&cv.bId, sizeof(uint32_t) * C); add(&cv.eId, sizeof(uint32_t) * C); add(&cv.trans, sizeof(double) * C);
    add(&cv.upblock, sizeof(uint32_t) * C * np); add(&cv.dP, sizeof(double) * C * np);
    add(&cv.flux_vj, sizeof(double) * C * np); add(&cv.flux_ni, sizeof(double) * C * nc);
    add(&cv.row_ptr, sizeof(uint32_t) * (nb + 1)); add(&cv.row_conn, sizeof(uint32_t) * (row_conn.size() + 1));
    add(&ctx->resRelV, D); add(&ctx->resRelN, D);
    add(&ctx->rownorm, sizeof(RowNorm) * (size_t)nb); add(&ctx->norm_out, sizeof(RowNorm));
    add(&ctx->norm_part, sizeof(RowNorm) * NORM_PARTS);
    add(&ctx->flags, sizeof(uint32_t) * 4);
    ctx->defer_cap = std::max(1024, nb / 4);
    add(&ctx->order, sizeof(int) * (size_t)nb); add(&ctx->cost_hist, sizeof(unsigned) * COST_BUCKETS);
    add(&ctx->defer_rec, sizeof(DeferRec) * (size_t)ctx->defer_cap); add(&ctx->defer_count, sizeof(unsigned) * 40);
    add(&ctx->defer_rec2, sizeof(DeferRec) * (size_t)ctx->defer_cap);
    add(&ctx->pe_res, sizeof(PERes) * (size_t)ctx->defer_cap);
    add(&ctx->pre_rec, sizeof(DeferRec) * (size_t)ctx->defer_cap); add(&ctx->pre_res, sizeof(PERes) * (size_t)ctx->defer_cap);
    add(&ctx->pre_flag, (size_t)nb); add(&ctx->adapt_level, sizeof(int) * 4);
    // Newton / time-step control: last Newton iterate, last time step (P, T, S;
    // Ni's is b.lNi), reduction candidates, results
    add(&ctx->nr_lP, D); add(&ctx->nr_lT, D); add(&ctx->nr_lN, D * nc); add(&ctx->nr_lS, D * np);
    add(&ctx->ts_lP, D); add(&ctx->ts_lT, D); add(&ctx->ts_lS, D * np);
    add(&ctx->maxch_partial, (size_t)MAX_CHANGE_BLOCKS * 5 * 16);
    add(&ctx->nr_stats, sizeof(double) * 5); add(&ctx->ts_stats, sizeof(double) * 5);
    add(&ctx->nr_res0, sizeof(double)); add(&ctx->nr_state, sizeof(int)); add(&ctx->nr_dt, sizeof(double) * 2);
    add(&ctx->bmat, sizeof(double) * C * 2 * bsize);
    // the recompute mode's slab scratch, outside the checkpointed state range
    if (recompute) {
        ctx->dsec_slab = std::min(nb, RECOMPUTE_SLAB_CELLS);
        add(&ctx->dsec_scratch, sizeof(double) * (size_t)ctx->dsec_slab * lend);
    }
    add(&ctx->adj_conn, sizeof(double) * C);
    // field transfers go through the staging buffer in chunks; stored
    // dSec_dPri moves in one piece
    size_t staging = recompute ? D * std::max({np * nc, np * np, 5}) : D * lend;
    staging = std::max(staging, sizeof(double) * C * nc);
    staging = std::max(staging, sizeof(double) * lend);
    add(&ctx->staging, staging);
    ctx->staging_bytes = staging;
    size_t total = 0;
    for (auto& s : slots) total += align256(s.bytes);
    if (cudaMalloc(&ctx->arena, total) != cudaSuccess) {
        delete ctx;
        return fail(OCPX_CUDA_ERROR, "cudaMalloc of " + std::to_string(total) + " bytes failed");
    }
    ctx->arena_bytes = total;
    size_t off = 0;
    for (auto& s : slots) { *s.p = ctx->arena + off; off += align256(s.bytes); }
    cudaMemset(ctx->arena, 0, total);
    // the per-cell state occupies one contiguous range of the arena: P .. iters
    ctx->state_off = (size_t)((char*)b.P - ctx->arena);
    ctx->state_bytes = (size_t)((char*)b.iters + align256(sizeof(int32_t) * (size_t)nb * 5) - (char*)b.P);

    auto fail_ctx = [&](ocpx_status s2, const std::string& m) { ocpx_destroy(ctx); return fail(s2, m); };
    {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        ctx->prio_hi = hi;
        if (cudaStreamCreateWithPriority(&ctx->stream2, cudaStreamNonBlocking, hi) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess)
            return fail_ctx(OCPX_CUDA_ERROR, "stream/event creation failed");
    }
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail_ctx(OCPX_CUDA_ERROR, "stream creation failed");
    if (ctx->ncm > 0 && setup_flash_batched(ctx->ncm, ctx->excl_smem) != cudaSuccess)
        return fail_ctx(OCPX_CUDA_ERROR, "flash kernel set-up failed");
    if (cudaMalloc(&ctx->d_model, sizeof(Model)) != cudaSuccess) return fail_ctx(OCPX_CUDA_ERROR, "model alloc failed");
    if (cudaMallocHost(&ctx->h_flags, sizeof(uint32_t) * 4) != cudaSuccess ||
        cudaMallocHost(&ctx->h_norm, sizeof(RowNorm)) != cudaSuccess)
        return fail_ctx(OCPX_CUDA_ERROR, "pinned alloc failed");
    cudaMemcpy(ctx->d_model, &ctx->host_model, sizeof(Model), cudaMemcpyHostToDevice);
    cudaMemcpy((void*)b.v, gd->v, D, cudaMemcpyHostToDevice);
    cudaMemcpy((void*)b.depth, gd->depth, D, cudaMemcpyHostToDevice);
    cudaMemcpy((void*)b.poroInit, gd->poro_init, D, cudaMemcpyHostToDevice);
    if (nconn > 0) {
        cudaMemcpy((void*)cv.bId, gd->conn_b, sizeof(uint32_t) * nconn, cudaMemcpyHostToDevice);
        cudaMemcpy((void*)cv.eId, gd->conn_e, sizeof(uint32_t) * nconn, cudaMemcpyHostToDevice);
        cudaMemcpy((void*)cv.trans, gd->conn_trans, sizeof(double) * nconn, cudaMemcpyHostToDevice);
    }
    cudaMemcpy((void*)cv.row_ptr, row_ptr.data(), sizeof(uint32_t) * (nb + 1), cudaMemcpyHostToDevice);
    if (!row_conn.empty())
        cudaMemcpy((void*)cv.row_conn, row_conn.data(), sizeof(uint32_t) * row_conn.size(), cudaMemcpyHostToDevice);
    ctx->h_row_ptr = std::move(row_ptr);
    ctx->h_row_conn = std::move(row_conn);
    ctx->h_conn_b.assign(gd->conn_b, gd->conn_b + nconn);
    ctx->h_conn_e.assign(gd->conn_e, gd->conn_e + nconn);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail_ctx(OCPX_CUDA_ERROR, std::string("context setup: ") + cudaGetErrorString(e));
    {
        const ocpx_status sst = build_system(ctx, nullptr, nullptr);
        if (sst != OCPX_OK) { const std::string m = g_err; ocpx_destroy(ctx); return fail(sst, m); }
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    ctx->coop_blocks = sms * 4;
    ctx->sms = sms;
    // the fused batched flash: one block of four warps per SM on small grids,
    // where the longest cells set the time (36,000 cells: 15.0 ms per step
    // against 16.8 ms for the tuned two-stream form); more on large ones,
    // where the per-lane work dominates and more warps hide the per-thread
    // frames' memory latency.  At 182 registers a thread two blocks fit on an
    // SM, so the four per SM launched run two at a time, the later blocks
    // finding the work taken (4,000,000 cells: 1,289 ms against 1,484 ms with
    // one block per SM and 1,439 ms two-stream; 304 to 912 blocks all within
    // 0.2 % of each other)
    ctx->fused_blocks = nb < 131072 ? sms : 4 * sms;
    ctx->fused_coop_blocks = -1;
    // a tighter budget on small grids, where the cooperative-only blocks take
    // the over-budget cells
    ctx->flash_budget = nb < 131072 ? 32 : 48;
    *out = ctx;
    return OCPX_OK;
}

void ocpx_destroy(ocpx_ctx* ctx)
{
    if (!ctx) return;
    ctx->drop_graph();
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (char* c : ctx->ckpt)
        if (c) cudaFree(c);
    for (auto& m : ctx->marks) { cudaEventDestroy(m.a); cudaEventDestroy(m.b); }
    for (auto e : ctx->free_events) cudaEventDestroy(e);
    if (ctx->arena) cudaFree(ctx->arena);
    if (ctx->ls_scratch) cudaFree(ctx->ls_scratch);
    if (ctx->split_state) cudaFree(ctx->split_state);
    if (ctx->step_adj) cudaFree(ctx->step_adj);
    if (ctx->sys) cudaFree(ctx->sys);
    if (ctx->wbuf) cudaFree(ctx->wbuf);
    if (ctx->weval) cudaFree(ctx->weval);
    if (ctx->d_model) cudaFree(ctx->d_model);
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->h_norm) cudaFreeHost(ctx->h_norm);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    delete ctx;
}

void* ocpx_stream(ocpx_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
uint64_t ocpx_launch_count(ocpx_ctx* ctx) { return ctx ? ctx->launches : 0; }

ocpx_status ocpx_set_field(ocpx_ctx* ctx, ocpx_field f, const void* host, size_t count)
{
    if (!ctx || !host) return fail(OCPX_INVALID_ARG, "null argument");
    if (f == OCPX_F_DSEC_DPRI && ctx->recompute)
        return fail(OCPX_INVALID_ARG, "dSec_dPri is recomputed, not stored: it cannot be set");
    const FieldInfo fi = ctx->field(f);
    if (!fi.dev || !fi.writable) return fail(OCPX_INVALID_ARG, "field not writable: " + std::to_string((int)f));
    const size_t expect = (size_t)fi.n * fi.width;
    if (count != expect)
        return fail(OCPX_INVALID_ARG, "field " + std::to_string((int)f) + ": expected " + std::to_string(expect) +
                                          " elements, got " + std::to_string(count));
    return ocpx_set_field_range(ctx, f, 0, (size_t)fi.n, host);
}

ocpx_status ocpx_get_field(ocpx_ctx* ctx, ocpx_field f, void* host, size_t count)
{
    if (!ctx || !host) return fail(OCPX_INVALID_ARG, "null argument");
    const FieldInfo fi = ctx->field(f);
    if (!fi.dev) return fail(OCPX_INVALID_ARG, "unknown field " + std::to_string((int)f));
    const size_t expect = (size_t)fi.n * fi.width;
    if (count != expect)
        return fail(OCPX_INVALID_ARG, "field " + std::to_string((int)f) + ": expected " + std::to_string(expect) +
                                          " elements, got " + std::to_string(count));
    return ocpx_get_field_range(ctx, f, 0, (size_t)fi.n, host);
}

}  // extern "C"

namespace {
// entities [first, first + n) of a field between the host (reference layout)
// and the device
ocpx_status field_transfer(ocpx_ctx* ctx, ocpx_field f, size_t first, size_t n, void* host, bool to_device)
{
    if (!ctx || (!host && n)) return fail(OCPX_INVALID_ARG, "null argument");
    if (f == OCPX_F_DSEC_DPRI && ctx->recompute) {
        // recomputed from the state the last flash left (P, T, Ni, phase labels,
        // x_ij, phase mole numbers), chunk by chunk through the staging buffer
        if (to_device) return fail(OCPX_INVALID_ARG, "dSec_dPri is recomputed, not stored: it cannot be set");
        const size_t lend = (size_t)ctx->np * (ctx->nc + 1) * (ctx->nc + 1);
        if (first > (size_t)ctx->nb || n > (size_t)ctx->nb - first)
            return fail(OCPX_INVALID_ARG, "dSec_dPri: range outside the cells");
        const size_t chunk = ctx->staging_bytes / (sizeof(double) * lend);
        for (size_t k = 0; k < n; k += chunk) {
            const size_t m = std::min(chunk, n - k);
            OCPX_CUDA(launch_dsec_cells(ctx->ncm, ctx->d_model, ctx->b, nullptr, (int)(first + k), (int)m,
                                        (double*)ctx->staging, 0, ctx->stream));
            ctx->launches++;
            OCPX_CUDA(cudaMemcpyAsync((double*)host + k * lend, ctx->staging, sizeof(double) * m * lend,
                                      cudaMemcpyDeviceToHost, ctx->stream));
            OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
        }
        return OCPX_OK;
    }
    const FieldInfo fi = ctx->field(f);
    if (!fi.dev) return fail(OCPX_INVALID_ARG, "unknown field " + std::to_string((int)f));
    if (to_device && !fi.writable) return fail(OCPX_INVALID_ARG, "field not writable: " + std::to_string((int)f));
    if (first > (size_t)fi.n || n > (size_t)fi.n - first)
        return fail(OCPX_INVALID_ARG, "field " + std::to_string((int)f) + ": range [" + std::to_string(first) + ", " +
                                          std::to_string(first + n) + ") outside " + std::to_string(fi.n) + " entities");
    if (!n) return OCPX_OK;
    if (to_device) ctx->state_gen++;
    const size_t ebytes = (size_t)fi.width * fi.elem;  // one entity
    const cudaMemcpyKind kind = to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    if (fi.width == 1 || !fi.soa) {
        char* dev = (char*)fi.dev + first * ebytes;
        OCPX_CUDA(cudaMemcpyAsync(to_device ? (void*)dev : host, to_device ? (const void*)host : (const void*)dev,
                                  n * ebytes, kind, ctx->stream));
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
        return OCPX_OK;
    }
    // SoA fields through the staging buffer, as many entities at a time as it holds
    const size_t chunk = ctx->staging_bytes / ebytes;
    for (size_t k = 0; k < n; k += chunk) {
        const size_t m = std::min(chunk, n - k);
        char* h = (char*)host + k * ebytes;
        if (to_device) {
            OCPX_CUDA(cudaMemcpyAsync(ctx->staging, h, m * ebytes, kind, ctx->stream));
            OCPX_CUDA(launch_transpose(fi.dev, ctx->staging, (int)m, fi.width, fi.elem, true, ctx->stream, fi.n,
                                       first + k));
        }
        else {
            OCPX_CUDA(launch_transpose(ctx->staging, fi.dev, (int)m, fi.width, fi.elem, false, ctx->stream, fi.n,
                                       first + k));
            OCPX_CUDA(cudaMemcpyAsync(h, ctx->staging, m * ebytes, kind, ctx->stream));
        }
        ctx->launches++;
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return OCPX_OK;
}
}  // namespace

extern "C" {

ocpx_status ocpx_set_field_range(ocpx_ctx* ctx, ocpx_field f, size_t first, size_t n, const void* host)
{
    return field_transfer(ctx, f, first, n, const_cast<void*>(host), true);
}

ocpx_status ocpx_get_field_range(ocpx_ctx* ctx, ocpx_field f, size_t first, size_t n, void* host)
{
    return field_transfer(ctx, f, first, n, host, false);
}

}  // extern "C"

namespace {

// CheckNi/CheckP + flash + kr/Pc + rock, all asynchronous
ocpx_status enqueue_properties(ocpx_ctx* ctx)
{
    cudaStream_t s = ctx->stream;
    ctx->state_gen++;
    OCPX_CUDA(cudaMemsetAsync(ctx->flags, 0, sizeof(uint32_t) * 4, s));
    int mk = ctx->stage_begin(0);
    OCPX_CUDA(launch_check(ctx->b, ctx->flags, ctx->block_cell, s));
    ctx->stage_end(mk);
    ctx->launches++;
    const int mk_flash = ctx->stage_begin(1);
    if (ctx->host_model.mixture == 1) {
        if (ctx->variant == 1) {
            // cells expensive in their last flash go to the cooperative kernel at
            // once, on a second (high-priority) stream, concurrently with the
            // per-cell kernel; cells that turn out expensive now follow after it
            const bool pre = ctx->predefer > 0;
            // list counts [0] late, [1] pre-deferred; [2], [3] the cooperative kernels' next-slot
            // counters; [4] the persistent per-cell kernel's position counter; [8 + r], [16 + r]
            // the count and position counter of re-budgeting round r; [32..35] the fused kernel's;
            // [36], [37] the split cells' refill and resume position counters
            OCPX_CUDA(cudaMemsetAsync(ctx->defer_count, 0, sizeof(unsigned) * 40, s));
            mk = ctx->stage_begin(9);
            OCPX_CUDA(launch_cost_order(ctx->d_model, ctx->b, ctx->cost_hist, ctx->order, (unsigned)ctx->coop_cells,
                                        pre ? ctx->predefer : (long long)ctx->flash_budget, ctx->adapt_level, s));
            ctx->launches += 3;
            if (pre) {
                const DeferSink sinkA{ctx->pre_rec, ctx->defer_count + 1, ctx->defer_cap};
                OCPX_CUDA(launch_predefer(ctx->d_model, ctx->b, ctx->order, ctx->cost_hist, ctx->predefer,
                                          ctx->adapt_level, sinkA, ctx->pre_flag, s));
                ctx->launches++;
            }
            ctx->stage_end(mk);
            unsigned* const cnt = ctx->defer_count;
            FlashBatch fbA{ctx->flash_budget, ctx->block_cell, ctx->coop_blocks, ctx->defer_cap,
                                 ctx->pre_rec, cnt + 1, ctx->pre_res, nullptr, nullptr, ctx->prio_hi,
                                 ctx->pre_blocks, ctx->excl_smem[0], 0, nullptr, cnt + 3, nullptr, nullptr, 0};
            // with re-budgeting rounds the rounds, not a budget raised to the
            // adaptive level, keep the cooperative list short: the per-cell
            // kernel then starts from the plain budget
            FlashBatch fbB{ctx->flash_budget, ctx->block_cell, ctx->coop_blocks, ctx->defer_cap,
                           ctx->defer_rec, cnt, ctx->pe_res, pre ? ctx->pre_flag : nullptr,
                           ctx->rounds > 0 ? nullptr : ctx->adapt_level, 0, 0, 0, ctx->cell_blocks, cnt + 4, cnt + 2,
                           nullptr, nullptr, 0};
            fbA.post_block = ctx->post_block;
            fbB.post_block = ctx->post_block;
            if (ctx->fused_blocks > 0) {
                // one persistent kernel on this stream: pre-deferred cells first, then
                // the cost-ordered cells, then the over-budget cells as they are published
                OCPX_CUDA(cudaMemsetAsync(ctx->defer_rec, 0, sizeof(DeferRec) * (size_t)ctx->defer_cap, s));
                FlashBatch ff = fbB;
                ff.rin = pre ? ctx->pre_rec : nullptr;
                ff.rin_count = pre ? cnt + 1 : nullptr;
                ff.pe_pre = ctx->pre_res;
                ff.cell_blocks = ctx->fused_blocks;
                ff.cell_next = cnt + 32;
                ff.excl_blocks = ctx->fused_excl && ctx->fused_blocks <= ctx->sms ? 1 : 0;
                ff.excl_smem_fused = ctx->excl_smem[1];
                const int coop_only = fused_coop_blocks(ctx);
                if (coop_only >= ctx->fused_blocks)
                    return fail(OCPX_INVALID_ARG, "FUSED_COOP_BLOCKS must be smaller than FUSED_BLOCKS");
                // the cooperative-only blocks wait for the others, so all must be
                // resident at once; the form is kept to one block per SM (a
                // cooperative launch of two blocks per SM without the SM-exclusive
                // reservation once faulted, for a cause not found)
                if (coop_only > 0 && (ctx->fused_blocks > ctx->sms || ctx->excl_smem[2] < 1))
                    return fail(OCPX_INVALID_ARG, "FUSED_COOP_BLOCKS needs all FUSED_BLOCKS resident at once, one "
                                                  "block per SM (at most " + std::to_string(ctx->sms) + " here)");
                ff.coop_only_blocks = coop_only;
                ff.watchdog = ctx->flags + 1;
                mk = ctx->stage_begin(10);
                if (ctx->split_refill && ctx->split_state) {
                    // the split cells (the order's first class) first: their first
                    // loop with lane refill, then the rest of their flash; the fused
                    // kernel then starts at the order's second class
                    const unsigned* n_split = ctx->cost_hist + 63;
                    const uint8_t* pf = pre ? ctx->pre_flag : nullptr;
                    OCPX_CUDA(launch_split_refill(ctx->ncm, ctx->d_model, ctx->b, ctx->order, n_split, pf,
                                                  ctx->split_state, cnt + 36, ctx->fused_blocks, s));
                    OCPX_CUDA(launch_split_resume(ctx->ncm, ctx->d_model, ctx->b, ctx->order, n_split, pf,
                                                  ctx->split_state, cnt + 37, ctx->fused_blocks, ff, s));
                    OCPX_CUDA(cudaMemcpyAsync(cnt + 33, n_split, sizeof(unsigned), cudaMemcpyDeviceToDevice, s));
                    ctx->launches += 2;
                }
                OCPX_CUDA(launch_flash_batched(ctx->ncm, ctx->d_model, ctx->b, ctx->order, ff, 4, s));
                ctx->stage_end(mk);
                ctx->late_count = 0;
                // both lists' cells finished by one launch: each thread's chain
                // is long, so two launches in a row would take twice as long
                mk = ctx->stage_begin(12);
                FlashBatch fp = fbB;
                if (pre) {
                    fp.rec2 = ctx->pre_rec;
                    fp.count2 = cnt + 1;
                    fp.pe2 = ctx->pre_res;
                }
                OCPX_CUDA(launch_flash_batched(ctx->ncm, ctx->d_model, ctx->b, ctx->order, fp, 2, s));
                ctx->stage_end(mk);
                ctx->launches += 2;
            }
            else {
                if (pre) {
                    // the pre-deferred cells' equilibrium and FlashDer on the second
                    // stream; the per-cell kernel skips them, so nothing else
                    // touches their state until the join
                    OCPX_CUDA(cudaEventRecord(ctx->ev_fork, s));
                    OCPX_CUDA(cudaStreamWaitEvent(ctx->stream2, ctx->ev_fork, 0));
                    mk = ctx->stage_begin(11, ctx->stream2);
                    OCPX_CUDA(launch_flash_batched(ctx->ncm, ctx->d_model, ctx->b, ctx->order, fbA, 1, ctx->stream2));
                    OCPX_CUDA(launch_flash_batched(ctx->ncm, ctx->d_model, ctx->b, ctx->order, fbA, 2, ctx->stream2));
                    ctx->stage_end(mk);
                    OCPX_CUDA(cudaEventRecord(ctx->ev_join, ctx->stream2));
                    ctx->launches += 2;
                }
                mk = ctx->stage_begin(10);
                OCPX_CUDA(launch_flash_batched(ctx->ncm, ctx->d_model, ctx->b, ctx->order, fbB, 0, s));
                // re-budgeting rounds: list r-1 -> list r with budget x G^r, alternating
                // between the two late lists; counts cnt[8 + r], position counters cnt[16 + r]
                long long mult = 1;
                for (int r = 1; r <= ctx->rounds; r++) {
                    mult *= ctx->round_growth;
                    FlashBatch fr = fbB;
                    fr.rin = fbB.rec;
                    fr.rin_count = fbB.count;
                    fr.rec = (r & 1) ? ctx->defer_rec2 : ctx->defer_rec;
                    fr.count = cnt + 8 + r;
                    fr.cell_next = cnt + 16 + r;
                    fr.mult = mult;
                    OCPX_CUDA(launch_flash_batched(ctx->ncm, ctx->d_model, ctx->b, ctx->order, fr, 3, s));
                    ctx->launches++;
                    fbB.rec = fr.rec;
                    fbB.count = fr.count;
                }
                ctx->late_count = (int)(fbB.count - cnt);
                ctx->stage_end(mk);
                mk = ctx->stage_begin(13);
                OCPX_CUDA(launch_flash_batched(ctx->ncm, ctx->d_model, ctx->b, ctx->order, fbB, 1, s));
                ctx->stage_end(mk);
                ctx->launches += 2;
                mk = ctx->stage_begin(12);
                OCPX_CUDA(launch_flash_batched(ctx->ncm, ctx->d_model, ctx->b, ctx->order, fbB, 2, s));
                ctx->launches++;
                ctx->stage_end(mk);
                if (pre) OCPX_CUDA(cudaStreamWaitEvent(s, ctx->ev_join, 0));
            }
        }
        else {
            OCPX_CUDA(launch_flash_comp(ctx->ncm, ctx->d_model, ctx->b, ctx->block_cell, s));
            ctx->launches++;
        }
    }
    else {
        OCPX_CUDA(launch_flash_bo(ctx->d_model, ctx->b, ctx->block_cell, s));
        ctx->launches++;
    }
    ctx->stage_end(mk_flash);
    mk = ctx->stage_begin(2);
    OCPX_CUDA(launch_krpc_rock(ctx->d_model, ctx->b, ctx->block_cell, s));
    ctx->stage_end(mk);
    ctx->launches++;
    mk = ctx->stage_begin(3);
    OCPX_CUDA(launch_report(ctx->b, ctx->flags + 1, ctx->block_cell, s));
    ctx->stage_end(mk);
    ctx->launches++;
    return OCPX_OK;
}

ocpx_status enqueue_calres(ocpx_ctx* ctx, double dt)
{
    cudaStream_t s = ctx->stream;
    ctx->last_dt = dt;
    int mk = ctx->stage_begin(4);
    OCPX_CUDA(launch_conn_flux(ctx->d_model, ctx->b, ctx->cv, ctx->block_conn, s));
    ctx->stage_end(mk);
    mk = ctx->stage_begin(5);
    const bool wells = ctx->ws.nw > 0;
    OCPX_CUDA(launch_residual(ctx->b, ctx->cv, dt, ctx->res, ctx->resRelV, ctx->resRelN, ctx->rownorm,
                              wells ? nullptr : ctx->norm_out, ctx->norm_part, ctx->block_cell, s));
    if (wells) {
        // CalResFIM of every well after the bulk rows, then the norms
        if (ctx->recompute) {
            OCPX_CUDA(launch_dsec_cells(ctx->ncm, ctx->d_model, ctx->b, ctx->ws.pc_cell, 0, ctx->ws.npc, ctx->ws.dsec,
                                        0, s));
            ctx->launches++;
        }
        OCPX_CUDA(launch_wells_res(ctx->b, ctx->ws, dt, ctx->res, ctx->resRelV, ctx->resRelN, ctx->rownorm, s));
        OCPX_CUDA(launch_norm_reduce(ctx->rownorm, ctx->nbI, ctx->norm_out, ctx->norm_part, s));
        ctx->launches += 3;
    }
    ctx->stage_end(mk);
    ctx->launches += 3;
    ctx->res_gen = ctx->state_gen;
    return OCPX_OK;
}

ocpx_status enqueue_assemble(ocpx_ctx* ctx, double dt)
{
    cudaStream_t s = ctx->stream;
    int mk = ctx->stage_begin(6);
    if (ctx->recompute) {
        // slab by slab: the slab's dSec_dPri into the scratch, then the side
        // blocks of the slab's cells
        for (int c0 = 0; c0 < ctx->nb; c0 += ctx->dsec_slab) {
            const int n = std::min(ctx->dsec_slab, ctx->nb - c0);
            OCPX_CUDA(launch_dsec_slab(ctx->ncm, ctx->d_model, ctx->b, c0, n, ctx->dsec_scratch, (size_t)n, s));
            OCPX_CUDA(launch_jac_side(ctx->nct_cap, ctx->d_model, ctx->b, ctx->cv, dt, c0, ctx->h_row_ptr[c0],
                                      ctx->h_row_ptr[c0 + n], ctx->dsec_scratch, (size_t)n, ctx->bmat,
                                      ctx->block_conn, s));
            ctx->launches += 2;
        }
        ctx->launches--;  // counted once below
    }
    else {
        OCPX_CUDA(launch_jac_conn(ctx->nct_cap, ctx->d_model, ctx->b, ctx->cv, dt, ctx->bmat, ctx->block_conn, s));
    }
    ctx->stage_end(mk);
    mk = ctx->stage_begin(7);
    OCPX_CUDA(launch_jac_rows(ctx->b, ctx->cv, ctx->bmat, ctx->jac_rowptr, ctx->jac_val, ctx->block_cell, s));
    if (ctx->ws.nw > 0) {
        // AssembleMatWells after AssembleMatBulks, from the terms of the last ocpx_calres
        OCPX_CUDA(launch_wells_jac(ctx->b, ctx->ws, dt, ctx->jac_rowptr, ctx->jac_val, s));
        ctx->launches += 2;
    }
    ctx->stage_end(mk);
    ctx->launches += 2;
    return OCPX_OK;
}

ocpx_status report_from_flags(ocpx_ctx* ctx, ocpx_report* rep)
{
    OCPX_CUDA(cudaMemcpyAsync(ctx->h_flags, ctx->flags, sizeof(uint32_t) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    const uint32_t chk = ctx->h_flags[0];
    if (rep) {
        rep->status_or = ctx->h_flags[1] | chk;
        rep->n_two_phase = (int)ctx->h_flags[2];
        rep->n_flagged = (int)ctx->h_flags[3];
    }
    if (chk & ST_NEG_NI) return fail(OCPX_NEGATIVE_NI, "negative moles beyond the clamp rule (Bulk::CheckNi)");
    if (chk & ST_NEG_P) return fail(OCPX_NEGATIVE_P, "negative pressure (Bulk::CheckP)");
    const uint32_t f = ctx->h_flags[1];
    if (f & ST_NONFINITE) return fail(OCPX_NONFINITE, "non-finite flash result");
    if (f & ST_ITER_CAP) return fail(OCPX_WATCHDOG, "flash iteration cap reached");
    return OCPX_OK;
}

}  // namespace

extern "C" {

ocpx_status ocpx_update_properties(ocpx_ctx* ctx, ocpx_report* rep)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    ocpx_status st = enqueue_properties(ctx);
    if (st != OCPX_OK) return st;
    return report_from_flags(ctx, rep);
}

ocpx_status ocpx_calres(ocpx_ctx* ctx, double dt, ocpx_norms* norms)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    ocpx_status st = enqueue_calres(ctx, dt);
    if (st != OCPX_OK) return st;
    if (norms) {
        OCPX_CUDA(cudaMemcpyAsync(ctx->h_norm, ctx->norm_out, sizeof(RowNorm), cudaMemcpyDeviceToHost, ctx->stream));
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
        norms->maxRelRes_V = ctx->h_norm->maxV;
        norms->maxId_V = ctx->h_norm->idV;
        norms->maxRelRes_N = ctx->h_norm->maxN;
        norms->maxId_N = ctx->h_norm->idN;
    }
    return OCPX_OK;
}

ocpx_status ocpx_assemble(ocpx_ctx* ctx, double dt)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    return enqueue_assemble(ctx, dt);
}

namespace {
// checks shared by the two forms of the solve; allocates the work space on
// the first call, which must not be inside a stream capture
ocpx_status linsolve_prepare(ocpx_ctx* ctx, double tol, int maxit)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    if (!(tol > 0) || maxit < 1) return fail(OCPX_INVALID_ARG, "tol must be > 0 and maxit >= 1");
    if (ctx->nbI < ctx->nb) return fail(OCPX_INVALID_ARG, "the device solve needs a single domain (no ghost cells)");
    if (!ctx->ls_scratch) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        OCPX_CUDA(cudaStreamIsCapturing(ctx->stream, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return fail(OCPX_INVALID_ARG, "the solver's work space is allocated by the first solve, outside a capture");
        OCPX_CUDA(cudaMalloc(&ctx->ls_scratch, sizeof(double) * linsolve_scratch_doubles(ctx->nrow, ctx->nc + 1)));
    }
    return OCPX_OK;
}
}  // namespace

ocpx_status ocpx_linsolve_async(ocpx_ctx* ctx, double tol, int maxit)
{
    const ocpx_status st = linsolve_prepare(ctx, tol, maxit);
    if (st != OCPX_OK) return st;
    OCPX_CUDA(linsolve_async(ctx->jac_rowptr, ctx->jac_col, ctx->jac_val, ctx->nrow, ctx->nc + 1, ctx->res, ctx->u,
                             ctx->ls_scratch, tol, maxit, 10, &ctx->launches, ctx->stream));
    return OCPX_OK;
}

ocpx_status ocpx_linsolve_report(ocpx_ctx* ctx, ocpx_solve_report* rep)
{
    if (!ctx || !rep) return fail(OCPX_INVALID_ARG, "null argument");
    if (!ctx->ls_scratch) return fail(OCPX_INVALID_ARG, "no solve has run on this context");
    LinsolveResult r{};
    OCPX_CUDA(linsolve_read(ctx->ls_scratch, ctx->nrow, ctx->nc + 1, &r, ctx->stream));
    *rep = ocpx_solve_report{r.iterations, r.relres, r.converged, r.breakdown};
    return OCPX_OK;
}

ocpx_status ocpx_linsolve(ocpx_ctx* ctx, double tol, int maxit, double* u_host, ocpx_solve_report* rep)
{
    const ocpx_status st = linsolve_prepare(ctx, tol, maxit);
    if (st != OCPX_OK) return st;
    const int dim = ctx->nc + 1;
    LinsolveResult r{};
    OCPX_CUDA(linsolve(ctx->jac_rowptr, ctx->jac_col, ctx->jac_val, ctx->nrow, dim, ctx->res, ctx->u,
                       ctx->ls_scratch, tol, maxit, 10, &r, &ctx->launches, ctx->stream));
    if (u_host) {
        OCPX_CUDA(cudaMemcpyAsync(u_host, ctx->u, sizeof(double) * ctx->nv(), cudaMemcpyDeviceToHost, ctx->stream));
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    if (rep) *rep = ocpx_solve_report{r.iterations, r.relres, r.converged, r.breakdown};
    return OCPX_OK;
}

namespace {
// GetSolution of the cells, with dSec_dPri stored or recomputed
cudaError_t newton_update(ocpx_ctx* ctx, double dSmax)
{
    if (ctx->recompute) return launch_newton_update_recompute(ctx->ncm, ctx->d_model, ctx->b, ctx->u, dSmax, ctx->stream);
    return launch_newton_update(ctx->b, ctx->u, dSmax, ctx->block_cell, ctx->stream);
}
}  // namespace

ocpx_status ocpx_newton_update_device(ocpx_ctx* ctx, double dSmax)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    const int mk = ctx->stage_begin(8);
    OCPX_CUDA(newton_update(ctx, dSmax));
    OCPX_CUDA(launch_wells_update(ctx->b, ctx->ws, ctx->u, ctx->stream));
    ctx->stage_end(mk);
    ctx->launches += ctx->ws.nw > 0 ? 2 : 1;
    ctx->state_gen++;
    return OCPX_OK;
}

ocpx_status ocpx_newton_update(ocpx_ctx* ctx, const double* u_host, double dSmax)
{
    if (!ctx || !u_host) return fail(OCPX_INVALID_ARG, "null argument");
    const size_t bytes = sizeof(double) * ctx->nv();
    OCPX_CUDA(cudaMemcpyAsync(ctx->u, u_host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    const int mk = ctx->stage_begin(8);
    OCPX_CUDA(newton_update(ctx, dSmax));
    OCPX_CUDA(launch_wells_update(ctx->b, ctx->ws, ctx->u, ctx->stream));
    ctx->stage_end(mk);
    ctx->launches += ctx->ws.nw > 0 ? 2 : 1;
    ctx->state_gen++;
    return OCPX_OK;
}

}  // extern "C"

namespace {

// the adjoint products of the step (ocpx_set_adjoint_seed), after its Jacobian
ocpx_status enqueue_step_adjoint(ocpx_ctx* ctx)
{
    cudaStream_t s = ctx->stream;
    const size_t nv = ctx->nv();
    const double* lam = ctx->step_adj;
    const int mk = ctx->stage_begin(14);
    OCPX_CUDA(launch_jt_lambda(ctx->b, ctx->cv, ctx->jac_rowptr, ctx->jac_val, ctx->jac_slot, lam,
                               ctx->step_adj + nv, ctx->block_cell, s));
    if (ctx->ws.nw > 0) {
        OCPX_CUDA(launch_wells_jt(ctx->b, ctx->ws, ctx->jac_rowptr, ctx->jac_val, lam, ctx->step_adj + nv, s));
        ctx->launches += 2;
    }
    OCPX_CUDA(launch_vjp_poro(ctx->d_model, ctx->b, lam, ctx->step_adj + 2 * nv, ctx->block_cell, s));
    ctx->launches += 2;
    if (ctx->nconn) {
        OCPX_CUDA(launch_vjp_trans(ctx->b, ctx->cv, ctx->last_dt, lam, ctx->step_adj + 2 * nv + ctx->nb,
                                   ctx->block_conn, s));
        ctx->launches++;
    }
    ctx->stage_end(mk);
    return OCPX_OK;
}

ocpx_status enqueue_step_kernels(ocpx_ctx* ctx, double dt)
{
    ocpx_status st;
    if ((st = enqueue_properties(ctx)) != OCPX_OK) return st;
    if ((st = enqueue_calres(ctx, dt)) != OCPX_OK) return st;
    if ((st = enqueue_assemble(ctx, dt)) != OCPX_OK) return st;
    return ctx->adj_in_step ? enqueue_step_adjoint(ctx) : OCPX_OK;
}

// Capture the step into a CUDA graph (batched variant).  The graph holds no
// host work, so one launch replays every kernel and memset of the step.
ocpx_status capture_step(ocpx_ctx* ctx, double dt)
{
    ctx->drop_graph();
    const uint64_t l0 = ctx->launches;
    OCPX_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const ocpx_status st = enqueue_step_kernels(ctx, dt);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (st != OCPX_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return fail(OCPX_CUDA_ERROR, std::string("graph capture: ") + cudaGetErrorString(e));
    const cudaError_t ei = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        ctx->graph_exec = nullptr;
        return fail(OCPX_CUDA_ERROR, std::string("graph instantiate: ") + cudaGetErrorString(ei));
    }
    ctx->graph_dt = dt;
    ctx->graph_launches = ctx->launches - l0;
    ctx->launches = l0;
    return OCPX_OK;
}

}  // namespace

extern "C" {

ocpx_status ocpx_enqueue_step(ocpx_ctx* ctx, double dt)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    // stage profiling records events between the kernels: run those steps eagerly
    if (ctx->variant != 1 || ctx->prof) return enqueue_step_kernels(ctx, dt);
    if (!ctx->graph_exec || ctx->graph_dt != dt) {
        const ocpx_status st = capture_step(ctx, dt);
        if (st != OCPX_OK) return st;
    }
    OCPX_CUDA(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    ctx->launches += ctx->graph_launches;
    return OCPX_OK;
}

ocpx_status ocpx_step_report(ocpx_ctx* ctx, ocpx_report* rep)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    return report_from_flags(ctx, rep);
}

ocpx_status ocpx_profile_enable(ocpx_ctx* ctx, int enable)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->prof = enable != 0;
    for (auto& m : ctx->marks) { ctx->free_events.push_back(m.a); ctx->free_events.push_back(m.b); }
    ctx->marks.clear();
    for (int s = 0; s < OCPX_STAGE_COUNT; s++) { ctx->prof_ms[s] = 0; ctx->prof_n[s] = 0; }
    return OCPX_OK;
}

ocpx_status ocpx_profile_read(ocpx_ctx* ctx, double* ms, uint64_t* launches)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    for (auto& m : ctx->marks) {
        float t = 0;
        OCPX_CUDA(cudaEventElapsedTime(&t, m.a, m.b));
        ctx->prof_ms[m.stage] += t;
        ctx->prof_n[m.stage]++;
        ctx->free_events.push_back(m.a);
        ctx->free_events.push_back(m.b);
    }
    ctx->marks.clear();
    for (int s = 0; s < OCPX_STAGE_COUNT; s++) {
        if (ms) ms[s] = ctx->prof_ms[s];
        if (launches) launches[s] = ctx->prof_n[s];
    }
    return OCPX_OK;
}

ocpx_status ocpx_update_last_step(ocpx_ctx* ctx)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    const size_t D = sizeof(double) * (size_t)ctx->nb;
    OCPX_CUDA(cudaMemcpyAsync(ctx->b.lNi, ctx->b.Ni, D * ctx->nc, cudaMemcpyDeviceToDevice, ctx->stream));
    // lP, lT, lS of BulkVarSet, read by CalMaxChangeTime and OCPNRsuite::InitStep
    OCPX_CUDA(cudaMemcpyAsync(ctx->ts_lP, ctx->b.P, D, cudaMemcpyDeviceToDevice, ctx->stream));
    OCPX_CUDA(cudaMemcpyAsync(ctx->ts_lT, ctx->b.T, D, cudaMemcpyDeviceToDevice, ctx->stream));
    OCPX_CUDA(cudaMemcpyAsync(ctx->ts_lS, ctx->b.S, D * ctx->np, cudaMemcpyDeviceToDevice, ctx->stream));
    return OCPX_OK;
}

ocpx_status ocpx_nr_init_step(ocpx_ctx* ctx)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    const size_t D = sizeof(double) * (size_t)ctx->nb;
    cudaStream_t s = ctx->stream;
    OCPX_CUDA(cudaMemcpyAsync(ctx->nr_lP, ctx->ts_lP, D, cudaMemcpyDeviceToDevice, s));
    OCPX_CUDA(cudaMemcpyAsync(ctx->nr_lT, ctx->ts_lT, D, cudaMemcpyDeviceToDevice, s));
    OCPX_CUDA(cudaMemcpyAsync(ctx->nr_lN, ctx->b.lNi, D * ctx->nc, cudaMemcpyDeviceToDevice, s));
    OCPX_CUDA(cudaMemcpyAsync(ctx->nr_lS, ctx->ts_lS, D * ctx->np, cudaMemcpyDeviceToDevice, s));
    OCPX_CUDA(cudaMemcpyAsync(ctx->nr_res0, &ctx->norm_out->maxV, sizeof(double), cudaMemcpyDeviceToDevice, s));
    return OCPX_OK;
}

namespace {
ocpx_status read_change(ocpx_ctx* ctx, const double* dev, ocpx_change_max* out)
{
    if (!out) return OCPX_OK;
    double v[5];
    OCPX_CUDA(cudaMemcpyAsync(v, dev, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = ocpx_change_max{v[0], v[1], v[2], v[3], v[4]};
    return OCPX_OK;
}
}  // namespace

ocpx_status ocpx_nr_max_change(ocpx_ctx* ctx, ocpx_change_max* out)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    OCPX_CUDA(launch_max_change(0, ctx->b, ctx->nr_lP, ctx->nr_lT, ctx->nr_lN, ctx->nr_lS, ctx->maxch_partial,
                                ctx->nr_stats, ctx->stream));
    ctx->launches += 2;
    return read_change(ctx, ctx->nr_stats, out);
}

ocpx_status ocpx_step_max_change(ocpx_ctx* ctx, ocpx_change_max* out)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    OCPX_CUDA(launch_max_change(1, ctx->b, ctx->ts_lP, ctx->ts_lT, nullptr, ctx->ts_lS, ctx->maxch_partial,
                                ctx->ts_stats, ctx->stream));
    ctx->launches += 2;
    return read_change(ctx, ctx->ts_stats, out);
}

ocpx_status ocpx_nr_check_converge(ocpx_ctx* ctx, const ocpx_nr_control* c, int* state)
{
    if (!ctx || !c) return fail(OCPX_INVALID_ARG, "null argument");
    OCPX_CUDA(launch_nr_converge(*c, ctx->nr_stats, ctx->norm_out, ctx->nr_res0,
                                 ctx->ws.nw > 0 ? ctx->ws.maxrel : nullptr, ctx->nr_state, ctx->stream));
    ctx->launches++;
    if (state) {
        OCPX_CUDA(cudaMemcpyAsync(state, ctx->nr_state, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return OCPX_OK;
}

ocpx_status ocpx_next_time_step(ocpx_ctx* ctx, const ocpx_nr_control* c, double* next_dt, double* predict_dt)
{
    if (!ctx || !c) return fail(OCPX_INVALID_ARG, "null argument");
    OCPX_CUDA(launch_next_dt(*c, ctx->ts_stats, ctx->nr_dt, ctx->stream));
    ctx->launches++;
    if (next_dt || predict_dt) {
        double v[2];
        OCPX_CUDA(cudaMemcpyAsync(v, ctx->nr_dt, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
        if (next_dt) *next_dt = v[0];
        if (predict_dt) *predict_dt = v[1];
    }
    return OCPX_OK;
}

}  // extern "C"

namespace {
ocpx_status check_wells(const ocpx_ctx* ctx, int nwell, const ocpx_well* wells)
{
    if (nwell < 0 || (nwell > 0 && !wells)) return fail(OCPX_INVALID_ARG, "null argument");
    if (ctx->np != 3 || ctx->nc + 1 > NCT_MAX + 1) return fail(OCPX_INVALID_ARG, "wells need three phases");
    for (int w = 0; w < nwell; w++) {
        const ocpx_well& W = wells[w];
        if ((W.type != 0 && W.type != 1) || (W.mode != 0 && W.mode != 1) || W.nperf < 0)
            return fail(OCPX_INVALID_ARG, "well " + std::to_string(w) + ": type, mode or perforation count");
        if (W.nperf > 0 && (!W.cell || !W.WI || !W.dG || (W.type == 0 && !W.xi_inj)))
            return fail(OCPX_INVALID_ARG, "well " + std::to_string(w) + ": missing perforation data");
        if ((W.type == 0 && !W.inj_zi) || (W.mode == 1 && (!W.factor || W.tar_rate == 0.0)))
            return fail(OCPX_INVALID_ARG, "well " + std::to_string(w) + ": missing injection or rate data");
        for (int q = 0; q < W.nperf; q++)
            if (W.cell[q] < 0 || W.cell[q] >= ctx->nbI)
                return fail(OCPX_INVALID_ARG, "well " + std::to_string(w) + ": perforated cell out of range "
                                              "(or a ghost cell)");
    }
    return OCPX_OK;
}
}  // namespace

extern "C" {

ocpx_status ocpx_set_wells(ocpx_ctx* ctx, int nwell, const ocpx_well* wells)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    ocpx_status st = check_wells(ctx, nwell, wells);
    if (st != OCPX_OK) return st;
    if (nwell > 0 && ctx->nbI < ctx->nb) return fail(OCPX_INVALID_ARG, "wells in the step need a single domain");
    const int nc = ctx->nc, ncol = nc + 1;
    const size_t bs = (size_t)ncol * ncol;
    std::vector<int> cells, nperf;
    for (int w = 0; w < nwell; w++) {
        nperf.push_back(wells[w].nperf);
        for (int q = 0; q < wells[w].nperf; q++) cells.push_back(wells[w].cell[q]);
    }
    const bool same = cells == ctx->well_cells && nperf == ctx->well_nperf && (nwell == 0) == (ctx->wbuf == nullptr);
    if (!same) {
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
        if (ctx->wbuf) cudaFree(ctx->wbuf);
        ctx->wbuf = nullptr;
        ctx->wbuf_bytes = 0;
        ctx->ws = WellSys{};
        ctx->well_cells = cells;
        ctx->well_nperf = nperf;
        // the residual, update and adjoint vectors grow by the wells' rows
        if (ctx->step_adj) cudaFree(ctx->step_adj);
        ctx->step_adj = nullptr;
        ctx->adj_in_step = false;
        st = build_system(ctx, &ctx->h_slot_bw, &ctx->h_slot_wb);
        if (st != OCPX_OK) return st;
        ctx->res_gen = 0;
    }
    if (nwell == 0) return OCPX_OK;
    const int np_ = (int)cells.size();
    std::vector<WellDev> wd(nwell);
    std::vector<double> bhp(nwell), zi((size_t)nwell * nc, 0.0), fac((size_t)nwell * nc, 0.0);
    std::vector<WellPerf> perf;
    int p0 = 0;
    for (int w = 0; w < nwell; w++) {
        const ocpx_well& W = wells[w];
        wd[w] = WellDev{W.type, W.mode, p0, p0 + W.nperf, W.tar_bhp, W.tar_rate};
        bhp[w] = W.bhp;
        for (int i = 0; i < nc; i++) {
            if (W.inj_zi) zi[(size_t)w * nc + i] = W.inj_zi[i];
            if (W.factor) fac[(size_t)w * nc + i] = W.factor[i];
        }
        for (int q = 0; q < W.nperf; q++)
            perf.push_back(WellPerf{W.cell[q], w, W.type, W.mode, W.bhp, W.WI[q], W.dG[q],
                                    W.type == 0 ? W.xi_inj[q] : 0.0});
        p0 += W.nperf;
    }
    // perforations grouped by cell, each group in well then perforation order
    std::vector<int> order(np_);
    for (int q = 0; q < np_; q++) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cells[a] < cells[b]; });
    std::vector<int> pc_cell, pc_start;
    for (int k = 0; k < np_; k++)
        if (k == 0 || cells[order[k]] != cells[order[k - 1]]) {
            pc_cell.push_back(cells[order[k]]);
            pc_start.push_back(k);
        }
    pc_start.push_back(np_);
    const int npc = (int)pc_cell.size();
    // one buffer: inputs, the bhp with its two checkpoint slots, then the
    // per-perforation terms
    size_t off = 0;
    auto at = [&](size_t bytes) { const size_t o = off; off += align256(bytes ? bytes : 1); return o; };
    const size_t o_wd = at(sizeof(WellDev) * nwell), o_bhp = at(sizeof(double) * 3 * nwell);
    const size_t o_zi = at(sizeof(double) * zi.size()), o_fac = at(sizeof(double) * fac.size());
    const size_t o_perf = at(sizeof(WellPerf) * np_), o_sbw = at(sizeof(uint32_t) * np_);
    const size_t o_swb = at(sizeof(uint32_t) * np_), o_pcc = at(sizeof(int) * npc);
    const size_t o_pcs = at(sizeof(int) * (npc + 1)), o_pcp = at(sizeof(int) * np_);
    const size_t o_qi = at(sizeof(double) * np_ * nc), o_dqb = at(sizeof(double) * np_ * ncol);
    const size_t o_dqw = at(sizeof(double) * np_ * nc), o_S = at(sizeof(double) * np_ * bs);
    const size_t o_wrel = at(sizeof(double) * nwell), o_max = at(sizeof(double));
    const size_t o_ppc = at(sizeof(int) * np_);
    const size_t o_dsec = ctx->recompute ? at(sizeof(double) * (size_t)npc * ctx->np * bs) : 0;
    std::vector<int> perf_pc(np_);
    for (int g = 0; g < npc; g++)
        for (int k = pc_start[g]; k < pc_start[g + 1]; k++) perf_pc[order[k]] = g;
    if (!ctx->wbuf) {
        OCPX_CUDA(cudaMalloc(&ctx->wbuf, off));
        ctx->wbuf_bytes = off;
        // on the context's stream: a plain cudaMemset runs on the legacy
        // stream, which the context's non-blocking stream does not wait for,
        // and could clear the copies below after they land
        OCPX_CUDA(cudaMemsetAsync(ctx->wbuf, 0, off, ctx->stream));
    }
    char* B = ctx->wbuf;
    WellSys& ws = ctx->ws;
    ws.nw = nwell;
    ws.nperf = np_;
    ws.npc = npc;
    ws.well = (const WellDev*)(B + o_wd);
    ws.bhp = (double*)(B + o_bhp);
    ws.zi = (const double*)(B + o_zi);
    ws.factor = (const double*)(B + o_fac);
    ws.perf = (const WellPerf*)(B + o_perf);
    ws.slot_bw = (const uint32_t*)(B + o_sbw);
    ws.slot_wb = (const uint32_t*)(B + o_swb);
    ws.pc_cell = (const int*)(B + o_pcc);
    ws.pc_start = (const int*)(B + o_pcs);
    ws.pc_perf = (const int*)(B + o_pcp);
    ws.qi = (double*)(B + o_qi);
    ws.dqb = (double*)(B + o_dqb);
    ws.dqw = (double*)(B + o_dqw);
    ws.S = (double*)(B + o_S);
    ws.wrel = (double*)(B + o_wrel);
    ws.maxrel = (double*)(B + o_max);
    ws.perf_pc = (const int*)(B + o_ppc);
    ws.dsec = ctx->recompute ? (double*)(B + o_dsec) : nullptr;
    cudaStream_t s = ctx->stream;
    OCPX_CUDA(cudaMemcpyAsync(B + o_wd, wd.data(), sizeof(WellDev) * nwell, cudaMemcpyHostToDevice, s));
    OCPX_CUDA(cudaMemcpyAsync(B + o_bhp, bhp.data(), sizeof(double) * nwell, cudaMemcpyHostToDevice, s));
    OCPX_CUDA(cudaMemcpyAsync(B + o_zi, zi.data(), sizeof(double) * zi.size(), cudaMemcpyHostToDevice, s));
    OCPX_CUDA(cudaMemcpyAsync(B + o_fac, fac.data(), sizeof(double) * fac.size(), cudaMemcpyHostToDevice, s));
    if (np_ > 0) {
        OCPX_CUDA(cudaMemcpyAsync(B + o_perf, perf.data(), sizeof(WellPerf) * np_, cudaMemcpyHostToDevice, s));
        OCPX_CUDA(cudaMemcpyAsync(B + o_sbw, ctx->h_slot_bw.data(), sizeof(uint32_t) * np_, cudaMemcpyHostToDevice, s));
        OCPX_CUDA(cudaMemcpyAsync(B + o_swb, ctx->h_slot_wb.data(), sizeof(uint32_t) * np_, cudaMemcpyHostToDevice, s));
        OCPX_CUDA(cudaMemcpyAsync(B + o_pcc, pc_cell.data(), sizeof(int) * npc, cudaMemcpyHostToDevice, s));
        OCPX_CUDA(cudaMemcpyAsync(B + o_pcs, pc_start.data(), sizeof(int) * (npc + 1), cudaMemcpyHostToDevice, s));
        OCPX_CUDA(cudaMemcpyAsync(B + o_pcp, order.data(), sizeof(int) * np_, cudaMemcpyHostToDevice, s));
        OCPX_CUDA(cudaMemcpyAsync(B + o_ppc, perf_pc.data(), sizeof(int) * np_, cudaMemcpyHostToDevice, s));
    }
    OCPX_CUDA(cudaStreamSynchronize(s));
    ctx->state_gen++;
    return OCPX_OK;
}

ocpx_status ocpx_get_wells(ocpx_ctx* ctx, double* bhp, double* max_rel)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    if (ctx->ws.nw == 0) return fail(OCPX_INVALID_ARG, "no wells are set (ocpx_set_wells)");
    if (bhp)
        OCPX_CUDA(cudaMemcpyAsync(bhp, ctx->ws.bhp, sizeof(double) * ctx->ws.nw, cudaMemcpyDeviceToHost, ctx->stream));
    if (max_rel) OCPX_CUDA(cudaMemcpyAsync(max_rel, ctx->ws.maxrel, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    return OCPX_OK;
}

ocpx_status ocpx_wells_eval(ocpx_ctx* ctx, int nwell, const ocpx_well* wells, double dt, double* res_out,
                            double* blocks_out, double* max_rel)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null argument");
    ocpx_status cst = check_wells(ctx, nwell, wells);
    if (cst != OCPX_OK) return cst;
    if (ctx->ws.nw > 0)
        return fail(OCPX_INVALID_ARG, "the context holds wells in its step (ocpx_set_wells): their terms are "
                                      "already in its residual and Jacobian");
    if (res_out && ctx->res_gen != ctx->state_gen)
        return fail(OCPX_INVALID_ARG, "the bulk residual is older than the state: call ocpx_calres first");
    const int nb = ctx->nb, nc = ctx->nc, ncol = nc + 1;
    const size_t bs = (size_t)ncol * ncol;
    std::vector<WellPerf> perf;
    std::vector<double> zi((size_t)nwell * nc, 0.0), fac((size_t)nwell * nc, 0.0);
    for (int w = 0; w < nwell; w++) {
        const ocpx_well& W = wells[w];
        for (int i = 0; i < nc; i++) {
            if (W.inj_zi) zi[(size_t)w * nc + i] = W.inj_zi[i];
            if (W.factor) fac[(size_t)w * nc + i] = W.factor[i];
        }
        for (int q = 0; q < W.nperf; q++)
            perf.push_back(WellPerf{W.cell[q], w, W.type, W.mode, W.bhp, W.WI[q], W.dG[q],
                                    W.type == 0 ? W.xi_inj[q] : 0.0});
    }
    const int np_ = (int)perf.size();
    std::vector<double> qi((size_t)np_ * nc), dqw((size_t)np_ * nc), bb((size_t)np_ * bs), wb((size_t)np_ * bs);
    if (np_ > 0) {
        // the call's inputs and outputs in one buffer
        const size_t n_in = sizeof(WellPerf) * np_, n_z = sizeof(double) * zi.size();
        const size_t n_q = sizeof(double) * qi.size(), n_b = sizeof(double) * bb.size();
        char* buf = nullptr;
        const size_t off_z = align256(n_in), off_f = off_z + align256(n_z), off_q = off_f + align256(n_z);
        const size_t off_w = off_q + align256(n_q), off_bb = off_w + align256(n_q), off_wb = off_bb + align256(n_b);
        // the context's buffer for these calls, grown when a call needs more
        const size_t need = off_wb + align256(n_b);
        if (ctx->weval_bytes < need) {
            if (ctx->weval) cudaFree(ctx->weval);
            ctx->weval = nullptr;
            ctx->weval_bytes = 0;
            OCPX_CUDA(cudaMalloc(&ctx->weval, need));
            ctx->weval_bytes = need;
        }
        buf = ctx->weval;
        cudaStream_t s = ctx->stream;
        cudaError_t e = cudaMemcpyAsync(buf, perf.data(), n_in, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && n_z) e = cudaMemcpyAsync(buf + off_z, zi.data(), n_z, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && n_z) e = cudaMemcpyAsync(buf + off_f, fac.data(), n_z, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = launch_well_perf(ctx->b, (const WellPerf*)buf, np_, (const double*)(buf + off_z),
                                 (const double*)(buf + off_f), dt, (double*)(buf + off_q), (double*)(buf + off_w),
                                 (double*)(buf + off_bb), (double*)(buf + off_wb), s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(qi.data(), buf + off_q, n_q, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dqw.data(), buf + off_w, n_q, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(bb.data(), buf + off_bb, n_b, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(wb.data(), buf + off_wb, n_b, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        ctx->launches++;
        if (e != cudaSuccess) return fail(OCPX_CUDA_ERROR, std::string("wells: ") + cudaGetErrorString(e));
    }
    // the wells' rows and the perforated cells' rows, summed per well in
    // perforation order as CalResFIM does, on the residual before CalRes's
    // negation (negation is exact)
    double mrel = 0.0;
    std::vector<double> R;
    if (res_out) {
        R.assign((size_t)(nb + nwell) * ncol, 0.0);
        OCPX_CUDA(cudaMemcpyAsync(R.data(), ctx->res, sizeof(double) * (size_t)nb * ncol, cudaMemcpyDeviceToHost,
                                  ctx->stream));
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
        for (size_t k = 0; k < (size_t)nb * ncol; k++) R[k] = -R[k];
    }
    size_t q0 = 0;
    for (int w = 0; w < nwell; w++) {
        const ocpx_well& W = wells[w];
        std::vector<double> qw(nc, 0.0);
        for (int q = 0; q < W.nperf; q++) {
            const size_t pq = q0 + q;
            for (int i = 0; i < nc; i++) qw[i] += qi[pq * nc + i];
            if (res_out)
                for (int i = 0; i < nc; i++) R[(size_t)W.cell[q] * ncol + 1 + i] += qi[pq * nc + i] * dt;
        }
        double r;
        if (W.mode == 0) r = W.bhp - W.tar_bhp;
        else {
            r = W.type == 0 ? W.tar_rate : -W.tar_rate;
            for (int i = 0; i < nc; i++) r += qw[i] * W.factor[i];
            mrel = std::max(mrel, std::fabs(r / W.tar_rate));
        }
        if (res_out) R[(size_t)(nb + w) * ncol] = r;
        q0 += W.nperf;
    }
    if (res_out)
        for (size_t k = 0; k < R.size(); k++) res_out[k] = -R[k];
    if (blocks_out) {
        double* out = blocks_out;
        for (int pq = 0; pq < np_; pq++) {
            std::copy(bb.begin() + pq * bs, bb.begin() + (pq + 1) * bs, out);
            out += bs;
            std::fill(out, out + bs, 0.0);
            for (int i = 0; i < nc; i++) out[(size_t)(i + 1) * ncol] = dqw[(size_t)pq * nc + i] * dt;
            out += bs;
            if (perf[pq].mode == 1) std::copy(wb.begin() + pq * bs, wb.begin() + (pq + 1) * bs, out);
            else std::fill(out, out + bs, 0.0);
            out += bs;
        }
        q0 = 0;
        for (int w = 0; w < nwell; w++) {
            const ocpx_well& W = wells[w];
            std::fill(out, out + bs, 0.0);
            for (int q = 0; q < W.nperf; q++) {
                if (W.mode == 0) {
                    for (int i = 0; i < ncol; i++) out[(size_t)i * ncol + i] += 1.0;
                }
                else {
                    double d0 = 0.0;
                    for (int i = 0; i < nc; i++) d0 += dqw[(q0 + q) * nc + i] * W.factor[i];
                    out[0] += d0;
                    for (int i = 0; i < nc; i++) out[(size_t)(i + 1) * ncol + i + 1] += 1.0;
                }
            }
            out += bs;
            q0 += W.nperf;
        }
    }
    if (max_rel) *max_rel = mrel;
    return OCPX_OK;
}

ocpx_status ocpx_checkpoint(ocpx_ctx* ctx, int slot, int restore)
{
    if (!ctx || slot < 0 || slot > 1) return fail(OCPX_INVALID_ARG, "checkpoint slot must be 0 or 1");
    if (!ctx->ckpt[slot]) {
        if (restore) return fail(OCPX_INVALID_ARG, "checkpoint slot is empty");
        OCPX_CUDA(cudaMalloc(&ctx->ckpt[slot], ctx->state_bytes));
    }
    char* state = ctx->arena + ctx->state_off;
    // the wells' bottom-hole pressures travel with the bulk state
    // (ResetToLastTimeStep resets them too); their slots follow bhp[] in the
    // wells' buffer
    const size_t wb = sizeof(double) * ctx->ws.nw;
    double* wslot = ctx->ws.nw > 0 ? ctx->ws.bhp + (size_t)(1 + slot) * ctx->ws.nw : nullptr;
    if (restore) {
        OCPX_CUDA(cudaMemcpyAsync(state, ctx->ckpt[slot], ctx->state_bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        if (wslot) OCPX_CUDA(cudaMemcpyAsync(ctx->ws.bhp, wslot, wb, cudaMemcpyDeviceToDevice, ctx->stream));
        ctx->state_gen++;
    }
    else {
        OCPX_CUDA(cudaMemcpyAsync(ctx->ckpt[slot], state, ctx->state_bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        if (wslot) OCPX_CUDA(cudaMemcpyAsync(wslot, ctx->ws.bhp, wb, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return OCPX_OK;
}

ocpx_status ocpx_synchronize(ocpx_ctx* ctx)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    return OCPX_OK;
}

ocpx_status ocpx_jacobian_dims(ocpx_ctx* ctx, size_t* nrow, size_t* nnz_blocks, int* block_dim)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    if (nrow) *nrow = ctx->nrow;
    if (nnz_blocks) *nnz_blocks = ctx->jac_nnz;
    if (block_dim) *block_dim = ctx->nc + 1;
    return OCPX_OK;
}

ocpx_status ocpx_get_jacobian(ocpx_ctx* ctx, uint32_t* rowptr, uint32_t* col, double* val)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    const size_t bsize = (size_t)(ctx->nc + 1) * (ctx->nc + 1);
    if (rowptr)
        OCPX_CUDA(cudaMemcpyAsync(rowptr, ctx->jac_rowptr, sizeof(uint32_t) * (ctx->nrow + 1), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    if (col)
        OCPX_CUDA(cudaMemcpyAsync(col, ctx->jac_col, sizeof(uint32_t) * ctx->jac_nnz, cudaMemcpyDeviceToHost, ctx->stream));
    if (val)
        OCPX_CUDA(cudaMemcpyAsync(val, ctx->jac_val, sizeof(double) * ctx->jac_nnz * bsize, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    return OCPX_OK;
}

ocpx_status ocpx_get_jacobian_rows(ocpx_ctx* ctx, size_t r0, size_t r1, uint32_t* rowptr, uint32_t* col, double* val)
{
    if (!ctx || !rowptr) return fail(OCPX_INVALID_ARG, "null argument");
    if (r0 > r1 || r1 > (size_t)ctx->nrow) return fail(OCPX_INVALID_ARG, "row range outside the system's rows");
    const size_t bsize = (size_t)(ctx->nc + 1) * (ctx->nc + 1);
    OCPX_CUDA(cudaMemcpyAsync(rowptr, ctx->jac_rowptr + r0, sizeof(uint32_t) * (r1 - r0 + 1), cudaMemcpyDeviceToHost,
                              ctx->stream));
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    const size_t b0 = rowptr[0], nblk = rowptr[r1 - r0] - b0;
    if (col && nblk)
        OCPX_CUDA(cudaMemcpyAsync(col, ctx->jac_col + b0, sizeof(uint32_t) * nblk, cudaMemcpyDeviceToHost, ctx->stream));
    if (val && nblk)
        OCPX_CUDA(cudaMemcpyAsync(val, ctx->jac_val + b0 * bsize, sizeof(double) * nblk * bsize, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    return OCPX_OK;
}

ocpx_status ocpx_jacobian_device(ocpx_ctx* ctx, const uint32_t** rowptr, const uint32_t** col, const double** val)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    if (rowptr) *rowptr = ctx->jac_rowptr;
    if (col) *col = ctx->jac_col;
    if (val) *val = ctx->jac_val;
    return OCPX_OK;
}

ocpx_status ocpx_set_variant(ocpx_ctx* ctx, int variant)
{
    if (!ctx || (variant != 0 && variant != 1)) return fail(OCPX_INVALID_ARG, "variant must be 0 or 1");
    ctx->variant = variant;
    ctx->drop_graph();
    return OCPX_OK;
}

ocpx_status ocpx_set_param(ocpx_ctx* ctx, ocpx_param p, long long value)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    ctx->drop_graph();
    switch (p) {
    case OCPX_PARAM_FLASH_BUDGET:
        if (value < 0 || value > 0x7fffffffLL) return fail(OCPX_INVALID_ARG, "flash budget out of range");
        ctx->flash_budget = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_COOP_BLOCKS:
        if (value < 1 || value > 65535) return fail(OCPX_INVALID_ARG, "cooperative blocks out of range");
        ctx->coop_blocks = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_BLOCK_CELL:
        if (value != 32 && value != 64 && value != 128) return fail(OCPX_INVALID_ARG, "block size must be 32, 64 or 128");
        ctx->block_cell = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_PREDEFER:
        if (value < 0) return fail(OCPX_INVALID_ARG, "predefer threshold must be >= 0");
        ctx->predefer = value;
        return OCPX_OK;
    case OCPX_PARAM_COOP_CELLS:
        if (value < 0 || value > 0x7fffffffLL) return fail(OCPX_INVALID_ARG, "coop cells out of range");
        ctx->coop_cells = value;
        return OCPX_OK;
    case OCPX_PARAM_PRE_BLOCKS:
        if (value < 0 || value > 65535) return fail(OCPX_INVALID_ARG, "pre blocks out of range");
        ctx->pre_blocks = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_CELL_BLOCKS:
        if (value < 0 || value > 65535) return fail(OCPX_INVALID_ARG, "cell blocks out of range");
        ctx->cell_blocks = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_FUSED_BLOCKS:
        if (value < 0 || value > 65535) return fail(OCPX_INVALID_ARG, "fused blocks out of range");
        ctx->fused_blocks = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_FUSED_COOP_BLOCKS:
        if (value < -1 || value > 65535) return fail(OCPX_INVALID_ARG, "fused coop blocks out of range");
        ctx->fused_coop_blocks = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_FUSED_EXCL:
        if (value < 0 || value > 1) return fail(OCPX_INVALID_ARG, "fused excl must be 0 or 1");
        ctx->fused_excl = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_POST_BLOCK:
        if (value < 32 || value > 128 || value % 32) return fail(OCPX_INVALID_ARG, "post block must be 32, 64, 96 or 128");
        ctx->post_block = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_ROUNDS:
        if (value < 0 || value > 8) return fail(OCPX_INVALID_ARG, "rounds must be 0..8");
        ctx->rounds = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_ROUND_GROWTH:
        if (value < 2 || value > 64) return fail(OCPX_INVALID_ARG, "round growth must be 2..64");
        ctx->round_growth = (int)value;
        return OCPX_OK;
    case OCPX_PARAM_SPLIT_REFILL:
        if (value != 0 && value != 1) return fail(OCPX_INVALID_ARG, "split refill must be 0 or 1");
        if (value && !ctx->split_state) {
            if (cudaMalloc(&ctx->split_state, sizeof(SplitState) * (size_t)ctx->nb) != cudaSuccess) {
                ctx->split_state = nullptr;
                return fail(OCPX_CUDA_ERROR, "cudaMalloc of the split states failed");
            }
        }
        ctx->split_refill = (int)value;
        return OCPX_OK;
    default:
        return fail(OCPX_INVALID_ARG, "unknown or read-only parameter");
    }
}

}  // extern "C"

namespace {
// device memory the context holds: the arena, the linear system, the wells,
// the linear solver's and the adjoint's work space, the checkpoints
size_t device_bytes(const ocpx_ctx* ctx)
{
    size_t n = ctx->arena_bytes + ctx->sys_bytes + ctx->wbuf_bytes + ctx->weval_bytes;
    if (ctx->ls_scratch) n += sizeof(double) * linsolve_scratch_doubles(ctx->nrow, ctx->nc + 1);
    if (ctx->split_state) n += sizeof(SplitState) * (size_t)ctx->nb;
    if (ctx->step_adj) n += sizeof(double) * (2 * ctx->nv() + ctx->nb + (size_t)ctx->nconn);
    for (char* c : ctx->ckpt)
        if (c) n += ctx->state_bytes;
    return n;
}
}  // namespace

extern "C" {

ocpx_status ocpx_get_param(ocpx_ctx* ctx, ocpx_param p, long long* value)
{
    if (!ctx || !value) return fail(OCPX_INVALID_ARG, "null argument");
    switch (p) {
    case OCPX_PARAM_FLASH_BUDGET: *value = ctx->flash_budget; return OCPX_OK;
    case OCPX_PARAM_COOP_BLOCKS: *value = ctx->coop_blocks; return OCPX_OK;
    case OCPX_PARAM_BLOCK_CELL: *value = ctx->block_cell; return OCPX_OK;
    case OCPX_PARAM_PREDEFER: *value = ctx->predefer; return OCPX_OK;
    case OCPX_PARAM_COOP_CELLS: *value = ctx->coop_cells; return OCPX_OK;
    case OCPX_PARAM_PRE_BLOCKS: *value = ctx->pre_blocks; return OCPX_OK;
    case OCPX_PARAM_CELL_BLOCKS: *value = ctx->cell_blocks; return OCPX_OK;
    case OCPX_PARAM_ROUNDS: *value = ctx->rounds; return OCPX_OK;
    case OCPX_PARAM_FUSED_BLOCKS: *value = ctx->fused_blocks; return OCPX_OK;
    case OCPX_PARAM_FUSED_COOP_BLOCKS: *value = fused_coop_blocks(ctx); return OCPX_OK;
    case OCPX_PARAM_SMS: *value = ctx->sms; return OCPX_OK;
    case OCPX_PARAM_FUSED_EXCL: *value = ctx->fused_excl; return OCPX_OK;
    case OCPX_PARAM_POST_BLOCK: *value = ctx->post_block; return OCPX_OK;
    case OCPX_PARAM_ROUND_GROWTH: *value = ctx->round_growth; return OCPX_OK;
    case OCPX_PARAM_RECOMPUTE_FLASH_DER: *value = ctx->recompute ? 1 : 0; return OCPX_OK;
    case OCPX_PARAM_SPLIT_REFILL: *value = ctx->split_refill; return OCPX_OK;
    case OCPX_PARAM_DEVICE_BYTES: *value = (long long)device_bytes(ctx); return OCPX_OK;
    case OCPX_PARAM_DEFERRED: {
        unsigned n[2] = {0, 0};
        OCPX_CUDA(cudaMemcpyAsync(&n[0], ctx->defer_count + ctx->late_count, sizeof(unsigned),
                                  cudaMemcpyDeviceToHost, ctx->stream));
        OCPX_CUDA(cudaMemcpyAsync(&n[1], ctx->defer_count + 1, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                  ctx->stream));
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
        *value = (long long)std::min(n[0], (unsigned)ctx->defer_cap) + std::min(n[1], (unsigned)ctx->defer_cap);
        return OCPX_OK;
    }
    case OCPX_PARAM_PREDEFERRED: {
        unsigned n = 0;
        OCPX_CUDA(cudaMemcpyAsync(&n, ctx->defer_count + 1, sizeof(n), cudaMemcpyDeviceToHost, ctx->stream));
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
        *value = (long long)std::min(n, (unsigned)ctx->defer_cap);
        return OCPX_OK;
    }
    case OCPX_PARAM_LEVEL: {
        int L = 0;
        OCPX_CUDA(cudaMemcpyAsync(&L, ctx->adapt_level, sizeof(L), cudaMemcpyDeviceToHost, ctx->stream));
        OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
        *value = L;
        return OCPX_OK;
    }
    default:
        return fail(OCPX_INVALID_ARG, "unknown parameter");
    }
}

ocpx_status ocpx_adjoint(ocpx_ctx* ctx, const double* lambda, double* jt_lambda, double* dr_dtrans,
                         double* dr_dporo)
{
    if (!ctx || !lambda) return fail(OCPX_INVALID_ARG, "null argument");
    if (ctx->nbI < ctx->nb) return fail(OCPX_INVALID_ARG, "the adjoint needs a single domain (no ghost cells)");
    cudaStream_t s = ctx->stream;
    const size_t nv = ctx->nv();
    double* d_lam = ctx->adj;
    double* d_out = ctx->adj + nv;
    OCPX_CUDA(cudaMemcpyAsync(d_lam, lambda, sizeof(double) * nv, cudaMemcpyHostToDevice, s));
    if (jt_lambda) {
        OCPX_CUDA(launch_jt_lambda(ctx->b, ctx->cv, ctx->jac_rowptr, ctx->jac_val, ctx->jac_slot, d_lam, d_out,
                                   ctx->block_cell, s));
        ctx->launches++;
        if (ctx->ws.nw > 0) {
            OCPX_CUDA(launch_wells_jt(ctx->b, ctx->ws, ctx->jac_rowptr, ctx->jac_val, d_lam, d_out, s));
            ctx->launches += 2;
        }
        OCPX_CUDA(cudaMemcpyAsync(jt_lambda, d_out, sizeof(double) * nv, cudaMemcpyDeviceToHost, s));
    }
    if (dr_dtrans && ctx->nconn) {
        OCPX_CUDA(launch_vjp_trans(ctx->b, ctx->cv, ctx->last_dt, d_lam, ctx->adj_conn, ctx->block_conn, s));
        ctx->launches++;
        OCPX_CUDA(cudaMemcpyAsync(dr_dtrans, ctx->adj_conn, sizeof(double) * ctx->nconn, cudaMemcpyDeviceToHost, s));
    }
    if (dr_dporo) {
        OCPX_CUDA(launch_vjp_poro(ctx->d_model, ctx->b, d_lam, d_out, ctx->block_cell, s));
        ctx->launches++;
        OCPX_CUDA(cudaMemcpyAsync(dr_dporo, d_out, sizeof(double) * ctx->nb, cudaMemcpyDeviceToHost, s));
    }
    OCPX_CUDA(cudaStreamSynchronize(s));
    return OCPX_OK;
}

ocpx_status ocpx_set_adjoint_seed(ocpx_ctx* ctx, const double* lambda)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    if (lambda && ctx->nbI < ctx->nb)
        return fail(OCPX_INVALID_ARG, "the adjoint needs a single domain (no ghost cells)");
    ctx->drop_graph();
    if (!lambda) {
        ctx->adj_in_step = false;
        return OCPX_OK;
    }
    const size_t nv = ctx->nv();
    if (!ctx->step_adj)
        OCPX_CUDA(cudaMalloc(&ctx->step_adj, sizeof(double) * (2 * nv + ctx->nb + (size_t)ctx->nconn)));
    OCPX_CUDA(cudaMemcpyAsync(ctx->step_adj, lambda, sizeof(double) * nv, cudaMemcpyHostToDevice, ctx->stream));
    OCPX_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->adj_in_step = true;
    return OCPX_OK;
}

ocpx_status ocpx_get_adjoint(ocpx_ctx* ctx, double* jt_lambda, double* dr_dtrans, double* dr_dporo)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    if (!ctx->adj_in_step) return fail(OCPX_INVALID_ARG, "no adjoint seed is set (ocpx_set_adjoint_seed)");
    const size_t nv = ctx->nv();
    cudaStream_t s = ctx->stream;
    if (jt_lambda)
        OCPX_CUDA(cudaMemcpyAsync(jt_lambda, ctx->step_adj + nv, sizeof(double) * nv, cudaMemcpyDeviceToHost, s));
    if (dr_dporo)
        OCPX_CUDA(cudaMemcpyAsync(dr_dporo, ctx->step_adj + 2 * nv, sizeof(double) * ctx->nb, cudaMemcpyDeviceToHost,
                                  s));
    if (dr_dtrans && ctx->nconn)
        OCPX_CUDA(cudaMemcpyAsync(dr_dtrans, ctx->step_adj + 2 * nv + ctx->nb, sizeof(double) * ctx->nconn,
                                  cudaMemcpyDeviceToHost, s));
    OCPX_CUDA(cudaStreamSynchronize(s));
    return OCPX_OK;
}

ocpx_status ocpx_step(ocpx_ctx* ctx, const double* u_host, double dSmax, double dt, double* res_host,
                      double* jac_val_host, ocpx_report* rep)
{
    if (!ctx) return fail(OCPX_INVALID_ARG, "null context");
    ocpx_status st;
    if (u_host) {
        st = ocpx_newton_update(ctx, u_host, dSmax);
        if (st != OCPX_OK) return st;
    }
    if ((st = ocpx_enqueue_step(ctx, dt)) != OCPX_OK) return st;
    const size_t bsize = (size_t)(ctx->nc + 1) * (ctx->nc + 1);
    if (res_host)
        OCPX_CUDA(cudaMemcpyAsync(res_host, ctx->res, sizeof(double) * ctx->nv(), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    if (jac_val_host)
        OCPX_CUDA(cudaMemcpyAsync(jac_val_host, ctx->jac_val, sizeof(double) * ctx->jac_nnz * bsize,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    return report_from_flags(ctx, rep);
}

}  // extern "C"
