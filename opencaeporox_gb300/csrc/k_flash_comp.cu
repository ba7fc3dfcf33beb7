// Compositional FlashDer kernels, compiled once per component capacity
// (OCPX_NCM) so each build carries arrays sized for its component count.
#include "ocpx_kernels.h"
#include "cell_ops.cuh"
#include "flash_coop.cuh"
#include "tile_sort.cuh"

#ifndef OCPX_NCM
#error "compile with -DOCPX_NCM=<capacity>"
#endif
#ifndef OCPX_FLASH_PART
#error "compile with -DOCPX_FLASH_PART=<0..8>"
#endif

namespace ocpx {

template <int NCM>
__global__ void __launch_bounds__(128) k_flash_comp(const Model* __restrict__ M, BulkView b)
{
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= b.nb) return;
    CompCellUpdate<NCM> u;
    u.run(*M, b, cell);
}

// Batched form, step 1: one thread per cell in the order given by `order`
// (cells of similar predicted cost side by side), with a work budget on the
// phase equilibrium; cells over budget are appended to the deferral list and
// left untouched.  With `next` NULL the grid has one thread per position of
// `order`.  Otherwise the grid is persistent: each warp takes the next 32
// positions from the counter `next` (zero before the launch) until `order`
// is exhausted, so fewer warps are resident (and fewer per-thread frames are
// live at once) and a warp that finishes early moves on at once.
template <int NCM>
__device__ __forceinline__ void flash_budget_cell(const Model* __restrict__ M, const BulkView& b, int cell, int budget,
                                                  const DeferSink& sink, const uint8_t* __restrict__ pre,
                                                  const int* __restrict__ level)
{
    if (pre && pre[cell]) return;  // handled by the cooperative kernel
    if (level) {
        // at least the work of the adaptive level: only cells heavier than the
        // heaviest predicted ones are deferred now
        const long long lw = (long long)exp2f(0.25f * (float)level[0]);
        if (lw > budget) budget = lw > 0x7fffffffLL ? 0x7fffffff : (int)lw;
    }
    CompCellUpdate<NCM> u;
    u.run(*M, b, cell, budget, &sink);
}

template <int NCM>
__global__ void __launch_bounds__(128) k_flash_budget(const Model* __restrict__ M, BulkView b,
                                                      const int* __restrict__ order, int budget, DeferSink sink,
                                                      const uint8_t* __restrict__ pre, const int* __restrict__ level,
                                                      unsigned* __restrict__ next)
{
    if (!next) {
        const int p = blockIdx.x * blockDim.x + threadIdx.x;
        if (p < b.nb) flash_budget_cell<NCM>(M, b, order[p], budget, sink, pre, level);
        return;
    }
    const unsigned lane = threadIdx.x & 31;
    for (;;) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(next, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (unsigned)b.nb) break;
        const unsigned p = base + lane;
        if (p < (unsigned)b.nb) flash_budget_cell<NCM>(M, b, order[p], budget, sink, pre, level);
        __syncwarp();
    }
}

// Re-budgeting round: the cells of a deferral list, rerun one thread per cell
// from their (untouched) state with the round's budget, b0 * mult, where b0
// is the step-1 budget (raised to the adaptive level when `level` is given).
// Cells over it go to the next list.  Each warp takes 32 list entries at a time from `next`.
// Restarting a cell from scratch repeats exactly the arithmetic it would have
// done, so the result does not depend on the round a cell finishes in; with a
// budget growing by a factor G per round, the repeated work is at most
// 1 / (G - 1) of the work of the cells that go through the rounds, and warps
// hold cells whose work lies within one factor of G of each other.
template <int NCM>
__global__ void __launch_bounds__(128) k_flash_round(const Model* __restrict__ M, BulkView b,
                                                     const DeferRec* __restrict__ rin,
                                                     const unsigned* __restrict__ rin_count, int cap, int budget,
                                                     long long mult, DeferSink sink, const int* __restrict__ level,
                                                     unsigned* __restrict__ next)
{
    const unsigned n = min(*rin_count, (unsigned)cap);
    long long b0 = budget;
    if (level) {
        const long long lw = (long long)exp2f(0.25f * (float)level[0]);
        if (lw > b0) b0 = lw;
    }
    long long br = b0 * mult;
    if (br > 0x7fffffffLL || br < 0) br = 0x7fffffffLL;
    const unsigned lane = threadIdx.x & 31;
    for (;;) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(next, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const unsigned p = base + lane;
        if (p < n) {
            CompCellUpdate<NCM> u;
            u.run(*M, b, rin[p].cell, (int)br, &sink);
        }
        __syncwarp();
    }
}

// Fused batched flash: one persistent kernel does what the per-cell kernel
// and the two cooperative passes do on two streams, so the long cells never
// compete with the per-cell work for an SM sub-partition's FP64 pipe, and no
// block placement across streams decides when they start.  Each warp:
//   1. takes pre-deferred cells, one at a time, and runs their equilibrium
//      cooperatively (they are the longest chains, so they start first);
//   2. then, each time it is free: claims the next over-budget cell if one
//      is published and runs it cooperatively, else takes 32 cost-ordered
//      cells, one per lane, with the work budget (over-budget cells are
//      published to the late list); when both are exhausted it leaves.
// A late cell is claimed in list order and only once its record is
// published; a warp that meets an unpublished one takes cells instead or
// leaves, and the cell's own publisher, which looks for late cells right
// after publishing, claims it.  So every late cell is run exactly once and
// no warp ever waits on another.  The records are read
// through L2 (another record in the same line may be cached in L1 from
// before it was written).  Counters: ctr[0] pre slots, ctr[1] cell
// positions, ctr[2] late slots, all zero before the launch; the late list's
// seq fields are zero before the launch.
template <int NCM>
__global__ void __launch_bounds__(FUSED_WARPS * 32, 1) k_flash_fused(const Model* __restrict__ M, BulkView b,
                                                                const int* __restrict__ order, int budget,
                                                                const uint8_t* __restrict__ pre,
                                                                const int* __restrict__ level,
                                                                const DeferRec* __restrict__ pre_rec,
                                                                const unsigned* __restrict__ pre_count,
                                                                PERes* __restrict__ pre_pe, DeferSink late,
                                                                PERes* __restrict__ late_pe,
                                                                unsigned* __restrict__ ctr, int coop_n,
                                                                uint32_t* __restrict__ watchdog)
{
    __shared__ CoopSh<NCM> sh[FUSED_WARPS];
    const int warp = threadIdx.x >> 5;
    const unsigned lane = threadIdx.x & 31;
    const bool roles = coop_n > 0;
    const bool coop_only = roles && (int)blockIdx.x < coop_n;
    // claims the next published over-budget cell (lane 0), or returns none
    auto claim_late = [&]() -> unsigned {
        unsigned got = 0xffffffffu;
        if (lane == 0) {
            volatile unsigned* vctr = &ctr[2];
            volatile unsigned* vcount = late.count;
            unsigned cur = *vctr;
            for (;;) {
                const unsigned n = min(*vcount, (unsigned)late.cap);
                if (cur >= n) break;
                if (*(volatile unsigned*)&late.rec[cur].seq != late.seq) break;
                const unsigned prev = atomicCAS(&ctr[2], cur, cur + 1u);
                if (prev == cur) { got = cur; break; }
                cur = prev;
            }
        }
        return __shfl_sync(0xffffffffu, got, 0);
    };
    auto run_late = [&](unsigned got) {
        __threadfence();
        DeferRec r;
        r.cell = __ldcg(&late.rec[got].cell);
        r.ftype_in = __ldcg(&late.rec[got].ftype_in);
        r.lNP = __ldcg(&late.rec[got].lNP);
        r.seq = late.seq;
        CoopPE<NCM> pe(sh[warp], M->comp);
        pe.run(*M, b, r, late_pe[got]);
        __syncwarp();
    };
    // 1. pre-deferred cells (with roles, on the cooperative blocks only: the
    // other warps must not take slots from the shared counter at all)
    const unsigned npre = pre_count ? min(*pre_count, (unsigned)late.cap) : 0u;
    if (!roles || coop_only) {
        for (;;) {
            unsigned slot = 0;
            if (lane == 0) slot = atomicAdd(&ctr[0], 1u);
            slot = __shfl_sync(0xffffffffu, slot, 0);
            if (slot >= npre) break;
            CoopPE<NCM> pe(sh[warp], M->comp);
            pe.run(*M, b, pre_rec[slot], pre_pe[slot]);
            __syncwarp();
        }
    }
    if (coop_only) {
        // 3'. the cooperative blocks: over-budget cells until every per-lane warp
        // has finished and none is left.  The wait is bounded; past the bound
        // the kernel reports a watchdog status instead of waiting on.
        const unsigned expected = (gridDim.x - (unsigned)coop_n) * FUSED_WARPS;
        unsigned spins = 0;
        for (;;) {
            const unsigned got = claim_late();
            if (got != 0xffffffffu) { run_late(got); spins = 0; continue; }
            unsigned done = 0;
            if (lane == 0) done = *(volatile unsigned*)&ctr[3] >= expected ? 1u : 0u;
            done = __shfl_sync(0xffffffffu, done, 0);
            if (done) {
                const unsigned last = claim_late();
                if (last != 0xffffffffu) { run_late(last); continue; }
                break;
            }
            if (++spins > (1u << 24)) {
                if (lane == 0) atomicOr(watchdog, (uint32_t)ST_ITER_CAP);
                break;
            }
            __nanosleep(256);
        }
        return;
    }
    // 2. over-budget cells as soon as they are published, else the next 32
    // cost-ordered cells (one per lane): a long cell that the budget caught
    // starts its cooperative run at once instead of after the whole order.
    // With roles the per-lane blocks leave the over-budget cells to the
    // cooperative blocks until the order is exhausted, then help.
    bool cells_left = true;
    for (;;) {
        if (!roles || !cells_left) {
            const unsigned got = claim_late();
            if (got != 0xffffffffu) { run_late(got); continue; }
        }
        if (!cells_left) break;
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(&ctr[1], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (unsigned)b.nb) {
            cells_left = false;  // one more look for over-budget cells, then leave
            continue;
        }
        const unsigned p = base + lane;
        if (p < (unsigned)b.nb) flash_budget_cell<NCM>(M, b, order[p], budget, late, pre, level);
        __syncwarp();
    }
    if (roles && lane == 0) {
        __threadfence();
        atomicAdd(&ctr[3], 1u);  // this warp's over-budget cells are all published
    }
}

// Step 2: the phase equilibrium of every deferred cell on a whole warp
// (flash_coop.cuh).  Persistent: each warp takes the next list slot from the
// counter `next` (zero before the launch) until the list is exhausted, so a
// warp that drew a short cell moves on at once; the list is roughly
// heaviest first, so the long cells start first.
//
// WARPS = COOP_WARPS: small blocks that share SMs with the other kernels of
// the flash.  WARPS = EXCL_WARPS: one warp per SM sub-partition, launched with
// all the shared memory a block may hold, so that no other block is placed
// on the SM while it runs; its warps then have the FP64 pipes of their
// sub-partitions to themselves (one warp's dependent FP64 chain issues at the
// pipe's full rate, so the longest cells run at full speed).
template <int NCM, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_flash_pe_coop(const Model* __restrict__ M, BulkView b,
                                                              const DeferRec* __restrict__ rec,
                                                              const unsigned* __restrict__ count, int cap,
                                                              unsigned* __restrict__ next,
                                                              PERes* __restrict__ out)
{
    __shared__ CoopSh<NCM> sh[WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned n = min(*count, (unsigned)cap);
    for (;;) {
        unsigned slot = 0;
        if (lane == 0) slot = atomicAdd(next, 1u);
        slot = __shfl_sync(0xffffffffu, slot, 0);
        if (slot >= n) break;
        CoopPE<NCM> pe(sh[warp], M->comp);
        pe.run(*M, b, rec[slot], out[slot]);
        __syncwarp();
    }
}

// Step 3: properties, derivatives and skip state of the deferred cells from
// their equilibrium, one thread per deferred cell: the cells of the first list,
// then those of the second (rec2 NULL: none), so that the busy threads are the
// leading ones.  Each list holds at most cap cells.
template <int NCM>
__global__ void __launch_bounds__(128) k_flash_post(const Model* __restrict__ M, BulkView b,
                                                    const DeferRec* __restrict__ rec,
                                                    const unsigned* __restrict__ count, int cap,
                                                    const PERes* __restrict__ pe,
                                                    const DeferRec* __restrict__ rec2,
                                                    const unsigned* __restrict__ count2,
                                                    const PERes* __restrict__ pe2)
{
    unsigned slot = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned n = min(*count, (unsigned)cap);
    if (slot >= n) {
        if (!rec2) return;
        slot -= n;
        if (slot >= min(*count2, (unsigned)cap)) return;
        rec = rec2;
        pe = pe2;
    }
    CompCellUpdate<NCM> u;
    u.run(*M, b, rec[slot].cell, 0x7fffffff, nullptr, &pe[slot]);
}

// ---- flash derivatives recomputed where they are used (no dSec_dPri stored)

// dSec_dPri of the cells list[t] (or first + t): with soa = 0 into
// out[t][row * (nc + 1) + col], else into out[(row * (nc + 1) + col) * soa + t]
template <int NCM>
__global__ void __launch_bounds__(128) k_dsec_cells(const Model* __restrict__ M, BulkView b, const int* __restrict__ list,
                                                    int first, int n, double* __restrict__ out, size_t soa)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int cell = list ? list[t] : first + t;
    const int ncol = b.nc + 1, lend = b.np * ncol * ncol;
    CompCellUpdate<NCM> u;
    if (soa) u.recompute_dsec(*M, b, cell, out + t, soa);
    else u.recompute_dsec(*M, b, cell, out + (size_t)t * lend, 1);
}

// dSec_dPri of the cells [first, first + n) into out[k * soa + (cell - first)],
// tiles of DSEC_TILE cells per block sorted by phase count first, so that the
// two-phase cells' derivative solve runs on whole warps.
constexpr int DSEC_TILE = 512;
template <int NCM>
__global__ void __launch_bounds__(128) k_dsec_slab(const Model* __restrict__ M, BulkView b, int first, int n,
                                                   double* __restrict__ out, size_t soa)
{
    __shared__ unsigned cnt[32];
    __shared__ unsigned short key_s[DSEC_TILE];
    __shared__ unsigned short idx_s[DSEC_TILE];
    const int c0 = first + blockIdx.x * DSEC_TILE;
    const int m = min(DSEC_TILE, first + n - c0);
    tile_sort<32>(
        m,
        [&](int i) {
            const int cell = c0 + i;
            return (b.phaseExist[b.idx(0, cell)] && b.phaseExist[b.idx(1, cell)]) ? 0 : 1;
        },
        cnt, key_s, idx_s);
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int cell = c0 + idx_s[i];
        CompCellUpdate<NCM> u;
        u.recompute_dsec(*M, b, cell, out + (cell - first), soa);
    }
}

// GetSolution with the cell's dSec_dPri recomputed before its state changes;
// tiles of DSEC_TILE cells with the two-phase cells first (their phase labels
// read before any cell of the tile moves)
template <int NCM>
__global__ void __launch_bounds__(128) k_newton_update_recompute(const Model* __restrict__ M, BulkView b,
                                                                 const double* __restrict__ u, double dSmax)
{
    __shared__ unsigned cnt[32];
    __shared__ unsigned short key_s[DSEC_TILE];
    __shared__ unsigned short idx_s[DSEC_TILE];
    const int c0 = blockIdx.x * DSEC_TILE;
    const int m = min(DSEC_TILE, b.nb - c0);
    tile_sort<32>(
        m,
        [&](int i) {
            const int cell = c0 + i;
            return (b.phaseExist[b.idx(0, cell)] && b.phaseExist[b.idx(1, cell)]) ? 0 : 1;
        },
        cnt, key_s, idx_s);
    constexpr int NCT = NCM + 1;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int cell = c0 + idx_s[i];
        double ds[3 * (NCT + 1) * (NCT + 1)];
        CompCellUpdate<NCM> cu;
        cu.recompute_dsec(*M, b, cell, ds, 1);
        newton_update_cell(b, cell, u, dSmax, ds, 1);
    }
}

// ---- the split cells (flash type 2) with lane refill

// The split's first successive-substitution loop of the cells at positions
// [0, *n_split) of the cost order (the cells whose flash starts with the
// split), one pass per trip through the loop below.  A lane whose cell's
// loop ends saves the cell's state and waits; once SPLIT_REFILL_MIN lanes of
// the warp wait (or none runs), they take new cells together, so the passes
// run with most lanes busy whatever each cell's count, and a cell's set-up
// runs on many lanes at once.  Per lane, the arithmetic is the split's own
// (split_begin, split_ssm_step).  Pre-deferred cells (the cooperative
// kernel's) and cells that are not split cells are marked skip.  next: a
// position counter, zero before the launch.
constexpr int SPLIT_REFILL_MIN = 12;
template <int NCM>
__global__ void __launch_bounds__(128) k_split_refill(const Model* __restrict__ M, BulkView b,
                                                      const int* __restrict__ order,
                                                      const unsigned* __restrict__ n_split,
                                                      const uint8_t* __restrict__ pre, SplitState* __restrict__ st,
                                                      unsigned* __restrict__ next)
{
    const unsigned n = *n_split;
    CompCellUpdate<NCM> u;
    typename CompFlash<NCM>::SsmLoop L;
    unsigned p = 0;
    bool active = false, exhausted = false;
    for (;;) {
        const unsigned waiting = __ballot_sync(0xffffffffu, !active && !exhausted);
        const unsigned running = __ballot_sync(0xffffffffu, active);
        if (!running && !waiting) break;
        if (waiting && (__popc(waiting) >= SPLIT_REFILL_MIN || !running) && !active && !exhausted) {
            for (;;) {
                p = atomicAdd(next, 1u);
                if (p >= n) { exhausted = true; break; }
                const int cell = order[p];
                if ((pre && pre[cell]) || !u.split_begin(*M, b, cell, L)) {
                    st[p].skip = 1;
                    continue;
                }
                active = true;
                break;
            }
        }
        if (active && u.f.split_ssm_step(L)) {
            u.f.split_save(st[p]);
            st[p].skip = 0;
            active = false;
        }
    }
}

// The rest of those cells' flash, resumed from the saved state (run with
// resume), 32 positions per warp from the counter next (zero before the
// launch), under the per-lane work budget of the fused form: a cell over it
// (the split's Newton loop failing into restarts) is published to the late
// list, whose equilibria the fused kernel runs on whole warps.  Pre-deferred
// cells are left to the cooperative kernel.
template <int NCM>
__global__ void __launch_bounds__(128) k_split_resume(const Model* __restrict__ M, BulkView b,
                                                      const int* __restrict__ order,
                                                      const unsigned* __restrict__ n_split,
                                                      const uint8_t* __restrict__ pre,
                                                      const SplitState* __restrict__ st, unsigned* __restrict__ next,
                                                      int budget, const int* __restrict__ level, DeferSink late)
{
    if (level) {
        const long long lw = (long long)exp2f(0.25f * (float)level[0]);
        if (lw > budget) budget = lw > 0x7fffffffLL ? 0x7fffffff : (int)lw;
    }
    const unsigned n = *n_split;
    const unsigned lane = threadIdx.x & 31;
    for (;;) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(next, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const unsigned p = base + lane;
        if (p < n) {
            const int cell = order[p];
            if (!(pre && pre[cell])) {
                CompCellUpdate<NCM> u;
                u.run(*M, b, cell, budget, &late, nullptr, &st[p]);
            }
        }
        __syncwarp();
    }
}

#define OCPX_CAT2(a, b) a##b
#define OCPX_CAT(a, b) OCPX_CAT2(a, b)
#define OCPX_NAME(base) OCPX_CAT(base, OCPX_NCM)

// Each kernel of a capacity is compiled in its own translation unit
// (OCPX_FLASH_PART, build.py), so the large kernels compile in parallel.  Part
// 0 holds the plain kernel and the dispatch of the batched parts; the others
// hold one kernel each and the launch that uses it.
cudaError_t OCPX_NAME(flash_part_budget_)(const Model*, const BulkView&, const int*, const FlashBatch&, cudaStream_t);
cudaError_t OCPX_NAME(flash_part_fused_)(const Model*, const BulkView&, const int*, const FlashBatch&, cudaStream_t);
cudaError_t OCPX_NAME(flash_part_round_)(const Model*, const BulkView&, const FlashBatch&, cudaStream_t);
cudaError_t OCPX_NAME(flash_part_coop_)(const Model*, const BulkView&, const FlashBatch&, cudaStream_t);
cudaError_t OCPX_NAME(flash_part_post_)(const Model*, const BulkView&, const FlashBatch&, cudaStream_t);
cudaError_t OCPX_NAME(setup_flash_coop_)(int, int, int*);
cudaError_t OCPX_NAME(setup_flash_fused_)(int, int*);

// parts 1 and 2 carry their own launch priority, which a stream capture keeps
// in the graph's kernel node
static inline void priority_attr(cudaLaunchConfig_t& cfg, cudaLaunchAttribute* attr, const FlashBatch& fb,
                                 cudaStream_t s)
{
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = fb.prio;
    cfg = {};
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = fb.prio ? 1 : 0;
}

#if OCPX_FLASH_PART == 0
cudaError_t OCPX_NAME(launch_flash_comp_)(const Model* dm, const BulkView& b, int block, cudaStream_t s)
{
    if (b.nb == 0) return cudaSuccess;
    const int grid = (b.nb + block - 1) / block;
    k_flash_comp<OCPX_NCM><<<grid, block, 0, s>>>(dm, b);
    return cudaGetLastError();
}

cudaError_t OCPX_NAME(launch_flash_batched_)(const Model* dm, const BulkView& b, const int* order,
                                             const FlashBatch& fb, int part, cudaStream_t s)
{
    if (b.nb == 0) return cudaSuccess;
    switch (part) {
    case 0: return OCPX_NAME(flash_part_budget_)(dm, b, order, fb, s);
    case 4: return OCPX_NAME(flash_part_fused_)(dm, b, order, fb, s);
    case 3: return OCPX_NAME(flash_part_round_)(dm, b, fb, s);
    case 1: return OCPX_NAME(flash_part_coop_)(dm, b, fb, s);
    case 2:
    default: return OCPX_NAME(flash_part_post_)(dm, b, fb, s);
    }
}

// Once per device (that device current): the SM-exclusive cooperative kernel
// may use all the shared memory a block can opt into; excl_smem[0] receives
// the dynamic part that fills it, excl_smem[1] the fused kernel's, and
// excl_smem[2] the fused blocks resident per SM without it.
cudaError_t OCPX_NAME(setup_flash_batched_)(int* excl_smem)
{
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = OCPX_NAME(setup_flash_coop_)(dev, optin, excl_smem);
    if (e == cudaSuccess) e = OCPX_NAME(setup_flash_fused_)(optin, excl_smem);
    return e;
}
#endif

#if OCPX_FLASH_PART == 1
cudaError_t OCPX_NAME(flash_part_budget_)(const Model* dm, const BulkView& b, const int* order, const FlashBatch& fb,
                                          cudaStream_t s)
{
    const DeferSink sink{fb.rec, fb.count, fb.cap};
    const int grid = fb.cell_blocks > 0 ? fb.cell_blocks : (b.nb + fb.block - 1) / fb.block;
    k_flash_budget<OCPX_NCM><<<grid, fb.block, 0, s>>>(dm, b, order, fb.budget, sink, fb.pre, fb.level,
                                                       fb.cell_blocks > 0 ? fb.cell_next : nullptr);
    return cudaGetLastError();
}
#endif

#if OCPX_FLASH_PART == 2
cudaError_t OCPX_NAME(flash_part_fused_)(const Model* dm, const BulkView& b, const int* order, const FlashBatch& fb,
                                         cudaStream_t s)
{
    // fused: pre list (rin, rin_count, pe_pre) and late list (rec, count, pe)
    DeferSink late{fb.rec, fb.count, fb.cap};
    late.seq = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.stream = s;
    cfg.gridDim = dim3(fb.cell_blocks);
    cfg.blockDim = dim3(FUSED_WARPS * 32);
    cfg.dynamicSmemBytes = fb.excl_blocks ? fb.excl_smem_fused : 0;
    // without the SM-exclusive reservation the SM keeps as much L1 as the
    // static shared memory allows: the per-lane cells' thread frames live there.
    // With cooperative-only blocks, those blocks wait for the others: a
    // cooperative launch guarantees that all blocks are resident together
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributePreferredSharedMemoryCarveout;
    attr[0].val.sharedMemCarveout = fb.excl_blocks ? (unsigned)cudaSharedmemCarveoutMaxShared
                                                   : (unsigned)cudaSharedmemCarveoutMaxL1;
    attr[1].id = cudaLaunchAttributeCooperative;
    attr[1].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = fb.coop_only_blocks > 0 ? 2 : 1;
    return cudaLaunchKernelEx(&cfg, k_flash_fused<OCPX_NCM>, dm, b, order, fb.budget, fb.pre, fb.level, fb.rin,
                              fb.rin_count, fb.pe_pre, late, fb.pe, fb.cell_next, fb.coop_only_blocks, fb.watchdog);
}

// the fused kernel, when it holds an SM alone (one block per SM)
cudaError_t OCPX_NAME(setup_flash_fused_)(int optin, int* excl_smem)
{
    cudaFuncAttributes ff{};
    cudaError_t e = cudaFuncGetAttributes(&ff, k_flash_fused<OCPX_NCM>);
    if (e != cudaSuccess) return e;
    const int dynf = optin > (int)ff.sharedSizeBytes ? optin - (int)ff.sharedSizeBytes : 0;
    e = cudaFuncSetAttribute(k_flash_fused<OCPX_NCM>, cudaFuncAttributeMaxDynamicSharedMemorySize, dynf);
    // maximum L1 unless a launch asks for the SM-exclusive shared memory (whose
    // dynamic size forces the largest shared-memory configuration anyway): a
    // cooperative launch kept the function's preference over the launch's
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_flash_fused<OCPX_NCM>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxL1);
    excl_smem[1] = dynf;
    if (e != cudaSuccess) return e;
    // fused blocks resident per SM without the shared-memory reservation (for
    // the co-residency a cooperative launch needs)
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_flash_fused<OCPX_NCM>, FUSED_WARPS * 32, 0);
    excl_smem[2] = per_sm;
    return e;
}
#endif

#if OCPX_FLASH_PART == 3
cudaError_t OCPX_NAME(flash_part_round_)(const Model* dm, const BulkView& b, const FlashBatch& fb, cudaStream_t s)
{
    // re-budgeting round: from list (rin, rin_count) into (rec, count)
    const DeferSink sink{fb.rec, fb.count, fb.cap};
    const int grid = fb.cell_blocks > 0 ? fb.cell_blocks : 304;
    k_flash_round<OCPX_NCM><<<grid, fb.block, 0, s>>>(dm, b, fb.rin, fb.rin_count, fb.cap, fb.budget, fb.mult, sink,
                                                      fb.level, fb.cell_next);
    return cudaGetLastError();
}
#endif

#if OCPX_FLASH_PART == 4
cudaError_t OCPX_NAME(flash_part_coop_excl_)(const Model*, const BulkView&, const FlashBatch&, cudaStream_t);

cudaError_t OCPX_NAME(flash_part_coop_)(const Model* dm, const BulkView& b, const FlashBatch& fb, cudaStream_t s)
{
    if (fb.excl_blocks > 0) return OCPX_NAME(flash_part_coop_excl_)(dm, b, fb, s);
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg;
    priority_attr(cfg, attr, fb, s);
    cfg.gridDim = dim3(fb.coop_blocks);
    cfg.blockDim = dim3(COOP_WARPS * 32);
    return cudaLaunchKernelEx(&cfg, k_flash_pe_coop<OCPX_NCM, COOP_WARPS>, dm, b, (const DeferRec*)fb.rec,
                              (const unsigned*)fb.count, fb.cap, fb.coop_next, fb.pe);
}
#endif

#if OCPX_FLASH_PART == 5
cudaError_t OCPX_NAME(flash_part_coop_excl_)(const Model* dm, const BulkView& b, const FlashBatch& fb, cudaStream_t s)
{
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg;
    priority_attr(cfg, attr, fb, s);
    cfg.gridDim = dim3(fb.excl_blocks);
    cfg.blockDim = dim3(EXCL_WARPS * 32);
    cfg.dynamicSmemBytes = fb.excl_smem;
    return cudaLaunchKernelEx(&cfg, k_flash_pe_coop<OCPX_NCM, EXCL_WARPS>, dm, b, (const DeferRec*)fb.rec,
                              (const unsigned*)fb.count, fb.cap, fb.coop_next, fb.pe);
}

cudaError_t OCPX_NAME(setup_flash_coop_)(int dev, int optin, int* excl_smem)
{
    (void)dev;
    cudaFuncAttributes fa{};
    cudaError_t e = cudaFuncGetAttributes(&fa, k_flash_pe_coop<OCPX_NCM, EXCL_WARPS>);
    if (e != cudaSuccess) return e;
    const int dyn = optin > (int)fa.sharedSizeBytes ? optin - (int)fa.sharedSizeBytes : 0;
    e = cudaFuncSetAttribute(k_flash_pe_coop<OCPX_NCM, EXCL_WARPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_flash_pe_coop<OCPX_NCM, EXCL_WARPS>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    excl_smem[0] = dyn;
    return e;
}
#endif

#if OCPX_FLASH_PART == 7
cudaError_t OCPX_NAME(launch_dsec_cells_)(const Model* dm, const BulkView& b, const int* list, int first, int n,
                                          double* out, size_t soa, cudaStream_t s)
{
    if (n > 0) k_dsec_cells<OCPX_NCM><<<(n + 127) / 128, 128, 0, s>>>(dm, b, list, first, n, out, soa);
    return cudaGetLastError();
}
cudaError_t OCPX_NAME(launch_dsec_slab_)(const Model* dm, const BulkView& b, int first, int n, double* out,
                                         size_t soa, cudaStream_t s)
{
    if (n > 0) k_dsec_slab<OCPX_NCM><<<(n + DSEC_TILE - 1) / DSEC_TILE, 128, 0, s>>>(dm, b, first, n, out, soa);
    return cudaGetLastError();
}
cudaError_t OCPX_NAME(launch_newton_update_recompute_)(const Model* dm, const BulkView& b, const double* u,
                                                       double dSmax, cudaStream_t s)
{
    if (b.nb > 0)
        k_newton_update_recompute<OCPX_NCM><<<(b.nb + DSEC_TILE - 1) / DSEC_TILE, 128, 0, s>>>(dm, b, u, dSmax);
    return cudaGetLastError();
}
#endif

#if OCPX_FLASH_PART == 8
cudaError_t OCPX_NAME(launch_split_refill_)(const Model* dm, const BulkView& b, const int* order,
                                            const unsigned* n_split, const uint8_t* pre, SplitState* st,
                                            unsigned* next, int blocks, cudaStream_t s)
{
    if (blocks > 0) k_split_refill<OCPX_NCM><<<blocks, 128, 0, s>>>(dm, b, order, n_split, pre, st, next);
    return cudaGetLastError();
}
cudaError_t OCPX_NAME(launch_split_resume_)(const Model* dm, const BulkView& b, const int* order,
                                            const unsigned* n_split, const uint8_t* pre, const SplitState* st,
                                            unsigned* next, int blocks, const FlashBatch& fb, cudaStream_t s)
{
    DeferSink late{fb.rec, fb.count, fb.cap};
    late.seq = 1;
    if (blocks > 0)
        k_split_resume<OCPX_NCM><<<blocks, 128, 0, s>>>(dm, b, order, n_split, pre, st, next, fb.budget, fb.level,
                                                        late);
    return cudaGetLastError();
}
#endif

#if OCPX_FLASH_PART == 6
cudaError_t OCPX_NAME(flash_part_post_)(const Model* dm, const BulkView& b, const FlashBatch& fb, cudaStream_t s)
{
    // one thread per deferred cell; the SM's L1 as large as it goes, for the
    // threads' frames
    cudaLaunchAttribute attr[2];
    cudaLaunchConfig_t cfg;
    priority_attr(cfg, attr, fb, s);
    const int pb = fb.post_block > 0 ? fb.post_block : 128;
    const long long threads = (long long)fb.cap * (fb.rec2 ? 2 : 1);
    cfg.gridDim = dim3((unsigned)((threads + pb - 1) / pb));
    cfg.blockDim = dim3(pb);
    attr[cfg.numAttrs].id = cudaLaunchAttributePreferredSharedMemoryCarveout;
    attr[cfg.numAttrs].val.sharedMemCarveout = (unsigned)cudaSharedmemCarveoutMaxL1;
    cfg.numAttrs++;
    return cudaLaunchKernelEx(&cfg, k_flash_post<OCPX_NCM>, dm, b, (const DeferRec*)fb.rec,
                              (const unsigned*)fb.count, fb.cap, (const PERes*)fb.pe, fb.rec2, fb.count2, fb.pe2);
}
#endif

}  // namespace ocpx
