// Kernels of the FIM step other than the compositional flash.
#include "ocpx_kernels.h"
#include "cell_ops.cuh"
#include "conn_ops.cuh"
#include "adjoint.cuh"
#include "tile_sort.cuh"

#include <algorithm>

namespace ocpx {

__global__ void k_flash_bo(const Model* __restrict__ M, BulkView b)
{
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell < b.nb) bo_flash_der_cell(*M, b, cell);
}

__global__ void k_krpc_rock(const Model* __restrict__ M, BulkView b)
{
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell < b.nb) krpc_rock_cell(*M, b, cell);
}

// CheckNi / CheckP; flags[0] collects the OR of the failure bits.
__global__ void k_check(BulkView b, uint32_t* __restrict__ flags)
{
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t st = 0;
    if (cell < b.nb) st = check_cell(b, cell);
    // warp-level OR, one atomic per warp that saw a failure
    st = __reduce_or_sync(0xffffffffu, st);
    if ((threadIdx.x & 31) == 0 && st) atomicOr(flags, st);
}

__global__ void k_newton_update(BulkView b, const double* __restrict__ u, double dSmax)
{
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell < b.nb) newton_update_cell(b, cell, u, dSmax);
}

__global__ void k_conn_flux(const Model* __restrict__ M, BulkView b, ConnView cv)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < cv.nconn) conn_flux(*M, b, cv, c);
}

__global__ void k_residual(BulkView b, ConnView cv, double dt, double* __restrict__ res, double* __restrict__ resRelV,
                           double* __restrict__ resRelN, RowNorm* __restrict__ rn)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < b.nbI) cell_residual(b, cv, n, dt, res, resRelV, resRelN, rn + n);
}

// Global maxima with the reference's tie rule (the first cell in index order
// wins a tie: IsoT_FIM::CalRes keeps a maximum unless a later cell exceeds it).
// Value first, then the smaller cell index, so any order of combination gives
// the same result.
__device__ __forceinline__ bool norm_better(double v, int i, double bestv, int besti)
{
    return i >= 0 && (besti < 0 || v > bestv || (v == bestv && i < besti));
}

// Pass 1 (gridDim.x blocks): each block's maxima over a grid-stride share of
// the rows into out[blockIdx.x]; pass 2 (one block) over those partials.
__global__ void k_norm_reduce(const RowNorm* __restrict__ rn, int nb, RowNorm* __restrict__ out)
{
    __shared__ double sv[256], sn[256];
    __shared__ int iv[256], in_[256];
    double mv = 0, mN = 0;
    int bv = -1, bn = -1;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nb; n += gridDim.x * blockDim.x) {
        const RowNorm r = rn[n];
        if (norm_better(r.maxV, r.idV, mv, bv)) { mv = r.maxV; bv = r.idV; }
        if (norm_better(r.maxN, r.idN, mN, bn)) { mN = r.maxN; bn = r.idN; }
    }
    sv[threadIdx.x] = mv; iv[threadIdx.x] = bv;
    sn[threadIdx.x] = mN; in_[threadIdx.x] = bn;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            const int o = threadIdx.x + s;
            if (norm_better(sv[o], iv[o], sv[threadIdx.x], iv[threadIdx.x])) {
                sv[threadIdx.x] = sv[o]; iv[threadIdx.x] = iv[o];
            }
            if (norm_better(sn[o], in_[o], sn[threadIdx.x], in_[threadIdx.x])) {
                sn[threadIdx.x] = sn[o]; in_[threadIdx.x] = in_[o];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        RowNorm& o = out[blockIdx.x];
        if (gridDim.x > 1) {  // a partial: keep "none" as index -1
            o.maxV = sv[0]; o.idV = iv[0]; o.maxN = sn[0]; o.idN = in_[0];
        }
        else {
            o.maxV = iv[0] >= 0 ? sv[0] : 0.0; o.idV = iv[0] >= 0 ? iv[0] : 0;
            o.maxN = in_[0] >= 0 ? sn[0] : 0.0; o.idN = in_[0] >= 0 ? in_[0] : 0;
        }
    }
}

// The code path of a connection's blocks: per phase whether it flows (it
// exists in its upwind cell), whether the bId side is upwind, and whether the
// downwind cell holds the phase too (3 bits a phase).
constexpr int CONN_CLASSES = 512;
__device__ __forceinline__ int conn_class(const BulkView& b, const ConnView& cv, int c)
{
    const uint32_t bId = cv.bId[c], eId = cv.eId[c];
    int key = 0;
    for (int j = 0; j < b.np && j < 3; j++) {
        const uint32_t u = cv.upblock[j * cv.nconn + c];
        if (!b.phaseExist[b.idx(j, (int)u)]) continue;
        const uint32_t d = (u == bId) ? eId : bId;
        key |= (1 | ((u == bId) << 1) | ((b.phaseExist[b.idx(j, (int)d)] != 0) << 2)) << (3 * j);
    }
    return key;
}

// tiles of JAC_TILE connections (or incidence entries) per block, sorted by code path
constexpr int JAC_TILE = 4096;

// The connection blocks of a tile of JAC_TILE consecutive connections per
// block of 128 threads: the tile is first sorted by code path (tile_sort),
// then each warp takes 32 consecutive connections of the sorted tile, so its
// lanes take the same branches.  Every connection's blocks are computed by
// conn_jac_blocks as before; only which thread computes them changes.
template <int NCT>
__global__ void __launch_bounds__(128) k_jac_conn(const Model* __restrict__ M, BulkView b, ConnView cv, double dt,
                                                  double* __restrict__ bmat)
{
    __shared__ unsigned cnt[CONN_CLASSES];
    __shared__ unsigned short key_s[JAC_TILE];
    __shared__ unsigned short idx_s[JAC_TILE];
    const int c0 = blockIdx.x * JAC_TILE;
    const int n = min(JAC_TILE, cv.nconn - c0);
    tile_sort<CONN_CLASSES>(
        n, [&](int i) { return conn_class(b, cv, c0 + i); }, cnt, key_s, idx_s);
    const int bsize = (b.nc + 1) * (b.nc + 1);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int c = c0 + idx_s[i];
        conn_jac_blocks<NCT>(*M, b, cv, c, dt, bmat + (size_t)c * 2 * bsize, bmat + ((size_t)c * 2 + 1) * bsize);
    }
}

// The side blocks of the connections incident to the cells [c0, c1): the
// incidence entries row_conn[e0 .. e1) (e0 = row_ptr[c0], e1 = row_ptr[c1]),
// each the block k_jac_conn computes for that side, from a copy of the side
// cell's dSec_dPri at ds[k * soa + (cell - c0)].  Tiles of JAC_TILE entries,
// sorted by code path and side as k_jac_conn's are.
template <int NCT>
__global__ void __launch_bounds__(128) k_jac_side(const Model* __restrict__ M, BulkView b, ConnView cv, double dt,
                                                  int c0, uint32_t e0, uint32_t e1, const double* __restrict__ ds,
                                                  size_t soa, double* __restrict__ bmat)
{
    __shared__ unsigned cnt[2 * CONN_CLASSES];
    __shared__ unsigned short key_s[JAC_TILE];
    __shared__ unsigned short idx_s[JAC_TILE];
    const uint32_t t0 = e0 + blockIdx.x * JAC_TILE;
    const int n = (int)min((uint32_t)JAC_TILE, e1 - t0);
    tile_sort<2 * CONN_CLASSES>(
        n,
        [&](int i) {
            const uint32_t entry = cv.row_conn[t0 + i];
            return conn_class(b, cv, (int)(entry >> 1)) | (int)((entry & 1u) << 9);
        },
        cnt, key_s, idx_s);
    const int bsize = (b.nc + 1) * (b.nc + 1);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t entry = cv.row_conn[t0 + idx_s[i]];
        const int c = (int)(entry >> 1), side = (int)(entry & 1u);
        ConnPhase q;
        conn_phase(*M, b, cv, c, q);
        const int cell = side ? q.eId : q.bId;
        conn_jac_side<NCT>(b, q, side, ds + (cell - c0), soa, dt, bmat + ((size_t)c * 2 + side) * bsize);
    }
}

// one warp per Jacobian block row
__global__ void k_jac_rows(BulkView b, ConnView cv, const double* __restrict__ bmat, const uint32_t* __restrict__ rowptr,
                           double* __restrict__ val)
{
    const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r < b.nbI) row_assemble_warp(b, cv, (int)r, bmat, rowptr, val, threadIdx.x & 31);
}

// out[0]: OR of status bits, out[1]: two-phase cells, out[2]: flagged cells
__global__ void k_report(BulkView b, uint32_t* __restrict__ out)
{
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t st = 0, two = 0, fl = 0;
    if (cell < b.nb) {
        st = b.status[cell];
        two = (b.phaseExist[b.idx(0, cell)] && b.phaseExist[b.idx(1, cell)]) ? 1u : 0u;
        fl = st ? 1u : 0u;
    }
    const uint32_t sto = __reduce_or_sync(0xffffffffu, st);
    const uint32_t twos = __reduce_add_sync(0xffffffffu, two);
    const uint32_t fls = __reduce_add_sync(0xffffffffu, fl);
    if ((threadIdx.x & 31) == 0) {
        if (sto) atomicOr(out, sto);
        if (twos) atomicAdd(out + 1, twos);
        if (fls) atomicAdd(out + 2, fls);
    }
}

template <typename T>
__global__ void k_transpose(T* __restrict__ dst, const T* __restrict__ src, int n, int width, size_t N, size_t first,
                            bool to_soa)
{
    // entities [first, first + n) of an SoA array a[k * N + i] <-> an AoS
    // array of n entities; t runs over the strided side so that its accesses
    // are coalesced
    const size_t total = (size_t)n * width;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        if (to_soa) {
            const size_t k = t / n, i = t % n;
            dst[k * N + first + i] = src[i * width + k];
        }
        else {
            const size_t i = t / width, k = t % width;
            dst[t] = src[k * N + first + i];
        }
    }
}

static int grid_for(int n, int block) { return (n + block - 1) / block; }

cudaError_t launch_flash_bo(const Model* dm, const BulkView& b, int block, cudaStream_t s)
{
    if (b.nb) k_flash_bo<<<grid_for(b.nb, block), block, 0, s>>>(dm, b);
    return cudaGetLastError();
}
cudaError_t launch_krpc_rock(const Model* dm, const BulkView& b, int block, cudaStream_t s)
{
    if (b.nb) k_krpc_rock<<<grid_for(b.nb, block), block, 0, s>>>(dm, b);
    return cudaGetLastError();
}
cudaError_t launch_check(const BulkView& b, uint32_t* flags, int block, cudaStream_t s)
{
    if (b.nb) k_check<<<grid_for(b.nb, block), block, 0, s>>>(b, flags);
    return cudaGetLastError();
}
cudaError_t launch_newton_update(const BulkView& b, const double* u, double dSmax, int block, cudaStream_t s)
{
    if (b.nb) k_newton_update<<<grid_for(b.nb, block), block, 0, s>>>(b, u, dSmax);
    return cudaGetLastError();
}
cudaError_t launch_conn_flux(const Model* dm, const BulkView& b, const ConnView& cv, int block, cudaStream_t s)
{
    if (cv.nconn) k_conn_flux<<<grid_for(cv.nconn, block), block, 0, s>>>(dm, b, cv);
    return cudaGetLastError();
}
cudaError_t launch_residual(const BulkView& b, const ConnView& cv, double dt, double* res, double* resRelV,
                            double* resRelN, RowNorm* rn, RowNorm* rn_out, RowNorm* part, int block, cudaStream_t s)
{
    if (!b.nbI) return cudaSuccess;
    k_residual<<<grid_for(b.nbI, block), block, 0, s>>>(b, cv, dt, res, resRelV, resRelN, rn);
    if (rn_out) return launch_norm_reduce(rn, b.nbI, rn_out, part, s);
    return cudaGetLastError();
}
cudaError_t launch_norm_reduce(const RowNorm* rn, int nbI, RowNorm* rn_out, RowNorm* part, cudaStream_t s)
{
    if (!nbI) return cudaSuccess;
    const int g = std::min(NORM_PARTS, (nbI + 255) / 256);
    if (g > 1) {
        k_norm_reduce<<<g, 256, 0, s>>>(rn, nbI, part);
        k_norm_reduce<<<1, 256, 0, s>>>(part, g, rn_out);
    }
    else {
        k_norm_reduce<<<1, 256, 0, s>>>(rn, nbI, rn_out);
    }
    return cudaGetLastError();
}
cudaError_t launch_jac_conn(int nct, const Model* dm, const BulkView& b, const ConnView& cv, double dt, double* bmat,
                            int block, cudaStream_t s)
{
    if (!cv.nconn) return cudaSuccess;
    (void)block;  // tiles of JAC_TILE connections on 128 threads
    const int g = (cv.nconn + JAC_TILE - 1) / JAC_TILE;
    switch (nct) {
    case 3: k_jac_conn<3><<<g, 128, 0, s>>>(dm, b, cv, dt, bmat); break;
    case 5: k_jac_conn<5><<<g, 128, 0, s>>>(dm, b, cv, dt, bmat); break;
    case 7: k_jac_conn<7><<<g, 128, 0, s>>>(dm, b, cv, dt, bmat); break;
    case 9: k_jac_conn<9><<<g, 128, 0, s>>>(dm, b, cv, dt, bmat); break;
    case 11: k_jac_conn<11><<<g, 128, 0, s>>>(dm, b, cv, dt, bmat); break;
    case 13: k_jac_conn<13><<<g, 128, 0, s>>>(dm, b, cv, dt, bmat); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
cudaError_t launch_jac_side(int nct, const Model* dm, const BulkView& b, const ConnView& cv, double dt, int c0,
                            uint32_t e0, uint32_t e1, const double* ds, size_t soa, double* bmat, int block,
                            cudaStream_t s)
{
    if (e1 <= e0) return cudaSuccess;
    (void)block;  // tiles of JAC_TILE entries on 128 threads
    const int g = (int)((e1 - e0 + JAC_TILE - 1) / JAC_TILE);
    switch (nct) {
    case 3: k_jac_side<3><<<g, 128, 0, s>>>(dm, b, cv, dt, c0, e0, e1, ds, soa, bmat); break;
    case 5: k_jac_side<5><<<g, 128, 0, s>>>(dm, b, cv, dt, c0, e0, e1, ds, soa, bmat); break;
    case 7: k_jac_side<7><<<g, 128, 0, s>>>(dm, b, cv, dt, c0, e0, e1, ds, soa, bmat); break;
    case 9: k_jac_side<9><<<g, 128, 0, s>>>(dm, b, cv, dt, c0, e0, e1, ds, soa, bmat); break;
    case 11: k_jac_side<11><<<g, 128, 0, s>>>(dm, b, cv, dt, c0, e0, e1, ds, soa, bmat); break;
    case 13: k_jac_side<13><<<g, 128, 0, s>>>(dm, b, cv, dt, c0, e0, e1, ds, soa, bmat); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
cudaError_t launch_jac_rows(const BulkView& b, const ConnView& cv, const double* bmat, const uint32_t* rowptr,
                            double* val, int block, cudaStream_t s)
{
    const int wpb = block / 32;  // rows per block
    if (b.nbI) k_jac_rows<<<(b.nbI + wpb - 1) / wpb, block, 0, s>>>(b, cv, bmat, rowptr, val);
    return cudaGetLastError();
}
// Work level of a predicted work w >= 1: floor(4 log2 w), at most 63 (levels
// are 19 % apart and reach 2^15.75 work units).
__device__ __forceinline__ int cost_level(long long w)
{
    const int l = (int)(4.0f * __log2f((float)w));
    return l < 0 ? 0 : (l > 63 ? 63 : l);
}

// The flash type a cell's flash starts from (SkipPSAMethod01::CalFtype02 /
// IfSkip on the current state: 1 skips the equilibrium, 2 goes to the split,
// 0 runs the stability test) and the work the cell is predicted to need: the
// work its last flash used on the segments this type runs (none when it
// skips, the split's when it goes to the split, all otherwise).  A cell whose
// skip test fails now runs the equilibrium its flag promised to spare.
__device__ long long predicted_work_now(const Model& M, const BulkView& b, int cell, int& ftype_in, unsigned& npPE)
{
    const CompModel& m = M.comp;
    const int NC = m.nc, np = b.np;
    double Ni[NC_MAX + 1], Sin[3];
    for (int i = 0; i <= NC; i++) Ni[i] = b.Ni[b.idx(i, cell)];
    unsigned phaseNum = 0;
    for (int j = 0; j < np; j++) {
        Sin[j] = b.S[b.idx(j, cell)];
        if (b.phaseExist[b.idx(j, cell)]) phaseNum++;
    }
    double Nt = 0;
    for (int i = 0; i < NC; i++) Nt += Ni[i];
    const double P = b.P[cell], T = b.T[cell] + M.units.conv4;
    npPE = phaseNum - 1u;
    ftype_in = flash_type_in(m, b, cell, Ni, Nt, P, T, Sin, npPE);
    if (ftype_in == 1) return 3;
    const int32_t* it = b.iters;
    if (ftype_in == 2)
        return 3LL + WORK_SSM_SP * (long long)it[b.idx(2, cell)] + WORK_NR_SP * (long long)it[b.idx(3, cell)] +
               it[b.idx(4, cell)] / 5;
    return predicted_work(b, cell);
}

// Sort key of a cell for the batched flash: its class by the flash type it
// starts from (cells that skip the equilibrium; cells that go to the split and
// the two-phase derivatives; cells that run the stability test), then its
// predicted work level (predicted_work_now), in descending order.  Warps then
// hold cells on the same code path with similar work.
__device__ __forceinline__ int cost_bucket(const Model& M, const BulkView& b, int cell)
{
    int ftype_in;
    unsigned npPE;
    const int lvl = cost_level(predicted_work_now(M, b, cell, ftype_in, npPE));
    const int cls = ftype_in == 1 ? 2 : (ftype_in == 2 ? 0 : 1);
    return cls * 64 + (63 - lvl);
}

__global__ void k_cost_hist(const Model* __restrict__ M, BulkView b, unsigned* __restrict__ hist)
{
    __shared__ unsigned h[COST_BUCKETS];
    for (int k = threadIdx.x; k < COST_BUCKETS; k += blockDim.x) h[k] = 0;
    __syncthreads();
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell < b.nb) atomicAdd(&h[cost_bucket(*M, b, cell)], 1u);
    __syncthreads();
    for (int k = threadIdx.x; k < COST_BUCKETS; k += blockDim.x)
        if (h[k]) atomicAdd(&hist[k], h[k]);
}

// Exclusive scan of the bucket counts, in place (one block of COST_BUCKETS
// threads).  Also the adaptive work level, written to level[0].  It is 0 (no
// floor) unless more than coop_cells cells lie at or above the level of the
// deferral threshold `wt`; then it is the lowest level L such that at most
// coop_cells cells have a predicted level >= L.  The cooperative kernel then
// gets about that many cells even when most cells of the workload are
// expensive, and is left alone when only a tail of cells is.
__global__ void k_cost_scan(unsigned* __restrict__ hist, unsigned coop_cells, long long wt, int* __restrict__ level)
{
    __shared__ unsigned v[COST_BUCKETS];
    const int t = threadIdx.x;
    v[t] = hist[t];
    __syncthreads();
    if (t == 0) {
        int L = 0;
        unsigned above = 0;
        if (coop_cells)
            for (int l = 63; l >= cost_level(wt + 1); l--)
                for (int cls = 0; cls < COST_BUCKETS / 64; cls++) above += v[cls * 64 + (63 - l)];
        if (above > coop_cells) {
            unsigned cum = 0;
            L = 64;
            for (int l = 63; l >= 0; l--) {
                unsigned tot = 0;
                for (int cls = 0; cls < COST_BUCKETS / 64; cls++) tot += v[cls * 64 + (63 - l)];
                if (cum + tot > coop_cells) break;
                cum += tot;
                L = l;
            }
        }
        level[0] = L;
    }
    __syncthreads();
    for (int d = 1; d < COST_BUCKETS; d <<= 1) {
        const unsigned add = t >= d ? v[t - d] : 0u;
        __syncthreads();
        v[t] += add;
        __syncthreads();
    }
    hist[t] = v[t] - hist[t];
}

__global__ void k_cost_scatter(const Model* __restrict__ M, BulkView b, unsigned* __restrict__ offs,
                               int* __restrict__ order)
{
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= b.nb) return;
    const unsigned pos = atomicAdd(&offs[cost_bucket(*M, b, cell)], 1u);
    order[pos] = cell;
}

cudaError_t launch_cost_order(const Model* dm, const BulkView& b, unsigned* hist, int* order, unsigned coop_cells,
                              long long wt, int* level, cudaStream_t s)
{
    if (!b.nb) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(unsigned) * COST_BUCKETS, s);
    if (e != cudaSuccess) return e;
    const int block = 256;
    k_cost_hist<<<grid_for(b.nb, block), block, 0, s>>>(dm, b, hist);
    k_cost_scan<<<1, COST_BUCKETS, 0, s>>>(hist, coop_cells, wt, level);
    k_cost_scatter<<<grid_for(b.nb, block), block, 0, s>>>(dm, b, hist, order);
    return cudaGetLastError();
}

// Cells predicted to need more than `threshold` work units
// (predicted_work_now), and whose work level is at or above the adaptive
// level, are handed to the cooperative kernel before the per-cell kernel
// runs, so that both run at the same time (pre[cell] = 1).  Cells that the
// skip test will let through (flash type 1) stay with the per-cell kernel.  Thread q visits the q-th cell
// of the cost order taken level by level (all classes of the highest level
// first), so the list comes out roughly heaviest first whatever the class, and
// the cooperative warps, which take list slots in order, start with the
// longest cells.  bucket_end: the end of each cost bucket in the order.
__global__ void k_predefer(const Model* __restrict__ M, BulkView b, const int* __restrict__ order,
                           const unsigned* __restrict__ bucket_end, long long threshold,
                           const int* __restrict__ level, DeferSink sink, uint8_t* __restrict__ pre)
{
    constexpr int NCLS = COST_BUCKETS / 64;
    __shared__ unsigned cnt[COST_BUCKETS];
    __shared__ unsigned lstart[64];  // level-major position of level l's first cell
    for (int k = threadIdx.x; k < COST_BUCKETS; k += blockDim.x)
        cnt[k] = bucket_end[k] - (k ? bucket_end[k - 1] : 0u);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned acc = 0;
        for (int l = 63; l >= 0; l--) {
            lstart[l] = acc;
            for (int c = 0; c < NCLS; c++) acc += cnt[c * 64 + (63 - l)];
        }
    }
    __syncthreads();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= b.nb) return;
    // the level holding position q: the lowest l with lstart[l] <= q
    // (lstart falls as l rises)
    int lo = 0, hi = 63;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (lstart[mid] <= (unsigned)q) hi = mid;
        else lo = mid + 1;
    }
    unsigned r = (unsigned)q - lstart[lo];
    int p = -1;
    for (int c = 0; c < NCLS; c++) {
        const int k = c * 64 + (63 - lo);
        if (r < cnt[k]) { p = (int)(bucket_end[k] - cnt[k] + r); break; }
        r -= cnt[k];
    }
    if (p < 0) return;  // not reached: the buckets hold every cell once
    const int cell = order[p];
    pre[cell] = 0;
    int ftype_in;
    unsigned npPE;
    const long long w = predicted_work_now(*M, b, cell, ftype_in, npPE);
    if (w <= threshold || cost_level(w) < level[0]) return;
    if (ftype_in == 1) return;
    if (sink.push(cell, ftype_in, npPE)) pre[cell] = 1;
}

cudaError_t launch_predefer(const Model* dm, const BulkView& b, const int* order, const unsigned* bucket_end,
                            long long threshold, const int* level, const DeferSink& sink, uint8_t* pre,
                            cudaStream_t s)
{
    if (b.nb)
        k_predefer<<<grid_for(b.nb, 128), 128, 0, s>>>(dm, b, order, bucket_end, threshold, level, sink, pre);
    return cudaGetLastError();
}

__global__ void k_jt_lambda(BulkView b, ConnView cv, const uint32_t* __restrict__ rowptr,
                            const double* __restrict__ val, const uint32_t* __restrict__ slot,
                            const double* __restrict__ lam, double* __restrict__ out)
{
    const int dim = b.nc + 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)b.nb * dim) return;
    jt_lambda_entry(b, cv, rowptr, val, slot, lam, out, (int)(t / dim), (int)(t % dim));
}

__global__ void k_vjp_trans(BulkView b, ConnView cv, double dt, const double* __restrict__ lam, double* __restrict__ out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < cv.nconn) out[c] = vjp_trans_conn(b, cv, dt, lam, c);
}

__global__ void k_vjp_poro(const Model* __restrict__ M, BulkView b, const double* __restrict__ lam,
                           double* __restrict__ out)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < b.nb) out[n] = vjp_poro_cell(*M, b, lam, n);
}

cudaError_t launch_jt_lambda(const BulkView& b, const ConnView& cv, const uint32_t* rowptr, const double* val,
                             const uint32_t* slot, const double* lam, double* out, int block, cudaStream_t s)
{
    const long long n = (long long)b.nb * (b.nc + 1);
    if (n) k_jt_lambda<<<(int)((n + block - 1) / block), block, 0, s>>>(b, cv, rowptr, val, slot, lam, out);
    return cudaGetLastError();
}
cudaError_t launch_vjp_trans(const BulkView& b, const ConnView& cv, double dt, const double* lam, double* out,
                             int block, cudaStream_t s)
{
    if (cv.nconn) k_vjp_trans<<<grid_for(cv.nconn, block), block, 0, s>>>(b, cv, dt, lam, out);
    return cudaGetLastError();
}
cudaError_t launch_vjp_poro(const Model* dm, const BulkView& b, const double* lam, double* out, int block,
                            cudaStream_t s)
{
    if (b.nb) k_vjp_poro<<<grid_for(b.nb, block), block, 0, s>>>(dm, b, lam, out);
    return cudaGetLastError();
}

cudaError_t launch_report(const BulkView& b, uint32_t* out3, int block, cudaStream_t s)
{
    if (b.nb) k_report<<<grid_for(b.nb, block), block, 0, s>>>(b, out3);
    return cudaGetLastError();
}
cudaError_t launch_transpose(void* dst, const void* src, int n, int width, int elem_bytes, bool to_soa,
                             cudaStream_t s, size_t N, size_t first)
{
    const size_t total = (size_t)n * width;
    if (!total) return cudaSuccess;
    if (N == 0) N = (size_t)n;
    const int block = 256;
    const int grid = (int)((total + block - 1) / block < 4096 ? (total + block - 1) / block : 4096);
    switch (elem_bytes) {
    case 1: k_transpose<uint8_t><<<grid, block, 0, s>>>((uint8_t*)dst, (const uint8_t*)src, n, width, N, first, to_soa); break;
    case 4: k_transpose<uint32_t><<<grid, block, 0, s>>>((uint32_t*)dst, (const uint32_t*)src, n, width, N, first, to_soa); break;
    case 8: k_transpose<double><<<grid, block, 0, s>>>((double*)dst, (const double*)src, n, width, N, first, to_soa); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace ocpx
