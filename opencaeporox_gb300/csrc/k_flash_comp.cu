// Compositional FlashDer kernels, compiled once per component capacity
// (OCPX_NCM) so each build carries arrays sized for its component count.
#include "ocpx_kernels.h"
#include "flash_comp.cuh"

#ifndef OCPX_NCM
#error "compile with -DOCPX_NCM=<capacity>"
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

// Work-queue variant: each warp lane claims cells from a global counter in
// chunks of `chunk` consecutive cells until the grid is exhausted.  The loop
// is bounded by the number of cells.
template <int NCM>
__global__ void __launch_bounds__(128) k_flash_comp_queue(const Model* __restrict__ M, BulkView b,
                                                          unsigned* __restrict__ counter, int chunk)
{
    const int lane = threadIdx.x & 31;
    while (true) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(counter, 32u * (unsigned)chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (unsigned)b.nb) break;
        for (int k = 0; k < chunk; k++) {
            const unsigned cell = base + (unsigned)k * 32u + (unsigned)lane;
            if (cell < (unsigned)b.nb) {
                CompCellUpdate<NCM> u;
                u.run(*M, b, (int)cell);
            }
        }
    }
}

#define OCPX_CAT2(a, b) a##b
#define OCPX_CAT(a, b) OCPX_CAT2(a, b)

cudaError_t OCPX_CAT(launch_flash_comp_, OCPX_NCM)(const Model* dm, const BulkView& b, int block, cudaStream_t s)
{
    if (b.nb == 0) return cudaSuccess;
    const int grid = (b.nb + block - 1) / block;
    k_flash_comp<OCPX_NCM><<<grid, block, 0, s>>>(dm, b);
    return cudaGetLastError();
}

cudaError_t OCPX_CAT(launch_flash_comp_queue_, OCPX_NCM)(const Model* dm, const BulkView& b, unsigned* counter,
                                                         int grid, int block, int chunk, cudaStream_t s)
{
    if (b.nb == 0) return cudaSuccess;
    k_flash_comp_queue<OCPX_NCM><<<grid, block, 0, s>>>(dm, b, counter, chunk);
    return cudaGetLastError();
}

}  // namespace ocpx
