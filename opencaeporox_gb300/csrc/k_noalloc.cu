// Relative-residual norms without any allocation: the "Calculate RelRes" loop
// of IsoT_FIM::CalRes (src/IsoThermalMethod.cpp:1147-1167) over a residual
// that is already on the device, with its reduction scratch in a fixed,
// file-scope device array instead of memory the caller or the library
// allocates.
//
// Scratch (g_relres_scratch, 256-byte aligned, about 24 KB):
//   * per-block partial maxima (value, cell) for the volume and the
//     component norms, OCPX_RELRES_NOALLOC_MAX_BLOCKS entries each;
//   * `done`, the count of blocks that have stored their partials.  It must
//     be zero when a call starts: it is zero-initialised when the module is
//     loaded, and the last block of every call sets it back to zero after it
//     has read the partials.  A call that fails to launch leaves it zero.
//     Nothing else needs an initial value: every partial a call reads was
//     written earlier in the same call.
// One block covers RELRES_CELLS_PER_BLOCK cells, so the scratch bounds the
// grid size: nb above OCPX_RELRES_NOALLOC_MAX_CELLS is rejected.
//
// All calls in a process share the one scratch per device: two calls whose
// kernels overlap in time (different streams, different host threads, or a
// stream that does not order them) race on it and give wrong results.
// Callers serialise the calls, e.g. by issuing them on one stream.
#include <cuda_runtime.h>

#include "ocpx.h"

namespace {

constexpr int RELRES_THREADS = 256;
constexpr int RELRES_CELLS_PER_THREAD = 8;
constexpr int RELRES_CELLS_PER_BLOCK = RELRES_THREADS * RELRES_CELLS_PER_THREAD;
static_assert((long long)OCPX_RELRES_NOALLOC_MAX_BLOCKS * RELRES_CELLS_PER_BLOCK == OCPX_RELRES_NOALLOC_MAX_CELLS,
              "the header's cell limit must match the scratch size");

struct RelresScratch {
    double maxV[OCPX_RELRES_NOALLOC_MAX_BLOCKS];
    double maxN[OCPX_RELRES_NOALLOC_MAX_BLOCKS];
    int idV[OCPX_RELRES_NOALLOC_MAX_BLOCKS];
    int idN[OCPX_RELRES_NOALLOC_MAX_BLOCKS];
    ocpx_norms out;
    unsigned int done;
};

static __device__ __align__(256) RelresScratch g_relres_scratch;

// (v, id) beats (w, jd): larger value, or equal value and lower cell index;
// id < 0 marks "no value above zero yet" (the reference starts its maxima at
// 0 with a strict "<", so a cell whose terms are all zero never becomes the
// maximum).
__device__ __forceinline__ bool beats(double v, int id, double w, int jd)
{
    return id >= 0 && (jd < 0 || v > w || (v == w && id < jd));
}

__global__ void __launch_bounds__(RELRES_THREADS)
k_relres_noalloc(const double* __restrict__ res, const double* __restrict__ rockVp, const double* __restrict__ Nt,
                 int nb, int len, double* __restrict__ resRelV, double* __restrict__ resRelN)
{
    RelresScratch& s = g_relres_scratch;
    __shared__ double sv[RELRES_THREADS], sn[RELRES_THREADS];
    __shared__ int iv[RELRES_THREADS], in_[RELRES_THREADS];
    __shared__ bool last;
    double mv = 0, mN = 0;
    int bv = -1, bn = -1;
    const int first = blockIdx.x * RELRES_CELLS_PER_BLOCK + threadIdx.x;
    // each thread visits its cells in increasing index order, so a strict ">"
    // keeps the first cell of equal maxima, as the reference's loop does
    for (int k = 0; k < RELRES_CELLS_PER_THREAD; k++) {
        const int n = first + k * RELRES_THREADS;
        if (n >= nb) break;
        const double* r = res + (size_t)n * len;
        const double vp = rockVp[n], nt = Nt[n];
        double sV = 0, sN = 0;
        for (int i = 0; i < len; i++) {
            const double t = fabs(r[i] / vp);
            if (mv < t) { mv = t; bv = n; }
            sV += t * t;
        }
        for (int i = 1; i < len; i++) {
            const double t = fabs(r[i] / nt);
            if (mN < t) { mN = t; bn = n; }
            sN += t * t;
        }
        resRelV[n] = sqrt(sV);
        resRelN[n] = sqrt(sN);
    }
    sv[threadIdx.x] = mv; iv[threadIdx.x] = bv;
    sn[threadIdx.x] = mN; in_[threadIdx.x] = bn;
    __syncthreads();
    for (int h = RELRES_THREADS / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            const int o = threadIdx.x + h;
            if (beats(sv[o], iv[o], sv[threadIdx.x], iv[threadIdx.x])) { sv[threadIdx.x] = sv[o]; iv[threadIdx.x] = iv[o]; }
            if (beats(sn[o], in_[o], sn[threadIdx.x], in_[threadIdx.x])) { sn[threadIdx.x] = sn[o]; in_[threadIdx.x] = in_[o]; }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        s.maxV[blockIdx.x] = sv[0]; s.idV[blockIdx.x] = iv[0];
        s.maxN[blockIdx.x] = sn[0]; s.idN[blockIdx.x] = in_[0];
        __threadfence();
        last = atomicAdd(&s.done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // the last block to finish combines the partials of all blocks
    __threadfence();
    mv = 0; mN = 0; bv = -1; bn = -1;
    for (int g = threadIdx.x; g < (int)gridDim.x; g += RELRES_THREADS) {
        const double v = __ldcg(&s.maxV[g]), w = __ldcg(&s.maxN[g]);
        const int a = __ldcg(&s.idV[g]), c = __ldcg(&s.idN[g]);
        if (beats(v, a, mv, bv)) { mv = v; bv = a; }
        if (beats(w, c, mN, bn)) { mN = w; bn = c; }
    }
    sv[threadIdx.x] = mv; iv[threadIdx.x] = bv;
    sn[threadIdx.x] = mN; in_[threadIdx.x] = bn;
    __syncthreads();
    for (int h = RELRES_THREADS / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            const int o = threadIdx.x + h;
            if (beats(sv[o], iv[o], sv[threadIdx.x], iv[threadIdx.x])) { sv[threadIdx.x] = sv[o]; iv[threadIdx.x] = iv[o]; }
            if (beats(sn[o], in_[o], sn[threadIdx.x], in_[threadIdx.x])) { sn[threadIdx.x] = sn[o]; in_[threadIdx.x] = in_[o]; }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        s.out.maxRelRes_V = iv[0] >= 0 ? sv[0] : 0.0;
        s.out.maxId_V = iv[0] >= 0 ? iv[0] : 0;
        s.out.maxRelRes_N = in_[0] >= 0 ? sn[0] : 0.0;
        s.out.maxId_N = in_[0] >= 0 ? in_[0] : 0;
        s.done = 0;  // ready for the next call
    }
}

// Device address of the scratch in the current device's context, looked up on
// every call: the lookup allocates nothing and is cheap, and an address kept
// from an earlier call could be stale after the context was torn down and the
// module loaded again (cudaDeviceReset).
cudaError_t scratch_address(RelresScratch** out)
{
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_relres_scratch);
    if (e != cudaSuccess) return e;
    *out = static_cast<RelresScratch*>(p);
    return cudaSuccess;
}

}  // namespace

extern "C" ocpx_status ocpx_relres_noalloc(const double* d_res, const double* d_rockVp, const double* d_Nt, int nb,
                                           int len, double* d_resRelV, double* d_resRelN, void* stream,
                                           ocpx_norms* norms)
{
    if (!d_res || !d_rockVp || !d_Nt || !d_resRelV || !d_resRelN || !norms) return OCPX_INVALID_ARG;
    if (nb <= 0 || nb > OCPX_RELRES_NOALLOC_MAX_CELLS || len < 2) return OCPX_INVALID_ARG;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return OCPX_NO_DEVICE;
    RelresScratch* scratch = nullptr;
    if (scratch_address(&scratch) != cudaSuccess) return OCPX_CUDA_ERROR;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int blocks = (nb + RELRES_CELLS_PER_BLOCK - 1) / RELRES_CELLS_PER_BLOCK;
    k_relres_noalloc<<<blocks, RELRES_THREADS, 0, s>>>(d_res, d_rockVp, d_Nt, nb, len, d_resRelV, d_resRelN);
    if (cudaGetLastError() != cudaSuccess) return OCPX_CUDA_ERROR;
    if (cudaMemcpyAsync(norms, &scratch->out, sizeof(ocpx_norms), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return OCPX_CUDA_ERROR;
    if (cudaStreamSynchronize(s) != cudaSuccess) return OCPX_CUDA_ERROR;
    return OCPX_OK;
}
