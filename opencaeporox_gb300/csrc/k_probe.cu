// FP64 throughput probe: the denominator of the flash kernel's roofline.
// The measured-peaks file of this platform lists HBM bandwidth and bf16
// tensor throughput only, so the FP64 peak is measured here with a kernel of
// independent fused multiply-add chains (8 per thread, no memory traffic).
#include <cuda_runtime.h>
#include "ocpx.h"

namespace {

__global__ void k_dfma_chain(double* out, int iters, double a, double b)
{
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-9, x2 = x0 + 2e-9, x3 = x0 + 3e-9;
    double x4 = x0 + 4e-9, x5 = x0 + 5e-9, x6 = x0 + 6e-9, x7 = x0 + 7e-9;
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace

extern "C" ocpx_status ocpx_measure_fp64_tflops(int device, int iters, double* tflops)
{
    if (!tflops || iters <= 0) return OCPX_INVALID_ARG;
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return OCPX_NO_DEVICE;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return OCPX_CUDA_ERROR;
    const int block = 256, grid = sms * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_dfma_chain<<<grid, block>>>(out, iters / 10 + 1, 0.9999999, 1e-7);  // warm-up
    cudaEventRecord(e0);
    k_dfma_chain<<<grid, block>>>(out, iters, 0.9999999, 1e-7);
    cudaEventRecord(e1);
    const cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0) return OCPX_CUDA_ERROR;
    const double flops = 2.0 * 8.0 * (double)iters * (double)grid * (double)block;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return OCPX_OK;
}
