// Host-side launcher declarations shared by the C-ABI translation unit and
// the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include "bulk_view.cuh"
#include "conn_ops.cuh"

namespace ocpx {

// capacities the compositional kernels are compiled for (EoS components)
constexpr int kNcmCaps[] = {4, 6, 8, 10, 12};
// capacities of the Jacobian connection kernel (components incl. water)
constexpr int kNctCaps[] = {3, 5, 7, 9, 11, 13};

// Compositional FlashDer for cells [0, nb): one thread per cell.
cudaError_t launch_flash_comp(int ncm, const Model* dm, const BulkView& b, int block, cudaStream_t s);
// Persistent work-queue variant: cells are claimed from a global counter in
// chunks, so warps that finish cheap cells pick up new ones while others are
// still iterating.
cudaError_t launch_flash_comp_queue(int ncm, const Model* dm, const BulkView& b, unsigned* counter, int grid,
                                    int block, int chunk, cudaStream_t s);

cudaError_t launch_flash_bo(const Model* dm, const BulkView& b, int block, cudaStream_t s);
cudaError_t launch_krpc_rock(const Model* dm, const BulkView& b, int block, cudaStream_t s);
cudaError_t launch_check(const BulkView& b, uint32_t* flags, int block, cudaStream_t s);
cudaError_t launch_newton_update(const BulkView& b, const double* u, double dSmax, int block, cudaStream_t s);
cudaError_t launch_conn_flux(const Model* dm, const BulkView& b, const ConnView& cv, int block, cudaStream_t s);
cudaError_t launch_residual(const BulkView& b, const ConnView& cv, double dt, double* res, double* resRelV,
                            double* resRelN, RowNorm* rn, RowNorm* rn_out, int block, cudaStream_t s);
cudaError_t launch_jac_conn(int nct, const Model* dm, const BulkView& b, const ConnView& cv, double dt,
                            double* bmat, int block, cudaStream_t s);
cudaError_t launch_jac_rows(const BulkView& b, const ConnView& cv, const double* bmat, const uint32_t* rowptr,
                            double* val, int block, cudaStream_t s);
cudaError_t launch_report(const BulkView& b, uint32_t* out3, int block, cudaStream_t s);

// layout conversion between the reference's cell-major arrays and the
// device structure-of-arrays: dst[k*n + i] = src[i*width + k] (to_soa) and back
cudaError_t launch_transpose(void* dst, const void* src, int n, int width, int elem_bytes, bool to_soa,
                             cudaStream_t s);

}  // namespace ocpx
