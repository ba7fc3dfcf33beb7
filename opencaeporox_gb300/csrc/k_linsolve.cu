// Linear solve of the Newton system on the device: J u = rhs with the
// assembled block-CSR Jacobian (bulk rows) and the residual vector the
// reference hands to its solver (LinearSystem::CopyRhs of -R), by BiCGStab
// with right block-Jacobi preconditioning.
//
// The reference passes this system to an external solver (FASP, PETSc or
// PARDISO through src/LinearSystem.cpp:35-89); none of those is part of the
// reference's own sources.  This is a device solver of the same system,
// checked against a direct solve.
//
// Every reduction runs on a fixed grid with a fixed tree, so the iterates are
// reproducible from run to run.  The scalars of the method stay in device
// memory; the host reads the residual norm only every few iterations.
#include "ocpx_kernels.h"

namespace ocpx {

namespace {

constexpr int LS_THREADS = 256;
constexpr int MAXD = NCT_MAX + 1;   // largest block dimension

// Gauss-Jordan inverse of each diagonal block (the first block of each row),
// partial pivoting; a zero pivot sets flag[0].
__global__ void k_block_inv(const uint32_t* __restrict__ rowptr, const double* __restrict__ val, int nb, int dim,
                            double* __restrict__ dinv, unsigned* __restrict__ flag)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nb) return;
    const int bs = dim * dim;
    double a[MAXD * MAXD], x[MAXD * MAXD];
    const double* blk = val + (size_t)rowptr[r] * bs;
    for (int q = 0; q < bs; q++) { a[q] = blk[q]; x[q] = 0; }
    for (int i = 0; i < dim; i++) x[i * dim + i] = 1;
    for (int c = 0; c < dim; c++) {
        int piv = c;
        double best = fabs(a[c * dim + c]);
        for (int i = c + 1; i < dim; i++)
            if (fabs(a[i * dim + c]) > best) { best = fabs(a[i * dim + c]); piv = i; }
        if (!(best > 0)) { atomicOr(flag, 1u); return; }
        if (piv != c)
            for (int j = 0; j < dim; j++) {
                double t = a[c * dim + j]; a[c * dim + j] = a[piv * dim + j]; a[piv * dim + j] = t;
                t = x[c * dim + j]; x[c * dim + j] = x[piv * dim + j]; x[piv * dim + j] = t;
            }
        const double inv = 1.0 / a[c * dim + c];
        for (int j = 0; j < dim; j++) { a[c * dim + j] *= inv; x[c * dim + j] *= inv; }
        for (int i = 0; i < dim; i++) {
            if (i == c) continue;
            const double f = a[i * dim + c];
            if (f == 0) continue;
            for (int j = 0; j < dim; j++) {
                a[i * dim + j] -= f * a[c * dim + j];
                x[i * dim + j] -= f * x[c * dim + j];
            }
        }
    }
    double* out = dinv + (size_t)r * bs;
    for (int q = 0; q < bs; q++) out[q] = x[q];
}

// y = J x: one thread per (row, component)
__global__ void k_spmv(const uint32_t* __restrict__ rowptr, const uint32_t* __restrict__ col,
                       const double* __restrict__ val, int nb, int dim, const double* __restrict__ x,
                       double* __restrict__ y)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nb * dim) return;
    const int r = (int)(t / dim), i = (int)(t % dim);
    const int bs = dim * dim;
    double acc = 0;
    for (uint32_t k = rowptr[r]; k < rowptr[r + 1]; k++) {
        const double* brow = val + (size_t)k * bs + (size_t)i * dim;
        const double* xc = x + (size_t)col[k] * dim;
        for (int j = 0; j < dim; j++) acc = fma(brow[j], xc[j], acc);
    }
    y[t] = acc;
}

// y = D^{-1} x
__global__ void k_bdiag(const double* __restrict__ dinv, int nb, int dim, const double* __restrict__ x,
                        double* __restrict__ y)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nb * dim) return;
    const int r = (int)(t / dim), i = (int)(t % dim);
    const double* d = dinv + (size_t)r * dim * dim + (size_t)i * dim;
    const double* xr = x + (size_t)r * dim;
    double acc = 0;
    for (int j = 0; j < dim; j++) acc = fma(d[j], xr[j], acc);
    y[t] = acc;
}

__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double s[LS_THREADS];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int w = LS_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    const double r = s[0];
    __syncthreads();
    return r;
}

// partial[b] = sum over this block's grid-stride share of a.b
__global__ void __launch_bounds__(LS_THREADS) k_dot_part(const double* __restrict__ a, const double* __restrict__ b,
                                                         long long n, double* __restrict__ partial)
{
    double acc = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        acc = fma(a[t], b[t], acc);
    const double s = block_sum(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void __launch_bounds__(LS_THREADS) k_dot_final(const double* __restrict__ partial, int np_,
                                                          double* __restrict__ out)
{
    double acc = 0;
    for (int k = threadIdx.x; k < np_; k += blockDim.x) acc += partial[k];
    const double s = block_sum(acc);
    if (threadIdx.x == 0) *out = s;
}

// scalar slots of the method
enum { S_RHO, S_RHO_OLD, S_ALPHA, S_OMEGA, S_BETA, S_RV, S_TS, S_TT, S_RR, S_BB, S_FLAG, S_COUNT };

// p = r + beta (p - omega v); beta from rho / rho_old and alpha / omega (p = r at the start)
__global__ void k_update_p(double* __restrict__ S, int first, const double* __restrict__ r, double* __restrict__ p,
                           const double* __restrict__ v, long long n)
{
    double beta = 0;
    if (!first) beta = (S[S_RHO] / S[S_RHO_OLD]) * (S[S_ALPHA] / S[S_OMEGA]);
    const double omega = S[S_OMEGA];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = first ? r[t] : r[t] + beta * (p[t] - omega * v[t]);
}

// s = r - alpha v, alpha = rho / (rhat . v)
__global__ void k_update_s(const double* __restrict__ S, const double* __restrict__ r, const double* __restrict__ v,
                           double* __restrict__ s, long long n)
{
    const double alpha = S[S_RHO] / S[S_RV];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) s[t] = r[t] - alpha * v[t];
}

// x += alpha phat + omega shat; r = s - omega t, omega = (t . s) / (t . t)
__global__ void k_update_xr(const double* __restrict__ S, double* __restrict__ x, const double* __restrict__ phat,
                            const double* __restrict__ shat, const double* __restrict__ s, const double* __restrict__ tv,
                            double* __restrict__ r, long long n)
{
    const double alpha = S[S_RHO] / S[S_RV];
    const double omega = S[S_TT] > 0 ? S[S_TS] / S[S_TT] : 0.0;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        x[t] = x[t] + alpha * phat[t] + omega * shat[t];
        r[t] = s[t] - omega * tv[t];
    }
}

// end of an iteration: keep alpha, omega, rho for the next beta
__global__ void k_scalars_end(double* __restrict__ S)
{
    S[S_ALPHA] = S[S_RHO] / S[S_RV];
    S[S_OMEGA] = S[S_TT] > 0 ? S[S_TS] / S[S_TT] : 0.0;
    S[S_RHO_OLD] = S[S_RHO];
    if (!(S[S_RV] != 0) || !(S[S_OMEGA] != 0)) S[S_FLAG] = 1;  // breakdown
}

inline int grid_n(long long n) { return (int)((n + LS_THREADS - 1) / LS_THREADS); }

}  // namespace

constexpr int LS_DOT_BLOCKS = 608;

size_t linsolve_scratch_doubles(int nb, int dim)
{
    const size_t n = (size_t)nb * dim;
    return 8 * n + (size_t)nb * dim * dim + LS_DOT_BLOCKS + S_COUNT + 1;
}

cudaError_t linsolve(const uint32_t* rowptr, const uint32_t* col, const double* val, int nb, int dim,
                     const double* rhs, double* x, double* scratch, double tol, int maxit, int check_every,
                     LinsolveResult* res, uint64_t* launches, cudaStream_t s)
{
    const long long n = (long long)nb * dim;
    double* r = scratch;
    double* rhat = r + n;
    double* p = rhat + n;
    double* v = p + n;
    double* sv = v + n;
    double* tv = sv + n;
    double* phat = tv + n;
    double* shat = phat + n;
    double* dinv = shat + n;
    double* partial = dinv + (size_t)nb * dim * dim;
    double* S = partial + LS_DOT_BLOCKS;
    unsigned* flag = reinterpret_cast<unsigned*>(S + S_COUNT);
    cudaError_t e;
    uint64_t nl = 0;
    auto dot = [&](const double* a, const double* b, double* out) {
        k_dot_part<<<LS_DOT_BLOCKS, LS_THREADS, 0, s>>>(a, b, n, partial);
        k_dot_final<<<1, LS_THREADS, 0, s>>>(partial, LS_DOT_BLOCKS, out);
        nl += 2;
    };
    if ((e = cudaMemsetAsync(S, 0, sizeof(double) * (S_COUNT + 1), s)) != cudaSuccess) return e;
    k_block_inv<<<grid_n(nb), LS_THREADS, 0, s>>>(rowptr, val, nb, dim, dinv, flag);
    nl++;
    // x = 0, r = rhat = rhs
    if ((e = cudaMemsetAsync(x, 0, sizeof(double) * n, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(r, rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(rhat, rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    dot(rhs, rhs, S + S_BB);
    double host[S_COUNT + 1];
    if ((e = cudaMemcpyAsync(host, S, sizeof(host), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    const double bb = host[S_BB];
    res->iterations = 0;
    res->relres = 0;
    res->converged = 0;
    res->breakdown = 0;
    if (reinterpret_cast<unsigned*>(&host[S_COUNT])[0]) { res->breakdown = 2; *launches += nl; return cudaSuccess; }
    if (!(bb > 0)) { res->converged = 1; *launches += nl; return cudaSuccess; }
    const int gn = grid_n(n);
    for (int it = 0; it < maxit; it++) {
        dot(rhat, r, S + S_RHO);
        k_update_p<<<gn, LS_THREADS, 0, s>>>(S, it == 0, r, p, v, n);
        k_bdiag<<<gn, LS_THREADS, 0, s>>>(dinv, nb, dim, p, phat);
        k_spmv<<<gn, LS_THREADS, 0, s>>>(rowptr, col, val, nb, dim, phat, v);
        dot(rhat, v, S + S_RV);
        k_update_s<<<gn, LS_THREADS, 0, s>>>(S, r, v, sv, n);
        k_bdiag<<<gn, LS_THREADS, 0, s>>>(dinv, nb, dim, sv, shat);
        k_spmv<<<gn, LS_THREADS, 0, s>>>(rowptr, col, val, nb, dim, shat, tv);
        dot(tv, sv, S + S_TS);
        dot(tv, tv, S + S_TT);
        k_update_xr<<<gn, LS_THREADS, 0, s>>>(S, x, phat, shat, sv, tv, r, n);
        k_scalars_end<<<1, 1, 0, s>>>(S);
        nl += 8;
        const bool check = (it + 1) % check_every == 0 || it + 1 == maxit;
        if (!check) continue;
        dot(r, r, S + S_RR);
        if ((e = cudaMemcpyAsync(host, S, sizeof(host), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        res->iterations = it + 1;
        res->relres = sqrt(host[S_RR] / bb);
        if (host[S_FLAG] != 0) { res->breakdown = 1; break; }
        if (res->relres <= tol) { res->converged = 1; break; }
    }
    *launches += nl;
    return cudaGetLastError();
}

}  // namespace ocpx
