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
// memory, and so does the convergence test: every few iterations a one-thread
// kernel compares the residual norm with the tolerance and, once the solve
// has converged or broken down, sets a stop flag that makes every later
// kernel of the solve return at once.  The synchronous form reads that flag
// at each test and stops enqueuing; the enqueue-only form (linsolve_async)
// enqueues all maxit iterations and never waits, so it can be captured in a
// CUDA graph.  Both run the same arithmetic and leave the same result.
#include "ocpx_kernels.h"

namespace ocpx {

namespace {

constexpr int LS_THREADS = 256;
constexpr int MAXD = NCT_MAX + 1;   // largest block dimension

// scalar slots of the method; S_DONE: 0 running, 1 converged, 2 BiCGStab
// breakdown, 3 a singular diagonal block; S_ITERS / S_RELRES: iterations and
// relative residual at the last test
enum { S_RHO, S_RHO_OLD, S_ALPHA, S_OMEGA, S_BETA, S_RV, S_TS, S_TT, S_RR, S_BB, S_FLAG, S_DONE, S_ITERS, S_RELRES,
       S_COUNT };

__device__ __forceinline__ bool stopped(const double* S) { return S[S_DONE] != 0; }

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
                       double* __restrict__ y, const double* __restrict__ S)
{
    if (stopped(S)) return;
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
                        double* __restrict__ y, const double* __restrict__ S)
{
    if (stopped(S)) return;
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
                                                         long long n, double* __restrict__ partial,
                                                         const double* __restrict__ S)
{
    if (stopped(S)) return;   // the same for every thread of the block
    double acc = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        acc = fma(a[t], b[t], acc);
    const double s = block_sum(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void __launch_bounds__(LS_THREADS) k_dot_final(const double* __restrict__ partial, int np_,
                                                          double* __restrict__ out, const double* __restrict__ S)
{
    if (stopped(S)) return;
    double acc = 0;
    for (int k = threadIdx.x; k < np_; k += blockDim.x) acc += partial[k];
    const double s = block_sum(acc);
    if (threadIdx.x == 0) *out = s;
}


// p = r + beta (p - omega v); beta from rho / rho_old and alpha / omega (p = r at the start)
__global__ void k_update_p(double* __restrict__ S, int first, const double* __restrict__ r, double* __restrict__ p,
                           const double* __restrict__ v, long long n)
{
    if (stopped(S)) return;
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
    if (stopped(S)) return;
    const double alpha = S[S_RHO] / S[S_RV];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) s[t] = r[t] - alpha * v[t];
}

// x += alpha phat + omega shat; r = s - omega t, omega = (t . s) / (t . t)
__global__ void k_update_xr(const double* __restrict__ S, double* __restrict__ x, const double* __restrict__ phat,
                            const double* __restrict__ shat, const double* __restrict__ s, const double* __restrict__ tv,
                            double* __restrict__ r, long long n)
{
    if (stopped(S)) return;
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
    if (stopped(S)) return;
    S[S_ALPHA] = S[S_RHO] / S[S_RV];
    S[S_OMEGA] = S[S_TT] > 0 ? S[S_TS] / S[S_TT] : 0.0;
    S[S_RHO_OLD] = S[S_RHO];
    if (!(S[S_RV] != 0) || !(S[S_OMEGA] != 0)) S[S_FLAG] = 1;  // breakdown
}

// before the first iteration: a singular diagonal block, or a zero
// right-hand side (solved by u = 0)
__global__ void k_start(double* __restrict__ S, const unsigned* __restrict__ singular)
{
    if (*singular) S[S_DONE] = 3;
    else if (!(S[S_BB] > 0)) S[S_DONE] = 1;
}

// the convergence test after `iters` iterations (S_RR = r.r just computed)
__global__ void k_test(double* __restrict__ S, double tol, int iters)
{
    if (stopped(S)) return;
    const double relres = sqrt(S[S_RR] / S[S_BB]);
    S[S_ITERS] = iters;
    S[S_RELRES] = relres;
    if (S[S_FLAG] != 0) S[S_DONE] = 2;
    else if (relres <= tol) S[S_DONE] = 1;
}

inline int grid_n(long long n) { return (int)((n + LS_THREADS - 1) / LS_THREADS); }

}  // namespace

constexpr int LS_DOT_BLOCKS = 608;

size_t linsolve_scratch_doubles(int nb, int dim)
{
    const size_t n = (size_t)nb * dim;
    return 8 * n + (size_t)nb * dim * dim + LS_DOT_BLOCKS + S_COUNT + 1;
}

namespace {

struct Work {
    double *r, *rhat, *p, *v, *sv, *tv, *phat, *shat, *dinv, *partial, *S;
    unsigned* singular;
};

Work carve(double* scratch, int nb, int dim)
{
    const long long n = (long long)nb * dim;
    Work w;
    w.r = scratch;
    w.rhat = w.r + n;
    w.p = w.rhat + n;
    w.v = w.p + n;
    w.sv = w.v + n;
    w.tv = w.sv + n;
    w.phat = w.tv + n;
    w.shat = w.phat + n;
    w.dinv = w.shat + n;
    w.partial = w.dinv + (size_t)nb * dim * dim;
    w.S = w.partial + LS_DOT_BLOCKS;
    w.singular = reinterpret_cast<unsigned*>(w.S + S_COUNT);
    return w;
}

// The solve's launches: set-up, then the iterations with a convergence test
// every check_every of them (and after the last).  With host_check, the
// stop flag is read at each test and enqueuing ends once it is set;
// otherwise all maxit iterations are enqueued and the host never waits.
cudaError_t run(const uint32_t* rowptr, const uint32_t* col, const double* val, int nb, int dim, const double* rhs,
                double* x, double* scratch, double tol, int maxit, int check_every, bool host_check,
                uint64_t* launches, cudaStream_t s)
{
    const long long n = (long long)nb * dim;
    const Work w = carve(scratch, nb, dim);
    double* S = w.S;
    cudaError_t e;
    uint64_t nl = 0;
    auto dot = [&](const double* a, const double* b, double* out) {
        k_dot_part<<<LS_DOT_BLOCKS, LS_THREADS, 0, s>>>(a, b, n, w.partial, S);
        k_dot_final<<<1, LS_THREADS, 0, s>>>(w.partial, LS_DOT_BLOCKS, out, S);
        nl += 2;
    };
    if ((e = cudaMemsetAsync(S, 0, sizeof(double) * (S_COUNT + 1), s)) != cudaSuccess) return e;
    k_block_inv<<<grid_n(nb), LS_THREADS, 0, s>>>(rowptr, val, nb, dim, w.dinv, w.singular);
    // x = 0, r = rhat = rhs
    if ((e = cudaMemsetAsync(x, 0, sizeof(double) * n, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(w.r, rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(w.rhat, rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    dot(rhs, rhs, S + S_BB);
    k_start<<<1, 1, 0, s>>>(S, w.singular);
    nl += 2;
    double done = 0;
    if (host_check) {
        if ((e = cudaMemcpyAsync(&done, S + S_DONE, sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    }
    const int gn = grid_n(n);
    for (int it = 0; it < maxit && done == 0; it++) {
        dot(w.rhat, w.r, S + S_RHO);
        k_update_p<<<gn, LS_THREADS, 0, s>>>(S, it == 0, w.r, w.p, w.v, n);
        k_bdiag<<<gn, LS_THREADS, 0, s>>>(w.dinv, nb, dim, w.p, w.phat, S);
        k_spmv<<<gn, LS_THREADS, 0, s>>>(rowptr, col, val, nb, dim, w.phat, w.v, S);
        dot(w.rhat, w.v, S + S_RV);
        k_update_s<<<gn, LS_THREADS, 0, s>>>(S, w.r, w.v, w.sv, n);
        k_bdiag<<<gn, LS_THREADS, 0, s>>>(w.dinv, nb, dim, w.sv, w.shat, S);
        k_spmv<<<gn, LS_THREADS, 0, s>>>(rowptr, col, val, nb, dim, w.shat, w.tv, S);
        dot(w.tv, w.sv, S + S_TS);
        dot(w.tv, w.tv, S + S_TT);
        k_update_xr<<<gn, LS_THREADS, 0, s>>>(S, x, w.phat, w.shat, w.sv, w.tv, w.r, n);
        k_scalars_end<<<1, 1, 0, s>>>(S);
        nl += 8;
        const bool check = (it + 1) % check_every == 0 || it + 1 == maxit;
        if (!check) continue;
        dot(w.r, w.r, S + S_RR);
        k_test<<<1, 1, 0, s>>>(S, tol, it + 1);
        nl++;
        if (!host_check) continue;
        if ((e = cudaMemcpyAsync(&done, S + S_DONE, sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    }
    *launches += nl;
    return cudaGetLastError();
}

}  // namespace

cudaError_t linsolve_read(const double* scratch, int nb, int dim, LinsolveResult* res, cudaStream_t s)
{
    const Work w = carve(const_cast<double*>(scratch), nb, dim);
    double host[S_COUNT];
    cudaError_t e;
    if ((e = cudaMemcpyAsync(host, w.S, sizeof(host), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    const int done = (int)host[S_DONE];
    res->iterations = (int)host[S_ITERS];
    res->relres = host[S_RELRES];
    res->converged = done == 1;
    res->breakdown = done == 2 ? 1 : (done == 3 ? 2 : 0);
    return cudaSuccess;
}

cudaError_t linsolve(const uint32_t* rowptr, const uint32_t* col, const double* val, int nb, int dim,
                     const double* rhs, double* x, double* scratch, double tol, int maxit, int check_every,
                     LinsolveResult* res, uint64_t* launches, cudaStream_t s)
{
    cudaError_t e = run(rowptr, col, val, nb, dim, rhs, x, scratch, tol, maxit, check_every, true, launches, s);
    if (e != cudaSuccess) return e;
    return linsolve_read(scratch, nb, dim, res, s);
}

cudaError_t linsolve_async(const uint32_t* rowptr, const uint32_t* col, const double* val, int nb, int dim,
                           const double* rhs, double* x, double* scratch, double tol, int maxit, int check_every,
                           uint64_t* launches, cudaStream_t s)
{
    return run(rowptr, col, val, nb, dim, rhs, x, scratch, tol, maxit, check_every, false, launches, s);
}

}  // namespace ocpx
