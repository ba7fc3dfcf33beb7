// Newton-iteration and time-step control of a FIM run, bulk part, on the
// device.
//
// Reference: OCPNRsuite::InitStep / CalMaxChangeNR / CalMaxChangeTime
// (src/OCPNRsuite.cpp:70-232), ControlNR::CheckConverge
// (src/OCPControlNR.cpp:27-77), ControlTime::CalNextTimeStep
// (src/OCPControlTime.cpp:128-178).
//
// The maxima are signed: the reference keeps the value whose magnitude is
// largest, replacing it only when a later entry is strictly larger in
// magnitude, so the first entry in its loop order wins a tie and zeros never
// replace the initial 0.  Each entry here carries its position in that order
// (cell-major, then component or phase), and the reduction keeps the
// largest magnitude with the smallest position; it is associative and
// commutative, so the result is the reference's exactly whatever the
// reduction tree.  The per-cell change arrays the reference also stores (dP,
// dN, ...) are not kept: nothing on the FIM path reads them.
#include "ocpx_kernels.h"

namespace ocpx {

namespace {

struct Cand {
    double v;
    long long key;
};

// a and b: candidates, key < 0 meaning none (the reference's initial 0).  A
// selected candidate is always nonzero and not NaN (the reference never
// replaces its running value with those); among the rest the largest
// magnitude wins, then the smallest position.
__device__ __forceinline__ Cand pick(Cand a, Cand b)
{
    if (b.key < 0 || !(fabs(b.v) > 0)) return a;
    if (a.key < 0) return b;
    const double fa = fabs(a.v), fb = fabs(b.v);
    if (fb > fa) return b;
    if (fb == fa && b.key < a.key) return b;
    return a;
}

__device__ __forceinline__ Cand none() { return Cand{0.0, -1}; }

constexpr int NQ = 5;            // dP, dT, dN, dS, eV
constexpr int RED_THREADS = 256;

__device__ __forceinline__ void block_reduce(Cand (&c)[NQ], Cand* __restrict__ out)
{
    __shared__ double sv[NQ][RED_THREADS];
    __shared__ long long sk[NQ][RED_THREADS];
    const int t = threadIdx.x;
    for (int q = 0; q < NQ; q++) { sv[q][t] = c[q].v; sk[q][t] = c[q].key; }
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if (t < s)
            for (int q = 0; q < NQ; q++) {
                const Cand r = pick(Cand{sv[q][t], sk[q][t]}, Cand{sv[q][t + s], sk[q][t + s]});
                sv[q][t] = r.v;
                sk[q][t] = r.key;
            }
        __syncthreads();
    }
    if (t == 0)
        for (int q = 0; q < NQ; q++) out[q] = Cand{sv[q][0], sk[q][0]};
}

// MODE 0: CalMaxChangeNR against the last Newton iterate (lP, lT, lN, lS),
// which is then replaced by the current state.  MODE 1: CalMaxChangeTime
// against the last time step (lP, lT, lS and b.lNi).
template <int MODE>
__global__ void __launch_bounds__(RED_THREADS) k_max_change(BulkView b, double* __restrict__ lP,
                                                           double* __restrict__ lT, double* __restrict__ lN,
                                                           double* __restrict__ lS, Cand* __restrict__ partial)
{
    Cand c[NQ];
    for (int q = 0; q < NQ; q++) c[q] = none();
    const int nc = b.nc, np = b.np;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < b.nbI; n += gridDim.x * blockDim.x) {
        const double P = b.P[n], T = b.T[n];
        c[0] = pick(c[0], Cand{P - lP[n], n});
        c[1] = pick(c[1], Cand{T - lT[n], n});
        if (MODE == 0) {
            double Nt = 0;
            for (int i = 0; i < nc; i++) Nt += lN[b.idx(i, n)];
            for (int i = 0; i < nc; i++) {
                const double Ni = b.Ni[b.idx(i, n)];
                c[2] = pick(c[2], Cand{(Ni - lN[b.idx(i, n)]) / Nt, (long long)n * nc + i});
                lN[b.idx(i, n)] = Ni;
            }
        }
        else {
            for (int i = 0; i < nc; i++) {
                const double Ni = b.Ni[b.idx(i, n)], l = b.lNi[b.idx(i, n)];
                const double tmp = fabs(Ni < l ? l : Ni);  // fabs(std::max(Ni, lNi))
                if (tmp > 1e-8) c[2] = pick(c[2], Cand{(Ni - l) / tmp, (long long)n * nc + i});
            }
        }
        for (int j = 0; j < np; j++) {
            const double S = b.S[b.idx(j, n)];
            c[3] = pick(c[3], Cand{S - lS[b.idx(j, n)], (long long)n * np + j});
            if (MODE == 0) lS[b.idx(j, n)] = S;
        }
        c[4] = pick(c[4], Cand{(b.vf[n] - b.rockVp[n]) / b.rockVp[n], n});
        if (MODE == 0) { lP[n] = P; lT[n] = T; }
    }
    block_reduce(c, partial + (size_t)blockIdx.x * NQ);
}

__global__ void __launch_bounds__(RED_THREADS) k_max_change_final(const Cand* __restrict__ partial, int nblocks,
                                                                 double* __restrict__ out)
{
    Cand c[NQ];
    for (int q = 0; q < NQ; q++) c[q] = none();
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x)
        for (int q = 0; q < NQ; q++) c[q] = pick(c[q], partial[(size_t)k * NQ + q]);
    __shared__ Cand res[NQ];
    block_reduce(c, res);
    __syncthreads();
    if (threadIdx.x == 0)
        for (int q = 0; q < NQ; q++) out[q] = res[q].v;
}

// the reference's std::min(a, b) and std::max(a, b)
__device__ __forceinline__ double smin(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return a < b ? b : a; }

__global__ void k_nr_converge(NRControl c, const double* __restrict__ nr, const RowNorm* __restrict__ norm,
                              const double* __restrict__ res0, const double* __restrict__ wellrel,
                              int* __restrict__ state)
{
    const double V = c.res_from_host ? c.maxRelRes_V : norm->maxV;
    const double N = c.res_from_host ? c.maxRelRes_N : norm->maxN;
    const double V0 = c.res_from_host ? c.maxRelRes0_V : *res0;
    // the wells' rate equations: the device's own residual when it holds the wells
    const double W = (!c.res_from_host && wellrel) ? *wellrel : c.maxWellRelRes_mol;
    const double tmpfac = 1.0;
    bool conv = false;
    // "res"
    if ((V <= V0 * c.tol * tmpfac || V <= c.tol * tmpfac || N <= c.tol * tmpfac) &&
        W <= c.tol * tmpfac)
        conv = true;
    // "d": DPBmaxNRc, DSmaxNRc
    if (fabs(nr[0]) <= c.dPmin && fabs(nr[3]) <= c.dSmin) conv = true;
    *state = conv ? 0 : (c.iterNR >= c.maxIter ? 2 : 1);
}

__global__ void k_next_dt(NRControl c, const double* __restrict__ ts, double* __restrict__ out)
{
    const double current_time = c.current_time + c.current_dt;
    double factor = c.maxIncreFac;
    // CalMaxChangeTime: the bulk maximum unless a well's is larger in magnitude
    const double dPmaxT = fabs(ts[0]) < fabs(c.dPWmaxT) ? c.dPWmaxT : ts[0];
    const double dPmax = fabs(dPmaxT);
    const double dSmax = fabs(ts[3]);
    const double tiny = 1e-8;
    if (dPmax > tiny) factor = smin(factor, c.dPlim / dPmax);
    if (dSmax > tiny) factor = smin(factor, c.dSlim / dSmax);
    if (c.iterNR < 5)
        factor = smin(factor, 2.0);
    else if (c.iterNR > 10)
        factor = smin(factor, 0.5);
    else
        factor = smin(factor, 1.5);
    factor = smax(c.minChopFac, factor);
    double dt = c.current_dt * factor;
    if (dt > c.timeMax) dt = c.timeMax;
    if (dt < c.timeMin) dt = c.timeMin;
    const double predict = dt;
    if (dt > (c.end_time - current_time)) dt = (c.end_time - current_time);
    out[0] = dt;
    out[1] = predict;
}

}  // namespace

int max_change_blocks(int nb)
{
    const int g = (nb + RED_THREADS - 1) / RED_THREADS;
    return g < 1 ? 1 : (g > MAX_CHANGE_BLOCKS ? MAX_CHANGE_BLOCKS : g);
}

cudaError_t launch_max_change(int mode, const BulkView& b, double* lP, double* lT, double* lN, double* lS,
                              void* partial, double* out5, cudaStream_t s)
{
    const int g = max_change_blocks(b.nbI);
    Cand* part = static_cast<Cand*>(partial);
    if (mode == 0)
        k_max_change<0><<<g, RED_THREADS, 0, s>>>(b, lP, lT, lN, lS, part);
    else
        k_max_change<1><<<g, RED_THREADS, 0, s>>>(b, lP, lT, lN, lS, part);
    k_max_change_final<<<1, RED_THREADS, 0, s>>>(part, g, out5);
    return cudaGetLastError();
}

cudaError_t launch_nr_converge(const NRControl& c, const double* nr5, const RowNorm* norm, const double* res0,
                               const double* wellrel, int* state, cudaStream_t s)
{
    k_nr_converge<<<1, 1, 0, s>>>(c, nr5, norm, res0, wellrel, state);
    return cudaGetLastError();
}

cudaError_t launch_next_dt(const NRControl& c, const double* ts5, double* out2, cudaStream_t s)
{
    k_next_dt<<<1, 1, 0, s>>>(c, ts5, out2);
    return cudaGetLastError();
}

}  // namespace ocpx
