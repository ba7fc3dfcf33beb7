// Register/local-memory dense solvers for the per-cell NC x NC systems.
//
// The reference calls LAPACK: dsysv_ ('U', Bunch-Kaufman) for the stability
// and split Newton systems (src/OCPPhaseEquilibrium.cpp:493, 835 via
// src/DenseMat.cpp:107-123) and dgesv_ for the derivative system with NC+1
// right-hand sides (src/OCPMixtureMethodComp.cpp:488 via src/DenseMat.cpp:88-105),
// and ssyevd_ (FP32) for the minimum eigenvalue in the skip test
// (src/AcceleratePEC.cpp:156, src/DenseMat.cpp:126-145).
//
// Here: Gaussian elimination with partial pivoting (Doolittle order, the
// textbook algorithm), and a cyclic Jacobi eigen-solver.  Results agree with
// LAPACK to rounding, not bitwise.  As in LAPACK, a zero pivot leaves the
// right-hand side untouched and is reported.
#pragma once
#include "ocpx_common.cuh"

namespace ocpx {

// Factorise row-major A (n x n) in place with partial pivoting; piv[k] is the
// row swapped with row k.  Returns false on an exactly zero pivot.
template <int NM>
OCPX_HD_NOINLINE bool lu_factor(int n, double* A, int* piv)
{
    for (int k = 0; k < n; k++) {
        int p = k;
        double amax = fabs(A[k * NM + k]);
        for (int r = k + 1; r < n; r++) {
            const double a = fabs(A[r * NM + k]);
            if (a > amax) { amax = a; p = r; }
        }
        piv[k] = p;
        if (A[p * NM + k] == 0.0) return false;
        if (p != k)
            for (int c = 0; c < n; c++) { const double t = A[k * NM + c]; A[k * NM + c] = A[p * NM + c]; A[p * NM + c] = t; }
        const double inv = 1.0 / A[k * NM + k];
        for (int r = k + 1; r < n; r++) {
            const double l = A[r * NM + k] * inv;
            A[r * NM + k] = l;
            for (int c = k + 1; c < n; c++) A[r * NM + c] -= l * A[k * NM + c];
        }
    }
    return true;
}

// Solve with the factors; b is one column of length n.
template <int NM>
OCPX_HD_NOINLINE void lu_apply(int n, const double* A, const int* piv, double* b)
{
    // rows were swapped in full during the factorisation, so every
    // interchange is applied before the forward substitution (as dgetrs does)
    for (int k = 0; k < n; k++) {
        const int p = piv[k];
        if (p != k) { const double t = b[k]; b[k] = b[p]; b[p] = t; }
    }
    for (int k = 0; k < n; k++)
        for (int r = k + 1; r < n; r++) b[r] -= A[r * NM + k] * b[k];
    for (int k = n - 1; k >= 0; k--) {
        double v = b[k];
        for (int c = k + 1; c < n; c++) v -= A[k * NM + c] * b[c];
        b[k] = v / A[k * NM + k];
    }
}

// dsysv_('U', ...) semantics on a row-major buffer J (leading dimension n, as
// the reference stores it): LAPACK reads the column-major upper triangle,
// i.e. the row-major lower triangle J[max(a,b)*n + min(a,b)], and treats the
// matrix as symmetric.  Solves in place in b.  Returns false if singular
// (b unchanged).
template <int NM>
OCPX_HD bool sym_lower_solve(int n, const double* J, double* b, double* work)
{
    int piv[NM];
    for (int a = 0; a < n; a++)
        for (int c = 0; c < n; c++) work[a * NM + c] = (a >= c) ? J[a * n + c] : J[c * n + a];
    if (!lu_factor<NM>(n, work, piv)) return false;
    lu_apply<NM>(n, work, piv, b);
    return true;
}

// dgesv_ semantics: A column-major n x n given as the reference's buffer
// (A(r,c) = Abuf[c*n + r]), nrhs right-hand sides stored column after column
// (B(r,k) = B[k*n + r]).  Solves in place.  Returns false if singular.
template <int NM>
OCPX_HD bool gen_solve_colmajor(int n, const double* Abuf, double* B, int nrhs, double* work)
{
    int piv[NM];
    for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) work[r * NM + c] = Abuf[c * n + r];
    if (!lu_factor<NM>(n, work, piv)) return false;
    for (int k = 0; k < nrhs; k++) lu_apply<NM>(n, work, piv, B + k * n);
    return true;
}

// Smallest eigenvalue of a symmetric matrix given in single precision (the
// reference builds the skip-test matrix as float and calls ssyevd_, which
// works in single precision).  Cyclic Jacobi in single precision: on GB300
// the FP32 pipe issues 64 times the FP64 rate, and the skip test's tolerance
// is set by FP32 anyway.  The sweep count is capped.
template <int NM>
OCPX_HD_NOINLINE float sym_min_eig_f32(int n, const float* Af, float* A)
{
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) A[i * NM + j] = Af[i * n + j];
    for (int sweep = 0; sweep < 30; sweep++) {
        float off = 0, diag = 0;
        for (int i = 0; i < n; i++) {
            diag += A[i * NM + i] * A[i * NM + i];
            for (int j = i + 1; j < n; j++) off += A[i * NM + j] * A[i * NM + j];
        }
        if (off <= 1e-13f * diag || off == 0.0f) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                const float apq = A[p * NM + q];
                if (apq == 0.0f) continue;
                const float app = A[p * NM + p], aqq = A[q * NM + q];
                const float theta = (aqq - app) / (2.0f * apq);
                const float t = (theta >= 0 ? 1.0f : -1.0f) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
                const float c = 1.0f / sqrtf(t * t + 1.0f);
                const float s = t * c;
                for (int k = 0; k < n; k++) {
                    const float akp = A[k * NM + p], akq = A[k * NM + q];
                    A[k * NM + p] = c * akp - s * akq;
                    A[k * NM + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    const float apk = A[p * NM + k], aqk = A[q * NM + k];
                    A[p * NM + k] = c * apk - s * aqk;
                    A[q * NM + k] = s * apk + c * aqk;
                }
            }
    }
    float mn = A[0];
    for (int i = 1; i < n; i++) mn = A[i * NM + i] < mn ? A[i * NM + i] : mn;
    return mn;
}

}  // namespace ocpx
