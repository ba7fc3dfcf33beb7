/* BLAS/LAPACK entry points the reference declares (include/DenseMat.hpp:43-125),
 * forwarded to the scipy_-prefixed symbols of SciPy's bundled OpenBLAS
 * (LP64, reference LAPACK 3.x semantics).  Harness code for the oracle build:
 * the reference itself pins LAPACK 3.11.0 and recommends MKL, so results may
 * differ from an MKL build in the last bits. */
#include <stddef.h>

void scipy_dscal_(const int*, const double*, double*, const int*);
double scipy_ddot_(const int*, const double*, const int*, const double*, const int*);
void scipy_dcopy_(const int*, const double*, const int*, double*, const int*);
void scipy_daxpy_(const int*, const double*, const double*, const int*, double*, const int*);
double scipy_dnrm2_(const int*, const double*, const int*);
double scipy_dasum_(const int*, const double*, const int*);
void scipy_dgemm_(const char*, const char*, const int*, const int*, const int*, const double*,
                  const double*, const int*, const double*, const int*, const double*, double*,
                  const int*, size_t, size_t);
void scipy_dgesv_(const int*, const int*, double*, const int*, int*, double*, const int*, int*);
void scipy_dsysv_(const char*, const int*, const int*, double*, const int*, int*, double*,
                  const int*, double*, const int*, int*, size_t);
void scipy_ssyevd_(const char*, const char*, const int*, float*, const int*, float*, float*,
                   const int*, int*, const int*, int*, size_t, size_t);

void dscal_(const int* n, const double* a, double* x, const int* incx) { scipy_dscal_(n, a, x, incx); }
double ddot_(const int* n, double* a, const int* ia, double* b, const int* ib) { return scipy_ddot_(n, a, ia, b, ib); }
int dcopy_(const int* n, const double* x, const int* ix, double* y, const int* iy) { scipy_dcopy_(n, x, ix, y, iy); return 0; }
int daxpy_(const int* n, const double* a, const double* x, const int* ix, double* y, const int* iy)
{ scipy_daxpy_(n, a, x, ix, y, iy); return 0; }
double dnrm2_(const int* n, double* x, const int* ix) { return scipy_dnrm2_(n, x, ix); }
double dasum_(const int* n, double* x, const int* ix) { return scipy_dasum_(n, x, ix); }
int dgemm_(const char* ta, const char* tb, const int* m, const int* n, const int* k, const double* al,
           const double* A, const int* lda, const double* B, const int* ldb, const double* be,
           double* C, const int* ldc)
{ scipy_dgemm_(ta, tb, m, n, k, al, A, lda, B, ldb, be, C, ldc, 1, 1); return 0; }
void dgesv_(const int* n, const int* nrhs, double* A, const int* lda, int* piv, double* b,
            const int* ldb, int* info)
{ scipy_dgesv_(n, nrhs, A, lda, piv, b, ldb, info); }
void dsysv_(const char* uplo, const int* n, const int* nrhs, double* A, const int* lda, int* piv,
            double* b, const int* ldb, double* work, const int* lwork, int* info)
{ scipy_dsysv_(uplo, n, nrhs, A, lda, piv, b, ldb, work, lwork, info, 1); }
void ssyevd_(const char* jobz, const char* uplo, const int* n, float* A, const int* lda, float* w,
             float* work, const int* lwork, int* iwork, const int* liwork, int* info)
{ scipy_ssyevd_(jobz, uplo, n, A, lda, w, work, lwork, iwork, liwork, info, 1, 1); }
