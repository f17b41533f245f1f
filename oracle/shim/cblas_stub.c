/* Row-major GEMMs behind the CBLAS prototypes of the reference's own
 * src/common/cblas.h (plain triple loops, double accumulation), plus
 * aborting stand-ins for the LAPACK routines that only non-hot helpers of
 * src/common/blas_lapack.c reference.  Oracle build only. */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>

#define CBLAS_INT int
#include "cblas.h"

static int tr(CBLAS_TRANSPOSE t) { return t == CblasNoTrans ? 0 : (t == CblasTrans ? 1 : 2); }

#define GEMM_BODY(T, ACC)                                                                   \
    for (int i = 0; i < M; ++i)                                                            \
        for (int j = 0; j < N; ++j)                                                        \
        {                                                                                  \
            ACC acc = 0;                                                                   \
            for (int k = 0; k < K; ++k)                                                    \
            {                                                                              \
                T a = ta == 0 ? A[(size_t)i * lda + k] : A[(size_t)k * lda + i];           \
                T b = tb == 0 ? B[(size_t)k * ldb + j] : B[(size_t)j * ldb + k];           \
                if (ta == 2) a = CONJ(a);                                                  \
                if (tb == 2) b = CONJ(b);                                                  \
                acc += a * b;                                                              \
            }                                                                              \
            T* c = C + (size_t)i * ldc + j;                                                \
            *c = (beta == 0) ? (T)(alpha * acc) : (T)(alpha * acc + beta * (*c));          \
        }

void cblas_zgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE TransA, CBLAS_TRANSPOSE TransB, const CBLAS_INT M,
                 const CBLAS_INT N, const CBLAS_INT K, const void* alphap, const void* Ap, const CBLAS_INT lda,
                 const void* Bp, const CBLAS_INT ldb, const void* betap, void* Cp, const CBLAS_INT ldc)
{
    if (layout != CblasRowMajor) abort();
    const double _Complex alpha = *(const double _Complex*)alphap, beta = *(const double _Complex*)betap;
    const double _Complex* A = Ap;
    const double _Complex* B = Bp;
    double _Complex* C = Cp;
    int ta = tr(TransA), tb = tr(TransB);
#define CONJ conj
    GEMM_BODY(double _Complex, double _Complex)
#undef CONJ
}

void cblas_cgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE TransA, CBLAS_TRANSPOSE TransB, const CBLAS_INT M,
                 const CBLAS_INT N, const CBLAS_INT K, const void* alphap, const void* Ap, const CBLAS_INT lda,
                 const void* Bp, const CBLAS_INT ldb, const void* betap, void* Cp, const CBLAS_INT ldc)
{
    if (layout != CblasRowMajor) abort();
    const float _Complex alpha = *(const float _Complex*)alphap, beta = *(const float _Complex*)betap;
    const float _Complex* A = Ap;
    const float _Complex* B = Bp;
    float _Complex* C = Cp;
    int ta = tr(TransA), tb = tr(TransB);
#define CONJ conjf
    GEMM_BODY(float _Complex, float _Complex)
#undef CONJ
}

void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE TransA, CBLAS_TRANSPOSE TransB, const CBLAS_INT M,
                 const CBLAS_INT N, const CBLAS_INT K, const double alpha, const double* A, const CBLAS_INT lda,
                 const double* B, const CBLAS_INT ldb, const double beta, double* C, const CBLAS_INT ldc)
{
    if (layout != CblasRowMajor) abort();
    int ta = tr(TransA), tb = tr(TransB);
#define CONJ(x) (x)
    GEMM_BODY(double, double)
#undef CONJ
}

void cblas_sgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE TransA, CBLAS_TRANSPOSE TransB, const CBLAS_INT M,
                 const CBLAS_INT N, const CBLAS_INT K, const float alpha, const float* A, const CBLAS_INT lda,
                 const float* B, const CBLAS_INT ldb, const float beta, float* C, const CBLAS_INT ldc)
{
    if (layout != CblasRowMajor) abort();
    int ta = tr(TransA), tb = tr(TransB);
#define CONJ(x) (x)
    GEMM_BODY(float, float)
#undef CONJ
}

