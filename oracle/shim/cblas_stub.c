/* Row-major GEMMs behind the CBLAS prototypes of the reference's own
 * src/common/cblas.h, plus aborting stand-ins for the LAPACK routines that
 * only non-hot helpers of src/common/blas_lapack.c reference.  Oracle build
 * only.
 *
 * By default the GEMMs are plain triple loops (deterministic; the parity
 * fixtures are made this way).  With LELPH_REF_BLAS naming an OpenBLAS shared
 * library -- the BLAS of the reference's own build recipe
 * (sample_config/make_gcc_omp.inc: -lopenblas) -- they forward to its CBLAS
 * entry points (also under the scipy_ prefix of the OpenBLAS that SciPy
 * ships), which is how the timed CPU baseline runs. */
#include <complex.h>
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>

#define CBLAS_INT int
#include "cblas.h"

static int tr(CBLAS_TRANSPOSE t) { return t == CblasNoTrans ? 0 : (t == CblasTrans ? 1 : 2); }

typedef void (*gemm_v)(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int, int, int, const void*, const void*, int,
                       const void*, int, const void*, void*, int);
typedef void (*gemm_d)(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int, int, int, double, const double*, int,
                       const double*, int, double, double*, int);
typedef void (*gemm_s)(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int, int, int, float, const float*, int,
                       const float*, int, float, float*, int);
static int blas_looked = 0;
static gemm_v ext_zgemm = NULL, ext_cgemm = NULL;
static gemm_d ext_dgemm = NULL;
static gemm_s ext_sgemm = NULL;

static void* sym2(void* h, const char* a, const char* b)
{
    void* p = dlsym(h, a);
    return p ? p : dlsym(h, b);
}

static void look_blas(void)
{
    if (blas_looked) return;
    blas_looked = 1;
    const char* path = getenv("LELPH_REF_BLAS");
    if (!path || !*path) return;
    void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h)
    {
        fprintf(stderr, "cblas stand-in: cannot open %s, using loops\n", path);
        return;
    }
    ext_zgemm = (gemm_v)sym2(h, "cblas_zgemm", "scipy_cblas_zgemm");
    ext_cgemm = (gemm_v)sym2(h, "cblas_cgemm", "scipy_cblas_cgemm");
    ext_dgemm = (gemm_d)sym2(h, "cblas_dgemm", "scipy_cblas_dgemm");
    ext_sgemm = (gemm_s)sym2(h, "cblas_sgemm", "scipy_cblas_sgemm");
}

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
    look_blas();
    if (ext_zgemm)
    {
        ext_zgemm(layout, TransA, TransB, M, N, K, alphap, Ap, lda, Bp, ldb, betap, Cp, ldc);
        return;
    }
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
    look_blas();
    if (ext_cgemm)
    {
        ext_cgemm(layout, TransA, TransB, M, N, K, alphap, Ap, lda, Bp, ldb, betap, Cp, ldc);
        return;
    }
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
    look_blas();
    if (ext_dgemm)
    {
        ext_dgemm(layout, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
        return;
    }
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
    look_blas();
    if (ext_sgemm)
    {
        ext_sgemm(layout, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
        return;
    }
    int ta = tr(TransA), tb = tr(TransB);
#define CONJ(x) (x)
    GEMM_BODY(float, float)
#undef CONJ
}

