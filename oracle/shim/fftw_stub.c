/* In-house mixed-radix FFT behind the FFTW3 API subset of fftw3.h.
 *
 * Self-sorting (Stockham) decimation in time.  With n = p_1 p_2 ... p_s and
 * after the stages of p_1 .. p_i (L = p_1 ... p_i, M = n / L), the work array
 * holds the length-L transforms of the M interleaved subsequences,
 *   X[j][k] = sum_{t<L} x[k + M t] w_L^{j t}   (j < L, k < M, stored at j M + k),
 * and the stage of radix p (M' = M / p) forms
 *   X'[j + L s][k'] = sum_{q<p} w_p^{s q} (w_{Lp}^{j q} X[j][k' + M' q]),
 * so the last stage leaves the transform in natural order.  Radices 4, 2 and
 * 3 have their own butterflies, 5 and other primes a direct sum.  Twiddles
 * w_N^t = exp(sign 2 pi i t / N) are evaluated in long double from the exact
 * reduced fraction and rounded once to the working precision; the double
 * entry points compute in double, the float ones in float (as FFTW's
 * single-precision library does), so the reference's default build carries
 * the rounding of a float FFT.  Unnormalised, like FFTW.  Oracle build only. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

#define LELPH_MAX_STAGES 40

struct lelph_dft_plan
{
    int n, howmany, istride, idist, ostride, odist, sign, is_float;
    void* in;
    void* out;
    int nst;
    int radix[LELPH_MAX_STAGES];
    size_t tw_off[LELPH_MAX_STAGES];  /* twiddles of stage i: (L p) values w_{Lp}^{j q} at j p + q */
    size_t wp_off[LELPH_MAX_STAGES];  /* w_p^t, t < p, of stage i */
    double* tw;                       /* (re, im) pairs, double plans */
    float* twf;                       /* (re, im) pairs, float plans */
    double* wp;                       /* (re, im) pairs */
    float* wpf;
    void* buf;                        /* two work arrays of n complex */
};

static const long double TWO_PI_L = 6.283185307179586476925286766559005768L;

static int factorize(int n, int* r)
{
    int s = 0;
    while (n % 4 == 0 && s < LELPH_MAX_STAGES) { r[s++] = 4; n /= 4; }
    while (n % 2 == 0 && s < LELPH_MAX_STAGES) { r[s++] = 2; n /= 2; }
    for (int p = 3; n > 1 && s < LELPH_MAX_STAGES; p += 2)
        while (n % p == 0 && s < LELPH_MAX_STAGES) { r[s++] = p; n /= p; }
    return n == 1 ? s : -1;
}

/* One precision of the transform: T the real type, name suffix S. */
#define LELPH_FFT_IMPL(T, S)                                                                              \
    typedef struct { T re, im; } cx##S;                                                                    \
    static inline cx##S cmul##S(cx##S a, cx##S b)                                                          \
    {                                                                                                      \
        cx##S c = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};                                  \
        return c;                                                                                          \
    }                                                                                                      \
    static void stage##S(const cx##S* x, cx##S* y, int L, int M1, int p, const cx##S* tw, const cx##S* wp, \
                         int sign)                                                                         \
    {                                                                                                      \
        const T s = (T)sign;                                                                               \
        const int M = M1 * p;                                                                              \
        cx##S a[64];                                                                                       \
        for (int j = 0; j < L; ++j)                                                                        \
        {                                                                                                  \
            const cx##S* w = tw + (size_t)j * p;                                                           \
            const cx##S* xin = x + (size_t)j * M;                                                          \
            for (int k = 0; k < M1; ++k)                                                                   \
            {                                                                                              \
                cx##S* yo = y + (size_t)j * M1 + k;                                                        \
                const size_t ys = (size_t)L * M1;                                                          \
                if (p == 2)                                                                                \
                {                                                                                          \
                    cx##S u = xin[k], v = cmul##S(xin[k + M1], w[1]);                                      \
                    yo[0].re = u.re + v.re; yo[0].im = u.im + v.im;                                        \
                    yo[ys].re = u.re - v.re; yo[ys].im = u.im - v.im;                                      \
                }                                                                                          \
                else if (p == 4)                                                                           \
                {                                                                                          \
                    cx##S a0 = xin[k], a1 = cmul##S(xin[k + M1], w[1]);                                    \
                    cx##S a2 = cmul##S(xin[k + 2 * M1], w[2]), a3 = cmul##S(xin[k + 3 * M1], w[3]);        \
                    cx##S t0 = {a0.re + a2.re, a0.im + a2.im}, t1 = {a0.re - a2.re, a0.im - a2.im};        \
                    cx##S t2 = {a1.re + a3.re, a1.im + a3.im}, t3 = {a1.re - a3.re, a1.im - a3.im};        \
                    /* w_4 = exp(sign i pi / 2) = sign i: t3 * w_4 = (-sign t3.im, sign t3.re) */          \
                    cx##S r3 = {-s * t3.im, s * t3.re};                                                    \
                    yo[0].re = t0.re + t2.re; yo[0].im = t0.im + t2.im;                                    \
                    yo[ys].re = t1.re + r3.re; yo[ys].im = t1.im + r3.im;                                  \
                    yo[2 * ys].re = t0.re - t2.re; yo[2 * ys].im = t0.im - t2.im;                          \
                    yo[3 * ys].re = t1.re - r3.re; yo[3 * ys].im = t1.im - r3.im;                          \
                }                                                                                          \
                else if (p == 3)                                                                           \
                {                                                                                          \
                    const T c = (T)-0.5, d = (T)(0.86602540378443864676372317075294L) * s;                 \
                    cx##S a0 = xin[k], a1 = cmul##S(xin[k + M1], w[1]), a2 = cmul##S(xin[k + 2 * M1], w[2]); \
                    cx##S t = {a1.re + a2.re, a1.im + a2.im}, u = {a1.re - a2.re, a1.im - a2.im};          \
                    cx##S m = {a0.re + c * t.re, a0.im + c * t.im};                                        \
                    yo[0].re = a0.re + t.re; yo[0].im = a0.im + t.im;                                      \
                    yo[ys].re = m.re - d * u.im; yo[ys].im = m.im + d * u.re;                              \
                    yo[2 * ys].re = m.re + d * u.im; yo[2 * ys].im = m.im - d * u.re;                      \
                }                                                                                          \
                else                                                                                       \
                {                                                                                          \
                    /* direct sum: radix 5 and any other prime */                                          \
                    a[0] = xin[k];                                                                         \
                    for (int q = 1; q < p; ++q) a[q] = cmul##S(xin[k + (size_t)q * M1], w[q]);             \
                    for (int r = 0; r < p; ++r)                                                            \
                    {                                                                                      \
                        cx##S acc = a[0];                                                                  \
                        int e = 0;                                                                         \
                        for (int q = 1; q < p; ++q)                                                        \
                        {                                                                                  \
                            e += r;                                                                        \
                            if (e >= p) e -= p;                                                            \
                            cx##S v = cmul##S(a[q], wp[e]);                                                \
                            acc.re += v.re;                                                                \
                            acc.im += v.im;                                                                \
                        }                                                                                  \
                        yo[(size_t)r * ys] = acc;                                                          \
                    }                                                                                      \
                }                                                                                          \
            }                                                                                              \
        }                                                                                                  \
    }                                                                                                      \
    static void run##S(const struct lelph_dft_plan* P, const cx##S* in, cx##S* out, cx##S* work)           \
    {                                                                                                      \
        const int n = P->n;                                                                                \
        cx##S* x = work;                                                                                   \
        cx##S* y = work + n;                                                                               \
        for (int h = 0; h < P->howmany; ++h)                                                               \
        {                                                                                                  \
            const cx##S* src = in + (size_t)h * P->idist;                                                  \
            for (int i = 0; i < n; ++i) x[i] = src[(size_t)i * P->istride];                                \
            int L = 1, M = n;                                                                              \
            for (int st = 0; st < P->nst; ++st)                                                            \
            {                                                                                              \
                const int p = P->radix[st];                                                                \
                M /= p;                                                                                    \
                stage##S(x, y, L, M, p, (const cx##S*)(P->tw##S##_ptr) + P->tw_off[st],                     \
                         (const cx##S*)(P->wp##S##_ptr) + P->wp_off[st], P->sign);                         \
                L *= p;                                                                                    \
                cx##S* t = x;                                                                              \
                x = y;                                                                                     \
                y = t;                                                                                     \
            }                                                                                              \
            cx##S* dst = out + (size_t)h * P->odist;                                                       \
            for (int i = 0; i < n; ++i) dst[(size_t)i * P->ostride] = x[i];                                \
        }                                                                                                  \
    }

/* the plan's twiddle tables under names the macro can form */
#define twd_ptr tw
#define twf_ptr twf
#define wpd_ptr wp
#define wpf_ptr wpf
LELPH_FFT_IMPL(double, d)
LELPH_FFT_IMPL(float, f)

static struct lelph_dft_plan* make_plan(int rank, const int* n, int howmany, void* in, int istride, int idist,
                                        void* out, int ostride, int odist, int sign, int is_float)
{
    if (rank != 1 || n[0] < 1) return NULL;
    struct lelph_dft_plan* p = calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->n = n[0];
    p->howmany = howmany;
    p->istride = istride;
    p->idist = idist;
    p->ostride = ostride;
    p->odist = odist;
    p->sign = sign;
    p->is_float = is_float;
    p->in = in;
    p->out = out;
    p->nst = p->n == 1 ? 0 : factorize(p->n, p->radix);
    if (p->nst < 0 || (p->n > 1 && p->nst == 0))
    {
        free(p);
        return NULL;
    }
    size_t ntw = 0, nwp = 0;
    int L = 1;
    for (int s = 0; s < p->nst; ++s)
    {
        if (p->radix[s] > 64)
        {
            free(p);
            return NULL;  /* prime factors above 64: not used by any FFT box of the path */
        }
        p->tw_off[s] = ntw;
        p->wp_off[s] = nwp;
        ntw += (size_t)L * p->radix[s];
        nwp += (size_t)p->radix[s];
        L *= p->radix[s];
    }
    p->tw = malloc(sizeof(double) * 2 * (ntw + 1));
    p->twf = malloc(sizeof(float) * 2 * (ntw + 1));
    p->wp = malloc(sizeof(double) * 2 * (nwp + 1));
    p->wpf = malloc(sizeof(float) * 2 * (nwp + 1));
    p->buf = malloc((is_float ? sizeof(float) : sizeof(double)) * 4 * (size_t)p->n);
    L = 1;
    for (int s = 0; s < p->nst; ++s)
    {
        const int r = p->radix[s], N = L * r;
        for (int j = 0; j < L; ++j)
            for (int q = 0; q < r; ++q)
            {
                const long long t = ((long long)j * q) % N;
                const long double ang = TWO_PI_L * (long double)t / (long double)N;
                const size_t o = 2 * (p->tw_off[s] + (size_t)j * r + q);
                p->tw[o] = (double)cosl(ang);
                p->tw[o + 1] = (double)(sign * sinl(ang));
                p->twf[o] = (float)cosl(ang);
                p->twf[o + 1] = (float)(sign * sinl(ang));
            }
        for (int t = 0; t < r; ++t)
        {
            const long double ang = TWO_PI_L * (long double)t / (long double)r;
            const size_t o = 2 * (p->wp_off[s] + (size_t)t);
            p->wp[o] = (double)cosl(ang);
            p->wp[o + 1] = (double)(sign * sinl(ang));
            p->wpf[o] = (float)cosl(ang);
            p->wpf[o + 1] = (float)(sign * sinl(ang));
        }
        L = N;
    }
    return p;
}

static void run_plan(const struct lelph_dft_plan* p, void* in, void* out)
{
    if (p->is_float)
        runf(p, (const cxf*)in, (cxf*)out, (cxf*)p->buf);
    else
        rund(p, (const cxd*)in, (cxd*)out, (cxd*)p->buf);
}

static void free_plan(struct lelph_dft_plan* p)
{
    if (!p) return;
    free(p->tw);
    free(p->twf);
    free(p->wp);
    free(p->wpf);
    free(p->buf);
    free(p);
}

fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed,
                             int istride, int idist, fftw_complex* out, const int* onembed, int ostride,
                             int odist, int sign, unsigned flags)
{
    (void)inembed; (void)onembed; (void)flags;
    return make_plan(rank, n, howmany, in, istride, idist, out, ostride, odist, sign, 0);
}
void fftw_execute(const fftw_plan p) { run_plan(p, p->in, p->out); }
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) { run_plan(p, in, out); }
void fftw_destroy_plan(fftw_plan p) { free_plan(p); }
int fftw_alignment_of(double* p) { return (int)((uintptr_t)p % 16); }
void* fftw_malloc(size_t n) { return aligned_alloc(64, (n + 63) / 64 * 64); }
void fftw_free(void* p) { free(p); }
void fftw_cleanup(void) {}

fftwf_plan fftwf_plan_many_dft(int rank, const int* n, int howmany, fftwf_complex* in, const int* inembed,
                               int istride, int idist, fftwf_complex* out, const int* onembed, int ostride,
                               int odist, int sign, unsigned flags)
{
    (void)inembed; (void)onembed; (void)flags;
    return make_plan(rank, n, howmany, in, istride, idist, out, ostride, odist, sign, 1);
}
void fftwf_execute(const fftwf_plan p) { run_plan(p, p->in, p->out); }
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out) { run_plan(p, in, out); }
void fftwf_destroy_plan(fftwf_plan p) { free_plan(p); }
int fftwf_alignment_of(float* p) { return (int)((uintptr_t)p % 16); }
void* fftwf_malloc(size_t n) { return aligned_alloc(64, (n + 63) / 64 * 64); }
void fftwf_free(void* p) { free(p); }
void fftwf_cleanup(void) {}
