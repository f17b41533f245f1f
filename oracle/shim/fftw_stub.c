/* In-house mixed-radix DFT behind the FFTW3 API subset of fftw3.h.
 *
 * Recursive decimation in time on the smallest prime factor p of n:
 *   X[k + m q] = sum_{r<p} W_n^{r (k + m q)} Y_r[k],  n = p m,
 * with Y_r the length-m transforms of x[r], x[r+p], ...  Twiddles
 * W_n^t = exp(sign 2 pi i t / n) are evaluated in long double from the exact
 * reduced fraction t/n and rounded once to the working precision.  The
 * double entry points compute in double; the float entry points compute every
 * butterfly in float, as FFTW's single-precision library does, so that the
 * reference's default (FP32) build carries the rounding of a float FFT.
 * Oracle build only. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

struct lelph_dft_plan
{
    int n, howmany, istride, idist, ostride, odist, sign, is_float;
    void* in;
    void* out;
    double _Complex* tw; /* tw[t] = exp(sign 2 pi i t / n), t < n */
    double _Complex* buf;
    double _Complex* scratch;
    float _Complex* twf; /* the same in float (float plans) */
    float _Complex* buff;
    float _Complex* scratchf;
};

static const long double TWO_PI_L = 6.283185307179586476925286766559005768L;

static int smallest_factor(int n)
{
    for (int p = 2; p * p <= n; ++p)
        if (n % p == 0) return p;
    return n;
}

/* in: n elements with stride s; out: n contiguous elements; tw: table of the
 * full length N (W_N^t), twstride = N / n.  Instantiated for double and float. */
#define LELPH_DFT_REC(NAME, CT)                                                                        \
    static void NAME(const CT* in, CT* out, int n, int s, const CT* tw, int twstride, int N, CT* scratch) \
    {                                                                                                  \
        if (n == 1)                                                                                    \
        {                                                                                              \
            out[0] = in[0];                                                                            \
            return;                                                                                    \
        }                                                                                              \
        int p = smallest_factor(n);                                                                    \
        int m = n / p;                                                                                 \
        for (int r = 0; r < p; ++r)                                                                    \
            NAME(in + (size_t)r * s, out + (size_t)r * m, m, s * p, tw, twstride * p, N, scratch + n); \
        CT* t = scratch;                                                                               \
        for (int k = 0; k < m; ++k)                                                                    \
        {                                                                                              \
            for (int r = 0; r < p; ++r)                                                                \
            {                                                                                          \
                long long e = ((long long)r * k * twstride) % N;                                       \
                t[r] = out[(size_t)r * m + k] * tw[e];                                                 \
            }                                                                                          \
            for (int q = 0; q < p; ++q)                                                                \
            {                                                                                          \
                CT acc = 0;                                                                            \
                for (int r = 0; r < p; ++r)                                                            \
                {                                                                                      \
                    long long e = ((long long)r * q * m * twstride) % N;                               \
                    acc += t[r] * tw[e];                                                               \
                }                                                                                      \
                t[p + q] = acc;                                                                        \
            }                                                                                          \
            for (int q = 0; q < p; ++q) out[(size_t)q * m + k] = t[p + q];                             \
        }                                                                                              \
    }
LELPH_DFT_REC(dft_rec, double _Complex)
LELPH_DFT_REC(dft_rec_f, float _Complex)

static struct lelph_dft_plan* make_plan(int rank, const int* n, int howmany, void* in, int istride, int idist,
                                        void* out, int ostride, int odist, int sign, int is_float)
{
    if (rank != 1) return NULL;
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
    p->tw = malloc(sizeof(double _Complex) * (size_t)p->n);
    p->buf = malloc(sizeof(double _Complex) * (size_t)p->n * 2);
    p->scratch = malloc(sizeof(double _Complex) * (size_t)p->n * 8 + 64);
    p->twf = malloc(sizeof(float _Complex) * (size_t)p->n);
    p->buff = malloc(sizeof(float _Complex) * (size_t)p->n * 2);
    p->scratchf = malloc(sizeof(float _Complex) * (size_t)p->n * 8 + 64);
    for (int t = 0; t < p->n; ++t)
    {
        long double ang = TWO_PI_L * (long double)t / (long double)p->n;
        p->tw[t] = (double)cosl(ang) + (double)(sign * sinl(ang)) * I;
        p->twf[t] = (float)cosl(ang) + (float)(sign * sinl(ang)) * I;
    }
    return p;
}

static void run_plan(const struct lelph_dft_plan* p, void* in, void* out)
{
    for (int h = 0; h < p->howmany; ++h)
    {
        if (p->is_float)
        {
            float _Complex* x = p->buff;
            float _Complex* y = p->buff + p->n;
            const float _Complex* src = (const float _Complex*)in + (size_t)h * p->idist;
            for (int i = 0; i < p->n; ++i) x[i] = src[(size_t)i * p->istride];
            dft_rec_f(x, y, p->n, 1, p->twf, 1, p->n, p->scratchf);
            float _Complex* dst = (float _Complex*)out + (size_t)h * p->odist;
            for (int i = 0; i < p->n; ++i) dst[(size_t)i * p->ostride] = y[i];
        }
        else
        {
            double _Complex* x = p->buf;
            double _Complex* y = p->buf + p->n;
            const double _Complex* src = (const double _Complex*)in + (size_t)h * p->idist;
            for (int i = 0; i < p->n; ++i) x[i] = src[(size_t)i * p->istride];
            dft_rec(x, y, p->n, 1, p->tw, 1, p->n, p->scratch);
            double _Complex* dst = (double _Complex*)out + (size_t)h * p->odist;
            for (int i = 0; i < p->n; ++i) dst[(size_t)i * p->ostride] = y[i];
        }
    }
}

static void free_plan(struct lelph_dft_plan* p)
{
    if (!p) return;
    free(p->tw);
    free(p->buf);
    free(p->scratch);
    free(p->twf);
    free(p->buff);
    free(p->scratchf);
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
