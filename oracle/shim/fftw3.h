/* Stand-in for the subset of the FFTW3 API the reference's FFT layer calls
 * (src/fft/*.c): 1-D many-transform plans, execute, new-array execute,
 * alignment query, malloc/free.  The transforms are an in-house mixed-radix
 * DFT (fftw_stub.c), unnormalised, FFTW_FORWARD = -1 (e^{-i}) and
 * FFTW_BACKWARD = +1 (e^{+i}).  Oracle build only. */
#pragma once
#include <complex.h>
#include <stddef.h>

typedef double _Complex fftw_complex;
typedef float _Complex fftwf_complex;
typedef struct lelph_dft_plan* fftw_plan;
typedef struct lelph_dft_plan* fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_PATIENT (1U << 5)

fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed,
                             int istride, int idist, fftw_complex* out, const int* onembed, int ostride,
                             int odist, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_destroy_plan(fftw_plan p);
int fftw_alignment_of(double* p);
void* fftw_malloc(size_t n);
void fftw_free(void* p);
void fftw_cleanup(void);

fftwf_plan fftwf_plan_many_dft(int rank, const int* n, int howmany, fftwf_complex* in, const int* inembed,
                               int istride, int idist, fftwf_complex* out, const int* onembed, int ostride,
                               int odist, int sign, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out);
void fftwf_destroy_plan(fftwf_plan p);
int fftwf_alignment_of(float* p);
void* fftwf_malloc(size_t n);
void fftwf_free(void* p);
void fftwf_cleanup(void);
