// Real spherical harmonics in FP64: the associated Legendre recurrence and all
// (l, m) at once by the angle-addition recurrence.
#pragma once
#include "lelph_common.cuh"

__device__ __forceinline__ double ylm_legendre(int l, int m, double x)
{
    // associated Legendre function without the Condon-Shortley phase, m >= 0
    double val = 1.0;
    if (l == 0 && m == 0) return 1.0;
    if (m > l) return 0.0;
    double sq = sqrt(1.0 - x * x);
    for (int im = 1; im <= m; ++im) val *= (2 * im - 1) * sq;
    if (l == m) return val;
    double vmm = val;
    val *= (2 * m + 1) * x;
    if (l == m + 1) return val;
    for (int im = m + 2; im <= l; ++im)
    {
        double tmp = val;
        val = (2 * im - 1) * x * val - (im + m - 1) * vmm;
        val = val / (im - m);
        vmm = tmp;
    }
    return val;
}

// Real spherical harmonics of all (l, m), l <= lmax, at K, written to y[l*l + l + m]:
// cos(m phi), sin(m phi) by the angle-addition recurrence from cos(phi), sin(phi).
__device__ __forceinline__ void ylm_all(int lmax, double vx, double vy, double vz, double* y)
{
    const double fact[8] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0};
    const double norm = sqrt(vx * vx + vy * vy + vz * vz);
    if (norm < 1e-6)
    {
        for (int i = 0; i < (lmax + 1) * (lmax + 1); ++i) y[i] = 0.0;
        y[0] = 1.0 / sqrt(4 * LELPH_PI_T);
        return;
    }
    const double cost = vz / norm;
    const double rxy = sqrt(vx * vx + vy * vy);
    const double c1 = rxy > 0.0 ? vx / rxy : 1.0, s1 = rxy > 0.0 ? vy / rxy : 0.0;
    double cm = 1.0, sm = 0.0;  // cos(m phi), sin(m phi)
    for (int m = 0; m <= lmax; ++m)
    {
        for (int l = m; l <= lmax; ++l)
        {
            double p = ylm_legendre(l, m, cost) * sqrt(fact[l - m] * (2 * l + 1) / (4 * LELPH_PI_T * fact[l + m]));
            if (m == 0)
                y[l * l + l] = p;
            else
            {
                y[l * l + l + m] = sqrt(2.0) * cm * p;
                y[l * l + l - m] = sqrt(2.0) * sm * p;
            }
        }
        const double cn = cm * c1 - sm * s1, sn = sm * c1 + cm * s1;
        cm = cn;
        sm = sn;
    }
}


// The same in FP32 (the mixed form's tensor-core projections): identical
// recurrences and normalisation, evaluated in single precision as the
// reference's default single-precision build does.
__device__ __forceinline__ float ylm_legendre_f(int l, int m, float x)
{
    float val = 1.f;
    if (l == 0 && m == 0) return 1.f;
    if (m > l) return 0.f;
    const float sq = sqrtf(fmaxf(1.f - x * x, 0.f));
    for (int im = 1; im <= m; ++im) val *= (float)(2 * im - 1) * sq;
    if (l == m) return val;
    float vmm = val;
    val *= (float)(2 * m + 1) * x;
    if (l == m + 1) return val;
    for (int im = m + 2; im <= l; ++im)
    {
        const float tmp = val;
        val = ((float)(2 * im - 1) * x * val - (float)(im + m - 1) * vmm) / (float)(im - m);
        vmm = tmp;
    }
    return val;
}

// y[(l*l + l + m) * stride] (y in shared memory: no local array)
__device__ __forceinline__ void ylm_all_f(int lmax, float vx, float vy, float vz, float* y, int stride)
{
    const float norm = sqrtf(vx * vx + vy * vy + vz * vz);
    if (norm < 1e-6f)
    {
        for (int i = 0; i < (lmax + 1) * (lmax + 1); ++i) y[i * stride] = 0.f;
        y[0] = 1.f / sqrtf(4.f * (float)LELPH_PI_T);
        return;
    }
    const float cost = vz / norm;
    const float rxy = sqrtf(vx * vx + vy * vy);
    const float c1 = rxy > 0.f ? vx / rxy : 1.f, s1 = rxy > 0.f ? vy / rxy : 0.f;
    float cm = 1.f, sm = 0.f;
    for (int m = 0; m <= lmax; ++m)
    {
        for (int l = m; l <= lmax; ++l)
        {
            float ratio = 1.f;  // (l - m)! / (l + m)!
            for (int i = l - m + 1; i <= l + m; ++i) ratio /= (float)i;
            const float p = ylm_legendre_f(l, m, cost) * sqrtf(ratio * (float)(2 * l + 1) / (4.f * (float)LELPH_PI_T));
            if (m == 0)
                y[(l * l + l) * stride] = p;
            else
            {
                y[(l * l + l + m) * stride] = 1.41421356f * cm * p;
                y[(l * l + l - m) * stride] = 1.41421356f * sm * p;
            }
        }
        const float cn = cm * c1 - sm * s1, sn = sm * c1 + cm * s1;
        cm = cn;
        sm = sn;
    }
}
