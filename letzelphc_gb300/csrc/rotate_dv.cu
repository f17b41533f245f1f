// dV_scf of S q from dV_scf of q (rotate_dvscf, src/symmetries/rotate_dvscf.c:22-368):
// output point r takes input point S^-1 (r - tau) of the FFT box (an integer
// permutation, checked to map the grid onto itself), times the phase
// e^{-i (S q).tau}; for non-collinear magnetism (nmag = 4) the spin part is
// rotated as U (V + B.sigma) U^dagger; time-reversed operations conjugate.
// One thread per output point; every (mode, component) of that point is
// gathered from the same source point.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"

#define LELPH_EPS_ROT 1e-5

__device__ __forceinline__ void su2_sandwich(const double2* u, double2& d0, double2& d1, double2& d2, double2& d3)
{
    const double2 c0 = cconj(u[0]), c1 = cconj(u[1]), c2 = cconj(u[2]), c3 = cconj(u[3]);
    const double2 a0 = cadd(cmul(d0, c0), cmul(d1, c1)), a1 = cadd(cmul(d2, c0), cmul(d3, c1));
    const double2 b0 = cadd(cmul(d0, c2), cmul(d1, c3)), b1 = cadd(cmul(d2, c2), cmul(d3, c3));
    const double2 m0 = cadd(cmul(u[0], a0), cmul(u[1], a1));
    const double2 m1 = cadd(cmul(u[0], b0), cmul(u[1], b1));
    const double2 m2 = cadd(cmul(u[2], a0), cmul(u[3], a1));
    const double2 m3 = cadd(cmul(u[2], b0), cmul(u[3], b1));
    d0 = m0;
    d1 = m1;
    d2 = m2;
    d3 = m3;
}

__global__ void __launch_bounds__(256) k_rotate_dvscf(RotDvDesc rd, const double2* __restrict__ in,
                                                      double2* __restrict__ out, unsigned* __restrict__ status)
{
    const long long N = (long long)rd.Nx * rd.Ny * rd.Nz;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int n3[3] = {rd.Nx, rd.Ny, rd.Nz};
    const long long Nyz = (long long)rd.Ny * rd.Nz;
    const double ii[3] = {(double)(i / Nyz), (double)((i % Nyz) / rd.Nz), (double)((i % Nyz) % rd.Nz)};
    double t[3];
    for (int x = 0; x < 3; ++x) t[x] = ii[x] / n3[x] - rd.tau_red[x];
    long long src = 0;
    bool ok = true;
    for (int x = 0; x < 3; ++x)
    {
        double v = rd.sym_red[3 * x] * t[0] + rd.sym_red[3 * x + 1] * t[1] + rd.sym_red[3 * x + 2] * t[2];
        v -= floor(v);
        v -= floor(v + LELPH_EPS_ROT);
        v -= LELPH_EPS_ROT;
        v *= n3[x];
        const double r = rint(v);
        if (fabs(v - r) > 1e-3 + 5e-5 * fabs(v)) ok = false;
        long long ir = (long long)r;
        if (ir < 0 || ir >= n3[x]) ok = false;
        src = src * n3[x] + (ir < 0 ? 0 : (ir >= n3[x] ? 0 : ir));
    }
    if (!ok)
    {
        atomicOr(status, LELPH_DEV_ERR_BOUNDS);
        for (int e = 0; e < rd.nmodes * rd.nmag; ++e) out[(size_t)e * N + i] = make_double2(0.0, 0.0);
        return;
    }
    for (int m = 0; m < rd.nmodes; ++m)
    {
        const double2* pin = in + (size_t)m * rd.nmag * N;
        double2* pout = out + (size_t)m * rd.nmag * N;
        if (rd.nmag == 4)
        {
            double2 d0 = cmul(rd.ph, pin[src]), d1 = cmul(rd.ph, pin[N + src]);
            double2 d2 = cmul(rd.ph, pin[2 * N + src]), d3 = cmul(rd.ph, pin[3 * N + src]);
            if (!rd.composite)
            {
                // [V, Bx, By, Bz] -> [V + Bz, Bx - i By, Bx + i By, V - Bz]
                const double2 iBy = make_double2(-d2.y, d2.x);
                const double2 e0 = cadd(d0, d3), e1 = csub(d1, iBy), e2 = cadd(d1, iBy), e3 = csub(d0, d3);
                d0 = e0;
                d1 = e1;
                d2 = e2;
                d3 = e3;
            }
            su2_sandwich(rd.su2, d0, d1, d2, d3);
            if (!rd.composite)
            {
                // back to [V, Bx, By, Bz]
                const double2 v = make_double2(0.5 * (d0.x + d3.x), 0.5 * (d0.y + d3.y));
                const double2 bx = make_double2(0.5 * (d1.x + d2.x), 0.5 * (d1.y + d2.y));
                const double2 df = make_double2(0.5 * (d2.x - d1.x), 0.5 * (d2.y - d1.y));
                const double2 by = make_double2(df.y, -df.x);  // -i (M2 - M1) / 2
                const double2 bz = make_double2(0.5 * (d0.x - d3.x), 0.5 * (d0.y - d3.y));
                d0 = v;
                d1 = bx;
                d2 = by;
                d3 = bz;
            }
            if (rd.trev)
            {
                d0 = cconj(d0);
                d1 = cconj(d1);
                d2 = cconj(d2);
                d3 = cconj(d3);
            }
            pout[i] = d0;
            pout[N + i] = d1;
            pout[2 * N + i] = d2;
            pout[3 * N + i] = d3;
        }
        else
        {
            for (int c = 0; c < rd.nmag; ++c)
            {
                double2 v = cmul(rd.ph, pin[(size_t)c * N + src]);
                if (rd.trev) v = cconj(v);
                pout[(size_t)c * N + i] = v;
            }
        }
    }
}

void lelph_launch_rotate_dvscf(const RotDvDesc& rd, const double2* in, double2* out, unsigned* status,
                               cudaStream_t st)
{
    const long long N = (long long)rd.Nx * rd.Ny * rd.Nz;
    k_rotate_dvscf<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(rd, in, out, status);
}
