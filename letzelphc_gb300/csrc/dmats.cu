// Electronic representation matrices of the symmetry operations (Dmats):
// D[spin, b, a] = <psi_{Rk,b} | U(R) | psi_{k,a}>  (electronic_reps,
// src/symmetries/elec_reps.c:16-413, driven per (symmetry, full-BZ k) by
// compute_and_write_dmats, src/elph/compute_dmats.c:20-131).
//
// Both sides of a job are unfolded from the irreducible wedge: k = S1 k1 and
// Rk = S2 k2.  The right operand is psi_{k1} carried by U(R) U(S1) onto the
// plane-wave list of k1 rotated by R S1; the left operand is psi_{k2}
// reordered onto that same list: plane wave p of k1 (Miller m) takes the k2
// coefficient whose Miller index is W2^-1 (W_RS1 m - G0), G0 = S2 k2 - R S1 k1,
// looked up in a per-k Miller -> position table of the FFT box and checked
// (absent: zero), which is the reference's find_gvecs_idxs match
// (src/wfc/gsort.c:49-93) read from the other side.  The SU(2) factors,
// fractional-translation phases and conjugations of the reference's sequence
// (elec_reps.c:301-372) fold per job into one 2x2 spinor matrix, one conjugation
// flag, one constant phase and one phase vector t; the plane-wave phase
// e^{-i 2 pi m.t} is the product of three per-axis factors tabulated per job.
// D is then one complex contraction over (spinor, plane wave), tiled 32 x 32
// and four-by-four per thread, with the operands staged in shared memory.
//
// Plain form: FP64 throughout.  Mixed form: the per-axis phase angles are
// reduced in FP64, the operands and the contraction are FP32, and the FP32
// partial sums are flushed into FP64 accumulators every DM_GROUP chunks.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"

#define DM_TB 32       // D tile (bands) per CTA, both sides
#define DM_KC 32       // plane waves per staged chunk
#define DM_THREADS 64  // 8 x 8 threads, 4 x 4 complex entries of the tile each
#define DM_GROUP 16    // chunks summed in FP32 before the FP64 flush (mixed form)

// element (kk, col) of a staged operand: 16-byte pairs of columns XOR-swizzled by kk
__device__ __forceinline__ int dm_idx(int kk, int col)
{
    return kk * DM_TB + ((((col >> 1) ^ (kk & 15)) << 1) | (col & 1));
}

template <typename T2> struct DmReal;
template <> struct DmReal<float2> { typedef float type; };
template <> struct DmReal<double2> { typedef double type; };

// e^{-i 2 pi_T x} for a per-axis angle x (in turns): the reduction to
// [-1/2, 1/2] is FP64, the evaluation in the operand type.
template <typename T2> __device__ __forceinline__ T2 dm_phase(double x);
template <> __device__ __forceinline__ double2 dm_phase<double2>(double x)
{
    double u = x * (LELPH_PI_T / 3.14159265358979323846);
    u -= rint(u);
    double s, c;
    sincospi(2.0 * u, &s, &c);
    return make_double2(c, -s);
}
template <> __device__ __forceinline__ float2 dm_phase<float2>(double x)
{
    double u = x * (LELPH_PI_T / 3.14159265358979323846);
    u -= rint(u);
    float s, c;
    sincospif((float)(2.0 * u), &s, &c);
    return make_float2(c, -s);
}

template <typename T2> __device__ __forceinline__ T2 dm_cvt(double2 v);
template <> __device__ __forceinline__ double2 dm_cvt<double2>(double2 v) { return v; }
template <> __device__ __forceinline__ float2 dm_cvt<float2>(double2 v) { return make_float2((float)v.x, (float)v.y); }

template <typename T2> __device__ __forceinline__ void dm_ld_pair(const T2* p, T2& a, T2& b);
template <> __device__ __forceinline__ void dm_ld_pair<float2>(const float2* p, float2& a, float2& b)
{
    const float4 v = *reinterpret_cast<const float4*>(p);
    a = make_float2(v.x, v.y);
    b = make_float2(v.z, v.w);
}
template <> __device__ __forceinline__ void dm_ld_pair<double2>(const double2* p, double2& a, double2& b)
{
    a = p[0];
    b = p[1];
}

template <typename T2> __device__ __forceinline__ void dm_cfma(T2& acc, T2 v, T2 w)
{
    acc.x = fma(v.x, w.x, acc.x);
    acc.x = fma(-v.y, w.y, acc.x);
    acc.y = fma(v.x, w.y, acc.y);
    acc.y = fma(v.y, w.x, acc.y);
}

// Stage one operand row segment: coefficient(s) x of band row `row` at
// position j, conjugated if asked, spinor-mixed by M, times the position's
// phase c, into the shared tile.
template <typename T2>
__device__ __forceinline__ void dm_stage(T2* tile, int j, int r, int ns, const double2* x, bool cj, const T2* M, T2 c)
{
    T2 y0 = dm_cvt<T2>(x[0]), y1 = dm_cvt<T2>(x[1]);
    if (cj)
    {
        y0 = cconj(y0);
        y1 = cconj(y1);
    }
    if (ns == 2)
    {
        const T2 z0 = cadd(cmul(M[0], y0), cmul(M[1], y1));
        const T2 z1 = cadd(cmul(M[2], y0), cmul(M[3], y1));
        tile[dm_idx(DM_KC + j, r)] = cmul(z1, c);
        y0 = z0;
    }
    tile[dm_idx(j, r)] = cmul(y0, c);
}

template <typename T2>
__global__ void __launch_bounds__(DM_THREADS) k_dmats(const DmatJob* __restrict__ jobs, DmatGeom dg,
                                                      const double2* __restrict__ coef,
                                                      const long long* __restrict__ coef_off,
                                                      const int* __restrict__ miller,
                                                      const long long* __restrict__ pw_off,
                                                      const int* __restrict__ npw_arr, const int* __restrict__ gtab,
                                                      double2* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char dm_smem[];
    const int ns = dg.nspinor, nb = dg.nb;
    const int KCS = ns * DM_KC;
    T2* sv = reinterpret_cast<T2*>(dm_smem);
    T2* sw = sv + KCS * DM_TB;
    T2* tabw = sw + KCS * DM_TB;               // per-axis phase factors, (Nx+1) + (Ny+1) + (Nz+1)
    T2* tabv = tabw + dg.ntab;
    T2* scw = tabv + dg.ntab;                  // per-position phases of the chunk
    T2* scv = scw + DM_KC;
    int* sii = reinterpret_cast<int*>(scv + DM_KC);  // k2 position of each k1 plane wave (-1: absent)
    __shared__ DmatJob J;

    const int t = threadIdx.x;
    const long long ijob = blockIdx.x;
    const int ntile = (nb + DM_TB - 1) / DM_TB;
    const int b0 = (blockIdx.y / ntile) * DM_TB, a0 = (blockIdx.y % ntile) * DM_TB;
    const int spin = blockIdx.z;
    if (t == 0) J = jobs[ijob];
    __syncthreads();

    // per-axis phase tables over the box's Miller range [-N/2, N/2]
    const int Nax[3] = {dg.Nx, dg.Ny, dg.Nz};
    {
        int base = 0;
        for (int ax = 0; ax < 3; ++ax)
        {
            for (int i = t; i <= Nax[ax]; i += DM_THREADS)
            {
                const double m = (double)(i - Nax[ax] / 2);
                tabw[base + i] = dm_phase<T2>(m * J.tw[ax]);
                tabv[base + i] = dm_phase<T2>(m * J.tv[ax]);
            }
            base += Nax[ax] + 1;
        }
    }
    T2 Mw[4], Mv[4];
#pragma unroll
    for (int e = 0; e < 4; ++e)
    {
        Mw[e] = dm_cvt<T2>(J.Mw[e]);
        Mv[e] = dm_cvt<T2>(J.Mv[e]);
    }
    const T2 Cw = dm_cvt<T2>(J.Cw), Cv = dm_cvt<T2>(J.Cv);
    const int npw1 = npw_arr[J.ik1], npw2 = npw_arr[J.ik2];
    const int* mil1 = miller + 3 * pw_off[J.ik1];
    const int* mil2 = miller + 3 * pw_off[J.ik2];
    const double2* c1 = coef + coef_off[J.ik1] + (long long)spin * nb * ns * npw1;
    const double2* c2 = coef + coef_off[J.ik2] + (long long)spin * nb * ns * npw2;
    const long long Nbox = (long long)dg.Nx * dg.Ny * dg.Nz;
    const int* tab2 = gtab + (long long)J.ik2 * Nbox;
    const int oy = dg.Nx + 1, oz = dg.Nx + dg.Ny + 2;

    const int rb = t >> 3, ca = t & 7;
    T2 acc[4][4];
    double2 accd[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            acc[i][j] = mk2<T2>(0.0, 0.0);
            accd[i][j] = make_double2(0.0, 0.0);
        }

    const int nchunk = (npw1 + DM_KC - 1) / DM_KC;
    for (int ch = 0; ch < nchunk; ++ch)
    {
        const int p0 = ch * DM_KC;
        __syncthreads();  // previous chunk's contraction is done with the tiles
        if (t < DM_KC)
        {
            // right operand phase of plane wave p (k1 list, Miller m)
            const int p = p0 + t;
            T2 c = mk2<T2>(0.0, 0.0);
            if (p < npw1)
            {
                const int* m = mil1 + 3 * p;
                c = cmul(cmul(tabw[m[0] + dg.Nx / 2], tabw[oy + m[1] + dg.Ny / 2]), tabw[oz + m[2] + dg.Nz / 2]);
                c = cmul(c, Cw);
            }
            scw[t] = c;
        }
        else
        {
            // left operand: the k2 plane wave landing on p, and its phase
            const int j = t - DM_KC, p = p0 + j;
            T2 c = mk2<T2>(0.0, 0.0);
            int ii = -1;
            if (p < npw1)
            {
                const int* m = mil1 + 3 * p;
                int g[3], n[3];
#pragma unroll
                for (int r = 0; r < 3; ++r)
                    g[r] = J.WRS1[3 * r] * m[0] + J.WRS1[3 * r + 1] * m[1] + J.WRS1[3 * r + 2] * m[2] - J.ulm[r];
#pragma unroll
                for (int r = 0; r < 3; ++r) n[r] = J.W2inv[3 * r] * g[0] + J.W2inv[3 * r + 1] * g[1] + J.W2inv[3 * r + 2] * g[2];
                const int bx = ((n[0] % dg.Nx) + dg.Nx) % dg.Nx, by = ((n[1] % dg.Ny) + dg.Ny) % dg.Ny,
                          bz = ((n[2] % dg.Nz) + dg.Nz) % dg.Nz;
                const int cand = tab2[((long long)bx * dg.Ny + by) * dg.Nz + bz];
                if (cand >= 0 && cand < npw2)
                {
                    const int* mc = mil2 + 3 * cand;
                    if (mc[0] == n[0] && mc[1] == n[1] && mc[2] == n[2]) ii = cand;
                }
                if (ii >= 0)
                {
                    c = cmul(cmul(tabv[m[0] + dg.Nx / 2], tabv[oy + m[1] + dg.Ny / 2]), tabv[oz + m[2] + dg.Nz / 2]);
                    c = cmul(c, Cv);
                }
            }
            sii[j] = ii;
            scv[j] = c;
        }
        __syncthreads();
        {
            const int j = t & (DM_KC - 1);
            const int p = p0 + j;
            const int ii = sii[j];
            const T2 cw = scw[j], cv = scv[j];
            for (int r = t >> 5; r < DM_TB; r += DM_THREADS / DM_KC)
            {
                double2 x[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
                const int a = a0 + r;
                if (a < nb && p < npw1)
                    for (int s = 0; s < ns; ++s) x[s] = c1[((long long)a * ns + s) * npw1 + p];
                dm_stage<T2>(sw, j, r, ns, x, J.conj_w != 0, Mw, cw);
                x[0] = x[1] = make_double2(0.0, 0.0);
                const int b = b0 + r;
                if (b < nb && ii >= 0)
                    for (int s = 0; s < ns; ++s) x[s] = c2[((long long)b * ns + s) * npw2 + ii];
                dm_stage<T2>(sv, j, r, ns, x, J.conj_v != 0, Mv, cv);
            }
        }
        __syncthreads();
        for (int kk = 0; kk < KCS; ++kk)
        {
            T2 v[4], w[4];
            dm_ld_pair<T2>(sv + dm_idx(kk, 4 * rb), v[0], v[1]);
            dm_ld_pair<T2>(sv + dm_idx(kk, 4 * rb + 2), v[2], v[3]);
            dm_ld_pair<T2>(sw + dm_idx(kk, 4 * ca), w[0], w[1]);
            dm_ld_pair<T2>(sw + dm_idx(kk, 4 * ca + 2), w[2], w[3]);
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) dm_cfma(acc[i][j], v[i], w[j]);
        }
        if (sizeof(T2) == sizeof(float2) && ((ch + 1) % DM_GROUP == 0 || ch + 1 == nchunk))
        {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                {
                    accd[i][j].x += (double)acc[i][j].x;
                    accd[i][j].y += (double)acc[i][j].y;
                    acc[i][j] = mk2<T2>(0.0, 0.0);
                }
        }
    }
    double2* D = out + (ijob * dg.nspin + spin) * (long long)nb * nb;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            const int b = b0 + 4 * rb + i, a = a0 + 4 * ca + j;
            if (b < nb && a < nb)
                D[(long long)b * nb + a] = sizeof(T2) == sizeof(float2)
                                               ? accd[i][j]
                                               : make_double2((double)acc[i][j].x, (double)acc[i][j].y);
        }
}

// Miller -> position table of every iBZ plane-wave list on the FFT box
// (entries not on a list stay -1).
__global__ void k_dm_gtab(const int* __restrict__ miller, const long long* __restrict__ pw_off,
                          const int* __restrict__ npw_arr, int nk, int Nx, int Ny, int Nz, int* __restrict__ gtab)
{
    const int ik = blockIdx.y;
    if (ik >= nk) return;
    const int npw = npw_arr[ik];
    const int* mil = miller + 3 * pw_off[ik];
    int* tab = gtab + (long long)ik * Nx * Ny * Nz;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < npw; g += gridDim.x * blockDim.x)
    {
        const int bx = ((mil[3 * g] % Nx) + Nx) % Nx, by = ((mil[3 * g + 1] % Ny) + Ny) % Ny,
                  bz = ((mil[3 * g + 2] % Nz) + Nz) % Nz;
        tab[((long long)bx * Ny + by) * Nz + bz] = g;
    }
}

size_t lelph_dmats_smem_bytes(const DmatGeom& dg, int fp64)
{
    const size_t e = fp64 ? sizeof(double2) : sizeof(float2);
    return e * (2 * (size_t)dg.nspinor * DM_KC * DM_TB + 2 * (size_t)dg.ntab + 2 * DM_KC) + sizeof(int) * DM_KC;
}

void lelph_launch_dm_gtab(const int* miller, const long long* pw_off, const int* npw, int nk, int npw_max, int Nx,
                          int Ny, int Nz, int* gtab, cudaStream_t st)
{
    dim3 grid((unsigned)((npw_max + 255) / 256), (unsigned)nk);
    k_dm_gtab<<<grid, 256, 0, st>>>(miller, pw_off, npw, nk, Nx, Ny, Nz, gtab);
}

int lelph_launch_dmats(const DmatJob* jobs, long long njobs, const DmatGeom& dg, int fp64, const double2* coef,
                       const long long* coef_off, const int* miller, const long long* pw_off, const int* npw,
                       const int* gtab, double2* out, cudaStream_t st)
{
    if (njobs <= 0) return 0;
    if (njobs > 0x7fffffffLL) return -1;
    const int ntile = (dg.nb + DM_TB - 1) / DM_TB;
    const size_t smem = lelph_dmats_smem_bytes(dg, fp64);
    dim3 grid((unsigned)njobs, (unsigned)(ntile * ntile), (unsigned)dg.nspin);
    if (fp64)
    {
        if (cudaFuncSetAttribute(k_dmats<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return -1;
        k_dmats<double2><<<grid, DM_THREADS, smem, st>>>(jobs, dg, coef, coef_off, miller, pw_off, npw, gtab, out);
    }
    else
    {
        if (cudaFuncSetAttribute(k_dmats<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return -1;
        k_dmats<float2><<<grid, DM_THREADS, smem, st>>>(jobs, dg, coef, coef_off, miller, pw_off, npw, gtab, out);
    }
    return 0;
}
