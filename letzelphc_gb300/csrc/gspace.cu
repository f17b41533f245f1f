// G-space route of the local sandwich: the reference's own order of work
// (elphLocal, src/dvloc/compute_Vbare_loc.c:264-310, with fft_convolution3D,
// src/fft/convolution.c:13-...): for each mode nu and band m of k,
//   F_{nu m s}(G) = sum_r e^{-i G.r} P_{nu m s}(r),
//   P_{nu m s} = dV_nu psi_{k m}  (nmag 1/2)  or  sum_s' dV_nu[s s'] psi_{k m s'}  (nmag 4),
// then one GEMM over the k+q sphere,
//   glocal[nu m][n] = (1/M) sum_{s, G in sphere(k+q)} F_{nu m s}(G) conj(c_{k+q n s}(G)).
// Everything runs on the product grid with the pair's dV window (as in the
// real-space route), so F is needed only on the k+q sphere, and the forward
// transform is pruned accordingly:
// * k_gs_plane: one (x plane, band, mode) per CTA: the product plane is formed
//   on load, transformed along z then y in shared memory, and only the (y, z)
//   columns that hold a plane wave of the k+q sphere are written out;
// * k_gs_xpass: the x transform of those columns, whose epilogue writes the
//   sphere's values in the sphere's sorted order (column, x) -- the K order of
//   the GEMM; the k+q coefficients are stored permuted to the same order;
// * k_gs_gemm: SIMT complex GEMM over one K chunk (FP32 in the mixed form,
//   FP64 in the plain form); chunk partials are summed in FP64 by k_gs_reduce,
//   which also applies 1/M and writes the FP64 local term the finish kernel
//   consumes.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "fft_smem.cuh"
#include "lelph_common.cuh"
#include "lelph_internal.h"

#define GS_THREADS 256
#define GS_CB 32   // columns per CTA of the x pass
#define GS_BM 64
#define GS_BN 64
#define GS_BK 16

// ------------------------------------------------------------------ plane pass
// grid: (nub modes, nb bands, Nx planes); mode fastest so that the CTAs that
// run together share the psi plane (from L2) and the window planes stay in L2.
template <typename T2, typename T>
__global__ void __launch_bounds__(GS_THREADS) k_gs_plane(const T2* __restrict__ psi, const T2* __restrict__ win,
                                                         GsGeom gg, int nu0, FftPlan1D py, FftPlan1D pz,
                                                         const T2* __restrict__ twy, const T2* __restrict__ twz,
                                                         const int* __restrict__ cols, int ncol, T2* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char gsp_smem[];
    const int Ny = gg.Ny, Nz = gg.Nz, NP = Ny * Nz;
    T2* a = reinterpret_cast<T2*>(gsp_smem);
    T2* b = a + NP;
    T2* ty = b + NP;
    T2* tz = ty + Ny;
    const int nul = blockIdx.x, m = blockIdx.y, x = blockIdx.z;
    const int nu = nu0 + nul;
    for (int t = threadIdx.x; t < Ny; t += blockDim.x) ty[t] = twy[t];
    for (int t = threadIdx.x; t < Nz; t += blockDim.x) tz[t] = twz[t];
    const long long M = (long long)gg.Nx * NP;
    const size_t xoff = (size_t)x * NP;
    const T2* pm = psi + (size_t)m * gg.nspinor * M + xoff;           // psi_k, band m, spinor 0, plane x
    const T2* dv = win + (size_t)nu * gg.nmag * M + xoff;             // window of mode nu, component 0, plane x
    for (int s = 0; s < gg.nspinor; ++s)
    {
        for (int e = threadIdx.x; e < NP; e += blockDim.x)
        {
            T2 v;
            if (gg.nmag == 4)
                v = cadd(cmul(dv[(size_t)(2 * s) * M + e], pm[e]), cmul(dv[(size_t)(2 * s + 1) * M + e], pm[M + e]));
            else
                v = cmul(dv[(size_t)(gg.nmag == 2 ? gg.spin : 0) * M + e], pm[(size_t)s * M + e]);
            a[e] = v;
        }
        __syncthreads();
        T2* r = fft_smem<T2, T>(a, b, Ny, 1, Nz, pz, tz, -1);       // z lines
        T2* o = r == a ? b : a;
        r = fft_smem<T2, T>(r, o, Nz, Nz, 1, py, ty, -1);           // y lines
        T2* dst = out + (((size_t)(nul * gg.nb + m) * gg.nspinor + s) * gg.Nx + x) * ncol;
        for (int c = threadIdx.x; c < ncol; c += blockDim.x) dst[c] = r[cols[c]];
        __syncthreads();
    }
}

// -------------------------------------------------------------------- x pass
// grid: (ceil(ncol / GS_CB), rows of the block x nspinor); the tile [x][column]
// is read along the columns (coalesced), transformed along x, and the sphere
// points of the block's columns -- a contiguous K range, sorted by (column, x)
// -- are written in order.
template <typename T2, typename T>
__global__ void __launch_bounds__(GS_THREADS) k_gs_xpass(const T2* __restrict__ in, int Nx, int ncol,
                                                         FftPlan1D px, const T2* __restrict__ twx,
                                                         const int* __restrict__ cst, const int* __restrict__ kcx,
                                                         int npad, T2* __restrict__ A)
{
    extern __shared__ __align__(16) unsigned char gsx_smem[];
    T2* a = reinterpret_cast<T2*>(gsx_smem);
    T2* b = a + Nx * GS_CB;
    T2* tx = b + Nx * GS_CB;
    const int c0 = blockIdx.x * GS_CB;
    const int rb = blockIdx.y;
    for (int t = threadIdx.x; t < Nx; t += blockDim.x) tx[t] = twx[t];
    const T2* src = in + (size_t)rb * Nx * ncol;
    for (int e = threadIdx.x; e < Nx * GS_CB; e += blockDim.x)
    {
        const int x = e / GS_CB, cc = e - x * GS_CB;
        const int c = c0 + cc;
        a[e] = c < ncol ? src[(size_t)x * ncol + c] : mk2<T2>(0.0, 0.0);
    }
    __syncthreads();
    T2* r = fft_smem<T2, T>(a, b, GS_CB, GS_CB, 1, px, tx, -1);
    const int k0 = cst[c0], k1 = cst[min(c0 + GS_CB, ncol)];
    T2* dst = A + (size_t)rb * npad;
    for (int K = k0 + threadIdx.x; K < k1; K += blockDim.x)
    {
        const int v = kcx[K];
        const int c = v / Nx, x = v - c * Nx;
        dst[K] = r[x * GS_CB + (c - c0)];
    }
}

// ---------------------------------------------------------------------- GEMM
// part[chunk][rowoff + row][n] = sum_{K in chunk} A[row][K] conj(B[n][K]);
// A: nrows x Ktot, B: nb x Ktot, both K-contiguous.  64 x 64 tile, 16-deep K
// steps staged through shared memory with a register prefetch; each thread
// holds 4 rows x 4 columns (columns tx + 16 j, conflict-free reads).
template <typename T, typename T2>
__global__ void __launch_bounds__(GS_THREADS) k_gs_gemm(const T2* __restrict__ A, const T2* __restrict__ B, int nrows,
                                                        int nb, int Ktot, int kchunk, int rowoff, int nrows_total,
                                                        T2* __restrict__ part)
{
    __shared__ T2 As[GS_BK][GS_BM + 1];
    __shared__ T2 Bs[GS_BK][GS_BN + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int lk = tid & 15, lr = tid >> 4;
    const int r0 = blockIdx.x * GS_BM, n0 = blockIdx.y * GS_BN;
    const int kbeg = blockIdx.z * kchunk, kend = min(Ktot, kbeg + kchunk);
    T2 acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = mk2<T2>(0.0, 0.0);
    T2 ra[4], rbv[4];
    auto load = [&](int k0) {
        const int k = k0 + lk;
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            const int row = r0 + lr + 16 * i, n = n0 + lr + 16 * i;
            ra[i] = (row < nrows && k < kend) ? A[(size_t)row * Ktot + k] : mk2<T2>(0.0, 0.0);
            rbv[i] = (n < nb && k < kend) ? B[(size_t)n * Ktot + k] : mk2<T2>(0.0, 0.0);
        }
    };
    load(kbeg);
    for (int k0 = kbeg; k0 < kend; k0 += GS_BK)
    {
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            As[lk][lr + 16 * i] = ra[i];
            Bs[lk][lr + 16 * i] = rbv[i];
        }
        __syncthreads();
        if (k0 + GS_BK < kend) load(k0 + GS_BK);
#pragma unroll
        for (int kk = 0; kk < GS_BK; ++kk)
        {
            T2 av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                {
                    // a * conj(b)
                    acc[i][j].x = fma(av[i].x, bv[j].x, acc[i][j].x);
                    acc[i][j].x = fma(av[i].y, bv[j].y, acc[i][j].x);
                    acc[i][j].y = fma(av[i].y, bv[j].x, acc[i][j].y);
                    acc[i][j].y = fma(-av[i].x, bv[j].y, acc[i][j].y);
                }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        const int row = r0 + ty * 4 + i;
        if (row >= nrows) continue;
        T2* dst = part + ((size_t)blockIdx.z * nrows_total + rowoff + row) * nb;
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            const int n = n0 + tx + 16 * j;
            if (n < nb) dst[n] = acc[i][j];
        }
    }
}

// glocal[row][n] = invM * sum_c part[c][row][n], summed in FP64
template <typename T2>
__global__ void k_gs_reduce(const T2* __restrict__ part, long long nel, int nchunks, double invM,
                            double2* __restrict__ glocal)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x)
    {
        double re = 0.0, im = 0.0;
        for (int c = 0; c < nchunks; ++c)
        {
            const T2 v = part[(size_t)c * nel + e];
            re += (double)v.x;
            im += (double)v.y;
        }
        glocal[e] = make_double2(re * invM, im * invM);
    }
}

// ------------------------------------------------- permuted k+q coefficients
// Bp[k][set][s][K] = c_k(set, s, perm_k[K]) for K < npw_k, zero up to npad_k.
// grid: (ceil(npad_max / 256), nsets * nspinor, nk)
template <typename T2>
__global__ void k_gs_bperm(const double2* __restrict__ chat, const long long* __restrict__ chat_off,
                           const int* __restrict__ npw_k, const int* __restrict__ npad_k,
                           const long long* __restrict__ perm_off, const int* __restrict__ perm,
                           const long long* __restrict__ bp_off, int k0, int nrowk, T2* __restrict__ Bp)
{
    const int k = k0 + blockIdx.z;
    const int npw = npw_k[k], npad = npad_k[k];
    const int K = blockIdx.x * blockDim.x + threadIdx.x;
    if (K >= npad) return;
    const int rs = blockIdx.y;  // set * nspinor + s
    (void)nrowk;
    T2 v = mk2<T2>(0.0, 0.0);
    if (K < npw)
    {
        const double2 c = chat[chat_off[k] + (size_t)rs * npw + perm[perm_off[k] + K]];
        v = mk2<T2>(c.x, c.y);
    }
    Bp[bp_off[k] + (size_t)rs * npad + K] = v;
}

// ------------------------------------------------------------------ launchers

size_t lelph_gs_plane_smem(const GsGeom& gg, int fp64)
{
    const size_t e = fp64 ? sizeof(double2) : sizeof(float2);
    return e * (2 * (size_t)gg.Ny * gg.Nz + gg.Ny + gg.Nz);
}

size_t lelph_gs_xpass_smem(const GsGeom& gg, int fp64)
{
    const size_t e = fp64 ? sizeof(double2) : sizeof(float2);
    return e * (2 * (size_t)gg.Nx * GS_CB + gg.Nx);
}

int lelph_launch_gs_plane(const GsGeom& gg, int fp64, const void* psi, const void* win, int nu0, int nub,
                          const FftPlan1D& py, const FftPlan1D& pz, const void* twy, const void* twz, const int* cols,
                          int ncol, void* out, cudaStream_t st)
{
    const size_t smem = lelph_gs_plane_smem(gg, fp64);
    if (smem > 220 * 1024 || nub > 65535 || gg.nb > 65535 || gg.Nx > 65535) return -1;
    dim3 grid((unsigned)nub, (unsigned)gg.nb, (unsigned)gg.Nx);
    if (fp64)
    {
        if (cudaFuncSetAttribute(k_gs_plane<double2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        k_gs_plane<double2, double><<<grid, GS_THREADS, smem, st>>>(
            (const double2*)psi, (const double2*)win, gg, nu0, py, pz, (const double2*)twy, (const double2*)twz,
            cols, ncol, (double2*)out);
    }
    else
    {
        if (cudaFuncSetAttribute(k_gs_plane<float2, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        k_gs_plane<float2, float><<<grid, GS_THREADS, smem, st>>>((const float2*)psi, (const float2*)win, gg, nu0,
                                                                  py, pz, (const float2*)twy, (const float2*)twz,
                                                                  cols, ncol, (float2*)out);
    }
    return 0;
}

int lelph_launch_gs_xpass(const GsGeom& gg, int fp64, const void* in, int nrb, int ncol, const FftPlan1D& px,
                          const void* twx, const int* cst, const int* kcx, int npad, void* A, cudaStream_t st)
{
    const size_t smem = lelph_gs_xpass_smem(gg, fp64);
    if (smem > 220 * 1024 || nrb > 65535) return -1;
    dim3 grid((unsigned)((ncol + GS_CB - 1) / GS_CB), (unsigned)nrb);
    if (fp64)
    {
        if (cudaFuncSetAttribute(k_gs_xpass<double2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        k_gs_xpass<double2, double><<<grid, GS_THREADS, smem, st>>>((const double2*)in, gg.Nx, ncol, px,
                                                                    (const double2*)twx, cst, kcx, npad,
                                                                    (double2*)A);
    }
    else
    {
        if (cudaFuncSetAttribute(k_gs_xpass<float2, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        k_gs_xpass<float2, float><<<grid, GS_THREADS, smem, st>>>((const float2*)in, gg.Nx, ncol, px,
                                                                  (const float2*)twx, cst, kcx, npad, (float2*)A);
    }
    return 0;
}

int lelph_launch_gs_gemm(int fp64, const void* A, const void* B, int nrows, int nb, int Ktot, int kchunk,
                         int rowoff, int nrows_total, void* part, cudaStream_t st)
{
    const int nch = (Ktot + kchunk - 1) / kchunk;
    const int gy = (nb + GS_BN - 1) / GS_BN;
    if (nch > 65535 || gy > 65535) return -1;
    dim3 grid((unsigned)((nrows + GS_BM - 1) / GS_BM), (unsigned)gy, (unsigned)nch);
    if (fp64)
        k_gs_gemm<double, double2><<<grid, GS_THREADS, 0, st>>>((const double2*)A, (const double2*)B, nrows, nb, Ktot,
                                                                kchunk, rowoff, nrows_total, (double2*)part);
    else
        k_gs_gemm<float, float2><<<grid, GS_THREADS, 0, st>>>((const float2*)A, (const float2*)B, nrows, nb, Ktot,
                                                              kchunk, rowoff, nrows_total, (float2*)part);
    return 0;
}

void lelph_launch_gs_reduce(int fp64, const void* part, long long nel, int nchunks, double invM, double2* glocal,
                            cudaStream_t st)
{
    const int blocks = (int)std::min<long long>(4096, (nel + 255) / 256);
    if (fp64)
        k_gs_reduce<double2><<<blocks, 256, 0, st>>>((const double2*)part, nel, nchunks, invM, glocal);
    else
        k_gs_reduce<float2><<<blocks, 256, 0, st>>>((const float2*)part, nel, nchunks, invM, glocal);
}

int lelph_launch_gs_bperm(int fp64, const double2* chat, const long long* chat_off, const int* npw_k,
                          const int* npad_k, const long long* perm_off, const int* perm, const long long* bp_off,
                          int k0, int nk, int rows_per_k, int npad_max, void* Bp, cudaStream_t st)
{
    if (rows_per_k > 65535 || nk > 65535) return -1;
    dim3 grid((unsigned)((npad_max + 255) / 256), (unsigned)rows_per_k, (unsigned)nk);
    if (fp64)
        k_gs_bperm<double2><<<grid, 256, 0, st>>>(chat, chat_off, npw_k, npad_k, perm_off, perm, bp_off, k0,
                                                  rows_per_k, (double2*)Bp);
    else
        k_gs_bperm<float2><<<grid, 256, 0, st>>>(chat, chat_off, npw_k, npad_k, perm_off, perm, bp_off, k0,
                                                 rows_per_k, (float2*)Bp);
    return 0;
}
