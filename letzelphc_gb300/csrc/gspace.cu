// G-space route of the local sandwich: the reference's own order of work
// (elphLocal, src/dvloc/compute_Vbare_loc.c:264-310, with fft_convolution3D,
// src/fft/convolution.c:13-189): for each mode nu and band m of k,
//   F_{nu m s}(G) = sum_r e^{-i G.r} P_{nu m s}(r),
//   P_{nu m s} = dV_nu psi_{k m}  (nmag 1/2)  or  sum_s' dV_nu[s s'] psi_{k m s'}  (nmag 4),
// then one GEMM over the k+q sphere,
//   glocal[nu m][n] = (1/M) sum_{s, G in sphere(k+q)} F_{nu m s}(G) conj(c_{k+q n s}(G)).
// Everything runs on the product grid with the pair's dV window (as in the
// real-space route), so F is needed only on the k+q sphere, and the forward
// transform is pruned accordingly:
// * plane pass (k_gs_plane; k_gs_plane_ct / k_gs_plane_ct1 for square planes
//   of the common sizes): the product plane dV psi_k of one x is formed on
//   load, transformed along z then y in shared memory (y only on the z lines
//   the sphere reaches), and only the (y, z) columns that hold a plane wave
//   of the k+q sphere are written out;
// * x pass (k_gs_xpass; k_gs_xpass_ct): the x transform of those columns,
//   whose epilogue writes the sphere's values in the sphere's sorted order
//   (column, x) -- the K order of the GEMM; the k+q coefficients are stored
//   permuted to the same order (k_gs_bperm);
// * GEMM (k_gs_gemm_f32x2 in the mixed form, k_gs_gemm in FP64): complex
//   product over one K chunk; chunk partials are summed in FP64 by
//   k_gs_reduce, which also applies 1/M and writes the FP64 local term the
//   finish kernel consumes.
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

// ------------------------------------------- plane pass, compile-time sizes
// The same transform for square planes of the common product-grid sizes with
// the compile-time Stockham schedule (ct_fft, fft_smem.cuh).  The z lines sit
// at a padded stride (Nz + 1), so consecutive threads, taking consecutive
// lines, hit distinct banks; the second (y) transform runs only on the z
// lines that hold a column of the k+q sphere (their list zl; the result is
// compact, element y of line l at l + y nzl).

// grid and output as k_gs_plane; cols2[c] = y nzl + l(z) indexes the compact
// result of the pruned y transform.
template <typename T2, typename T, int NY, int NZ>
__global__ void __launch_bounds__(GS_THREADS) k_gs_plane_ct(const T2* __restrict__ psi, const T2* __restrict__ win,
                                                            GsGeom gg, int nu0, const T2* __restrict__ twy,
                                                            const T2* __restrict__ twz, const int* __restrict__ cols2,
                                                            int ncol, const int* __restrict__ zl, int nzl,
                                                            T2* __restrict__ out)
{
    static_assert(ct_smooth(NY) && ct_smooth(NZ), "2, 3, 5-smooth plane");
    constexpr int NZP = NZ + 1;       // padded z-line stride
    constexpr int NP = NY * NZP;
    extern __shared__ __align__(16) unsigned char gsc_smem[];
    T2* a = reinterpret_cast<T2*>(gsc_smem);
    T2* b = a + NP;
    T2* ty = b + NP;
    T2* tz = ty + NY;
    int* szl = reinterpret_cast<int*>(tz + NZ);
    const int nul = blockIdx.x, m = blockIdx.y, x = blockIdx.z;
    const int nu = nu0 + nul;
    for (int t = threadIdx.x; t < NY; t += blockDim.x) ty[t] = twy[t];
    for (int t = threadIdx.x; t < NZ; t += blockDim.x) tz[t] = twz[t];
    for (int t = threadIdx.x; t < nzl; t += blockDim.x) szl[t] = zl[t];
    constexpr int NPL = NY * NZ;      // points of a plane in global memory
    const long long M = (long long)gg.Nx * NPL;
    const size_t xoff = (size_t)x * NPL;
    const T2* pm = psi + (size_t)m * gg.nspinor * M + xoff;
    const T2* dv = win + (size_t)nu * gg.nmag * M + xoff;
    for (int s = 0; s < gg.nspinor; ++s)
    {
        if (gg.nmag == 4)
        {
            const T2* d0 = dv + (size_t)(2 * s) * M;
            const T2* d1 = d0 + M;
            for (int e = threadIdx.x; e < NPL; e += GS_THREADS)
                a[e + e / NZ] = cadd(cmul(d0[e], pm[e]), cmul(d1[e], pm[M + e]));
        }
        else
        {
            const T2* d0 = dv + (size_t)(gg.nmag == 2 ? gg.spin : 0) * M;
            const T2* p0 = pm + (size_t)s * M;
            for (int e = threadIdx.x; e < NPL; e += GS_THREADS) a[e + e / NZ] = cmul(d0[e], p0[e]);
        }
        __syncthreads();
        // z lines (line y at y NZP), then the y transform of the sphere's z lines
        T2* r = ct_fft<T2, T, NZ, 0, 1, true, NY>(a, b, NY, 1, NZP, nullptr, 1, NZP, tz, -1);
        T2* o = r == a ? b : a;
        r = ct_fft<T2, T, NY, 0, 1, true, 0>(r, o, nzl, NZP, 1, szl, nzl, 1, ty, -1);
        T2* dst = out + (((size_t)(nul * gg.nb + m) * gg.nspinor + s) * gg.Nx + x) * ncol;
        for (int c = threadIdx.x; c < ncol; c += GS_THREADS) dst[c] = r[cols2[c]];
        __syncthreads();
    }
}

// Epilogue store of one sphere value: as it is, or (FP32 operand of the
// tensor-core GEMM, lo given) as its TF32-rounded value and the TF32-rounded
// remainder.
__device__ __forceinline__ void gs_store(double2* hi, double2* lo, int K, double2 v)
{
    (void)lo;
    hi[K] = v;
}
__device__ __forceinline__ void gs_store(float2* hi, float2* lo, int K, float2 v)
{
    if (!lo)
    {
        hi[K] = v;
        return;
    }
    const float2 h = make_float2(tf32_rn(v.x), tf32_rn(v.y));
    hi[K] = h;
    lo[K] = make_float2(tf32_rn(v.x - h.x), tf32_rn(v.y - h.y));
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
                                                         int npad, T2* __restrict__ A, T2* __restrict__ A_lo)
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
        gs_store(dst, A_lo ? A_lo + (size_t)rb * npad : nullptr, K, r[x * GS_CB + (c - c0)]);
    }
}

// x pass for the compile-time sizes: CB columns per CTA, every load of the
// tile issued before the first is used (the generic pass waits on each), the
// x transform with the compile-time schedule, consecutive threads on
// consecutive columns (conflict-free).
template <typename T2, typename T, int NX, int CB>
__global__ void __launch_bounds__(GS_THREADS) k_gs_xpass_ct(const T2* __restrict__ in, int ncol,
                                                            const T2* __restrict__ twx, const int* __restrict__ cst,
                                                            const int* __restrict__ kcx, int npad,
                                                            T2* __restrict__ A, T2* __restrict__ A_lo)
{
    constexpr int NE = NX * CB;
    constexpr int PER = (NE + GS_THREADS - 1) / GS_THREADS;
    extern __shared__ __align__(16) unsigned char gsxc_smem[];
    T2* a = reinterpret_cast<T2*>(gsxc_smem);
    T2* b = a + NE;
    T2* tx = b + NE;
    const int c0 = blockIdx.x * CB;
    const int rb = blockIdx.y;
    for (int t = threadIdx.x; t < NX; t += blockDim.x) tx[t] = twx[t];
    const T2* src = in + (size_t)rb * NX * ncol + c0;
    T2 v[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i)
    {
        const int e = threadIdx.x + i * GS_THREADS;
        const int x = e / CB, cc = e - x * CB;
        v[i] = (e < NE && c0 + cc < ncol) ? src[(size_t)x * ncol + cc] : mk2<T2>(0.0, 0.0);
    }
#pragma unroll
    for (int i = 0; i < PER; ++i)
    {
        const int e = threadIdx.x + i * GS_THREADS;
        if (e < NE) a[e] = v[i];
    }
    __syncthreads();
    T2* r = ct_fft<T2, T, NX, 0, 1, true, CB>(a, b, CB, CB, 1, nullptr, CB, 1, tx, -1);
    const int k0 = cst[c0], k1 = cst[min(c0 + CB, ncol)];
    T2* dst = A + (size_t)rb * npad;
    T2* dlo = A_lo ? A_lo + (size_t)rb * npad : nullptr;
    for (int K = k0 + threadIdx.x; K < k1; K += blockDim.x)
    {
        const int w = kcx[K];
        const int c = w / NX, x = w - c * NX;
        gs_store(dst, dlo, K, r[x * CB + (c - c0)]);
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

// The same product for FP32 operands with a tile shaped to the band count:
// 256 threads as 32 row groups x 8 column groups, TM rows x TN columns per
// thread (columns tx + 8 j), BM = 32 TM rows, BN = 8 TN columns; BN is
// picked at launch so that the bands fill whole tiles (200 bands: 5 tiles
// of 40).  The K steps are double-buffered in shared memory by cp.async
// (8-byte copies into the K-major tiles; out-of-range elements are
// zero-filled), so no registers hold staged tiles.
__device__ __forceinline__ void gs_cp8(uint32_t dst, const void* src, bool valid)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 8 : 0)
                 : "memory");
}
__device__ __forceinline__ void gs_cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void gs_cp_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void gs_cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// A is kept planar in shared memory (real and imaginary parts in separate
// K-major tiles, copied by 4-byte cp.async), so a thread's two adjacent rows
// form one FP32x2 operand and every complex multiply-add of a row pair is two
// packed FMAs per part (5 % faster than four scalar FMAs per element):
//   re(i, i+1) += (a_re) b.x + (a_im) b.y,  im(i, i+1) += (a_im) b.x - (a_re) b.y.
template <int TM, int TN>
__global__ void __launch_bounds__(GS_THREADS, 2) k_gs_gemm_f32x2(const float2* __restrict__ A,
                                                                 const float2* __restrict__ B, int nrows, int nb,
                                                                 int Ktot, int kchunk, int rowoff, int nrows_total,
                                                                 float2* __restrict__ part)
{
    static_assert(TM % 2 == 0, "row pairs");
    constexpr int BM = 32 * TM, BN = 8 * TN, BMP = BM + 2;
    constexpr int AL = BM * GS_BK / GS_THREADS;
    constexpr int BL = (BN * GS_BK + GS_THREADS - 1) / GS_THREADS;
    extern __shared__ __align__(16) unsigned char gsx2_smem[];
    auto Are = reinterpret_cast<float(*)[GS_BK][BMP]>(gsx2_smem);                                // [2][BK][BMP]
    auto Aim = reinterpret_cast<float(*)[GS_BK][BMP]>(gsx2_smem + sizeof(float) * 2 * GS_BK * BMP);
    auto Bs = reinterpret_cast<float2(*)[GS_BK][BN + 1]>(gsx2_smem + sizeof(float) * 4 * GS_BK * BMP);
    const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3;
    const int lk = tid & 15, lr = tid >> 4;
    const int r0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * kchunk, kend = min(Ktot, kbeg + kchunk);
    float2 re[TM / 2][TN], im[TM / 2][TN];
#pragma unroll
    for (int i = 0; i < TM / 2; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) re[i][j] = im[i][j] = make_float2(0.f, 0.f);
    auto issue = [&](int k0, int buf) {
        const int k = k0 + lk;
#pragma unroll
        for (int i = 0; i < AL; ++i)
        {
            const int row = r0 + lr + 16 * i;
            const bool ok = row < nrows && k < kend;
            const float* src = ok ? reinterpret_cast<const float*>(A + (size_t)row * Ktot + k)
                                  : reinterpret_cast<const float*>(A);
            const uint32_t dre = (uint32_t)__cvta_generic_to_shared(&Are[buf][lk][lr + 16 * i]);
            const uint32_t dim_ = (uint32_t)__cvta_generic_to_shared(&Aim[buf][lk][lr + 16 * i]);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dre), "l"(src), "r"(ok ? 4 : 0)
                         : "memory");
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dim_), "l"(src + 1), "r"(ok ? 4 : 0)
                         : "memory");
        }
#pragma unroll
        for (int i = 0; i < BL; ++i)
        {
            const int e = tid + i * GS_THREADS;
            if (e < BN * GS_BK)
            {
                const int n = n0 + (e >> 4), kk = k0 + (e & 15);
                const bool ok = n < nb && kk < kend;
                gs_cp8((uint32_t)__cvta_generic_to_shared(&Bs[buf][e & 15][e >> 4]),
                       ok ? (const void*)(B + (size_t)n * Ktot + kk) : (const void*)B, ok);
            }
        }
        gs_cp_commit();
    };
    issue(kbeg, 0);
    int buf = 0;
    for (int k0 = kbeg; k0 < kend; k0 += GS_BK, buf ^= 1)
    {
        if (k0 + GS_BK < kend)
        {
            issue(k0 + GS_BK, buf ^ 1);
            gs_cp_wait1();
        }
        else
            gs_cp_wait0();
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GS_BK; ++kk)
        {
            float2 ar[TM / 2], ai[TM / 2];
#pragma unroll
            for (int i = 0; i < TM / 2; ++i)
            {
                ar[i] = *reinterpret_cast<const float2*>(&Are[buf][kk][ty * TM + 2 * i]);
                ai[i] = *reinterpret_cast<const float2*>(&Aim[buf][kk][ty * TM + 2 * i]);
            }
#pragma unroll
            for (int j = 0; j < TN; ++j)
            {
                const float2 b = Bs[buf][kk][tx + 8 * j];
                const float2 bxx = make_float2(b.x, b.x), byy = make_float2(b.y, b.y);
                const float2 nbyy = make_float2(-b.y, -b.y);
#pragma unroll
                for (int i = 0; i < TM / 2; ++i)
                {
                    re[i][j] = __ffma2_rn(ar[i], bxx, re[i][j]);
                    re[i][j] = __ffma2_rn(ai[i], byy, re[i][j]);
                    im[i][j] = __ffma2_rn(ai[i], bxx, im[i][j]);
                    im[i][j] = __ffma2_rn(ar[i], nbyy, im[i][j]);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM / 2; ++i)
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            const int row = r0 + ty * TM + 2 * i + h;
            if (row >= nrows) continue;
            float2* dst = part + ((size_t)blockIdx.z * nrows_total + rowoff + row) * nb;
#pragma unroll
            for (int j = 0; j < TN; ++j)
            {
                const int n = n0 + tx + 8 * j;
                if (n < nb) dst[n] = h ? make_float2(re[i][j].y, im[i][j].y) : make_float2(re[i][j].x, im[i][j].x);
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

// FP32, one spinor component: each CTA takes one (band, x plane) and NUC (8)
// consecutive modes; the psi plane stays in registers for all of them.  At
// most 85 registers, so three CTAs share an SM (their shared memory fits
// too) and hide each other's barriers and window loads.  (Measured: keeping
// the next window plane in registers as well, two CTAs per SM, was 9 %
// slower; two planes per CTA with 512 threads, 4 % slower; the y transform
// with radices <= 5, 12 % slower.)
template <int NY, int NZ, int NUC>
__global__ void __launch_bounds__(GS_THREADS, 3) k_gs_plane_ct1(const float2* __restrict__ psi,
                                                               const float2* __restrict__ win, GsGeom gg, int nu0,
                                                               int nub, const float2* __restrict__ twy,
                                                               const float2* __restrict__ twz,
                                                               const int* __restrict__ cols2, int ncol,
                                                               const int* __restrict__ zl, int nzl,
                                                               float2* __restrict__ out)
{
    constexpr int NZP = NZ + 1;
    constexpr int NP = NY * NZP;
    constexpr int NPL = NY * NZ;
    constexpr int PER = (NPL + GS_THREADS - 1) / GS_THREADS;
    extern __shared__ __align__(16) unsigned char gs1_smem[];
    float2* a = reinterpret_cast<float2*>(gs1_smem);
    float2* b = a + NP;
    float2* ty = b + NP;
    float2* tz = ty + NY;
    int* szl = reinterpret_cast<int*>(tz + NZ);
    const int m = blockIdx.y, x = blockIdx.z;
    const int nl0 = blockIdx.x * NUC, nl1 = min(nub, nl0 + NUC);
    for (int t = threadIdx.x; t < NY; t += blockDim.x) ty[t] = twy[t];
    for (int t = threadIdx.x; t < NZ; t += blockDim.x) tz[t] = twz[t];
    for (int t = threadIdx.x; t < nzl; t += blockDim.x) szl[t] = zl[t];
    const long long M = (long long)gg.Nx * NPL;
    const size_t xoff = (size_t)x * NPL;
    const float2* pm = psi + (size_t)m * M + xoff;
    const int comp = gg.nmag == 2 ? gg.spin : 0;
    float2 ps[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i)
    {
        const int e = threadIdx.x + i * GS_THREADS;
        ps[i] = e < NPL ? pm[e] : make_float2(0.f, 0.f);
    }
    for (int nul = nl0; nul < nl1; ++nul)
    {
        const float2* d0 = win + ((size_t)(nu0 + nul) * gg.nmag + comp) * M + xoff;
#pragma unroll
        for (int i = 0; i < PER; ++i)
        {
            const int e = threadIdx.x + i * GS_THREADS;
            if (e < NPL) a[e + e / NZ] = cmul(d0[e], ps[i]);
        }
        __syncthreads();
        float2* r = ct_fft<float2, float, NZ, 0, 1, true, NY>(a, b, NY, 1, NZP, nullptr, 1, NZP, tz, -1);
        float2* o = r == a ? b : a;
        r = ct_fft<float2, float, NY, 0, 1, true, 0>(r, o, nzl, NZP, 1, szl, nzl, 1, ty, -1);
        float2* dst = out + ((size_t)(nul * gg.nb + m) * gg.Nx + x) * ncol;
        for (int c = threadIdx.x; c < ncol; c += GS_THREADS) dst[c] = r[cols2[c]];
        __syncthreads();
    }
}

template <typename T2, typename T, int N>
static int gs_plane_ct(const GsGeom& gg, const void* psi, const void* win, int nu0, int nub, const void* twy,
                       const void* twz, const int* cols2, int ncol, const int* zl, int nzl, void* out, cudaStream_t st)
{
    const size_t smem = sizeof(T2) * (2 * (size_t)N * (N + 1) + 2 * N) + sizeof(int) * N;
    // (planes up to 64 x 64: the psi and window planes of a thread fit its registers)
    if constexpr (sizeof(T2) == sizeof(float2) && N * N <= 4096)
    {
        if (gg.nspinor == 1)
        {
            constexpr int NUC = 8;
            dim3 g1((unsigned)((nub + NUC - 1) / NUC), (unsigned)gg.nb, (unsigned)gg.Nx);
            static bool attr1 = false;
            if (!attr1)
            {
                if (cudaFuncSetAttribute(k_gs_plane_ct1<N, N, NUC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem) != cudaSuccess)
                    return -1;
                attr1 = true;
            }
            k_gs_plane_ct1<N, N, NUC><<<g1, GS_THREADS, smem, st>>>((const float2*)psi, (const float2*)win, gg, nu0, nub,
                                                                    (const float2*)twy, (const float2*)twz, cols2, ncol,
                                                                    zl, nzl, (float2*)out);
            return 0;
        }
    }
    static bool attr = false;
    if (!attr)
    {
        if (cudaFuncSetAttribute(k_gs_plane_ct<T2, T, N, N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        attr = true;
    }
    dim3 grid((unsigned)nub, (unsigned)gg.nb, (unsigned)gg.Nx);
    k_gs_plane_ct<T2, T, N, N><<<grid, GS_THREADS, smem, st>>>((const T2*)psi, (const T2*)win, gg, nu0,
                                                               (const T2*)twy, (const T2*)twz, cols2, ncol, zl, nzl,
                                                               (T2*)out);
    return 0;
}

bool lelph_gs_plane_fixed(const GsGeom& gg, int fp64)
{
    if (gg.Ny != gg.Nz) return false;
    switch (gg.Ny)
    {
    case 36: case 48: case 60: case 64: case 72: case 80: return true;
    case 96: return !fp64;  // two FP64 96 x 96 planes exceed shared memory
    default: return false;
    }
}

int lelph_launch_gs_plane(const GsGeom& gg, int fp64, const void* psi, const void* win, int nu0, int nub,
                          const FftPlan1D& py, const FftPlan1D& pz, const void* twy, const void* twz, const int* cols,
                          int ncol, const int* cols2, const int* zl, int nzl, void* out, cudaStream_t st)
{
    const size_t smem = lelph_gs_plane_smem(gg, fp64);
    if (smem > 220 * 1024 || nub > 65535 || gg.nb > 65535 || gg.Nx > 65535) return -1;
    if (lelph_gs_plane_fixed(gg, fp64) && cols2 && zl)
    {
#define GS_CT(N)                                                                                                       case N:                                                                                                                return fp64 ? gs_plane_ct<double2, double, N>(gg, psi, win, nu0, nub, twy, twz, cols2, ncol, zl, nzl, out, st)                     : gs_plane_ct<float2, float, N>(gg, psi, win, nu0, nub, twy, twz, cols2, ncol, zl, nzl, out, st);
        switch (gg.Ny)
        {
            GS_CT(36)
            GS_CT(48)
            GS_CT(60)
            GS_CT(64)
            GS_CT(72)
            GS_CT(80)
        case 96:
            if (fp64) break;
            return gs_plane_ct<float2, float, 96>(gg, psi, win, nu0, nub, twy, twz, cols2, ncol, zl, nzl, out, st);
        default:
            break;
        }
#undef GS_CT
    }
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

template <typename T2, typename T, int NX, int CB>
static int gs_xpass_ct(int nrb, int ncol, const void* twx, const int* cst, const int* kcx, int npad, const void* in,
                       void* A, void* A_lo, cudaStream_t st)
{
    const size_t smem = sizeof(T2) * (2 * (size_t)NX * CB + NX);
    static bool attr = false;
    if (!attr)
    {
        if (cudaFuncSetAttribute(k_gs_xpass_ct<T2, T, NX, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        attr = true;
    }
    dim3 grid((unsigned)((ncol + CB - 1) / CB), (unsigned)nrb);
    k_gs_xpass_ct<T2, T, NX, CB><<<grid, GS_THREADS, smem, st>>>((const T2*)in, ncol, (const T2*)twx, cst, kcx, npad,
                                                                (T2*)A, (T2*)A_lo);
    return 0;
}

int lelph_launch_gs_xpass(const GsGeom& gg, int fp64, const void* in, int nrb, int ncol, const FftPlan1D& px,
                          const void* twx, const int* cst, const int* kcx, int npad, void* A, cudaStream_t st,
                          void* A_lo)
{
    if (fp64) A_lo = nullptr;
    const size_t smem = lelph_gs_xpass_smem(gg, fp64);
    if (smem > 220 * 1024 || nrb > 65535) return -1;
#define GS_XC(N)                                                                                            \
    case N:                                                                                                 \
        return fp64 ? gs_xpass_ct<double2, double, N, 32>(nrb, ncol, twx, cst, kcx, npad, in, A, A_lo, st)  \
                    : gs_xpass_ct<float2, float, N, 64>(nrb, ncol, twx, cst, kcx, npad, in, A, A_lo, st);
    switch (gg.Nx)
    {
        GS_XC(36)
        GS_XC(48)
        GS_XC(60)
        GS_XC(64)
        GS_XC(72)
        GS_XC(80)
        GS_XC(96)
    default:
        break;
    }
#undef GS_XC
    dim3 grid((unsigned)((ncol + GS_CB - 1) / GS_CB), (unsigned)nrb);
    if (fp64)
    {
        if (cudaFuncSetAttribute(k_gs_xpass<double2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        k_gs_xpass<double2, double><<<grid, GS_THREADS, smem, st>>>((const double2*)in, gg.Nx, ncol, px,
                                                                    (const double2*)twx, cst, kcx, npad,
                                                                    (double2*)A, nullptr);
    }
    else
    {
        if (cudaFuncSetAttribute(k_gs_xpass<float2, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        k_gs_xpass<float2, float><<<grid, GS_THREADS, smem, st>>>((const float2*)in, gg.Nx, ncol, px,
                                                                  (const float2*)twx, cst, kcx, npad, (float2*)A,
                                                                  (float2*)A_lo);
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
    {
        k_gs_gemm<double, double2><<<grid, GS_THREADS, 0, st>>>((const double2*)A, (const double2*)B, nrows, nb, Ktot,
                                                                kchunk, rowoff, nrows_total, (double2*)part);
        return 0;
    }
    // FP32: column tile of 32, 40, 48 or 64 bands, the one wasting the fewest columns
    int best = 64, waste = 1 << 30;
    for (int bn : {64, 48, 40, 32})
    {
        const int w = (nb + bn - 1) / bn * bn - nb;
        if (w < waste)
        {
            waste = w;
            best = bn;
        }
    }
    // 256-row tiles (8 rows per thread) for the narrow column tiles when the rows fill them
    const bool tall = best <= 40 && nrows >= 2048;
    const int bm = tall ? 256 : 128;
    dim3 g2((unsigned)((nrows + bm - 1) / bm), (unsigned)((nb + best - 1) / best), (unsigned)nch);
#define GS_G2(TM, TN)                                                                                            \
    do                                                                                                           \
    {                                                                                                            \
        const int sm = (int)(sizeof(float) * 4 * GS_BK * (32 * TM + 2) + sizeof(float2) * 2 * GS_BK * (8 * TN + 1)); \
        static bool at = false;                                                                                  \
        if (!at)                                                                                                 \
        {                                                                                                        \
            if (cudaFuncSetAttribute(k_gs_gemm_f32x2<TM, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) != \
                cudaSuccess)                                                                                     \
                return -1;                                                                                       \
            at = true;                                                                                           \
        }                                                                                                        \
        k_gs_gemm_f32x2<TM, TN><<<g2, GS_THREADS, sm, st>>>((const float2*)A, (const float2*)B, nrows, nb, Ktot,  \
                                                            kchunk, rowoff, nrows_total, (float2*)part);         \
    } while (0)
    if (best == 64) GS_G2(4, 8);
    else if (best == 48) GS_G2(4, 6);
    else if (best == 40) { if (tall) GS_G2(8, 5); else GS_G2(4, 5); }
    else { if (tall) GS_G2(8, 4); else GS_G2(4, 4); }
#undef GS_G2
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
