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
// (src/wfc/gsort.c:49-93) read from the other side; a first kernel writes
// these maps for every job.  The SU(2) factors, fractional-translation phases
// and conjugations of the reference's sequence (elec_reps.c:301-372) fold per
// job onto the k2 side: D = sum_p v(p) . psi_k1(p)^(c) with
// v = C e^{-i 2 pi m.t} M psi_k2^(c'), so the k1 rows are staged into shared
// memory unchanged by asynchronous copies (double-buffered, one chunk ahead)
// and only the gathered k2 rows are transformed; the plane-wave phase is the
// product of three per-axis factors tabulated per job.  D is one complex
// contraction over (spinor, plane wave), tiled 32 x 32 and four-by-four per
// thread.
//
// Plain form: FP64 throughout.  Mixed form: the per-axis phase angles are
// reduced in FP64, operands and contraction are FP32 (an FP32 copy of the
// coefficients), with partial sums over DM_GROUP chunks added into a second
// FP32 accumulator (pairwise summation).
#include <cuda_runtime.h>
#include <stdint.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"

#define DM_TB 32       // D tile (bands) per CTA, both sides
#define DM_KC 32       // plane waves per staged chunk
#define DM_THREADS 64  // 8 x 8 threads, 4 x 4 complex entries of the tile each
#define DM_GROUP 16    // chunks per partial sum (mixed form)

#define DM_TBP 34      // staged row stride (complex): 16-byte aligned rows, 2-way conflicts on the column writes

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

template <int B> __device__ __forceinline__ void dm_cp(uint32_t dst, const void* src, int src_bytes);
template <> __device__ __forceinline__ void dm_cp<8>(uint32_t dst, const void* src, int src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
template <> __device__ __forceinline__ void dm_cp<16>(uint32_t dst, const void* src, int src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void dm_cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void dm_cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// acc += v w (CJ: acc += v conj(w))
template <bool CJ, typename T2> __device__ __forceinline__ void dm_cfma(T2& acc, T2 v, T2 w)
{
    if (CJ)
    {
        acc.x = fma(v.x, w.x, acc.x);
        acc.x = fma(v.y, w.y, acc.x);
        acc.y = fma(v.y, w.x, acc.y);
        acc.y = fma(-v.x, w.y, acc.y);
    }
    else
    {
        acc.x = fma(v.x, w.x, acc.x);
        acc.x = fma(-v.y, w.y, acc.x);
        acc.y = fma(v.x, w.y, acc.y);
        acc.y = fma(v.y, w.x, acc.y);
    }
}

// k2 position of every plane wave of the k1 list, per job (-1: not in the k2
// list): the reference's find_gvecs_idxs match read from the k1 side.
__global__ void __launch_bounds__(256) k_dm_map(const DmatJob* __restrict__ jobs, DmatGeom dg,
                                                const int* __restrict__ miller, const long long* __restrict__ pw_off,
                                                const int* __restrict__ npw_arr, const int* __restrict__ gtab,
                                                int stride, int* __restrict__ map)
{
    __shared__ DmatJob J;
    const long long ijob = blockIdx.x;
    if (threadIdx.x == 0) J = jobs[ijob];
    __syncthreads();
    const int p = blockIdx.y * blockDim.x + threadIdx.x;
    const int npw1 = npw_arr[J.ik1];
    if (p >= npw1) return;
    const int npw2 = npw_arr[J.ik2];
    const int* m = miller + 3 * (pw_off[J.ik1] + p);
    const int* mil2 = miller + 3 * pw_off[J.ik2];
    int g[3], n[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) g[r] = J.WRS1[3 * r] * m[0] + J.WRS1[3 * r + 1] * m[1] + J.WRS1[3 * r + 2] * m[2] - J.ulm[r];
#pragma unroll
    for (int r = 0; r < 3; ++r) n[r] = J.W2inv[3 * r] * g[0] + J.W2inv[3 * r + 1] * g[1] + J.W2inv[3 * r + 2] * g[2];
    const int bx = ((n[0] % dg.Nx) + dg.Nx) % dg.Nx, by = ((n[1] % dg.Ny) + dg.Ny) % dg.Ny,
              bz = ((n[2] % dg.Nz) + dg.Nz) % dg.Nz;
    const int cand = gtab[(long long)J.ik2 * dg.Nx * dg.Ny * dg.Nz + ((long long)bx * dg.Ny + by) * dg.Nz + bz];
    int ii = -1;
    if (cand >= 0 && cand < npw2)
    {
        const int* mc = mil2 + 3 * cand;
        if (mc[0] == n[0] && mc[1] == n[1] && mc[2] == n[2]) ii = cand;
    }
    map[ijob * stride + p] = ii;
}

// The contraction of one job (CJ: the k1 operand enters conjugated).
template <typename T2, int NS, bool CJ>
__device__ __forceinline__ void dm_body(const DmatJob& J, const DmatGeom& dg, const T2* __restrict__ coef,
                                        const long long* __restrict__ coef_off, const int* __restrict__ miller,
                                        const long long* __restrict__ pw_off, const int* __restrict__ npw_arr,
                                        const int* __restrict__ jmap, int spin, int b0, int a0, T2* sv, T2* sw,
                                        const T2* tab, T2* sc, int* sii, double2* __restrict__ D)
{
    constexpr bool F32 = sizeof(T2) == sizeof(float2);
    constexpr int KCS = NS * DM_KC;
    constexpr int RB = 8 / NS;  // rows loaded per batch by each thread
    const int t = threadIdx.x;
    const int nb = dg.nb;
    T2 M[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) M[e] = dm_cvt<T2>(J.M[e]);
    const bool cjv = J.conj_v != 0;
    const T2 C = dm_cvt<T2>(J.C);
    const int npw1 = npw_arr[J.ik1], npw2 = npw_arr[J.ik2];
    const int* mil1 = miller + 3 * pw_off[J.ik1];
    const T2* c1 = coef + coef_off[J.ik1] + (long long)spin * nb * NS * npw1;
    const T2* c2 = coef + coef_off[J.ik2] + (long long)spin * nb * NS * npw2;
    const int oy = dg.Nx + 1, oz = dg.Nx + dg.Ny + 2;
    const int rb = t >> 3, ca = t & 7;
    const int j = t & (DM_KC - 1), r0 = t >> 5;
    const uint32_t sw0 = smem_u32(sw);

    // the k1 rows of chunk c, copied as they are into w buffer c & 1
    auto issue_w = [&](int c) {
        const int p = c * DM_KC + j;
        const uint32_t base = sw0 + (uint32_t)((c & 1) * KCS * DM_TBP * sizeof(T2));
#pragma unroll
        for (int i = 0; i < DM_TB / 2; ++i)
        {
            const int r = r0 + 2 * i, a = a0 + r;
            const bool ok = a < nb && p < npw1;
#pragma unroll
            for (int s = 0; s < NS; ++s)
                dm_cp<sizeof(T2)>(base + (uint32_t)(((s * DM_KC + j) * DM_TBP + r) * sizeof(T2)),
                                  ok ? (const void*)(c1 + ((long long)a * NS + s) * npw1 + p) : (const void*)c1,
                                  ok ? (int)sizeof(T2) : 0);
        }
    };

    T2 acc[4][4], acc2[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[i][k] = acc2[i][k] = mk2<T2>(0.0, 0.0);

    // per-position data of the next chunk, prefetched one chunk ahead
    int pm[3] = {0, 0, 0}, pii = -1;
    if (t < DM_KC && t < npw1)
    {
        pm[0] = mil1[3 * t];
        pm[1] = mil1[3 * t + 1];
        pm[2] = mil1[3 * t + 2];
        pii = jmap[t];
    }
    issue_w(0);
    dm_cp_commit();

    const int nchunk = (npw1 + DM_KC - 1) / DM_KC;
    for (int ch = 0; ch < nchunk; ++ch)
    {
        const int p0 = ch * DM_KC;
        if (t < DM_KC)
        {
            T2 c = mk2<T2>(0.0, 0.0);
            const bool in = p0 + t < npw1;
            if (in && pii >= 0)
            {
                c = cmul(cmul(tab[pm[0] + dg.Nx / 2], tab[oy + pm[1] + dg.Ny / 2]), tab[oz + pm[2] + dg.Nz / 2]);
                c = cmul(c, C);
            }
            sc[t] = c;
            sii[t] = in ? pii : -1;
            const int pn = p0 + DM_KC + t;
            if (pn < npw1)
            {
                pm[0] = mil1[3 * pn];
                pm[1] = mil1[3 * pn + 1];
                pm[2] = mil1[3 * pn + 2];
                pii = jmap[pn];
            }
        }
        __syncthreads();  // positions of this chunk visible; the previous contraction is done
        if (ch + 1 < nchunk) issue_w(ch + 1);
        dm_cp_commit();
        {
            // k2 rows: gathered, conjugated if asked, spinor-mixed, times the phase
            const int ii = sii[j];
            const T2 c = sc[j];
#pragma unroll
            for (int bt = 0; bt < (DM_TB / 2) / RB; ++bt)
            {
                T2 x[RB][NS];
#pragma unroll
                for (int i = 0; i < RB; ++i)
                {
                    const int b = b0 + r0 + 2 * (bt * RB + i);
#pragma unroll
                    for (int s = 0; s < NS; ++s)
                        x[i][s] = (b < nb && ii >= 0) ? c2[((long long)b * NS + s) * npw2 + ii] : mk2<T2>(0.0, 0.0);
                }
#pragma unroll
                for (int i = 0; i < RB; ++i)
                {
                    const int r = r0 + 2 * (bt * RB + i);
                    T2 y0 = x[i][0];
                    if (cjv) y0 = cconj(y0);
                    if (NS == 2)
                    {
                        T2 y1 = x[i][NS - 1];
                        if (cjv) y1 = cconj(y1);
                        const T2 z0 = cadd(cmul(M[0], y0), cmul(M[1], y1));
                        const T2 z1 = cadd(cmul(M[2], y0), cmul(M[3], y1));
                        sv[(DM_KC + j) * DM_TBP + r] = cmul(z1, c);
                        y0 = z0;
                    }
                    sv[j * DM_TBP + r] = cmul(y0, c);
                }
            }
        }
        dm_cp_wait1();    // this chunk's k1 rows have landed (the next chunk's may be in flight)
        __syncthreads();
        const T2* wb = sw + (ch & 1) * KCS * DM_TBP;
#pragma unroll 8
        for (int kk = 0; kk < KCS; ++kk)
        {
            T2 v[4], w[4];
            dm_ld_pair<T2>(sv + kk * DM_TBP + 4 * rb, v[0], v[1]);
            dm_ld_pair<T2>(sv + kk * DM_TBP + 4 * rb + 2, v[2], v[3]);
            dm_ld_pair<T2>(wb + kk * DM_TBP + 4 * ca, w[0], w[1]);
            dm_ld_pair<T2>(wb + kk * DM_TBP + 4 * ca + 2, w[2], w[3]);
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int k = 0; k < 4; ++k) dm_cfma<CJ>(acc[i][k], v[i], w[k]);
        }
        if (F32 && ((ch + 1) % DM_GROUP == 0 || ch + 1 == nchunk))
        {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int k = 0; k < 4; ++k)
                {
                    acc2[i][k] = cadd(acc2[i][k], acc[i][k]);
                    acc[i][k] = mk2<T2>(0.0, 0.0);
                }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            const int b = b0 + 4 * rb + i, a = a0 + 4 * ca + k;
            const T2 r = F32 ? acc2[i][k] : acc[i][k];
            if (b < nb && a < nb) D[(long long)b * nb + a] = make_double2((double)r.x, (double)r.y);
        }
}

template <typename T2, int NS>
__global__ void __launch_bounds__(DM_THREADS, 8) k_dmats(const DmatJob* __restrict__ jobs, DmatGeom dg,
                                                         const T2* __restrict__ coef,
                                                         const long long* __restrict__ coef_off,
                                                         const int* __restrict__ miller,
                                                         const long long* __restrict__ pw_off,
                                                         const int* __restrict__ npw_arr, const int* __restrict__ map,
                                                         int stride, double2* __restrict__ out)
{
    constexpr int KCS = NS * DM_KC;
    extern __shared__ __align__(16) unsigned char dm_smem[];
    T2* sv = reinterpret_cast<T2*>(dm_smem);
    T2* sw = sv + KCS * DM_TBP;        // two buffers
    T2* tab = sw + 2 * KCS * DM_TBP;   // per-axis phase factors, (Nx+1) + (Ny+1) + (Nz+1)
    T2* sc = tab + dg.ntab;            // per-position phases of the chunk
    int* sii = reinterpret_cast<int*>(sc + DM_KC);
    __shared__ DmatJob J;

    const int t = threadIdx.x;
    const long long ijob = blockIdx.x;
    const int ntile = (dg.nb + DM_TB - 1) / DM_TB;
    const int b0 = (blockIdx.y / ntile) * DM_TB, a0 = (blockIdx.y % ntile) * DM_TB;
    const int spin = blockIdx.z;
    if (t == 0) J = jobs[ijob];
    __syncthreads();
    {
        const int Nax[3] = {dg.Nx, dg.Ny, dg.Nz};
        int base = 0;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax)
        {
            for (int i = t; i <= Nax[ax]; i += DM_THREADS) tab[base + i] = dm_phase<T2>((double)(i - Nax[ax] / 2) * J.t[ax]);
            base += Nax[ax] + 1;
        }
    }
    // (the tables are published by the first __syncthreads of the chunk loop)
    double2* D = out + (ijob * dg.nspin + spin) * (long long)dg.nb * dg.nb;
    const int* jmap = map + ijob * stride;
    if (J.conj_w)
        dm_body<T2, NS, true>(J, dg, coef, coef_off, miller, pw_off, npw_arr, jmap, spin, b0, a0, sv, sw, tab, sc,
                              sii, D);
    else
        dm_body<T2, NS, false>(J, dg, coef, coef_off, miller, pw_off, npw_arr, jmap, spin, b0, a0, sv, sw, tab, sc,
                               sii, D);
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
    return e * (3 * (size_t)dg.nspinor * DM_KC * DM_TBP + (size_t)dg.ntab + DM_KC) + sizeof(int) * DM_KC;
}

void lelph_launch_dm_gtab(const int* miller, const long long* pw_off, const int* npw, int nk, int npw_max, int Nx,
                          int Ny, int Nz, int* gtab, cudaStream_t st)
{
    dim3 grid((unsigned)((npw_max + 255) / 256), (unsigned)nk);
    k_dm_gtab<<<grid, 256, 0, st>>>(miller, pw_off, npw, nk, Nx, Ny, Nz, gtab);
}

// FP32 copy of the iBZ coefficients (the mixed form's operands)
__global__ void k_dm_c64(const double2* __restrict__ in, long long n, float2* __restrict__ out)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

void lelph_launch_dm_c64(const double2* in, long long n, float2* out, cudaStream_t st)
{
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (blocks < 1) blocks = 1;
    k_dm_c64<<<(unsigned)blocks, 256, 0, st>>>(in, n, out);
}

template <typename T2, int NS>
static int launch_dm(dim3 grid, size_t smem, cudaStream_t st, const DmatJob* jobs, const DmatGeom& dg,
                     const T2* coef, const long long* coef_off, const int* miller, const long long* pw_off,
                     const int* npw, const int* map, int stride, double2* out)
{
    if (cudaFuncSetAttribute(k_dmats<T2, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    k_dmats<T2, NS><<<grid, DM_THREADS, smem, st>>>(jobs, dg, coef, coef_off, miller, pw_off, npw, map, stride, out);
    return 0;
}

int lelph_launch_dmats(const DmatJob* jobs, long long njobs, const DmatGeom& dg, const double2* coef64,
                       const float2* coef32,
                       const long long* coef_off, const int* miller, const long long* pw_off, const int* npw,
                       const int* gtab, int npw_max, int* map, double2* out, cudaStream_t st)
{
    if (njobs <= 0) return 0;
    if (njobs > 0x7fffffffLL || npw_max <= 0) return -1;
    // index maps first (one thread per (job, plane wave)), then the contraction
    dim3 mgrid((unsigned)njobs, (unsigned)((npw_max + 255) / 256));
    k_dm_map<<<mgrid, 256, 0, st>>>(jobs, dg, miller, pw_off, npw, gtab, npw_max, map);
    const int ntile = (dg.nb + DM_TB - 1) / DM_TB;
    const size_t smem = lelph_dmats_smem_bytes(dg, coef32 ? 0 : 1);
    dim3 grid((unsigned)njobs, (unsigned)(ntile * ntile), (unsigned)dg.nspin);
    if (!coef32)
        return dg.nspinor == 2 ? launch_dm<double2, 2>(grid, smem, st, jobs, dg, coef64, coef_off, miller, pw_off,
                                                       npw, map, npw_max, out)
                               : launch_dm<double2, 1>(grid, smem, st, jobs, dg, coef64, coef_off, miller, pw_off,
                                                       npw, map, npw_max, out);
    return dg.nspinor == 2 ? launch_dm<float2, 2>(grid, smem, st, jobs, dg, coef32, coef_off, miller, pw_off, npw,
                                                  map, npw_max, out)
                           : launch_dm<float2, 1>(grid, smem, st, jobs, dg, coef32, coef_off, miller, pw_off, npw,
                                                  map, npw_max, out);
}
