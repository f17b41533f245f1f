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

#include <algorithm>

#include "lelph_common.cuh"
#include "lelph_internal.h"
#include "tc_operands.cuh"

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

// FP32 copy of the iBZ coefficients with the plane wave outermost within each
// (k, spin) block, [pw][band][spinor]: the tensor-core Dmats gather all bands
// of one matched plane wave in one coalesced read
__global__ void k_dm_c64t(const double2* __restrict__ in, const long long* __restrict__ coef_off,
                          const int* __restrict__ npw_arr, int nspin, int nb, int ns, float2* __restrict__ out)
{
    const int ik = blockIdx.y;
    const int npw = npw_arr[ik];
    const long long base = coef_off[ik];
    const long long n = (long long)nspin * nb * ns * npw;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        // i in the output order (spin, pw, band, spinor)
        const int t = (int)(i % ns);
        long long r = i / ns;
        const int b = (int)(r % nb);
        r /= nb;
        const int g = (int)(r % npw);
        const int sp = (int)(r / npw);
        const double2 v = in[base + (((long long)sp * nb + b) * ns + t) * npw + g];
        out[base + i] = make_float2((float)v.x, (float)v.y);
    }
}

void lelph_launch_dm_c64t(const double2* in, const long long* coef_off, const int* npw, int nk, int nspin, int nb,
                          int ns, float2* out, cudaStream_t st)
{
    k_dm_c64t<<<dim3(64, (unsigned)nk), 256, 0, st>>>(in, coef_off, npw, nspin, nb, ns, out);
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

// ============================================================ tensor cores
//
// Mixed form on tcgen05 (k_dmats_tc).  Jobs that share the irreducible k1 and
// the conjugation of its rows share the right operand, so a work unit is a
// group of up to JB such jobs, one spin, one 128-row tile of the k1 side and
// one tile of k2 bands.  As a real GEMM with K = (re, im) over (spinor,
// plane wave of k1):
//   A row 2a     = (yr, -yi)  [y~ = y]      or (yr, yi)   [y~ = conj y]
//   A row 2a + 1 = (yi, yr)                 or (-yi, yr)
//   B row (j, b) = (vr, vi)
// so D[2a][(j, b)] = Re D_j[b][a] and D[2a + 1][(j, b)] = Im D_j[b][a].
// Producer warps build both operands per 16-plane-wave stage in shared memory
// as TF32 (hi, lo) pairs in the 128-byte swizzled K-major layout: the k1 rows
// from the FP32 coefficients; the k2 rows gathered through the job's map,
// conjugated, spinor-mixed and multiplied by the plane-wave phase, which comes
// from per-job per-axis tables (angles reduced in FP64) and is formed with the
// map lookups once per 8 stages.  The MMA issue, the two accumulators (hi.hi;
// hi.lo + lo.hi), the drains and the FP64 output sums are those of the
// tensor-core projections (projections_tc.cu).

#define DT_G 16          // plane waves per stage
#define DT_CH 16         // stages per FP32 sum
// producer warps: 8, or 7 with two drain groups (512 threads: 128 registers a thread)
#define DT_PW(NDR) ((NDR) == 1 ? 8 : 7)
#define DT_JB 8          // jobs per unit at most
#define DT_PG 8          // stages per position-data phase
#define DT_NST_MAX 4
#define DT_SMEM_LIMIT (227 * 1024)
#define DT_THREADS(NDR) (32 * (1 + DT_PW(NDR) + 4 * (NDR)))

// per-job data of a unit in shared memory
struct DtJobS
{
    float2 M[4];
    float2 C;
    long long c2off;  // FP32 coefficients of k2 for the unit's spin
    int npw2, conj_v, pad[2];
};

struct DtLayout
{
    uint32_t a_bytes, b_bytes, stage_bytes, nst;
    uint32_t job_off, tab_off, pos_off, pos_n, bar_off, total;
};

__host__ __device__ inline DtLayout dt_layout(int NT, int ntab)
{
    DtLayout L;
    L.a_bytes = 128 * 128;
    L.b_bytes = (uint32_t)NT * 128;
    L.stage_bytes = 2 * L.a_bytes + 2 * L.b_bytes;
    L.pos_n = DT_PG * DT_G * DT_JB;  // (stage, position, job) entries per buffer
    const uint32_t job_bytes = DT_JB * sizeof(DtJobS);
    const uint32_t tab_bytes = (DT_JB * (uint32_t)ntab * 8 + 15) / 16 * 16;
    const uint32_t pos_bytes = 2 * L.pos_n * 12;  // two buffers of (int map, float2 phase)
    const uint32_t other = job_bytes + tab_bytes + pos_bytes + 256 + 1024;
    L.nst = other < DT_SMEM_LIMIT ? (DT_SMEM_LIMIT - other) / L.stage_bytes : 0;
    if (L.nst > DT_NST_MAX) L.nst = DT_NST_MAX;
    L.job_off = L.nst * L.stage_bytes;
    L.tab_off = L.job_off + job_bytes;
    L.pos_off = L.tab_off + tab_bytes;
    L.bar_off = L.pos_off + pos_bytes;
    L.total = L.bar_off + 256 + 1024;
    return L;
}

struct DtUnit
{
    int grp, spin, mt, nt;
};

__device__ __forceinline__ DtUnit dt_unit(int u, int nspin, int mtiles, int ntiles)
{
    DtUnit w;
    w.nt = u % ntiles;
    int t = u / ntiles;
    w.mt = t % mtiles;
    t /= mtiles;
    w.spin = t % nspin;
    w.grp = t / nspin;
    return w;
}

template <int NDR, int NS>
__global__ void __launch_bounds__(DT_THREADS(NDR), 1)
    k_dmats_tc(const DmatGroup* __restrict__ groups, const int* __restrict__ perm, int nunits, int mtiles, int ntiles,
               int NT, int nbt, const DmatJob* __restrict__ jobs, DmatGeom dg, const float2* __restrict__ coef,
               const float2* __restrict__ coefT, const long long* __restrict__ coef_off,
               const int* __restrict__ miller,
               const long long* __restrict__ pw_off, const int* __restrict__ npw_arr, const int* __restrict__ map,
               int stride, double2* __restrict__ out, unsigned* __restrict__ status, unsigned long long wait_ns)
{
    extern __shared__ __align__(1024) uint8_t dt_raw[];
    uint8_t* sm = dt_raw + ((1024u - (smem_u32(dt_raw) & 1023u)) & 1023u);
    const DtLayout L = dt_layout(NT, dg.ntab);
    uint64_t* sfull = reinterpret_cast<uint64_t*>(sm + L.bar_off);
    uint64_t* sfree = sfull + DT_NST_MAX;
    uint64_t* accf = sfree + DT_NST_MAX;
    uint64_t* acce = accf + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    DtJobS* jobs_s = reinterpret_cast<DtJobS*>(sm + L.job_off);
    float2* tab_s = reinterpret_cast<float2*>(sm + L.tab_off);  // [DT_JB][ntab]
    int* pos_ii = reinterpret_cast<int*>(sm + L.pos_off);       // [2][pos_n]
    float2* pos_c = reinterpret_cast<float2*>(pos_ii + 2 * L.pos_n);
    const int NST = (int)L.nst;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ndrain = 4 * NDR;
    const int nb = dg.nb;
    const uint32_t tcols = (4 * NT <= 64) ? 64u : (4 * NT <= 128) ? 128u : (4 * NT <= 256) ? 256u : 512u;
    constexpr int PW = DT_PW(NDR), PTH = 32 * PW;
    constexpr int NA = (512 + PTH - 1) / PTH;  // k1-row tasks (64 row pairs x 8 chunks) per producer thread

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < NST; ++s)
        {
            mbar_init(&sfull[s], PW);
            mbar_init(&sfree[s], 1);
        }
        for (int b = 0; b < 2; ++b)
        {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], ndrain);
        }
        *abort_flag = 0;
        fence_barrier_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, tcols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0)
    {
        if (lane == 0)
        {
            // ---------------- MMA issue: hi.hi into one accumulator, the cross terms into a second
            const uint32_t idesc = umma_idesc_tf32(128u, (uint32_t)NT);
            int s = 0, b = 0;
            uint32_t phs = 0, phb = 0;
            uint64_t* last_commit = nullptr;
            uint32_t last_par = 0;
            bool stop = false;
            for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
            {
                const DtUnit w = dt_unit(u, dg.nspin, mtiles, ntiles);
                const int npw1 = npw_arr[groups[w.grp].ik1];
                const int nstage = NS * ((npw1 + DT_G - 1) / DT_G);
                for (int it = 0; it < nstage; ++it)
                {
                    bool ok = mbar_wait_bounded(&acce[b], phb ^ 1u, wait_ns) && mbar_wait_bounded(&sfull[s], phs, wait_ns);
                    if (!ok)
                    {
                        *abort_flag = 1;
                        atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t base = smem_u32(sm + s * L.stage_bytes);
                    const uint64_t ahi = umma_desc_sw128(base), alo = umma_desc_sw128(base + L.a_bytes);
                    const uint64_t bhi = umma_desc_sw128(base + 2 * L.a_bytes);
                    const uint64_t blo = umma_desc_sw128(base + 2 * L.a_bytes + L.b_bytes);
                    const uint32_t dacc = tmem + (uint32_t)b * 2u * (uint32_t)NT, dx = dacc + (uint32_t)NT;
#pragma unroll
                    for (int k = 0; k < 4; ++k) umma_tf32(dacc, ahi + 2 * k, bhi + 2 * k, idesc, k > 0 ? 1u : 0u);
#pragma unroll
                    for (int k = 0; k < 4; ++k) umma_tf32(dx, ahi + 2 * k, blo + 2 * k, idesc, k > 0 ? 1u : 0u);
#pragma unroll
                    for (int k = 0; k < 4; ++k) umma_tf32(dx, alo + 2 * k, bhi + 2 * k, idesc, 1u);
                    umma_commit(&sfree[s]);
                    umma_commit(&accf[b]);
                    last_commit = &accf[b];
                    last_par = phb;
                    if (++s == NST)
                    {
                        s = 0;
                        phs ^= 1u;
                    }
                    if (++b == 2)
                    {
                        b = 0;
                        phb ^= 1u;
                    }
                }
            }
            if (last_commit) mbar_wait_bounded(last_commit, last_par);
        }
    }
    else if (warp <= PW)
    {
        // ---------------- producers
        const int p = threadIdx.x - 32;
        const int oy = dg.Nx + 1, oz = dg.Nx + dg.Ny + 2;
        int s = 0, npg = 0;
        uint32_t phs = 0;
        bool failed = false;
        for (int u = blockIdx.x; u < nunits; u += gridDim.x)
        {
            const DtUnit w = dt_unit(u, dg.nspin, mtiles, ntiles);
            const DmatGroup G = groups[w.grp];
            const int npw1 = npw_arr[G.ik1];
            const int nps = (npw1 + DT_G - 1) / DT_G;
            const int nstage = NS * nps;
            const int* mil1 = miller + 3 * pw_off[G.ik1];
            const float2* c1 = coef + coef_off[G.ik1] + (long long)w.spin * nb * NS * npw1;
            // the previous unit's stages are formed before its job data is replaced
            if (tc_producer_bar_any<PTH>(failed)) break;
            for (int e = p; e < G.count * (1 + dg.ntab); e += PTH)
            {
                const int j = e / (1 + dg.ntab), i = e % (1 + dg.ntab);
                const DmatJob& J = jobs[perm[G.first + j]];
                if (i == 0)
                {
                    DtJobS js;
                    for (int m = 0; m < 4; ++m) js.M[m] = dm_cvt<float2>(J.M[m]);
                    js.C = dm_cvt<float2>(J.C);
                    js.npw2 = npw_arr[J.ik2];
                    js.c2off = coef_off[J.ik2] + (long long)w.spin * nb * NS * js.npw2;
                    js.conj_v = J.conj_v;
                    jobs_s[j] = js;
                }
                else
                {
                    // per-axis phase factors e^{-i 2 pi_T (m - N/2 ... ) t_ax}
                    const int ti = i - 1;
                    const int ax = ti <= dg.Nx ? 0 : (ti <= dg.Nx + dg.Ny + 1 ? 1 : 2);
                    const int base = ax == 0 ? 0 : (ax == 1 ? oy : oz);
                    const int Nax = ax == 0 ? dg.Nx : (ax == 1 ? dg.Ny : dg.Nz);
                    tab_s[j * dg.ntab + ti] = dm_phase<float2>((double)(ti - base - Nax / 2) * J.t[ax]);
                }
            }
            if (tc_producer_bar_any<PTH>(failed)) break;
            bool leave = false;
            int cur = 0;  // position-data buffer of the current group of stages
            for (int it = 0; it < nstage; ++it)
            {
                const int sg = it % DT_PG;
                if (sg == 0)
                {
                    // map lookups and plane-wave phases of the next DT_PG stages
                    cur = npg & 1;
                    ++npg;
                    int* pii = pos_ii + cur * L.pos_n;
                    float2* pc = pos_c + cur * L.pos_n;
                    for (int e = p; e < DT_PG * DT_G * DT_JB; e += PTH)
                    {
                        const int pp = e % DT_G, j = (e / DT_G) % DT_JB, sgi = e / (DT_JB * DT_G);
                        const int st_i = it + sgi;
                        int ii = -1;
                        float2 c = make_float2(0.f, 0.f);
                        if (st_i < nstage && j < G.count)
                        {
                            const int pw = (st_i % nps) * DT_G + pp;
                            if (pw < npw1)
                            {
                                ii = map[(long long)perm[G.first + j] * stride + pw];
                                if (ii >= 0)
                                {
                                    const float2* tb = tab_s + j * dg.ntab;
                                    const int* m = mil1 + 3 * pw;
                                    c = cmul(cmul(tb[m[0] + dg.Nx / 2], tb[oy + m[1] + dg.Ny / 2]),
                                             tb[oz + m[2] + dg.Nz / 2]);
                                    c = cmul(c, jobs_s[j].C);
                                }
                            }
                        }
                        pii[e] = ii;
                        pc[e] = c;
                    }
                    if (tc_producer_bar_any<PTH>(failed))
                    {
                        leave = true;
                        break;
                    }
                }
                const int sp = it / nps, p0 = (it % nps) * DT_G;
                // the slot wait, decided for the whole warp: the fill below ends in a
                // __syncwarp, which every lane must reach
                if (!failed)
                {
                    const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&sfree[s], phs ^ 1u, wait_ns));
                    if (!ok)
                    {
                        failed = true;
                        if (lane == 0)
                        {
                            *abort_flag = 1;
                            atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                        }
                    }
                }
                if (!failed)
                {
                    uint8_t* st = sm + s * L.stage_bytes;
                    uint8_t* Ahi = st;
                    uint8_t* Alo = st + L.a_bytes;
                    uint8_t* Bhi = st + 2 * L.a_bytes;
                    uint8_t* Blo = Bhi + L.b_bytes;
                    // A: k1 rows a of the tile, chunk c = plane waves 2c, 2c + 1
#pragma unroll
                    for (int i = 0; i < NA; ++i)
                    {
                        const int tau = p + PTH * i;
                        if (tau >= 512) break;
                        const int rp = tau >> 3, c = tau & 7;
                        const int a = w.mt * 64 + rp;
                        float2 y[2];
#pragma unroll
                        for (int e = 0; e < 2; ++e)
                        {
                            const int pw = p0 + 2 * c + e;
                            y[e] = (a < nb && pw < npw1) ? c1[((long long)a * NS + sp) * npw1 + pw] : make_float2(0.f, 0.f);
                        }
                        float4 r0, r1;
                        if (G.conj_w)
                        {
                            r0 = make_float4(y[0].x, y[0].y, y[1].x, y[1].y);
                            r1 = make_float4(-y[0].y, y[0].x, -y[1].y, y[1].x);
                        }
                        else
                        {
                            r0 = make_float4(y[0].x, -y[0].y, y[1].x, -y[1].y);
                            r1 = make_float4(y[0].y, y[0].x, y[1].y, y[1].x);
                        }
                        float4 h, l;
                        tc_split4_tf32(r0, h, l);
                        *reinterpret_cast<float4*>(Ahi + tc_swz128(2 * rp, c)) = h;
                        *reinterpret_cast<float4*>(Alo + tc_swz128(2 * rp, c)) = l;
                        tc_split4_tf32(r1, h, l);
                        *reinterpret_cast<float4*>(Ahi + tc_swz128(2 * rp + 1, c)) = h;
                        *reinterpret_cast<float4*>(Alo + tc_swz128(2 * rp + 1, c)) = l;
                    }
                    // B: k2 rows (job j, band b), chunk c
                    const int* pii = pos_ii + cur * L.pos_n + sg * DT_G * DT_JB;
                    const float2* pc = pos_c + cur * L.pos_n + sg * DT_G * DT_JB;
                    // lanes over consecutive rows (bands of a job) of one chunk: the bands
                    // of a matched plane wave are contiguous in the plane-wave-major copy,
                    // and the chunk's map and phase entries are read by broadcast.  First
                    // every gather of the stage, then the transforms and stores.
                    constexpr int NBT = (128 * 8 + PTH - 1) / PTH;
                    float2 xg[NBT][2][NS];
#pragma unroll
                    for (int i = 0; i < NBT; ++i)
                    {
                        const int tau = p + PTH * i;
                        const int n = tau % NT, c = tau / NT;
                        const int j = n / nbt, b = w.nt * nbt + n % nbt;
                        const bool row_ok = tau < NT * 8 && j < G.count && b < nb;
#pragma unroll
                        for (int e = 0; e < 2; ++e)
                        {
                            const int ii = row_ok ? pii[j * DT_G + 2 * c + e] : -1;
                            const float2* c2 = coefT + (row_ok ? jobs_s[j].c2off : 0);
#pragma unroll
                            for (int t = 0; t < NS; ++t)
                                xg[i][e][t] = ii >= 0 ? c2[((long long)ii * nb + b) * NS + t] : make_float2(0.f, 0.f);
                        }
                    }
#pragma unroll
                    for (int i = 0; i < NBT; ++i)
                    {
                        const int tau = p + PTH * i;
                        if (tau < NT * 8)
                        {
                            const int n = tau % NT, c = tau / NT;
                            const int j = min(n / nbt, DT_JB - 1), b = w.nt * nbt + n % nbt;
                            const bool row_ok = n / nbt < G.count && b < nb;
                            const DtJobS& js = jobs_s[j];
                            float2 v[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
                            for (int e = 0; e < 2 && row_ok; ++e)
                            {
                                float2 y0 = xg[i][e][0];
                                if (js.conj_v) y0 = cconj(y0);
                                float2 r = y0;
                                if (NS == 2)
                                {
                                    float2 y1 = xg[i][e][NS - 1];
                                    if (js.conj_v) y1 = cconj(y1);
                                    r = sp == 0 ? cadd(cmul(js.M[0], y0), cmul(js.M[1], y1))
                                                : cadd(cmul(js.M[2], y0), cmul(js.M[3], y1));
                                }
                                // unmatched or padding entries gathered zeros; the phase is zero there too
                                v[e] = cmul(r, pc[j * DT_G + 2 * c + e]);
                            }
                            float4 h, l;
                            tc_split4_tf32(make_float4(v[0].x, v[0].y, v[1].x, v[1].y), h, l);
                            *reinterpret_cast<float4*>(Bhi + tc_swz128(n, c)) = h;
                            *reinterpret_cast<float4*>(Blo + tc_swz128(n, c)) = l;
                        }
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&sfull[s]);
                }
                if (++s == NST)
                {
                    s = 0;
                    phs ^= 1u;
                }
            }
            if (leave) break;
        }
    }
    else if (warp < 1 + PW + ndrain)
    {
        // ---------------- drains: lane quadrant warp % 4, columns [64 cg, 64 cg + 64)
        const int dw = warp - 1 - PW;
        const int q = warp & 3, cg = dw >> 2;
        const int r = q * 32 + lane;
        const int part = r & 1;
        int b = 0;
        uint32_t phb = 0;
        bool stop = false;
        for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
        {
            const DtUnit w = dt_unit(u, dg.nspin, mtiles, ntiles);
            const DmatGroup G = groups[w.grp];
            const int npw1 = npw_arr[G.ik1];
            const int nstage = NS * ((npw1 + DT_G - 1) / DT_G);
            const int a = (w.mt * 128 + r) >> 1;
            float acc[64];
#pragma unroll
            for (int j = 0; j < 64; ++j) acc[j] = 0.f;
            for (int it = 0; it < nstage; ++it)
            {
                bool ok = (*abort_flag == 0) && mbar_wait_bounded(&accf[b], phb, wait_ns);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok)
                {
                    if (lane == 0 && *abort_flag == 0)
                    {
                        *abort_flag = 1;
                        atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                    }
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t ta =
                    tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)b * 2u * (uint32_t)NT + (uint32_t)(cg * 64);
#pragma unroll
                for (int c = 0; c < 64; c += 16)
                    if (cg * 64 + c < NT)
                    {
                        float v[16], x[16];
                        tmem_ld16(ta + (uint32_t)c, v);
                        tmem_ld16(ta + (uint32_t)(NT + c), x);
#pragma unroll
                        for (int j = 0; j < 16; ++j) acc[c + j] += v[j] + x[j];
                    }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acce[b]);
                if (++b == 2)
                {
                    b = 0;
                    phb ^= 1u;
                }
                if ((it % DT_CH) == DT_CH - 1 || it == nstage - 1)
                {
                    // this chunk's FP32 sums into the FP64 output (even lane of a row pair)
#pragma unroll
                    for (int c = 0; c < 64; c += 8)
                    {
#pragma unroll
                        for (int jj = 0; jj < 8; ++jj)
                        {
                            const int n = cg * 64 + c + jj;
                            const float other = __shfl_xor_sync(0xffffffffu, acc[c + jj], 1);
                            const int j = n / nbt, bb = w.nt * nbt + n % nbt;
                            if (part == 0 && a < nb && n < NT && n < DT_JB * nbt && j < G.count && bb < nb)
                            {
                                double2* o = out + ((long long)perm[G.first + j] * dg.nspin + w.spin) * nb * nb +
                                             (long long)bb * nb + a;
                                double2 t = *o;
                                t.x += (double)acc[c + jj];
                                t.y += (double)other;
                                *o = t;
                            }
                            acc[c + jj] = 0.f;
                        }
                        asm volatile("" ::: "memory");
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
    {
        tc_fence_after();
        tmem_dealloc(tmem, tcols);
    }
}

// jobs per unit (JB), k2 bands per tile (nbt), B rows (NT) and band tiles:
// up to 64 bands, JB = 128 / nb jobs (at most 8) of all bands; more bands, one
// job per unit in tiles of at most 128 bands
void lelph_dmats_tc_config(int nb, int* JB, int* nbt, int* NT, int* ntiles)
{
    if (nb <= 64)
    {
        *JB = std::min(DT_JB, 128 / nb);
        *nbt = nb;
        *ntiles = 1;
        *NT = (*JB * nb + 15) / 16 * 16;
    }
    else
    {
        *JB = 1;
        const int nt = (nb + 127) / 128;
        *nbt = ((nb + nt - 1) / nt + 15) / 16 * 16;
        *ntiles = (nb + *nbt - 1) / *nbt;
        *NT = *nbt;
    }
}

int lelph_dmats_tc_supported(const DmatGeom& dg)
{
    int JB, nbt, NT, ntiles;
    lelph_dmats_tc_config(dg.nb, &JB, &nbt, &NT, &ntiles);
    return NT <= 128 && dt_layout(NT, dg.ntab).nst >= 2 && (dg.nspinor == 1 || dg.nspinor == 2);
}

template <int NDR, int NS>
static int dt_launch(int grid, size_t smem, cudaStream_t st, const DmatGroup* groups, const int* perm, int units,
                     int mtiles, int ntiles, int NT, int nbt, const DmatJob* jobs, const DmatGeom& dg,
                     const float2* coef, const float2* coefT, const long long* coef_off, const int* miller,
                     const long long* pw_off,
                     const int* npw, const int* map, int stride, double2* out, unsigned* status,
                     unsigned long long wait_ns)
{
    if (cudaFuncSetAttribute(k_dmats_tc<NDR, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return -1;
    k_dmats_tc<NDR, NS><<<grid, DT_THREADS(NDR), smem, st>>>(groups, perm, units, mtiles, ntiles, NT, nbt, jobs, dg,
                                                              coef, coefT, coef_off, miller, pw_off, npw, map, stride,
                                                              out, status, wait_ns);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int lelph_launch_dmats_tc(const DmatJob* jobs, long long njobs, const DmatGroup* groups, const int* perm,
                          int ngroups, const DmatGeom& dg, const float2* coef32, const float2* coef32t,
                          const long long* coef_off, const int* miller, const long long* pw_off, const int* npw,
                          const int* gtab, int npw_max, int* map, double2* out, unsigned* status,
                          unsigned long long wait_ns, cudaStream_t st)
{
    if (njobs <= 0) return 0;
    if (njobs > 0x7fffffffLL || npw_max <= 0 || !lelph_dmats_tc_supported(dg)) return -1;
    if (wait_ns == 0) wait_ns = LELPH_WAIT_LIMIT_NS;
    dim3 mgrid((unsigned)njobs, (unsigned)((npw_max + 255) / 256));
    k_dm_map<<<mgrid, 256, 0, st>>>(jobs, dg, miller, pw_off, npw, gtab, npw_max, map);
    if (cudaMemsetAsync(out, 0, sizeof(double2) * (size_t)njobs * dg.nspin * dg.nb * dg.nb, st) != cudaSuccess)
        return -1;
    int JB, nbt, NT, ntiles;
    lelph_dmats_tc_config(dg.nb, &JB, &nbt, &NT, &ntiles);
    const int mtiles = (dg.nb + 63) / 64;
    const long long units = (long long)ngroups * dg.nspin * mtiles * ntiles;
    if (units <= 0 || units > (1LL << 30)) return -1;
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<long long>(units, nsm);
    const size_t smem = dt_layout(NT, dg.ntab).total;
    const int ndr = (NT + 63) / 64;
#define DT_ARGS grid, smem, st, groups, perm, (int)units, mtiles, ntiles, NT, nbt, jobs, dg, coef32, coef32t, \
                coef_off, miller, pw_off, npw, map, npw_max, out, status, wait_ns
    if (dg.nspinor == 2) return ndr == 1 ? dt_launch<1, 2>(DT_ARGS) : dt_launch<2, 2>(DT_ARGS);
    return ndr == 1 ? dt_launch<1, 1>(DT_ARGS) : dt_launch<2, 1>(DT_ARGS);
#undef DT_ARGS
}
