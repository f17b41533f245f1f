// G-space route, mixed form: the band sandwich over the k+q sphere on the
// 5th-generation tensor cores.
//
//   part[chunk][rowoff + row][n] = sum_{K in chunk} A[row][K] conj(B[n][K])
//
// is the product of elphLocal (src/dvloc/compute_Vbare_loc.c:323-326, the
// matmul_cmplx of the convolved rows against the k+q coefficients).  It runs
// as a real GEMM with K = (re, im) interleaved:
//   Re = sum ar br + ai bi  ->  B row 2n     = (br, bi)
//   Im = sum ai br - ar bi  ->  B row 2n + 1 = (-bi, br)
// so the accumulator columns 2n, 2n + 1 are the (re, im) pair of band n and
// a row of the partials is the float2 layout k_gs_reduce reads.
//
// Precision: TF32 operands split into hi = rn_tf32(v) and lo = rn_tf32(v - hi)
// (about 22 significant bits together, the 8-bit exponent of FP32: no operand
// scaling), three products hi hi + hi lo + lo hi per K step (kind::tf32,
// K = 8), FP32 accumulation in tensor memory.  The accumulator loses low-order
// bits on every accumulation, so each chain is one 32-element K stage (12
// MMAs); drain warps add every finished chain into FP32 registers and write
// one partial per K chunk, summed in FP64 by k_gs_reduce.
//
// k_gs_gemm_tc: persistent, one CTA per SM over units (K chunk, 128-row
// tile, N tile), N tile fastest so that the CTAs that share an A tile run
// together (A read from HBM once, its other reads hit L2) and chunk slowest
// so that the B chunk in flight stays in L2.  Warp 0 issues the TMA loads of a
// stage (A hi, A lo: 128 x 32 FP32; B hi, B lo: NT x 32 FP32; 128-byte
// swizzle), warp 1 owns the tensor memory and issues the MMAs, warps 2-5
// drain the two accumulators (lane quadrant = warp % 4).  Every wait is
// bounded and raises LELPH_DEV_ERR_TIMEOUT instead of hanging.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "lelph_common.cuh"
#include "lelph_internal.h"

#define GT_THREADS 192
#define GT_NST_MAX 8
#define GT_SMEM_LIMIT (227 * 1024)

struct GtLayout
{
    uint32_t a_bytes, b_bytes, stage_bytes, nst, bar_off, total, acc_stride, tmem_cols;
};

__host__ __device__ inline GtLayout gt_layout(int NT)
{
    GtLayout L;
    L.a_bytes = 128 * 128;                 // 128 rows x 32 FP32
    L.b_bytes = (uint32_t)NT * 128;        // NT rows x 32 FP32
    L.stage_bytes = 2 * L.a_bytes + 2 * L.b_bytes;  // multiple of 1024 (NT % 8 == 0)
    L.nst = (GT_SMEM_LIMIT - 2048) / L.stage_bytes;
    if (L.nst > GT_NST_MAX) L.nst = GT_NST_MAX;
    L.bar_off = L.nst * L.stage_bytes;
    L.total = L.bar_off + 256 + 1024;      // barriers, alignment slack
    L.acc_stride = ((uint32_t)NT + 31) / 32 * 32;  // the two accumulators start on 32-column boundaries
    L.tmem_cols = 2 * L.acc_stride <= 256 ? 256 : 512;
    return L;
}

// N tile: at most 144 columns (three 32-deep stages in shared memory), a
// multiple of 16, as few tiles as possible and as little padding as possible
int lelph_gs_tc_ntile(int nb, int* ntiles)
{
    const int ncols = 2 * nb;
    int nt = (ncols + 143) / 144;
    int NT = (ncols + nt - 1) / nt;
    NT = (NT + 15) / 16 * 16;
    if (NT < 16) NT = 16;
    *ntiles = (ncols + NT - 1) / NT;
    return NT;
}

int lelph_gs_tc_supported(int nb)
{
    int nt = 0;
    const int NT = lelph_gs_tc_ntile(nb, &nt);
    return NT <= 256 && gt_layout(NT).nst >= 3;
}

template <int NT>
__global__ void __launch_bounds__(GT_THREADS, 1)
    k_gs_gemm_tc(const __grid_constant__ CUtensorMap tmA_hi, const __grid_constant__ CUtensorMap tmA_lo,
                 const __grid_constant__ CUtensorMap tmB_hi, const __grid_constant__ CUtensorMap tmB_lo, int nrows,
                 int nb, int kreal, int kchunk_real, int nrt, int nnt, int nunits, int rowoff, int nrows_total,
                 float2* __restrict__ part, unsigned* __restrict__ status, unsigned long long wait_ns)
{
    extern __shared__ __align__(1024) uint8_t gt_raw[];
    // aligned by pointer arithmetic on the shared array itself (not through an
    // integer), so that the compiler keeps the shared address space and emits
    // shared-memory loads with 32-bit addresses rather than generic ones
    uint8_t* sm = gt_raw + ((1024u - (smem_u32(gt_raw) & 1023u)) & 1023u);
    const GtLayout L = gt_layout(NT);
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + L.bar_off);
    uint64_t* empty = full + GT_NST_MAX;
    uint64_t* accf = empty + GT_NST_MAX;  // [2] accumulator b complete (MMA -> drains)
    uint64_t* acce = accf + 2;            // [2] accumulator b drained (drains -> MMA)
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const int NST = (int)L.nst;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < NST; ++s)
        {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b)
        {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], 4);
        }
        *abort_flag = 0;
        fence_barrier_init();
    }
    if (warp == 1) tmem_alloc(tmem_slot, L.tmem_cols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // unit u -> (chunk, row tile, N tile), N tile fastest, chunk slowest
    auto unit = [&](int u, int& ch, int& rt, int& ntl) {
        ntl = u % nnt;
        const int t = u / nnt;
        rt = t % nrt;
        ch = t / nrt;
    };

    if (warp == 0)
    {
        if (lane == 0)
        {
            prefetch_tmap(&tmA_hi);
            prefetch_tmap(&tmA_lo);
            prefetch_tmap(&tmB_hi);
            prefetch_tmap(&tmB_lo);
            int s = 0;
            uint32_t ph = 0;
            long long issued = 0;
            bool stop = false;
            for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
            {
                int ch, rt, ntl;
                unit(u, ch, rt, ntl);
                const int k0 = ch * kchunk_real, k1 = min(kreal, k0 + kchunk_real);
                for (int k = k0; k < k1; k += 32, s = (s + 1 == NST) ? 0 : s + 1, ph ^= (s == 0) ? 1u : 0u)
                {
                    if (!mbar_wait_bounded(&empty[s], ph ^ 1u, wait_ns) || *abort_flag)
                    {
                        if (!*abort_flag) atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                        *abort_flag = 1;
                        stop = true;
                        break;
                    }
                    uint8_t* st = sm + s * L.stage_bytes;
                    mbar_arrive_expect_tx(&full[s], L.stage_bytes);
                    tma_load_2d(st, &tmA_hi, &full[s], k, rt * 128);
                    tma_load_2d(st + L.a_bytes, &tmA_lo, &full[s], k, rt * 128);
                    tma_load_2d(st + 2 * L.a_bytes, &tmB_hi, &full[s], k, ntl * NT);
                    tma_load_2d(st + 2 * L.a_bytes + L.b_bytes, &tmB_lo, &full[s], k, ntl * NT);
                    ++issued;
                }
            }
            // every issued copy lands before the CTA can retire
            for (long long i = (issued > NST ? issued - NST : 0); i < issued; ++i)
                mbar_wait_bounded(&full[i % NST], (uint32_t)(i / NST) & 1u);
        }
    }
    else if (warp == 1)
    {
        if (lane == 0)
        {
            constexpr uint32_t idesc = umma_idesc_tf32(128u, (uint32_t)NT);
            int s = 0, b = 0;
            uint32_t ph = 0, phb = 0;
            bool stop = false;
            uint64_t* last_commit = nullptr;
            uint32_t last_par = 0;
            for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
            {
                int ch, rt, ntl;
                unit(u, ch, rt, ntl);
                const int k0 = ch * kchunk_real, k1 = min(kreal, k0 + kchunk_real);
                for (int k = k0; k < k1; k += 32)
                {
                    bool ok = mbar_wait_bounded(&acce[b], phb ^ 1u, wait_ns) && mbar_wait_bounded(&full[s], ph, wait_ns);
                    if (!ok || *abort_flag)
                    {
                        if (!*abort_flag) atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                        *abort_flag = 1;
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t base = smem_u32(sm + s * L.stage_bytes);
                    const uint32_t dacc = tmem + (uint32_t)b * L.acc_stride;
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                    {
                        const uint64_t ah = umma_desc_sw128(base + 32u * kk);
                        const uint64_t al = umma_desc_sw128(base + L.a_bytes + 32u * kk);
                        const uint64_t bh = umma_desc_sw128(base + 2 * L.a_bytes + 32u * kk);
                        const uint64_t bl = umma_desc_sw128(base + 2 * L.a_bytes + L.b_bytes + 32u * kk);
                        umma_tf32(dacc, ah, bh, idesc, kk > 0 ? 1u : 0u);
                        umma_tf32(dacc, ah, bl, idesc, 1u);
                        umma_tf32(dacc, al, bh, idesc, 1u);
                    }
                    umma_commit(&empty[s]);
                    umma_commit(&accf[b]);
                    last_commit = &accf[b];
                    last_par = phb;
                    s = (s + 1 == NST) ? 0 : s + 1;
                    if (s == 0) ph ^= 1u;
                    if (++b == 2)
                    {
                        b = 0;
                        phb ^= 1u;
                    }
                }
            }
            // every MMA issued completes before the tensor memory is released
            if (last_commit) mbar_wait_bounded(last_commit, last_par);
        }
    }
    else
    {
        // drains: lane quadrant q = warp % 4 (rows 32 q .. 32 q + 31), all NT columns
        const int q = warp & 3;
        int b = 0;
        uint32_t phb = 0;
        bool stop = false;
        for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
        {
            int ch, rt, ntl;
            unit(u, ch, rt, ntl);
            const int k0 = ch * kchunk_real, k1 = min(kreal, k0 + kchunk_real);
            float acc[NT];
#pragma unroll
            for (int i = 0; i < NT; ++i) acc[i] = 0.f;
            for (int k = k0; k < k1; k += 32, b ^= 1, phb ^= (b == 0) ? 1u : 0u)
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
                const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)b * L.acc_stride;
#pragma unroll
                for (int c = 0; c < NT; c += 16)
                {
                    float v[16];
                    tmem_ld16(ta + (uint32_t)c, v);
#pragma unroll
                    for (int i = 0; i < 16; ++i) acc[c + i] += v[i];
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acce[b]);
            }
            if (stop) break;
            const int row = rt * 128 + q * 32 + lane;
            if (row < nrows)
            {
                float2* dst = part + ((size_t)ch * nrows_total + rowoff + row) * nb;
                const int n0 = ntl * (NT / 2);
#pragma unroll
                for (int c = 0; c < NT; c += 2)
                    if (n0 + c / 2 < nb) dst[n0 + c / 2] = make_float2(acc[c], acc[c + 1]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1)
    {
        tc_fence_after();
        tmem_dealloc(tmem, L.tmem_cols);
    }
}

// Bq[h][2n + t][K'] from the k+q coefficients Bp[n][K] (complex, K = spinor x
// npad): t = 0 -> (br, bi), t = 1 -> (-bi, br) at K' = 2K, 2K + 1; h = 0 the
// TF32-rounded value, h = 1 the TF32-rounded remainder.
__global__ void k_gs_bsplit(const float2* __restrict__ Bp, int nb, int Ktot, float* __restrict__ Bq)
{
    const size_t plane = (size_t)2 * nb * 2 * Ktot;
    const long long n_el = (long long)nb * Ktot;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n_el;
         e += (long long)gridDim.x * blockDim.x)
    {
        const int n = (int)(e / Ktot);
        const int K = (int)(e - (long long)n * Ktot);
        const float2 v = Bp[e];
        float h[4], l[4];
        const float w[4] = {v.x, v.y, -v.y, v.x};
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            h[i] = tf32_rn(w[i]);
            l[i] = tf32_rn(w[i] - h[i]);
        }
        float* r0 = Bq + ((size_t)(2 * n) * 2 * Ktot + 2 * (size_t)K);
        float* r1 = r0 + 2 * (size_t)Ktot;
        *reinterpret_cast<float2*>(r0) = make_float2(h[0], h[1]);
        *reinterpret_cast<float2*>(r1) = make_float2(h[2], h[3]);
        *reinterpret_cast<float2*>(r0 + plane) = make_float2(l[0], l[1]);
        *reinterpret_cast<float2*>(r1 + plane) = make_float2(l[2], l[3]);
    }
}

size_t lelph_gs_tc_smem(int nb)
{
    int nt = 0;
    return gt_layout(lelph_gs_tc_ntile(nb, &nt)).total;
}

void lelph_launch_gs_bsplit(const float2* Bp, int nb, int Ktot, float* Bq, cudaStream_t st)
{
    const long long n = (long long)nb * Ktot;
    const int blocks = (int)std::min<long long>(4096, (n + 255) / 256);
    k_gs_bsplit<<<blocks, 256, 0, st>>>(Bp, nb, Ktot, Bq);
}

template <int NT>
static int gt_launch(const CUtensorMap* m, int nrows, int nb, int Ktot, int kchunk, int rowoff, int nrows_total,
                     float2* part, unsigned* status, unsigned long long wait_ns, cudaStream_t st)
{
    const GtLayout L = gt_layout(NT);
    static bool attr = false;
    if (!attr)
    {
        if (cudaFuncSetAttribute(k_gs_gemm_tc<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total) !=
            cudaSuccess)
            return -1;
        attr = true;
    }
    int nnt = 0;
    lelph_gs_tc_ntile(nb, &nnt);
    const int nrt = (nrows + 127) / 128;
    const int kreal = 2 * Ktot, kch = 2 * kchunk;
    const int nch = (kreal + kch - 1) / kch;
    const long long units = (long long)nch * nrt * nnt;
    if (units <= 0 || units > (1ll << 30)) return -1;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<long long>(units, std::max(1, nsm));
    k_gs_gemm_tc<NT><<<grid, GT_THREADS, L.total, st>>>(m[0], m[1], m[2], m[3], nrows, nb, kreal, kch, nrt, nnt,
                                                        (int)units, rowoff, nrows_total, part, status,
                                                        wait_ns ? wait_ns : LELPH_WAIT_LIMIT_NS);
    return 0;
}

int lelph_launch_gs_gemm_tc(const void* tmaps, int nrows, int nb, int Ktot, int kchunk, int rowoff,
                            int nrows_total, float2* part, unsigned* status, unsigned long long wait_ns,
                            cudaStream_t st)
{
    int nnt = 0;
    const int NT = lelph_gs_tc_ntile(nb, &nnt);
    const CUtensorMap* m = static_cast<const CUtensorMap*>(tmaps);
    switch (NT)
    {
#define GT_CASE(N) \
    case N: return gt_launch<N>(m, nrows, nb, Ktot, kchunk, rowoff, nrows_total, part, status, wait_ns, st);
        GT_CASE(16) GT_CASE(32) GT_CASE(48) GT_CASE(64) GT_CASE(80) GT_CASE(96) GT_CASE(112) GT_CASE(128)
        GT_CASE(144)
#undef GT_CASE
    default:
        return -1;
    }
}
