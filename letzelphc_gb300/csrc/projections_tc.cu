// Kleinman-Bylander projections of the mixed form on the 5th-generation
// tensor cores.
//
//   Pi[k][row][set] = sum_G beta_row(G) conj(c^_set(G))
//
// with beta_x(G) = F e^{-i 2pi K.tau} Y_lm(K) (1 | K_x sign), K = S (k + G),
// the projector rows of src/nonloc/Vbare_nloc.c:148-168 and 318-363, and c^
// the unfolded coefficients; the contraction is the one of
// src/nonloc/Vbare_nloc.c:412-418 (bandbuffer products).  It runs as a real
// GEMM with K = (re, im) interleaved over the plane waves:
//   A row 2s     = (cr, ci)    ->  D[2s][n]     = sum cr br + ci bi = Re
//   A row 2s + 1 = (-ci, cr)   ->  D[2s + 1][n] = sum cr bi - ci br = Im
//   B row n      = (br, bi)
// (M = coefficient rows of 64 sets per 128-row tile, N = projector rows).
//
// Both operands are built in shared memory by producer warps, one 16-plane-
// wave stage (32 real K elements, one 128-byte K atom) at a time, as TF32
// (hi, lo) pairs in the 128-byte swizzled K-major layout the MMA descriptors
// read: per stage the producers tabulate K and Y_lm (FP32, the recurrences of
// the FP64 form), the structure-factor phases (K.tau = (k + G).(R^T tau) and
// the angle reduced to one turn in FP64, sine and cosine in FP32) and F, then
// form beta and the expanded coefficient rows; the
// tables cover a group of up to 8 stages, so that the serial FP64 work of a
// table phase is shared by the group.  One thread issues per stage three
// products of four K = 8 steps (kind::tf32): hi hi into one tensor-memory
// accumulator, hi lo + lo hi into a second one (every accumulation rounds the
// running sum, so the large sum sees 4 accumulations per stage, not 12), with
// two such buffers in flight; drain warps add each stage's accumulators into
// FP32 registers and every 16 stages add those sums in FP64 into the output,
// which each work unit (k, set tile, projector tile) owns exclusively.  Every
// wait is bounded and raises LELPH_DEV_ERR_TIMEOUT instead of hanging; the
// producer warps leave their loops together, at a barrier that ORs their
// timeout flags.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "lelph_common.cuh"
#include "lelph_internal.h"
#include "tc_operands.cuh"
#include "ylm.cuh"

#define PT_G 16           // plane waves per stage
#define PT_CH 16          // stages per FP32 sum
// producer warps: 8, or 7 with two drain groups (512 threads: 128 registers a thread)
#define PT_PW(NDR) ((NDR) == 1 ? 8 : 7)
#define PT_NST_MAX 6
#define PT_SMEM_LIMIT (227 * 1024)
#define PT_MAXLM 16       // lmax <= 3
#define PT_MAXATOM 64     // atoms per projector tile
#define PT_MAXLT 32       // (l shell, type) pairs
#define PT_THREADS(NDR) (32 * (1 + PT_PW(NDR) + 4 * (NDR)))

struct PtLayout
{
    uint32_t a_bytes, b_bytes, stage_bytes, nst;
    uint32_t tab_off, tab_bytes, ylm, kx, f, ph;  // table buffer offsets (two buffers)
    uint32_t rinfo_off, taup_off, bar_off, total;
};

// tables of TG = tgs * PT_G plane waves: Y_lm (nlm rows), K (3 rows), F (nlt rows)
// as FP32, phases of up to natmax atoms as float2; two buffers
__host__ __device__ inline PtLayout pt_layout(int NTB, int nlm, int nlt, int natmax, int tgs)
{
    PtLayout L;
    const uint32_t TG = (uint32_t)tgs * PT_G;
    L.a_bytes = 128 * 128;            // 128 rows x 32 FP32
    L.b_bytes = (uint32_t)NTB * 128;  // NTB rows x 32 FP32
    L.stage_bytes = 2 * L.a_bytes + 2 * L.b_bytes;  // multiple of 1024 (NTB % 16 == 0)
    L.ylm = 0;
    L.kx = L.ylm + (uint32_t)nlm * TG * 4;
    L.f = L.kx + 3 * TG * 4;
    L.ph = L.f + (uint32_t)nlt * TG * 4;
    L.tab_bytes = (L.ph + (uint32_t)natmax * TG * 8 + 15) / 16 * 16;
    const uint32_t other = 2 * L.tab_bytes + 128 * 5 * 4 + (PT_MAXATOM * 3 + 12) * 8 + 256 + 1024;
    L.nst = other < PT_SMEM_LIMIT ? (PT_SMEM_LIMIT - other) / L.stage_bytes : 0;
    if (L.nst > PT_NST_MAX) L.nst = PT_NST_MAX;
    L.tab_off = L.nst * L.stage_bytes;
    L.rinfo_off = L.tab_off + 2 * L.tab_bytes;
    L.taup_off = L.rinfo_off + 128 * 5 * 4;  // k (3), R (9), R^T tau of the tile's atoms (FP64)
    L.bar_off = L.taup_off + (PT_MAXATOM * 3 + 12) * 8;
    L.total = L.bar_off + 256 + 1024;  // barriers, alignment slack
    return L;
}

__device__ __forceinline__ float2 pt_c32(double2 v) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ float2 pt_c32(float2 v) { return v; }

struct PtUnit
{
    int kbz, mt, nt;
};

__device__ __forceinline__ PtUnit pt_unit(int u, int k0, int mtiles, int ntiles)
{
    PtUnit w;
    w.nt = u % ntiles;
    const int t = u / ntiles;
    w.mt = t % mtiles;
    w.kbz = k0 + t / mtiles;
    return w;
}

// Persistent grid: one CTA per SM over units (k, set tile, projector tile),
// projector tile fastest.  Warp 0: tensor memory and MMA issue; warps
// 1..PW: producers; then 4*NDR drain warps (lane quadrant warp % 4,
// 64 accumulator columns each).  proj must be zero on entry.
template <int NDR, typename CT>
__global__ void __launch_bounds__(PT_THREADS(NDR), 1)
    k_projections_tc(int k0, int nunits, int mtiles, int ntiles, int NTB, int natmax, int tgs,
                     const KPointSym* __restrict__ ks, const double* __restrict__ gvec,
                     const long long* __restrict__ pw_off, const int* __restrict__ npw_arr,
                     const double* __restrict__ Fk, const long long* __restrict__ fk_off, const CT* __restrict__ chat,
                     const long long* __restrict__ chat_off, NonlocalDesc nl, int nsets, double2* __restrict__ proj,
                     unsigned* __restrict__ status, unsigned long long wait_ns)
{
    extern __shared__ __align__(1024) uint8_t pt_raw[];
    // aligned by pointer arithmetic on the shared array (keeps the shared address space)
    uint8_t* sm = pt_raw + ((1024u - (smem_u32(pt_raw) & 1023u)) & 1023u);
    const int nlt = nl.nltimesj * nl.ntype;
    const int nlm = (nl.lmax + 1) * (nl.lmax + 1);
    const PtLayout L = pt_layout(NTB, nlm, nlt, natmax, tgs);
    const int TG = tgs * PT_G;
    constexpr int PW = PT_PW(NDR), PTH = 32 * PW;
    constexpr int NA = (512 + PTH - 1) / PTH;  // coefficient tasks (64 sets x 8 chunks) per producer thread
    uint64_t* sfull = reinterpret_cast<uint64_t*>(sm + L.bar_off);  // stage written (producer warps)
    uint64_t* sfree = sfull + PT_NST_MAX;                           // stage read (MMA commit)
    uint64_t* accf = sfree + PT_NST_MAX;                            // [2] accumulator complete (MMA commit)
    uint64_t* acce = accf + 2;                                      // [2] accumulator drained (drain warps)
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    int* rinfo = reinterpret_cast<int*>(sm + L.rinfo_off);  // [NTB][5]: atom slot, lm, lt, x, sign bits
    const int NST = (int)L.nst;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ndrain = 4 * NDR;
    const int rows_tot = nl.natom * nl.nproj_max * 4;
    const int rows_atom = nl.nproj_max * 4;
    // two accumulator buffers of 2 NTB columns: [0, NTB) hi.hi, [NTB, 2 NTB) hi.lo + lo.hi
    const uint32_t tcols = (4 * NTB <= 64) ? 64u : (4 * NTB <= 128) ? 128u : (4 * NTB <= 256) ? 256u : 512u;

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
            // ---------------- MMA issue
            const uint32_t idesc = umma_idesc_tf32(128u, (uint32_t)NTB);
            int s = 0, b = 0;
            uint32_t phs = 0, phb = 0;
            uint64_t* last_commit = nullptr;
            uint32_t last_par = 0;
            bool stop = false;
            for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
            {
                const PtUnit w = pt_unit(u, k0, mtiles, ntiles);
                const int npw = npw_arr[ks[w.kbz].ik];
                const int nstage = (npw + PT_G - 1) / PT_G;
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
                    // the large hi.hi chain and the small cross terms in separate
                    // accumulators: each accumulation rounds the running sum, so the
                    // large sum takes 4 of the stage's 12 accumulations, not 12
                    const uint32_t dacc = tmem + (uint32_t)b * 2u * (uint32_t)NTB, dx = dacc + (uint32_t)NTB;
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
            // every MMA this thread issued completes before the tensor memory is released
            if (last_commit) mbar_wait_bounded(last_commit, last_par);
        }
    }
    else if (warp <= PW)
    {
        // ---------------- producers
        const int p = threadIdx.x - 32;
        int s = 0, ngroup = 0;
        uint32_t phs = 0;
        bool failed = false;  // this thread's wait on a stage slot ran out
        for (int u = blockIdx.x; u < nunits; u += gridDim.x)
        {
            const PtUnit w = pt_unit(u, k0, mtiles, ntiles);
            const KPointSym& S = ks[w.kbz];
            const int npw = npw_arr[S.ik];
            const int nstage = (npw + PT_G - 1) / PT_G;
            const double* G = gvec + 3 * pw_off[S.ik];
            const double* F = Fk + fk_off[S.ik];
            const CT* Cc = chat + chat_off[w.kbz];
            const int set0 = w.mt * 64, row0 = w.nt * NTB;
            const int a_first = row0 / rows_atom;
            const int a_last = min(nl.natom - 1, (row0 + NTB - 1) / rows_atom);
            const int natom_t = a_last - a_first + 1;
            // the previous unit's stages have been formed by every producer before the
            // row table is replaced
            if (tc_producer_bar_any<PTH>(failed)) break;
            if (p < NTB)
            {
                const int rg = row0 + p;
                int info[4] = {-1, 0, 0, 0};
                float sg = 1.f;
                if (rg < rows_tot)
                {
                    const int a = rg / rows_atom, pj = (rg / 4) % nl.nproj_max, x = rg % 4;
                    const int ity = nl.atom_type[a];
                    int np = 0;
                    for (int lidx = 0; lidx < nl.nltimesj; ++lidx)
                    {
                        const int l = (int)rint(nl.PP_table[(lidx * nl.ntype + ity) * 3] - 1.0);
                        if (l < 0) continue;
                        if (pj >= np && pj < np + 2 * l + 1)
                        {
                            info[0] = a - a_first;
                            info[1] = l * l + (pj - np);
                            info[2] = lidx * nl.ntype + ity;
                            info[3] = x;
                            sg = (float)nl.Fsign[lidx * nl.ntype + ity];
                        }
                        np += 2 * l + 1;
                    }
                }
                for (int c = 0; c < 4; ++c) rinfo[p * 5 + c] = info[c];
                rinfo[p * 5 + 4] = __float_as_int(sg);
            }
            // k and R of the unit, and R^T tau: K.tau = (k + G).(R^T tau) needs one
            // FP64 dot product per atom
            double* kR = reinterpret_cast<double*>(sm + L.taup_off);
            double* taup = kR + 12;
            if (p < 3) kR[p] = S.kcart[p];
            else if (p < 12) kR[p] = S.R[p - 3];
            else if (p < 12 + 3 * natom_t)
            {
                const int a = (p - 12) / 3, x = (p - 12) % 3;
                const double* ta = nl.atom_pos + 3 * (a_first + a);
                taup[p - 12] = S.R[x] * ta[0] + S.R[3 + x] * ta[1] + S.R[6 + x] * ta[2];
            }
            if (tc_producer_bar_any<PTH>(failed)) break;
            const float* ylm_s = nullptr;
            const float* kx_s = nullptr;
            const float* f_s = nullptr;
            const float2* ph_s = nullptr;
            float2 cvn[NA][2];
            auto load_cv = [&](int st_i) {
                const int g0 = st_i * PT_G;
#pragma unroll
                for (int i = 0; i < NA; ++i)
                {
                    const int tau = min(p + PTH * i, 511);
                    const int sl = tau >> 3, c = tau & 7;
                    const int set = set0 + sl, g = g0 + 2 * c;
                    cvn[i][0] = (set < nsets && g < npw) ? pt_c32(Cc[(size_t)set * npw + g]) : make_float2(0.f, 0.f);
                    cvn[i][1] =
                        (set < nsets && g + 1 < npw) ? pt_c32(Cc[(size_t)set * npw + g + 1]) : make_float2(0.f, 0.f);
                }
            };
            load_cv(0);
            bool leave = false;
            for (int it = 0; it < nstage; ++it)
            {
                const int gi = it % tgs;  // stage within its table group
                if (gi == 0)
                {
                    // tables of the group's TG plane waves (K and Y_lm in FP32, phases, F)
                    uint8_t* tab = sm + L.tab_off + (uint32_t)(ngroup & 1) * L.tab_bytes;
                    ++ngroup;
                    float* ylm_w = reinterpret_cast<float*>(tab + L.ylm);
                    float* kx_w = reinterpret_cast<float*>(tab + L.kx);
                    float* f_w = reinterpret_cast<float*>(tab + L.f);
                    float2* ph_w = reinterpret_cast<float2*>(tab + L.ph);
                    const int gbase = it * PT_G;
                    const int ntask = TG * (1 + natom_t + nlt);
                    for (int tau = p; tau < ntask; tau += PTH)
                    {
                        const int gg = tau % TG, kind = tau / TG;
                        const int g = gbase + gg;
                        if (kind < 1 + natom_t)
                        {
                            double v0 = 0.0, v1 = 0.0, v2 = 0.0;
                            if (g < npw)
                            {
                                v0 = kR[0] + G[3 * g];
                                v1 = kR[1] + G[3 * g + 1];
                                v2 = kR[2] + G[3 * g + 2];
                            }
                            if (kind == 0)
                            {
                                // K = R (k + G) and Y_lm(K) in FP32
                                const float f0 = (float)v0, f1 = (float)v1, f2 = (float)v2;
                                const double* R = kR + 3;
                                const float K0 = (float)R[0] * f0 + (float)R[1] * f1 + (float)R[2] * f2;
                                const float K1 = (float)R[3] * f0 + (float)R[4] * f1 + (float)R[5] * f2;
                                const float K2 = (float)R[6] * f0 + (float)R[7] * f1 + (float)R[8] * f2;
                                if (g < npw) ylm_all_f(nl.lmax, K0, K1, K2, ylm_w + gg, TG);
                                else
                                    for (int i = 0; i < nlm; ++i) ylm_w[i * TG + gg] = 0.f;
                                kx_w[0 * TG + gg] = K0;
                                kx_w[1 * TG + gg] = K1;
                                kx_w[2 * TG + gg] = K2;
                            }
                            else
                            {
                                const double* tp = taup + 3 * (kind - 1);
                                const double dot = v0 * tp[0] + v1 * tp[1] + v2 * tp[2];
                                // the angle 2 pi_T dot reduced to one turn in FP64 (pi_T the
                                // reference's truncated pi), sine and cosine in FP32
                                const double turns = dot * (LELPH_PI_T / 3.14159265358979323846);
                                float sn, cs;
                                sincospif(2.0f * (float)(turns - rint(turns)), &sn, &cs);
                                ph_w[(kind - 1) * TG + gg] = make_float2(cs, -sn);
                            }
                        }
                        else
                        {
                            const int lt = kind - 1 - natom_t;
                            f_w[lt * TG + gg] = g < npw ? (float)F[(size_t)lt * npw + g] : 0.f;
                        }
                    }
                    ylm_s = ylm_w;
                    kx_s = kx_w;
                    f_s = f_w;
                    ph_s = ph_w;
                    // tables complete; every producer leaves together when any one's wait ran out
                    if (tc_producer_bar_any<PTH>(failed))
                    {
                        leave = true;
                        break;
                    }
                }
                // this stage's coefficients (loaded one stage ahead) and the next
                // stage's loads, in flight while this stage is formed: tasks (set,
                // 2-plane-wave chunk)
                float2 cv[NA][2];
#pragma unroll
                for (int i = 0; i < NA; ++i)
                {
                    cv[i][0] = cvn[i][0];
                    cv[i][1] = cvn[i][1];
                }
                if (it + 1 < nstage) load_cv(it + 1);
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
                    // B: projector rows n, chunk c = plane waves 2c, 2c + 1 of the stage
                    // eight lanes per row, consecutive plane waves: a warp's table reads
                    // fall in consecutive words (no bank conflicts between rows)
                    constexpr int NBT = (128 * 8 + PTH - 1) / PTH;
#pragma unroll
                    for (int i = 0; i < NBT; ++i)
                    {
                        const int tau = p + PTH * i;
                        if (tau >= NTB * 8) break;
                        const int n = tau >> 3, c = tau & 7;
                        const int* ri = rinfo + n * 5;
                        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (ri[0] >= 0)
                        {
                            const float sg = __int_as_float(ri[4]);
                            float b2[4];
#pragma unroll
                            for (int e = 0; e < 2; ++e)
                            {
                                const int gg = gi * PT_G + 2 * c + e;
                                float fy = f_s[ri[2] * TG + gg] * ylm_s[ri[1] * TG + gg];
                                if (ri[3] > 0) fy *= kx_s[(ri[3] - 1) * TG + gg] * sg;
                                const float2 ph = ph_s[ri[0] * TG + gg];
                                b2[2 * e] = fy * ph.x;
                                b2[2 * e + 1] = fy * ph.y;
                            }
                            v = make_float4(b2[0], b2[1], b2[2], b2[3]);
                        }
                        float4 h, l;
                        tc_split4_tf32(v, h, l);
                        *reinterpret_cast<float4*>(Bhi + tc_swz128(n, c)) = h;
                        *reinterpret_cast<float4*>(Blo + tc_swz128(n, c)) = l;
                    }
                    // A: the coefficient rows 2 sl (cr, ci) and 2 sl + 1 (-ci, cr)
#pragma unroll
                    for (int i = 0; i < NA; ++i)
                    {
                        const int tau = p + PTH * i;
                        if (tau >= 512) break;
                        const int sl = tau >> 3, c = tau & 7;
                        const float cr0 = cv[i][0].x, ci0 = cv[i][0].y, cr1 = cv[i][1].x, ci1 = cv[i][1].y;
                        float4 h, l;
                        tc_split4_tf32(make_float4(cr0, ci0, cr1, ci1), h, l);
                        *reinterpret_cast<float4*>(Ahi + tc_swz128(2 * sl, c)) = h;
                        *reinterpret_cast<float4*>(Alo + tc_swz128(2 * sl, c)) = l;
                        tc_split4_tf32(make_float4(-ci0, cr0, -ci1, cr1), h, l);
                        *reinterpret_cast<float4*>(Ahi + tc_swz128(2 * sl + 1, c)) = h;
                        *reinterpret_cast<float4*>(Alo + tc_swz128(2 * sl + 1, c)) = l;
                    }
                    // generic-proxy writes -> the tensor core's async proxy
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
        const int r = q * 32 + lane;  // accumulator row: set 2 sl + part
        const int sl = r >> 1, part = r & 1;
        int b = 0;
        uint32_t phb = 0;
        bool stop = false;
        for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
        {
            const PtUnit w = pt_unit(u, k0, mtiles, ntiles);
            const int npw = npw_arr[ks[w.kbz].ik];
            const int nstage = (npw + PT_G - 1) / PT_G;
            const int set = w.mt * 64 + sl;
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
                    tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)b * 2u * (uint32_t)NTB + (uint32_t)(cg * 64);
#pragma unroll
                for (int c = 0; c < 64; c += 16)
                    if (cg * 64 + c < NTB)
                    {
                        float v[16], x[16];
                        tmem_ld16(ta + (uint32_t)c, v);
                        tmem_ld16(ta + (uint32_t)(NTB + c), x);
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
                if ((it % PT_CH) == PT_CH - 1 || it == nstage - 1)
                {
                    // this chunk's FP32 sums into the FP64 output: the even lane of a
                    // (Re, Im) row pair writes the pair
                    double2* o = proj + ((size_t)w.kbz * rows_tot + w.nt * NTB + cg * 64) * nsets + set;
#pragma unroll
                    for (int c = 0; c < 64; c += 8)
                    {
#pragma unroll
                        for (int jj = 0; jj < 8; ++jj)
                        {
                            const int j = c + jj;
                            const float other = __shfl_xor_sync(0xffffffffu, acc[j], 1);
                            if (part == 0 && set < nsets && cg * 64 + j < NTB && w.nt * NTB + cg * 64 + j < rows_tot)
                            {
                                double2 t = o[(size_t)j * nsets];
                                t.x += (double)acc[j];
                                t.y += (double)other;
                                o[(size_t)j * nsets] = t;
                            }
                            acc[j] = 0.f;
                        }
                        // eight columns at a time: keeps the loads from being hoisted
                        // (and their registers from spilling)
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

// projector tile: at most 128 rows, a multiple of 16, as few tiles as possible
static int pt_ntile(int rows, int* ntiles)
{
    int nt = (rows + 127) / 128;
    int NTB = (rows + nt - 1) / nt;
    NTB = (NTB + 15) / 16 * 16;
    *ntiles = (rows + NTB - 1) / NTB;
    return NTB;
}

struct PtConfig
{
    int NTB, ntiles, natmax, tgs;
    PtLayout L;
};

// the largest table group (stages per table phase) that leaves three stages of
// operands in shared memory
static bool pt_config(const NonlocalDesc& nl, PtConfig* c)
{
    const int rows = nl.natom * nl.nproj_max * 4;
    if (rows <= 0 || nl.lmax > 3 || nl.nltimesj * nl.ntype > PT_MAXLT) return false;
    c->NTB = pt_ntile(rows, &c->ntiles);
    c->natmax = std::min(nl.natom, c->NTB / (nl.nproj_max * 4) + 2);
    const int nlm = (nl.lmax + 1) * (nl.lmax + 1), nlt = nl.nltimesj * nl.ntype;
    for (int tgs = 8; tgs >= 1; tgs /= 2)
    {
        c->tgs = tgs;
        c->L = pt_layout(c->NTB, nlm, nlt, c->natmax, tgs);
        if (c->L.nst >= 3) return true;
    }
    return c->L.nst >= 2;
}

int lelph_projections_tc_supported(const NonlocalDesc& nl)
{
    PtConfig c;
    return pt_config(nl, &c) ? 1 : 0;
}

template <int NDR, typename CT>
static void pt_launch(const PtConfig& c, int grid, int k0, int units, int mtiles, const KPointSym* ksym_dev,
                      const double* gvec, const long long* pw_off, const int* npw, const double* Fk,
                      const long long* fk_off, const CT* chat, const long long* chat_off, const NonlocalDesc& nl,
                      int nsets, double2* proj, unsigned* status, unsigned long long wait_ns, cudaStream_t st)
{
    cudaFuncSetAttribute(k_projections_tc<NDR, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.L.total);
    k_projections_tc<NDR, CT><<<grid, PT_THREADS(NDR), c.L.total, st>>>(
        k0, units, mtiles, c.ntiles, c.NTB, c.natmax, c.tgs, ksym_dev, gvec, pw_off, npw, Fk, fk_off, chat, chat_off,
        nl, nsets, proj, status, wait_ns);
}

int lelph_launch_projections_tc(int k0, int nk, const KPointSym* ksym_dev, const double* gvec,
                                const long long* pw_off, const int* npw, const double* Fk, const long long* fk_off,
                                const void* chat, int chat_f32, const long long* chat_off, const NonlocalDesc& nl,
                                const GeomDev& g, double2* proj, unsigned* status, unsigned long long wait_ns,
                                cudaStream_t st)
{
    if (wait_ns == 0) wait_ns = LELPH_WAIT_LIMIT_NS;
    PtConfig c;
    if (!pt_config(nl, &c)) return -1;
    const int nsets = g.nspin * g.nbnds * g.nspinor;
    const int rows = nl.natom * nl.nproj_max * 4;
    const int mtiles = (nsets + 63) / 64;
    const long long units = (long long)nk * mtiles * c.ntiles;
    if (units <= 0) return 0;
    if (units > (1LL << 30)) return -1;
    if (cudaMemsetAsync(proj + (size_t)k0 * rows * nsets, 0, sizeof(double2) * (size_t)nk * rows * nsets, st) !=
        cudaSuccess)
        return -1;
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<long long>(units, nsm);
    const int ndr = (c.NTB + 63) / 64;
#define PT_ARGS c, grid, k0, (int)units, mtiles, ksym_dev, gvec, pw_off, npw, Fk, fk_off
#define PT_TAIL chat_off, nl, nsets, proj, status, wait_ns, st
    if (chat_f32)
    {
        if (ndr == 1) pt_launch<1, float2>(PT_ARGS, static_cast<const float2*>(chat), PT_TAIL);
        else pt_launch<2, float2>(PT_ARGS, static_cast<const float2*>(chat), PT_TAIL);
    }
    else
    {
        if (ndr == 1) pt_launch<1, double2>(PT_ARGS, static_cast<const double2*>(chat), PT_TAIL);
        else pt_launch<2, double2>(PT_ARGS, static_cast<const double2*>(chat), PT_TAIL);
    }
#undef PT_ARGS
#undef PT_TAIL
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
