// Local dV sandwich <psi_{m,k+q} | dV_nu | psi_{n,k}> in real space.
//
// The reference forms dV*psi_k on the FFT box, transforms it forward, keeps
// the k+q sphere and contracts with the k+q coefficients
// (src/dvloc/compute_Vbare_loc.c:286-341, src/fft/convolution.c:13-189).
// With psi(r) the unnormalised inverse transform of the zero-padded sphere on
// the product grid (M points) and dV_G0 the window of dV for the pair's
// umklapp shift G0 (built on the host side, see k_dv_window), Parseval turns
// that into one contraction over the grid:
//   g[nu][m][n] = (1/M) sum_{s,r} conj(psi_kq,n,s(r))
//                                 * sum_s' dV_G0,nu^{s s'}(r) psi_k,m,s'(r)
// i.e. a complex GEMM with
// M = (mode, band of k), N = band of k+q, K = (spinor, grid point), whose A
// operand is generated on the fly from dV and psi_k.
//
// * k_local_fp64: the plain form, FP64 SIMT.
// * k_local_tc:   the mixed form on the 5th-generation tensor cores: psi(r)
//   in FP32, split into 16-bit (hi, lo) pairs, three products
//   A_hi B_hi + A_hi B_lo + A_lo B_hi accumulated in FP32 in tensor memory per
//   K chunk; chunks are reduced in FP64 by the finish kernel.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"

// ================================================================ FP64 form

#define F64_TM 64
#define F64_TN 32
#define F64_KP 16

// grid: (ceil(nrows/64), ceil(nb/32), npairs*nspin); 256 threads
__global__ void __launch_bounds__(256) k_local_fp64(const PairInfo* __restrict__ pairs,
                                                    const double2* __restrict__ psi, const double2* __restrict__ dV,
                                                    GeomDev gd, double2* __restrict__ glocal)
{
    __shared__ double2 As[F64_TM][F64_KP + 1];
    __shared__ double2 Bs[F64_TN][F64_KP + 1];
    const int zp = blockIdx.z;
    const int pair = zp / gd.nspin;
    const int spin = zp - pair * gd.nspin;
    const PairInfo P = pairs[pair];
    const int nrows = gd.nmodes * gd.nbnds;
    const int row0 = blockIdx.x * F64_TM;
    const int col0 = blockIdx.y * F64_TN;
    const long long N = (long long)gd.Nx * gd.Ny * gd.Nz;
    const long long Ktot = (long long)gd.nspinor * N;
    const size_t box = (size_t)N;
    // psi layout [kbz][spin][band][spinor][r]
    const double2* psik = psi + ((size_t)P.kbz_k * gd.nspin + spin) * gd.nbnds * gd.nspinor * box;
    const double2* psikq = psi + ((size_t)P.kbz_kq * gd.nspin + spin) * gd.nbnds * gd.nspinor * box;
    const double2* dvq = dV + (size_t)P.dvslot * gd.nmodes * gd.nmag * box;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double2 acc[4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) acc[i][j] = make_double2(0.0, 0.0);
    __syncthreads();
    for (long long k0 = 0; k0 < Ktot; k0 += F64_KP)
    {
        // A tile: 64 rows x 16 points
        for (int e = threadIdx.x; e < F64_TM * F64_KP; e += blockDim.x)
        {
            int rr = e / F64_KP, p = e - rr * F64_KP;
            int row = row0 + rr;
            long long kc = k0 + p;
            double2 a = make_double2(0.0, 0.0);
            if (row < nrows && kc < Ktot)
            {
                int nu = row / gd.nbnds, m = row - nu * gd.nbnds;
                int s = (int)(kc / N);
                int r = (int)(kc - (long long)s * N);
                const double2* dvn = dvq + (size_t)nu * gd.nmag * box;
                const double2* pm = psik + (size_t)m * gd.nspinor * box;
                if (gd.nmag == 4)
                {
                    a = cadd(cmul(dvn[(size_t)(2 * s) * box + r], pm[r]),
                             cmul(dvn[(size_t)(2 * s + 1) * box + r], pm[box + r]));
                }
                else
                {
                    int comp = (gd.nmag == 2) ? spin : 0;
                    a = cmul(dvn[(size_t)comp * box + r], pm[(size_t)s * box + r]);
                }
            }
            As[rr][p] = a;
        }
        for (int e = threadIdx.x; e < F64_TN * F64_KP; e += blockDim.x)
        {
            int cc = e / F64_KP, p = e - cc * F64_KP;
            int n = col0 + cc;
            long long kc = k0 + p;
            double2 b = make_double2(0.0, 0.0);
            if (n < gd.nbnds && kc < Ktot)
            {
                int s = (int)(kc / N);
                int r = (int)(kc - (long long)s * N);
                b = cconj(psikq[((size_t)n * gd.nspinor + s) * box + r]);
            }
            Bs[cc][p] = b;
        }
        __syncthreads();
#pragma unroll 4
        for (int p = 0; p < F64_KP; ++p)
        {
            double2 av[4], bv[2];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[ty * 4 + i][p];
#pragma unroll
            for (int j = 0; j < 2; ++j) bv[j] = Bs[tx * 2 + j][p];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j)
                {
                    acc[i][j].x = fma(av[i].x, bv[j].x, acc[i][j].x);
                    acc[i][j].x = fma(-av[i].y, bv[j].y, acc[i][j].x);
                    acc[i][j].y = fma(av[i].x, bv[j].y, acc[i][j].y);
                    acc[i][j].y = fma(av[i].y, bv[j].x, acc[i][j].y);
                }
        }
        __syncthreads();
    }
    const double invN = 1.0 / (double)N;
    double2* go = glocal + (size_t)zp * nrows * gd.nbnds;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
        {
            int row = row0 + ty * 4 + i, n = col0 + tx * 2 + j;
            if (row < nrows && n < gd.nbnds)
                go[(size_t)row * gd.nbnds + n] = make_double2(acc[i][j].x * invN, acc[i][j].y * invN);
        }
}

void lelph_launch_local_fp64(const PairInfo* pairs, int npairs, const double2* psi, const double2* dV,
                             const GeomDev& g, double2* glocal, unsigned* status, cudaStream_t st)
{
    (void)status;
    int nrows = g.nmodes * g.nbnds;
    dim3 grid((nrows + F64_TM - 1) / F64_TM, (g.nbnds + F64_TN - 1) / F64_TN, npairs * g.nspin);
    k_local_fp64<<<grid, 256, 0, st>>>(pairs, psi, dV, g, glocal);
}

// ============================================================= mixed form
//
// Warp roles: warp 0 issues TMA, warp 1 owns tensor memory and issues the
// MMAs, warps 2-9 build the A operand, warps 10.. drain the accumulators
// (warp w reads TMEM lanes 32*(w%4)..+31, one 64-column half each).

#define TC_NST_MAX 4
#define TC_SMEM_LIMIT (227 * 1024)
#define TC_KPTS 32  // complex grid points per pipeline stage (64 16-bit K elements = 128 B rows)
#define TC_GROUP 2         // pipeline stages chained into one TMEM accumulator before it is drained
#define TC_MAX_THREADS 576 // 10 role warps + up to 8 drain warps

struct TcSmemLayout
{
    uint32_t a_hi, a_lo, b_hi, b_lo, p_hi, p_lo, dv;  // offsets of stage 0
    uint32_t a_bytes, b_bytes, p_bytes, dv_bytes;     // per stage per half
    uint32_t stage_bytes;
    uint32_t nst;
    uint32_t bar_off, total;
};

// whole modes per 128-row tile of (mode, band) rows
__host__ __device__ inline int tc_tile_modes(const GeomDev& g) { return g.mt_modes; }

__host__ __device__ inline TcSmemLayout tc_layout(const GeomDev& g)
{
    TcSmemLayout L;
    const uint32_t NT = 2 * g.nbp;
    const uint32_t nsp = (g.nmag == 4) ? 2 : 1;
    L.a_bytes = 128 * 128;
    L.b_bytes = NT * 128;
    L.p_bytes = nsp * g.nbp * 128;
    L.a_hi = 0;
    L.a_lo = L.a_hi + L.a_bytes;
    L.b_hi = L.a_lo + L.a_bytes;
    L.b_lo = L.b_hi + L.b_bytes;
    L.p_hi = L.b_lo + L.b_bytes;
    L.p_lo = L.p_hi + L.p_bytes;
    L.dv = L.p_lo + L.p_bytes;
    L.dv_bytes = tc_tile_modes(g) * g.nmag * TC_KPTS * 8;
    L.stage_bytes = (L.dv + L.dv_bytes + 1023) / 1024 * 1024;
    L.nst = (TC_SMEM_LIMIT - 2048) / L.stage_bytes;
    if (L.nst > TC_NST_MAX) L.nst = TC_NST_MAX;
    L.bar_off = L.nst * L.stage_bytes;
    L.total = L.bar_off + 256 + 1024;  // barriers + alignment slack
    return L;
}

int lelph_local_tc_smem_bytes(const GeomDev& g) { return (int)tc_layout(g).total; }
int lelph_local_tc_tile_modes(const GeomDev& g) { return tc_tile_modes(g); }

template <int BF16>
__device__ __forceinline__ void split_store(uint8_t* a_hi, uint8_t* a_lo, uint32_t off, float re, float im)
{
    uint32_t h, l;
    if (BF16)
    {
        __nv_bfloat162 hv = __floats2bfloat162_rn(re, im);
        float2 hf = __bfloat1622float2(hv);
        __nv_bfloat162 lv = __floats2bfloat162_rn(re - hf.x, im - hf.y);
        h = *reinterpret_cast<uint32_t*>(&hv);
        l = *reinterpret_cast<uint32_t*>(&lv);
    }
    else
    {
        __half2 hv = __floats2half2_rn(re, im);
        float2 hf = __half22float2(hv);
        __half2 lv = __floats2half2_rn(re - hf.x, im - hf.y);
        h = *reinterpret_cast<uint32_t*>(&hv);
        l = *reinterpret_cast<uint32_t*>(&lv);
    }
    *reinterpret_cast<uint32_t*>(a_hi + off) = h;
    *reinterpret_cast<uint32_t*>(a_lo + off) = l;
}

template <int BF16>
__device__ __forceinline__ float2 load_split(const uint8_t* hi, const uint8_t* lo, uint32_t off)
{
    uint32_t h = *reinterpret_cast<const uint32_t*>(hi + off);
    uint32_t l = *reinterpret_cast<const uint32_t*>(lo + off);
    float2 a, b;
    if (BF16)
    {
        a = __bfloat1622float2(*reinterpret_cast<__nv_bfloat162*>(&h));
        b = __bfloat1622float2(*reinterpret_cast<__nv_bfloat162*>(&l));
    }
    else
    {
        a = __half22float2(*reinterpret_cast<__half2*>(&h));
        b = __half22float2(*reinterpret_cast<__half2*>(&l));
    }
    return make_float2(a.x + b.x, a.y + b.y);
}

// A operand for one pipeline stage, fast path: nb % 8 == 0, one magnetic
// component per row.  Warp pw owns bands m = pw + 8j (j < BPW = nb/8); row
// (ml, m) = ml*nb + m keeps the swizzle phase of a band fixed, so each product
// costs one complex multiply, one (hi, lo) split and two shared stores.
template <int BF16, int BPW>
__device__ __forceinline__ void produce_fast(uint8_t* st, const TcSmemLayout& L, const float2* dvs, int MTa, int comp, int nmag, int nbnds, int pw, int lane,
                                             const uint32_t* off0)
{
    float2 psi[BPW];
#pragma unroll
    for (int j = 0; j < BPW; ++j)
        psi[j] = load_split<BF16>(st + L.p_hi, st + L.p_lo, (uint32_t)(pw + 8 * j) * 128 + 4 * lane);
    const uint32_t mstride = (uint32_t)(nbnds >> 3) * 1024u;
    for (int ml = 0; ml < MTa; ++ml)
    {
        const float2 dvp = dvs[(ml * nmag + comp) * TC_KPTS + lane];
#pragma unroll
        for (int j = 0; j < BPW; ++j)
        {
            const float2 a = cmul(dvp, psi[j]);
            split_store<BF16>(st + L.a_hi, st + L.a_lo, off0[j] + (uint32_t)ml * mstride, a.x, a.y);
        }
    }
}

// grid: (nchunks, mtiles, npairs*nspin); 32*(10 + ndrain) threads.
//
// The tensor-core accumulator loses low-order bits on every accumulation
// (its error grows linearly with the number of MMAs chained into one FP32
// accumulator), so accumulation chains are kept to TC_GROUP pipeline stages:
// the MMA warp alternates between two TMEM accumulators, and the drain warps
// add each finished accumulator into round-to-nearest FP32 registers, which
// are written out per K chunk and reduced in FP64 by the finish kernel.
template <int BF16>
__global__ void __launch_bounds__(TC_MAX_THREADS, 1)
    k_local_tc(const __grid_constant__ CUtensorMap tmapB, const __grid_constant__ CUtensorMap tmapA,
               const __grid_constant__ CUtensorMap tmapV, const PairInfo* __restrict__ pairs,
               const float* __restrict__ mode_scale, GeomDev gd, int chunk_pts, int nchunks,
               float* __restrict__ partials, unsigned* __restrict__ status)
{
    extern __shared__ __align__(1024) uint8_t smraw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    const TcSmemLayout L = tc_layout(gd);
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + L.bar_off);
    uint64_t* aready = full + TC_NST_MAX;
    uint64_t* empty = aready + TC_NST_MAX;
    uint64_t* accf = empty + TC_NST_MAX;  // [2] accumulator b complete (MMA -> drain)
    uint64_t* acce = accf + 2;            // [2] accumulator b drained (drain -> MMA)
    uint64_t* dvbar = acce + 2;           // [NST] scaled dV tile written (producers -> producers)
    const int NST = (int)L.nst;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(dvbar + TC_NST_MAX);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunk = blockIdx.x, mt = blockIdx.y, zp = blockIdx.z;
    const int pair = zp / gd.nspin, spin = zp - pair * gd.nspin;
    const PairInfo P = pairs[pair];
    const int NT = 2 * gd.nbp;
    const long long N = (long long)gd.Nx * gd.Ny * gd.Nz;
    const int nstage = chunk_pts / TC_KPTS;
    const int ngroup = (nstage + TC_GROUP - 1) / TC_GROUP;
    const int nsp = (gd.nmag == 4) ? 2 : 1;
    const int ndrain = 4 * ((NT + 63) / 64);
    const uint32_t ncols = 2 * NT <= 32 ? 32 : (2 * NT <= 64 ? 64 : (2 * NT <= 128 ? 128 : 256));

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < NST; ++s)
        {
            mbar_init(&full[s], 1);
            mbar_init(&aready[s], 8);
            mbar_init(&empty[s], 1);
            mbar_init(&dvbar[s], 8);
        }
        for (int b = 0; b < 2; ++b)
        {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], ndrain);
        }
        *abort_flag = 0;
        fence_barrier_init();
    }
    if (warp == 1) tmem_alloc(tmem_slot, ncols);
    // zero the A operand buffers once (rows past the last (mode, band) stay 0)
    for (int s = 0; s < NST; ++s)
    {
        uint32_t* a = reinterpret_cast<uint32_t*>(sm + s * L.stage_bytes + L.a_hi);
        for (int i = threadIdx.x; i < (int)(2 * L.a_bytes / 4); i += blockDim.x) a[i] = 0u;
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0)
    {
        if (lane == 0)
        {
            prefetch_tmap(&tmapB);
            prefetch_tmap(&tmapA);
            prefetch_tmap(&tmapV);
            const int rowB_hi = ((P.kbz_kq * gd.nspin + spin) * 2 + 0) * NT;
            const int rowB_lo = rowB_hi + NT;
            const int rowP_hi = ((P.kbz_k * gd.nspin + spin) * 2 + 0) * NT;
            const int rowP_lo = rowP_hi + NT;
            const uint32_t bytes = 2 * L.b_bytes + 2 * L.p_bytes + L.dv_bytes;
            const int rowV = (P.dvslot * gd.nmodes + mt * gd.mt_modes) * gd.nmag;
            int issued = 0;
            for (int it = 0; it < nstage; ++it)
            {
                const int s = it % NST;
                const uint32_t ph = (uint32_t)(it / NST) & 1u;
                if (!mbar_wait_bounded(&empty[s], ph ^ 1u))
                {
                    *abort_flag = 1;
                    atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                    break;
                }
                if (*abort_flag) break;
                uint8_t* st = sm + s * L.stage_bytes;
                const long long kc = (long long)chunk * chunk_pts + (long long)it * TC_KPTS;
                const int sp = (int)(kc / N);
                const long long r0 = kc - (long long)sp * N;
                mbar_arrive_expect_tx(&full[s], bytes);
                tma_load_2d(st + L.b_hi, &tmapB, &full[s], (int)(2 * kc), rowB_hi);
                tma_load_2d(st + L.b_lo, &tmapB, &full[s], (int)(2 * kc), rowB_lo);
                for (int q = 0; q < nsp; ++q)
                {
                    const int spp = (gd.nmag == 4) ? q : sp;
                    const int x = (int)(2 * ((long long)spp * N + r0));
                    tma_load_2d(st + L.p_hi + q * gd.nbp * 128, &tmapA, &full[s], x, rowP_hi);
                    tma_load_2d(st + L.p_lo + q * gd.nbp * 128, &tmapA, &full[s], x, rowP_lo);
                }
                // dV_nu(r) of the tile's modes, all magnetic components: rows (nu, comp) x 32 points
                tma_load_2d(st + L.dv, &tmapV, &full[s], (int)(2 * r0), rowV);
                issued = it + 1;
            }
            // let every issued copy land before the CTA can retire
            for (int it = (issued > NST ? issued - NST : 0); it < issued; ++it)
                mbar_wait_bounded(&full[it % NST], (uint32_t)(it / NST) & 1u);
        }
    }
    else if (warp == 1)
    {
        if (lane == 0)
        {
            const uint32_t idesc = umma_idesc_f16(BF16 ? 1u : 0u, 128u, (uint32_t)NT);
            for (int it = 0; it < nstage; ++it)
            {
                const int s = it % NST;
                const uint32_t ph = (uint32_t)(it / NST) & 1u;
                const int grp = it / TC_GROUP;
                const int b = grp & 1;
                const bool first = (it % TC_GROUP) == 0;
                const bool last = (it % TC_GROUP) == TC_GROUP - 1 || it == nstage - 1;
                bool ok = true;
                if (first) ok = mbar_wait_bounded(&acce[b], (uint32_t)((grp >> 1) & 1) ^ 1u);
                ok = ok && mbar_wait_bounded(&full[s], ph) && mbar_wait_bounded(&aready[s], ph);
                if (!ok)
                {
                    *abort_flag = 1;
                    atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                    break;
                }
                if (*abort_flag) break;
                tc_fence_after();
                const uint32_t base = smem_u32(sm + s * L.stage_bytes);
                const uint32_t dacc = tmem + (uint32_t)(b * NT);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                {
                    const uint64_t ah = umma_desc_sw128(base + L.a_hi + 32 * k);
                    const uint64_t al = umma_desc_sw128(base + L.a_lo + 32 * k);
                    const uint64_t bh = umma_desc_sw128(base + L.b_hi + 32 * k);
                    const uint64_t bl = umma_desc_sw128(base + L.b_lo + 32 * k);
                    umma_f16(dacc, ah, bh, idesc, (first && k == 0) ? 0u : 1u);
                    umma_f16(dacc, ah, bl, idesc, 1u);
                    umma_f16(dacc, al, bh, idesc, 1u);
                }
                umma_commit(&empty[s]);
                if (last) umma_commit(&accf[b]);
            }
        }
    }
    else if (warp < 10)
    {
        // ---------------- A producers: warps 2..9, lane = grid point in stage
        const int pw = warp - 2;  // 0..7
        const int MT = gd.mt_modes;
        const int nu0 = mt * MT;
        const int MTa = min(MT, gd.nmodes - nu0);  // modes present in this tile
        const bool fast = (gd.nbnds % 8 == 0) && (gd.nmag != 4) && gd.nbnds <= 64;
        const uint32_t chunk16 = (uint32_t)(lane >> 2), within = (uint32_t)(lane & 3) * 4;
        const int bpw = gd.nbnds >> 3;
        uint32_t off0[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
        {
            const uint32_t m = (uint32_t)(pw + 8 * j);
            off0[j] = (m >> 3) * 1024 + (m & 7) * 128 + ((chunk16 ^ (m & 7)) << 4) + within;
        }
        // a K chunk never straddles spinor components (chunk_pts divides N)
        const long long kc0 = (long long)chunk * chunk_pts;
        const int sp = (int)(kc0 / N);
        for (int it = 0; it < nstage; ++it)
        {
            const int s = it % NST;
            const uint32_t ph = (uint32_t)(it / NST) & 1u;
            bool ok = mbar_wait_bounded(&empty[s], ph ^ 1u) && mbar_wait_bounded(&full[s], ph);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok && lane == 0)
            {
                *abort_flag = 1;
                atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
            }
            if (__any_sync(0xffffffffu, !ok || *abort_flag != 0)) break;
            uint8_t* st = sm + s * L.stage_bytes;
            const float2* dvs = reinterpret_cast<const float2*>(st + L.dv);
            if (fast)
            {
                const int comp = (gd.nmag == 2) ? spin : 0;
                switch (bpw)
                {
                    case 1: produce_fast<BF16, 1>(st, L, dvs, MTa, comp, gd.nmag, gd.nbnds, pw, lane, off0); break;
                    case 2: produce_fast<BF16, 2>(st, L, dvs, MTa, comp, gd.nmag, gd.nbnds, pw, lane, off0); break;
                    case 3: produce_fast<BF16, 3>(st, L, dvs, MTa, comp, gd.nmag, gd.nbnds, pw, lane, off0); break;
                    case 4: produce_fast<BF16, 4>(st, L, dvs, MTa, comp, gd.nmag, gd.nbnds, pw, lane, off0); break;
                    case 5: produce_fast<BF16, 5>(st, L, dvs, MTa, comp, gd.nmag, gd.nbnds, pw, lane, off0); break;
                    case 6: produce_fast<BF16, 6>(st, L, dvs, MTa, comp, gd.nmag, gd.nbnds, pw, lane, off0); break;
                    case 7: produce_fast<BF16, 7>(st, L, dvs, MTa, comp, gd.nmag, gd.nbnds, pw, lane, off0); break;
                    default: produce_fast<BF16, 8>(st, L, dvs, MTa, comp, gd.nmag, gd.nbnds, pw, lane, off0); break;
                }
            }
            else
            {
                for (int m = pw; m < gd.nbnds; m += 8)
                {
                    float2 psi0 = load_split<BF16>(st + L.p_hi, st + L.p_lo, (uint32_t)m * 128 + 4 * lane);
                    float2 psi1 = make_float2(0.f, 0.f);
                    if (gd.nmag == 4)
                        psi1 = load_split<BF16>(st + L.p_hi + gd.nbp * 128, st + L.p_lo + gd.nbp * 128,
                                                (uint32_t)m * 128 + 4 * lane);
                    for (int ml = 0; ml < MTa; ++ml)
                    {
                        const int row = ml * gd.nbnds + m;
                        const float2* dvn = dvs + ml * gd.nmag * TC_KPTS + lane;
                        float2 a;
                        if (gd.nmag == 4)
                            a = cadd(cmul(dvn[(2 * sp) * TC_KPTS], psi0), cmul(dvn[(2 * sp + 1) * TC_KPTS], psi1));
                        else
                            a = cmul(dvn[((gd.nmag == 2) ? spin : 0) * TC_KPTS], psi0);
                        const uint32_t off = (uint32_t)(row >> 3) * 1024 + (uint32_t)(row & 7) * 128 +
                                             ((chunk16 ^ (uint32_t)(row & 7)) << 4) + within;
                        split_store<BF16>(st + L.a_hi, st + L.a_lo, off, a.x, a.y);
                    }
                }
            }
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&aready[s]);
        }
    }
    else if (warp < 10 + ndrain)
    {
        // ---------------- drain warps: TMEM lane quadrant warp%4, 64-column half
        const int dw = warp - 10;
        const int q = warp & 3;
        const int c0 = (dw >> 2) * 64;
        const int nc = min(64, NT - c0);
        float acc[64];
#pragma unroll
        for (int i = 0; i < 64; ++i) acc[i] = 0.f;
        bool good = true;
        for (int grp = 0; grp < ngroup; ++grp)
        {
            const int b = grp & 1;
            bool ok = (*abort_flag == 0) && mbar_wait_bounded(&accf[b], (uint32_t)(grp >> 1) & 1u);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok)
            {
                if (lane == 0 && *abort_flag == 0)
                {
                    *abort_flag = 1;
                    atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                }
                good = false;
                break;
            }
            tc_fence_after();
            const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * NT + c0);
#pragma unroll
            for (int c = 0; c < 64; c += 16)
            {
                if (c < nc)
                {
                    float v[16];
                    tmem_ld16(ta + (uint32_t)c, v);
#pragma unroll
                    for (int i = 0; i < 16; ++i) acc[c + i] += v[i];
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[b]);
        }
        if (good)
        {
            const int row = q * 32 + lane;
            const int mtiles = gridDim.y;
            float* out = partials + ((((size_t)zp * mtiles + mt) * nchunks + chunk) * 128 + row) * NT + c0;
#pragma unroll
            for (int c = 0; c < 64; c += 4)
                if (c < nc) *reinterpret_cast<float4*>(out + c) = make_float4(acc[c], acc[c + 1], acc[c + 2], acc[c + 3]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1)
    {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

void lelph_launch_local_tc(const PairInfo* pairs, int npairs, const void* tmapB, const void* tmapA,
                           const void* tmapV, const float* mode_scale, const GeomDev& g, int ab_bf16, int chunk_pts,
                           int nchunks, float* partials, unsigned* status, cudaStream_t st)
{
    const int mtiles = (g.nmodes + g.mt_modes - 1) / g.mt_modes;
    dim3 grid(nchunks, mtiles, npairs * g.nspin);
    const int smem = lelph_local_tc_smem_bytes(g);
    const int threads = 32 * (10 + 4 * ((2 * g.nbp + 63) / 64));
    const CUtensorMap* tB = static_cast<const CUtensorMap*>(tmapB);
    const CUtensorMap* tA = static_cast<const CUtensorMap*>(tmapA);
    const CUtensorMap* tV = static_cast<const CUtensorMap*>(tmapV);
    if (ab_bf16)
    {
        cudaFuncSetAttribute(k_local_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        k_local_tc<1><<<grid, threads, smem, st>>>(*tB, *tA, *tV, pairs, mode_scale, g, chunk_pts, nchunks,
                                                      partials, status);
    }
    else
    {
        cudaFuncSetAttribute(k_local_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        k_local_tc<0><<<grid, threads, smem, st>>>(*tB, *tA, *tV, pairs, mode_scale, g, chunk_pts, nchunks,
                                                      partials, status);
    }
}
