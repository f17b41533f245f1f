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
//   in FP32, A = dV psi_k formed in registers and written to tensor memory
//   as 16-bit (hi, lo) pairs, B = psi_k+q split likewise in shared memory,
//   three products A_hi B_hi + A_hi B_lo + A_lo B_hi accumulated in FP32 in
//   tensor memory per K chunk; chunks are reduced in FP64 by the finish kernel.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

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
// MMAs, warps 2 .. 2 + 4 PQ - 1 build the A operand directly in tensor
// memory, the next warps drain the accumulators.
//
// Tensor memory (512 columns): NACC (4, or 2 for wide tiles) accumulators,
// then NA A-operand slots of 128 columns (A_hi: 64 columns, A_lo: 64 columns;
// one column holds the (Re, Im) 16-bit pair of one grid point, lane = row).
// Shared memory holds only TMA tiles, so the TMA ring is up to 8 stages deep:
// per stage B (k+q split rows, 128-byte swizzle), the FP32 psi_k tile (two
// 16-point halves, 128-byte swizzle) and the FP32 dV tile of the tile's modes.

#define TC_NST_MAX 8
#define TC_NA_MAX 6
#define TC_NACC_MAX 4
#define TC_SMEM_LIMIT (227 * 1024)
// A pipeline stage is KP grid points (KP/32 K atoms of 128 bytes); one TMEM
// accumulator chains 64 points (two 32-point stages or one 64-point stage)
// before it is drained.
// producer warps per TMEM lane quadrant (each forms KP / PQ points of a stage,
// at least one 16-point block)
#define TC_PQ 2
template <int KP> __host__ __device__ constexpr int tc_pq() { return KP >= 16 * TC_PQ ? TC_PQ : KP / 16; }
// TMA and MMA warps, 4 PQ producer warps, 4 drain warps per 64 accumulator
// columns (NDR groups)
#define TC_THREADS(KP, NDR) (32 * (2 + 4 * tc_pq<KP>() + 4 * (NDR)))

struct TcSmemLayout
{
    uint32_t b_hi, b_lo, p, dv;               // offsets of stage 0 (B: K atom 0; atom j at + j * b_atom)
    uint32_t b_bytes, b_atom, p_half, p_bytes, dv_bytes, dv_block;
    uint32_t stage_bytes;
    uint32_t nst, na, nacc, accw, merged, a_col0;
    uint32_t bar_off, total;
};

// whole modes per 128-row tile of (mode, band) rows
__host__ __device__ inline int tc_tile_modes(const GeomDev& g) { return g.mt_modes; }

__host__ __device__ inline TcSmemLayout tc_layout(const GeomDev& g)
{
    TcSmemLayout L;
    const uint32_t NT = 2 * g.nbp;
    const uint32_t nsp = (g.nmag == 4) ? 2 : 1;
    // B per K atom (32 points): NT hi rows then NT lo rows, 128 B each, so the
    // merged N = 2 NT operand of an atom is one contiguous K-major tile
    L.b_bytes = NT * 128;
    L.b_atom = 2 * L.b_bytes;
    L.p_half = g.nbp * 128;  // 16 points x 8 B per band row
    const uint32_t natom = (uint32_t)g.kpts / 32;
    L.p_bytes = nsp * (2 * natom) * L.p_half;
    L.dv_block = tc_tile_modes(g) * g.nmag * 32 * 8;  // rows (mode, component) x 32 points
    L.dv_bytes = natom * L.dv_block;
    L.b_hi = 0;
    L.b_lo = L.b_hi + L.b_bytes;
    L.p = natom * L.b_atom;
    L.dv = L.p + L.p_bytes;
    L.stage_bytes = (L.dv + L.dv_bytes + 1023) / 1024 * 1024;
    L.nst = (TC_SMEM_LIMIT - 2048) / L.stage_bytes;
    if (L.nst > TC_NST_MAX) L.nst = TC_NST_MAX;
    // merged form (NT <= 64): one N = 2*NT MMA A_hi [B_hi; B_lo] and one N = NT
    // MMA A_lo B_hi per K step; accumulator columns [0, NT) collect hi.hi and
    // [NT, 2 NT) hi.lo + lo.hi.  Narrow N runs at a fixed per-instruction cost,
    // so the merge saves a third of the tensor time.  Wider tiles keep three
    // N = NT products into one accumulator.
    L.merged = (NT <= 64) ? 1 : 0;
    L.accw = L.merged ? 2 * NT : NT;
    L.nacc = (4 * L.accw + 4 * 64 <= 512) ? 4 : 2;
    L.a_col0 = L.nacc * L.accw;
    L.na = (512 - L.a_col0) / (2 * (uint32_t)g.kpts);
    if (L.na > TC_NA_MAX) L.na = TC_NA_MAX;
    L.bar_off = L.nst * L.stage_bytes;
    L.total = L.bar_off + 512 + 256 + 1024;  // barriers, a zero dV row, alignment slack
    return L;
}

int lelph_local_tc_smem_bytes(const GeomDev& g) { return (int)tc_layout(g).total; }
int lelph_local_tc_stages(const GeomDev& g) { return (int)tc_layout(g).nst; }
int lelph_local_tc_tile_modes(const GeomDev& g) { return tc_tile_modes(g); }
int lelph_local_tc_supported(const GeomDev& g)
{
    const TcSmemLayout L = tc_layout(g);
    return (2 * g.nbp <= 128) && L.nst >= 2 && L.na >= 2 && L.a_col0 + L.na * 2 * (uint32_t)g.kpts <= 512;
}

// (hi, lo) 16-bit split of a complex value: hi = rn(v), lo = rn(v - hi)
template <int BF16>
__device__ __forceinline__ void split_pair(float re, float im, uint32_t& h, uint32_t& l)
{
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
        // the residuals (re, im) - hi, exact; two scalar subtractions, which
        // measured faster than one packed FP32x2 FMA here
        const float2 d = make_float2(re - hf.x, im - hf.y);
        __half2 lv = __floats2half2_rn(d.x, d.y);
        h = *reinterpret_cast<uint32_t*>(&hv);
        l = *reinterpret_cast<uint32_t*>(&lv);
    }
}

// Tensor-memory stores of the A producers.  No "memory" clobber: they write
// tensor memory only, and a clobber would keep the compiler from issuing the
// next points' shared-memory loads before them.  The stage's
// tcgen05.wait::st (a volatile asm with a clobber) stays after them.
__device__ __forceinline__ void tmem_st8_a(uint32_t taddr, const uint32_t* r)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(r[0]),
                 "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]));
}
__device__ __forceinline__ void tmem_st16_a(uint32_t taddr, const uint32_t* r)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
                 ::"r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
                 "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]));
}
__device__ __forceinline__ void tmem_st4_a(uint32_t taddr, const uint32_t* r)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr), "r"(r[0]), "r"(r[1]),
                 "r"(r[2]), "r"(r[3]));
}

// The operands of SUB grid points of one row (one lane), NC dV components:
// psi (16-byte chunks of two points) and dV.
template <int SUB, int NC>
struct ProdFrag
{
    float4 ps[SUB / 2][NC];
    float4 dv[SUB / 2][NC];
};

// pp[c] points at the lane's psi row (128-byte swizzled half tile), dvp[c] at
// the row's dV (16 points of the half); j0 is the first point of the SUB.
template <int SUB, int NC>
__device__ __forceinline__ void prod_load(ProdFrag<SUB, NC>& f, const uint8_t* const* pp, const float4* const* dvp,
                                          uint32_t swz, int j0)
{
#pragma unroll
    for (int jj = 0; jj < SUB / 2; ++jj)
    {
        const int j = j0 / 2 + jj;  // 16-byte chunk = 2 points
#pragma unroll
        for (int c = 0; c < NC; ++c)
        {
            f.ps[jj][c] = *reinterpret_cast<const float4*>(pp[c] + ((((uint32_t)j) ^ swz) << 4));
            f.dv[jj][c] = dvp[c][j];
        }
    }
}

// A operand of the SUB points: a = sum_c dV^{c} psi^{c}, split and stored to
// the lane's TMEM row.
template <int BF16, int SUB, int NC>
__device__ __forceinline__ void prod_store(const ProdFrag<SUB, NC>& f, uint32_t tcol_hi, uint32_t tcol_lo)
{
    uint32_t hi[SUB], lo[SUB];
#pragma unroll
    for (int jj = 0; jj < SUB / 2; ++jj)
    {
        // the first component's product initialises the sum: 0 + x is not
        // foldable to x in IEEE arithmetic (-0), so a zero start costs an add
        float4 acc;
        {
            const float4 ps = f.ps[jj][0], dv = f.dv[jj][0];
            acc.x = dv.x * ps.x - dv.y * ps.y;
            acc.y = dv.x * ps.y + dv.y * ps.x;
            acc.z = dv.z * ps.z - dv.w * ps.w;
            acc.w = dv.z * ps.w + dv.w * ps.z;
        }
#pragma unroll
        for (int c = 1; c < NC; ++c)
        {
            const float4 ps = f.ps[jj][c], dv = f.dv[jj][c];
            acc.x += dv.x * ps.x - dv.y * ps.y;
            acc.y += dv.x * ps.y + dv.y * ps.x;
            acc.z += dv.z * ps.z - dv.w * ps.w;
            acc.w += dv.z * ps.w + dv.w * ps.z;
        }
        split_pair<BF16>(acc.x, acc.y, hi[2 * jj], lo[2 * jj]);
        split_pair<BF16>(acc.z, acc.w, hi[2 * jj + 1], lo[2 * jj + 1]);
    }
    if (SUB == 16)
    {
        tmem_st16_a(tcol_hi, hi);
        tmem_st16_a(tcol_lo, lo);
    }
    else if (SUB == 8)
    {
        tmem_st8_a(tcol_hi, hi);
        tmem_st8_a(tcol_lo, lo);
    }
    else
    {
        tmem_st4_a(tcol_hi, hi);
        tmem_st4_a(tcol_lo, lo);
    }
}

// A producer's share of one pipeline stage: points h*KP/PQ .. (h+1)*KP/PQ - 1,
// in 16-point psi blocks of 16/SUB pieces of SUB points each.  The pieces are
// software-pipelined: the shared-memory loads of piece t+1 are issued before
// piece t is formed and stored, so that their latency overlaps the work.
template <int BF16, int KP, int SUB, int NC, int PF>
__device__ __forceinline__ void produce_stage(const uint8_t* st, const TcSmemLayout& L, const float4* zero_dv,
                                              bool in_tile, int h, int m, int ml, int nmag, int comp0, int comp1,
                                              int nsp, uint32_t swz, uint32_t col_base)
{
    constexpr int NATOM = KP / 32;
    constexpr int PPW = KP / tc_pq<KP>();  // points of this warp
    static_assert(PPW % 16 == 0, "a producer warp forms whole 16-point blocks");
    constexpr int NBW = PPW / 16;    // 16-point blocks of this warp
    constexpr int PER_BLOCK = 16 / SUB;
    constexpr int NPIECE = NBW * PER_BLOCK;
    const uint8_t* pp[NBW][2];
    const float4* dvp[NBW][2];
#pragma unroll
    for (int b = 0; b < NBW; ++b)
    {
        const int p0 = h * PPW + 16 * b;  // first point of the block in the stage
        const int pb = p0 >> 4;                // 16-point psi block
        const float* dvs = reinterpret_cast<const float*>(st + L.dv + (uint32_t)(p0 >> 5) * L.dv_block);
        pp[b][0] = st + L.p + (0 * 2 * NATOM + pb) * L.p_half + (uint32_t)m * 128;
        pp[b][1] = st + L.p + ((nsp - 1) * 2 * NATOM + pb) * L.p_half + (uint32_t)m * 128;
        dvp[b][0] = in_tile ? reinterpret_cast<const float4*>(dvs + ((size_t)(ml * nmag + comp0) * 32 + (p0 & 31)) * 2)
                            : zero_dv;
        dvp[b][1] = in_tile ? reinterpret_cast<const float4*>(dvs + ((size_t)(ml * nmag + comp1) * 32 + (p0 & 31)) * 2)
                            : zero_dv;
    }
    if (PF)
    {
        ProdFrag<SUB, NC> f[2];
        prod_load<SUB, NC>(f[0], pp[0], dvp[0], swz, 0);
#pragma unroll
        for (int t = 0; t < NPIECE; ++t)
        {
            if (t + 1 < NPIECE)
            {
                const int bn = (t + 1) / PER_BLOCK;
                prod_load<SUB, NC>(f[(t + 1) & 1], pp[bn], dvp[bn], swz, ((t + 1) % PER_BLOCK) * SUB);
            }
            const int b = t / PER_BLOCK, j0 = (t % PER_BLOCK) * SUB;
            const uint32_t col_hi = col_base + (uint32_t)(h * PPW + 16 * b + j0);
            prod_store<BF16, SUB, NC>(f[t & 1], col_hi, col_hi + KP);
        }
    }
    else
    {
#pragma unroll
        for (int t = 0; t < NPIECE; ++t)
        {
            ProdFrag<SUB, NC> f;
            const int b = t / PER_BLOCK, j0 = (t % PER_BLOCK) * SUB;
            prod_load<SUB, NC>(f, pp[b], dvp[b], swz, j0);
            const uint32_t col_hi = col_base + (uint32_t)(h * PPW + 16 * b + j0);
            prod_store<BF16, SUB, NC>(f, col_hi, col_hi + KP);
        }
    }
}

// One pipeline stage of the merged split product (NT <= 64): per 16-wide K
// step k, A_hi [B_hi; B_lo] (N = 2 NT) into dacc and A_lo B_hi (N = NT) into
// dacc2.  B's descriptor advances by 32 bytes per step inside a 128-byte K
// atom (d0: atom 0, d1: atom 1) and A's tensor-memory column by 8, all by
// immediates inside one asm block, so that the issuing thread spends about
// three instructions per MMA pair: it shares its SM sub-partition with FMA-bound
// producer warps, and every instruction of it waits for an issue slot.
template <int KP>
__device__ __forceinline__ void umma_stage_merged(uint32_t dacc, uint32_t dacc2, uint32_t ahi, uint64_t d0,
                                                  uint64_t d1, uint32_t idesc2, uint32_t idesc, uint32_t en);
template <>
__device__ __forceinline__ void umma_stage_merged<64>(uint32_t dacc, uint32_t dacc2, uint32_t ahi, uint64_t d0,
                                                      uint64_t d1, uint32_t idesc2, uint32_t idesc, uint32_t en)
{
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t.reg .b64 d;\n\t.reg .b32 a;\n\t"
        "setp.ne.b32 p, %7, 0;\n\tsetp.eq.b32 q, %7, %7;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%2], %3, %5, p;\n\t"
        "add.u32 a, %2, 64;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], %3, %6, q;\n\t"
        "add.s64 d, %3, 2;\n\t"
        "add.u32 a, %2, 8;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], d, %5, q;\n\t"
        "add.u32 a, %2, 72;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], d, %6, q;\n\t"
        "add.s64 d, %3, 4;\n\t"
        "add.u32 a, %2, 16;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], d, %5, q;\n\t"
        "add.u32 a, %2, 80;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], d, %6, q;\n\t"
        "add.s64 d, %3, 6;\n\t"
        "add.u32 a, %2, 24;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], d, %5, q;\n\t"
        "add.u32 a, %2, 88;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], d, %6, q;\n\t"
        "add.u32 a, %2, 32;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], %4, %5, q;\n\t"
        "add.u32 a, %2, 96;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], %4, %6, q;\n\t"
        "add.s64 d, %4, 2;\n\t"
        "add.u32 a, %2, 40;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], d, %5, q;\n\t"
        "add.u32 a, %2, 104;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], d, %6, q;\n\t"
        "add.s64 d, %4, 4;\n\t"
        "add.u32 a, %2, 48;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], d, %5, q;\n\t"
        "add.u32 a, %2, 112;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], d, %6, q;\n\t"
        "add.s64 d, %4, 6;\n\t"
        "add.u32 a, %2, 56;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], d, %5, q;\n\t"
        "add.u32 a, %2, 120;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], d, %6, q;\n\t"
        "}"
        ::"r"(dacc), "r"(dacc2), "r"(ahi), "l"(d0), "l"(d1), "r"(idesc2), "r"(idesc), "r"(en)
        : "memory");
}
template <>
__device__ __forceinline__ void umma_stage_merged<32>(uint32_t dacc, uint32_t dacc2, uint32_t ahi, uint64_t d0,
                                                      uint64_t d1, uint32_t idesc2, uint32_t idesc, uint32_t en)
{
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t.reg .b64 d;\n\t.reg .b32 a;\n\t"
        "setp.ne.b32 p, %7, 0;\n\tsetp.eq.b32 q, %7, %7;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%2], %3, %5, p;\n\t"
        "add.u32 a, %2, 32;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], %3, %6, q;\n\t"
        "add.s64 d, %3, 2;\n\t"
        "add.u32 a, %2, 8;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], d, %5, q;\n\t"
        "add.u32 a, %2, 40;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], d, %6, q;\n\t"
        "add.s64 d, %3, 4;\n\t"
        "add.u32 a, %2, 16;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], d, %5, q;\n\t"
        "add.u32 a, %2, 48;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], d, %6, q;\n\t"
        "add.s64 d, %3, 6;\n\t"
        "add.u32 a, %2, 24;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [a], d, %5, q;\n\t"
        "add.u32 a, %2, 56;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%1], [a], d, %6, q;\n\t"
        "}"
        ::"r"(dacc), "r"(dacc2), "r"(ahi), "l"(d0), "l"(d1), "r"(idesc2), "r"(idesc), "r"(en)
        : "memory");
}

// Persistent grid: one CTA per SM; CTA c takes the work units u = c, c + G,
// c + 2G, ... with u = (pair*nspin + spin, mode tile, K chunk), chunk fastest.
// The barrier rings, the tensor memory and the TMA pipeline carry over from
// one unit to the next, so a unit's first tiles are in flight while the
// previous unit drains.  TC_THREADS(KP, NDR) threads.
//
// The tensor-core accumulator loses low-order bits on every accumulation
// (its error grows linearly with the number of MMAs chained into one FP32
// accumulator), so accumulation chains are kept to TC_GROUP pipeline stages:
// the MMA warp cycles through NACC TMEM accumulators, and the drain warps
// add each finished accumulator into round-to-nearest FP32 registers, which
// are written out per K chunk and reduced in FP64 by the finish kernel.
struct TcUnit
{
    int chunk, mt, zp, spin;
    PairInfo P;
};

__device__ __forceinline__ TcUnit tc_unit(int u, int nchunks, int mtiles, int nspin, const PairInfo* pairs)
{
    TcUnit w;
    w.chunk = u % nchunks;
    const int t = u / nchunks;
    w.mt = t % mtiles;
    w.zp = t / mtiles;
    const int pair = w.zp / nspin;
    w.spin = w.zp - pair * nspin;
    w.P = pairs[pair];
    return w;
}

template <int BF16, int KP, int NDR>
__global__ void __launch_bounds__(TC_THREADS(KP, NDR), 1)
    k_local_tc(const __grid_constant__ CUtensorMap tmapB, const __grid_constant__ CUtensorMap tmapP,
               const __grid_constant__ CUtensorMap tmapV, const PairInfo* __restrict__ pairs, GeomDev gd,
               int chunk_pts, int nchunks, int mtiles, int nunits, float* __restrict__ partials,
               unsigned* __restrict__ status, unsigned long long wait_ns)
{
    extern __shared__ __align__(1024) uint8_t smraw[];
    // aligned by pointer arithmetic on the shared array itself (not through an
    // integer), so that the compiler keeps the shared address space and emits
    // shared-memory loads with 32-bit addresses rather than generic ones
    uint8_t* sm = smraw + ((1024u - (smem_u32(smraw) & 1023u)) & 1023u);
    const TcSmemLayout L = tc_layout(gd);
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + L.bar_off);
    uint64_t* empty = full + TC_NST_MAX;    // TMA slot consumed: MMA commit + 4 PQ producer warps
    uint64_t* aready = empty + TC_NST_MAX;  // A slot written (producers -> MMA)
    uint64_t* afree = aready + TC_NA_MAX;   // A slot read (MMA commit -> producers)
    uint64_t* accf = afree + TC_NA_MAX;     // [nacc] accumulator b complete (MMA -> drain)
    uint64_t* acce = accf + TC_NACC_MAX;    // [nacc] accumulator b drained (drain -> MMA)
    const int NST = (int)L.nst, NA = (int)L.na, NACC = (int)L.nacc;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + TC_NACC_MAX);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const float4* zero_dv = reinterpret_cast<const float4*>(sm + L.bar_off + 512);  // 256 zero bytes

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NT = 2 * gd.nbp;
    const long long N = (long long)gd.Nx * gd.Ny * gd.Nz;
    constexpr int TC_GROUP = 64 / KP;
    constexpr int NATOM = KP / 32;
    const int nstage = chunk_pts / KP;
    const int ngroup = (nstage + TC_GROUP - 1) / TC_GROUP;
    const int nsp = (gd.nmag == 4) ? 2 : 1;
    const int ndrain = 4 * NDR;  // = 4 * ceil(NT / 64), chosen by the launcher

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < NST; ++s)
        {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1 + 4 * tc_pq<KP>());
        }
        for (int a = 0; a < NA; ++a)
        {
            mbar_init(&aready[a], 4 * tc_pq<KP>());
            mbar_init(&afree[a], 1);
        }
        for (int b = 0; b < NACC; ++b)
        {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], ndrain);
        }
        *abort_flag = 0;
        fence_barrier_init();
    }
    if (threadIdx.x < 64) reinterpret_cast<float*>(sm + L.bar_off + 512)[threadIdx.x] = 0.f;
    if (warp == 1) tmem_alloc(tmem_slot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0)
    {
        if (lane == 0)
        {
            prefetch_tmap(&tmapB);
            prefetch_tmap(&tmapP);
            prefetch_tmap(&tmapV);
            const int nkb = (int)((long long)gd.nspinor * N / 32);  // 32-point K blocks per row group
            const uint32_t bytes = NATOM * L.b_atom + L.p_bytes + L.dv_bytes;
            // ring positions advance incrementally: no runtime divisions on the issue paths
            int s = 0;
            uint32_t ph = 0;
            long long issued = 0;
            bool stop = false;
            for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
            {
                const TcUnit w = tc_unit(u, nchunks, mtiles, gd.nspin, pairs);
                // tile-major operands: z = (row group) * blocks + block
                const int zB_hi = ((w.P.kbz_kq * gd.nspin + w.spin) * 2 + 0) * nkb;
                const int zB_lo = zB_hi + nkb;
                const int zP = (w.P.kbz_k * gd.nspin + w.spin) * 2 * nkb;  // 16-point blocks
                const int zV = w.P.dvslot * (int)(N / 32);
                const int yV = w.mt * gd.mt_modes * gd.nmag;
                // a K chunk lies within one spinor component (chunk_pts divides N)
                const long long kc0 = (long long)w.chunk * chunk_pts;
                const int sp = (int)(kc0 / N);
                const long long r00 = kc0 - (long long)sp * N;
                for (int it = 0; it < nstage; ++it, s = (s + 1 == NST) ? 0 : s + 1, ph ^= (s == 0) ? 1u : 0u)
                {
                    if (!mbar_wait_bounded(&empty[s], ph ^ 1u, wait_ns))
                    {
                        *abort_flag = 1;
                        atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                        stop = true;
                        break;
                    }
                    if (*abort_flag)
                    {
                        stop = true;
                        break;
                    }
                    uint8_t* st = sm + s * L.stage_bytes;
                    const long long kc = kc0 + (long long)it * KP;
                    const long long r0 = r00 + (long long)it * KP;
                    mbar_arrive_expect_tx(&full[s], bytes);
                    for (int j = 0; j < NATOM; ++j)
                    {
                        tma_load_3d(st + j * L.b_atom + L.b_hi, &tmapB, &full[s], 0, 0, zB_hi + (int)(kc >> 5) + j);
                        tma_load_3d(st + j * L.b_atom + L.b_lo, &tmapB, &full[s], 0, 0, zB_lo + (int)(kc >> 5) + j);
                    }
                    for (int q = 0; q < nsp; ++q)
                    {
                        const int spp = (gd.nmag == 4) ? q : sp;
                        const long long kq = (long long)spp * N + r0;
                        // the stage's 16-point blocks in one box
                        tma_load_3d(st + L.p + 2 * NATOM * q * L.p_half, &tmapP, &full[s], 0, 0, zP + (int)(kq >> 4));
                    }
                    // dV_nu(r) of the tile's modes, all magnetic components: two blocks of
                    // rows (nu, comp) x 32 points
                    tma_load_3d(st + L.dv, &tmapV, &full[s], 0, yV, zV + (int)(r0 >> 5));
                    ++issued;
                }
            }
            // let every issued copy land before the CTA can retire
            for (long long i = (issued > NST ? issued - NST : 0); i < issued; ++i)
                mbar_wait_bounded(&full[i % NST], (uint32_t)(i / NST) & 1u);
        }
    }
    else if (warp == 1)
    {
        if (lane == 0)
        {
            const uint32_t idesc = umma_idesc_f16(BF16 ? 1u : 0u, 128u, (uint32_t)NT);
            const uint32_t idesc2 = umma_idesc_f16(BF16 ? 1u : 0u, 128u, (uint32_t)(2 * NT));
            const bool merged = L.merged != 0;
            int s = 0, a = 0, b = 0;
            uint32_t pha = 0, phb = 0;
            bool stop = false;
            uint64_t* last_commit = nullptr;  // the A-slot barrier of the latest commit, and its phase parity
            uint32_t last_par = 0;
            for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
            {
                for (int it = 0; it < nstage; ++it)
                {
                    const bool first = (it % TC_GROUP) == 0;
                    const bool last = (it % TC_GROUP) == TC_GROUP - 1 || it == nstage - 1;
                    // MMA issue blocks per instruction, so this thread checks one barrier
                    // per stage: the producers arrive on aready[a] only after they saw the
                    // stage's TMA tiles land (full[s]), which orders B for the MMAs too
                    bool ok = true;
                    if (first) ok = mbar_wait_bounded(&acce[b], phb ^ 1u, wait_ns);
                    ok = ok && mbar_wait_bounded(&aready[a], pha, wait_ns);
                    if (!ok)
                    {
                        *abort_flag = 1;
                        atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t base = smem_u32(sm + s * L.stage_bytes);
                    const uint32_t dacc = tmem + (uint32_t)b * L.accw;
                    const uint32_t ahi = tmem + L.a_col0 + (uint32_t)a * (2u * KP);
                    if (merged)
                    {
                        // rows [0, NT) of each atom's 2*NT-row tile are B_hi, [NT, 2NT) B_lo
                        const uint64_t d0 = umma_desc_sw128(base + L.b_hi);
                        const uint64_t d1 = d0 + (uint64_t)(L.b_atom >> 4);
                        umma_stage_merged<KP>(dacc, dacc + (uint32_t)NT, ahi, d0, d1, idesc2, idesc,
                                              first ? 0u : 1u);
                    }
                    else
#pragma unroll
                    for (int k = 0; k < KP / 8; ++k)
                    {
                        const uint32_t atom = base + (uint32_t)(k >> 2) * L.b_atom + 32u * (uint32_t)(k & 3);
                        const uint64_t bh = umma_desc_sw128(atom + L.b_hi);
                        const uint32_t en = (first && k == 0) ? 0u : 1u;
                        {
                            const uint64_t bl = umma_desc_sw128(atom + L.b_lo);
                            umma_f16_ta(dacc, ahi + 8 * k, bh, idesc, en);
                            umma_f16_ta(dacc, ahi + 8 * k, bl, idesc, 1u);
                            umma_f16_ta(dacc, ahi + KP + 8 * k, bh, idesc, 1u);
                        }
                    }
                    umma_commit(&empty[s]);
                    umma_commit(&afree[a]);
                    last_commit = &afree[a];
                    last_par = pha;
                    if (last) umma_commit(&accf[b]);
                    s = (s + 1 == NST) ? 0 : s + 1;
                    if (++a == NA)
                    {
                        a = 0;
                        pha ^= 1u;
                    }
                    if (last && ++b == NACC)
                    {
                        b = 0;
                        phb ^= 1u;
                    }
                }
            }
            // every MMA this thread issued completes before the tensor memory is
            // released, also when a wait above gave up (the commit tracks them all)
            if (last_commit) mbar_wait_bounded(last_commit, last_par);
        }
    }
    else if (warp < 2 + 4 * tc_pq<KP>())
    {
        // ---------------- A producers: lane quadrant q = warp % 4 (rows 32q..32q+31),
        // share h of the stage's points (KP / PQ of them)
        const int q = warp & 3;
        const int h = (warp - 2) >> 2;
        const int MT = gd.mt_modes;
        const int row = 32 * q + lane;
        const int ml = row / gd.nbnds, m = row - ml * gd.nbnds;
        const uint32_t swz = (uint32_t)(m & 7);
        const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
        int s = 0, a = 0;
        uint32_t ph = 0, pha = 0;
        bool stop = false;
        for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
        {
            const TcUnit w = tc_unit(u, nchunks, mtiles, gd.nspin, pairs);
            // rows of modes past nmodes read the TMA zero fill of the dV tile; rows
            // past the tile's MT*nb read the zero block
            const bool in_tile = ml < MT;
            // a K chunk never straddles spinor components (chunk_pts divides N)
            const int sp = (int)(((long long)w.chunk * chunk_pts) / N);
            int comp0, comp1;
            if (gd.nmag == 4)
            {
                comp0 = 2 * sp;
                comp1 = 2 * sp + 1;
            }
            else
            {
                comp0 = (gd.nmag == 2) ? w.spin : 0;
                comp1 = comp0;
            }
            for (int it = 0; it < nstage; ++it, s = (s + 1 == NST) ? 0 : s + 1, ph ^= (s == 0) ? 1u : 0u,
                     a = (a + 1 == NA) ? 0 : a + 1, pha ^= (a == 0) ? 1u : 0u)
            {
                bool ok = mbar_wait_bounded(&afree[a], pha ^ 1u, wait_ns) && mbar_wait_bounded(&full[s], ph, wait_ns);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok && lane == 0)
                {
                    *abort_flag = 1;
                    atomicOr(status, LELPH_DEV_ERR_TIMEOUT);
                }
                if (__any_sync(0xffffffffu, !ok || *abort_flag != 0))
                {
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint8_t* st = sm + s * L.stage_bytes;
                const uint32_t col_base = lane_base + L.a_col0 + (uint32_t)a * (2u * KP);
                if (gd.nmag == 4)
                    produce_stage<BF16, KP, 4, 2, (tc_pq<KP>() <= 2)>(st, L, zero_dv, in_tile, h, m, ml, gd.nmag, comp0, comp1, nsp,
                                                     swz, col_base);
                else
                    produce_stage<BF16, KP, 8, 1, (tc_pq<KP>() <= 2)>(st, L, zero_dv, in_tile, h, m, ml, gd.nmag, comp0, comp1, nsp,
                                                     swz, col_base);
                tmem_wait_st();
                tc_fence_before();
                __syncwarp();
                if (lane == 0)
                {
                    mbar_arrive(&aready[a]);
                    mbar_arrive(&empty[s]);
                }
            }
        }
    }
    else if (warp < 2 + 4 * tc_pq<KP>() + ndrain)
    {
        // ---------------- drain warps: TMEM lane quadrant warp%4, 64-column half
        const int dw = warp - 2 - 4 * tc_pq<KP>();
        const int q = warp & 3;
        const int c0 = (dw >> 2) * 64;
        const int nc = min(64, NT - c0);
        int b = 0;
        uint32_t phb = 0;
        bool stop = false;
        for (int u = blockIdx.x; u < nunits && !stop; u += gridDim.x)
        {
            float acc[64];
#pragma unroll
            for (int i = 0; i < 64; ++i) acc[i] = 0.f;
            for (int grp = 0; grp < ngroup; ++grp, b = (b + 1 == NACC) ? 0 : b + 1, phb ^= (b == 0) ? 1u : 0u)
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
                const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)b * L.accw + (uint32_t)c0;
#pragma unroll
                for (int c = 0; c < 64; c += 16)
                {
                    if (c < nc)
                    {
                        float v[16];
                        tmem_ld16(ta + (uint32_t)c, v);
#pragma unroll
                        for (int i = 0; i < 16; ++i) acc[c + i] += v[i];
                        if (L.merged)
                        {
                            tmem_ld16(ta + (uint32_t)(NT + c), v);
#pragma unroll
                            for (int i = 0; i < 16; ++i) acc[c + i] += v[i];
                        }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acce[b]);
            }
            if (stop) break;
            const TcUnit w = tc_unit(u, nchunks, mtiles, gd.nspin, pairs);
            const int row = q * 32 + lane;
            float* out = partials + lelph_tc_partial_offset(gd, nchunks, w.zp, w.mt, w.chunk, row) + c0;
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
        tmem_dealloc(tmem, 512);
    }
}

void lelph_launch_local_tc(const PairInfo* pairs, int npairs, const void* tmapB, const void* tmapP,
                           const void* tmapV, const GeomDev& g, int ab_bf16, int chunk_pts, int nchunks,
                           float* partials, unsigned* status, cudaStream_t st, unsigned long long wait_ns)
{
    if (wait_ns == 0) wait_ns = LELPH_WAIT_LIMIT_NS;
    const int mtiles = lelph_tc_mode_tiles(g);
    const long long units = (long long)npairs * g.nspin * mtiles * nchunks;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<long long>(units, std::max(1, nsm));
    const int smem = lelph_local_tc_smem_bytes(g);
    const int ndr = (2 * g.nbp + 63) / 64;  // drain groups of 64 accumulator columns (1 or 2)
    const CUtensorMap* tB = static_cast<const CUtensorMap*>(tmapB);
    const CUtensorMap* tP = static_cast<const CUtensorMap*>(tmapP);
    const CUtensorMap* tV = static_cast<const CUtensorMap*>(tmapV);
    if (units <= 0) return;
#define TC_LAUNCH(BF, KPV, NDR)                                                                                  \
    do                                                                                                           \
    {                                                                                                            \
        cudaFuncSetAttribute(k_local_tc<BF, KPV, NDR>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);        \
        k_local_tc<BF, KPV, NDR><<<grid, TC_THREADS(KPV, NDR), smem, st>>>(*tB, *tP, *tV, pairs, g, chunk_pts, nchunks, \
                                                                     mtiles, (int)units, partials, status,       \
                                                                     wait_ns);                                   \
    } while (0)
#define TC_LAUNCH_NDR(BF, KPV)                                                                                   \
    do                                                                                                           \
    {                                                                                                            \
        if (ndr == 1) TC_LAUNCH(BF, KPV, 1);                                                                     \
        else TC_LAUNCH(BF, KPV, 2);                                                                              \
    } while (0)
    if (ab_bf16)
    {
        if (g.kpts == 64) TC_LAUNCH_NDR(1, 64);
        else TC_LAUNCH_NDR(1, 32);
    }
    else
    {
        if (g.kpts == 64) TC_LAUNCH_NDR(0, 64);
        else TC_LAUNCH_NDR(0, 32);
    }
#undef TC_LAUNCH_NDR
#undef TC_LAUNCH
}
