// Wavefunction unfolding and batched 3-D FFTs for the electron-phonon path.
//
// * k_scatter: sphere -> box for every (full-BZ k, spin, band, spinor).  The
//   symmetry-rotated Miller index is integer arithmetic (W n, W the integer
//   action of the symmetry on the reciprocal lattice), so the plane-wave ->
//   box map is exact; it replaces rotateGvecs + rint + Sort_pw
//   (src/wfc/rotate_Gvecs.c:15-81, src/wfc/sortpw.c:95-315) and the
//   sphere->box step of invfft3D (src/fft/bwdfft.c:45-69).  SU(2) rotation
//   (src/wfc/su2rotate.c:13-41), the FP64 fractional-translation phase with
//   the truncated pi (src/wfc/trans_wfc.c:15-52) and the time-reversal conj
//   are applied on the fly.
// * k_fft_contig / k_fft_strided: batched 1-D Stockham passes (radix 2,3,4,5)
//   in shared memory, replacing the FFTW plans of src/fft/planner.c and the
//   slab transposes of src/fft/transpose.c.  Unnormalised, sign +1 is
//   FFTW_BACKWARD.
// * k_fft_x_split: the last (x) pass of the mixed form, whose epilogue writes
//   psi(r) straight into the split-precision tensor-core operand layout (the
//   k+q role) and as FP32 (the k role, from which the A operand is formed).
#include <cuda_runtime.h>
#include <stdint.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"
#include "fft_smem.cuh"

// ---------------------------------------------------- contiguous-line pass

// With a box mask, only the lines of occupied (x, y) columns are read,
// transformed and written back; the others are all zero and stay so.
// CTL > 0: the line length is the compile-time constant CTL (== p.L) and the
// compile-time Stockham schedule runs (ct_fft); 0: the run-time plan.
template <typename T2, typename T, int CTL>
__global__ void __launch_bounds__(256) k_fft_contig(T2* __restrict__ data, long long nlines, FftPlan1D p,
                                                    const T2* __restrict__ tw, int sign, int lpc, BoxMask mk)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* a = reinterpret_cast<T2*>(smraw);
    T2* b = a + (size_t)lpc * p.L;
    T2* tws = b + (size_t)lpc * p.L;
    int* act = reinterpret_cast<int*>(tws + p.L);  // [lpc] active lines of the block
    __shared__ int nact;
    for (int t = threadIdx.x; t < p.L; t += blockDim.x) tws[t] = tw[t];
    long long l0 = (long long)blockIdx.x * lpc;
    int nl = (int)min((long long)lpc, nlines - l0);
    T2* g = data + l0 * p.L;
    if (mk.col)
    {
        if (threadIdx.x == 0) nact = 0;
        __syncthreads();
        const long long ncol = (long long)mk.Nx * mk.Ny;
        if (nlines <= 0x7fffffffLL)
        {
            // 32-bit divisions (a 64-bit one is a long software sequence)
            const unsigned nc32 = (unsigned)ncol, nbk = (unsigned)mk.nbox_per_k;
            for (int j = threadIdx.x; j < nl; j += blockDim.x)
            {
                const unsigned line = (unsigned)(l0 + j);
                const unsigned box = line / nc32;
                const unsigned col = line - box * nc32;
                if (mk.col[(size_t)(box / nbk) * nc32 + col]) act[atomicAdd(&nact, 1)] = j;
            }
        }
        else
            for (int j = threadIdx.x; j < nl; j += blockDim.x)
            {
                const long long line = l0 + j;
                const long long box = line / ncol;
                const long long col = line - box * ncol;
                const long long kslot = box / mk.nbox_per_k;
                if (mk.col[kslot * ncol + col]) act[atomicAdd(&nact, 1)] = j;
            }
        __syncthreads();
        const int na = nact;
        if (na == 0) return;
        const RecipDiv dL = recip_div(p.L);
        if constexpr (CTL > 0 && CTL % 2 == 0 && sizeof(T2) == 8)
        {
            // two points per 16-byte load (lines start at even offsets)
            for (int i = 2 * threadIdx.x; i < na * CTL; i += 2 * blockDim.x)
            {
                const int j = i / CTL, e = i - j * CTL;  // a constant divisor
                *reinterpret_cast<float4*>(a + i) = *reinterpret_cast<const float4*>(g + (size_t)act[j] * CTL + e);
            }
        }
        else
            for (int i = threadIdx.x; i < na * p.L; i += blockDim.x)
            {
                int e, j;
                if constexpr (CTL > 0)
                {
                    j = i / CTL;  // a constant divisor: multiply and shift
                    e = i - j * CTL;
                }
                else
                    j = div_rem(i, dL, e);
                a[i] = g[(size_t)act[j] * p.L + e];
            }
        __syncthreads();
        T2* r;
        if constexpr (CTL > 0)
            r = ct_fft<T2, T, CTL, 0, 1, false, 0>(a, b, na, 1, CTL, nullptr, 1, CTL, tws, sign);
        else
            r = fft_smem<T2, T>(a, b, na, 1, p.L, p, tws, sign);
        if constexpr (CTL > 0 && CTL % 2 == 0 && sizeof(T2) == 8)
        {
            for (int i = 2 * threadIdx.x; i < na * CTL; i += 2 * blockDim.x)
            {
                const int j = i / CTL, e = i - j * CTL;
                *reinterpret_cast<float4*>(g + (size_t)act[j] * CTL + e) = *reinterpret_cast<const float4*>(r + i);
            }
        }
        else
            for (int i = threadIdx.x; i < na * p.L; i += blockDim.x)
            {
                int e, j;
                if constexpr (CTL > 0)
                {
                    j = i / CTL;  // a constant divisor: multiply and shift
                    e = i - j * CTL;
                }
                else
                    j = div_rem(i, dL, e);
                g[(size_t)act[j] * p.L + e] = r[i];
            }
        return;
    }
    int n = nl * p.L;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = g[i];
    __syncthreads();
    T2* r;
    if constexpr (CTL > 0)
        r = ct_fft<T2, T, CTL, 0, 1, false, 0>(a, b, nl, 1, CTL, nullptr, 1, CTL, tws, sign);
    else
        r = fft_smem<T2, T>(a, b, nl, 1, p.L, p, tws, sign);
    for (int i = threadIdx.x; i < n; i += blockDim.x) g[i] = r[i];
}

// ------------------------------------------------------- strided-line pass
// data viewed as [nouter][L][inner]; one CTA = one outer index and a chunk
// of `ich` inner positions, loaded as an [L][ich] tile (coalesced in inner).

// With a box mask (y pass: outer = (box, x)), empty x planes are skipped.
// CTL as in k_fft_contig.
// NLC > 0 (with CTL > 0): inner = ich = NLC, one chunk per line set, so the
// index divisions of the load, the passes and the store are by constants.
template <typename T2, typename T, int CTL, int NLC>
__global__ void __launch_bounds__(256) k_fft_strided(T2* __restrict__ data, long long nouter, int inner, int ich,
                                                     int nchunk, FftPlan1D p, const T2* __restrict__ tw, int sign,
                                                     BoxMask mk)
{
    static_assert(NLC == 0 || CTL > 0, "a compile-time line count needs a compile-time length");
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* a = reinterpret_cast<T2*>(smraw);
    T2* b = a + (size_t)ich * p.L;
    T2* tws = b + (size_t)ich * p.L;
    long long o = blockIdx.x / nchunk;
    // with a box mask: this plane's column flags (y pass: line element l = y),
    // unoccupied columns read as zero
    const uint8_t* cflag = nullptr;
    if (mk.xpl)
    {
        // blockIdx.x < 2^32: 32-bit divisions
        const unsigned o32 = (unsigned)o, nx = (unsigned)mk.Nx;
        const unsigned box = o32 / nx;
        const unsigned x = o32 - box * nx;
        const size_t kslot = box / (unsigned)mk.nbox_per_k;
        if (!mk.xpl[kslot * nx + x]) return;
        if (mk.col) cflag = mk.col + (kslot * nx + x) * (size_t)mk.Ny;
    }
    for (int t = threadIdx.x; t < p.L; t += blockDim.x) tws[t] = tw[t];
    if constexpr (NLC > 0)
    {
        // the block's CTL x NLC points are contiguous: idx = l * NLC + i
        T2* g = data + (size_t)o * (CTL * NLC);
        if constexpr (sizeof(T2) == 8 && (CTL * NLC) % 2 == 0)
        {
            // two points per 16-byte access (the block's start is even in points)
            for (int idx = threadIdx.x; idx < CTL * NLC / 2; idx += blockDim.x)
                reinterpret_cast<float4*>(a)[idx] = (cflag && !cflag[2 * idx / NLC])
                                                        ? make_float4(0.f, 0.f, 0.f, 0.f)
                                                        : reinterpret_cast<const float4*>(g)[idx];
            __syncthreads();
            T2* r = ct_fft<T2, T, CTL, 0, 1, true, NLC>(a, b, NLC, NLC, 1, nullptr, NLC, 1, tws, sign);
            for (int idx = threadIdx.x; idx < CTL * NLC / 2; idx += blockDim.x)
                reinterpret_cast<float4*>(g)[idx] = reinterpret_cast<const float4*>(r)[idx];
        }
        else
        {
            for (int idx = threadIdx.x; idx < CTL * NLC; idx += blockDim.x)
                a[idx] = (cflag && !cflag[idx / NLC]) ? T2{} : g[idx];
            __syncthreads();
            T2* r = ct_fft<T2, T, CTL, 0, 1, true, NLC>(a, b, NLC, NLC, 1, nullptr, NLC, 1, tws, sign);
            for (int idx = threadIdx.x; idx < CTL * NLC; idx += blockDim.x) g[idx] = r[idx];
        }
        return;
    }
    int c = blockIdx.x - (int)(o * nchunk);
    int i0 = c * ich;
    int ic = min(ich, inner - i0);
    T2* g = data + (size_t)o * p.L * inner + i0;
    int n = p.L * ic;
    const RecipDiv dc = recip_div(ic);
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x)
    {
        int i;
        const int l = div_rem(idx, dc, i);
        a[l * ic + i] = (cflag && !cflag[l]) ? T2{} : g[(size_t)l * inner + i];
    }
    __syncthreads();
    T2* r;
    if constexpr (CTL > 0)
        r = ct_fft<T2, T, CTL, 0, 1, true, 0>(a, b, ic, ic, 1, nullptr, ic, 1, tws, sign);
    else
        r = fft_smem<T2, T>(a, b, ic, ic, 1, p, tws, sign);
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x)
    {
        int i;
        const int l = div_rem(idx, dc, i);
        g[(size_t)l * inner + i] = r[l * ic + i];
    }
}

// x pass of the mixed form: boxes (nbox = nk*nspin*nb*nspinor) of FP32
// complex; result psi(r) * band_scale is split into (hi, lo) 16-bit floats and
// written to the operand layout
//   Bsplit[((kbz*nspin + s)*2 + hl)*(2*nbp) + row][2*kc + {0,1}],  kc = spinor*N + r
// row n < nbp holds (Re, Im) of band n, row nbp + n holds (-Im, Re).
template <int BF16>
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo)
{
    if (BF16)
    {
        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        float2 hf = __bfloat1622float2(h);
        __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
        hi = *reinterpret_cast<uint32_t*>(&h);
        lo = *reinterpret_cast<uint32_t*>(&l);
    }
    else
    {
        __half2 h = __floats2half2_rn(a, b);
        float2 hf = __half22float2(h);
        __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
        hi = *reinterpret_cast<uint32_t*>(&h);
        lo = *reinterpret_cast<uint32_t*>(&l);
    }
}

// NLC > 0 (with CTL > 0): every chunk holds exactly NLC columns (the host
// checks that they tile the plane), so the line count, and with it every
// index division of the load and of the passes, is a compile-time constant.
template <int BF16, int CTL, int NLC>
__global__ void __launch_bounds__(256) k_fft_x_split(const float2* __restrict__ boxes, int nbox, int k0, int ich,
                                                     int nchunk, FftPlan1D p, const float2* __restrict__ tw,
                                                     int sign, GeomDev gd, const float* __restrict__ band_scale,
                                                     uint16_t* __restrict__ Bsplit, float2* __restrict__ psi32,
                                                     BoxMask mk)
{
    static_assert(NLC == 0 || CTL > 0, "a compile-time line count needs a compile-time length");
    extern __shared__ __align__(16) unsigned char smraw[];
    float2* a = reinterpret_cast<float2*>(smraw);
    float2* b = a + (size_t)ich * p.L;
    float2* tws = b + (size_t)ich * p.L;
    for (int t = threadIdx.x; t < p.L; t += blockDim.x) tws[t] = tw[t];
    const int inner = gd.Ny * gd.Nz;
    const long long N = (long long)gd.Nx * inner;
    int o = blockIdx.x / nchunk;
    int c = blockIdx.x - o * nchunk;
    int i0 = c * ich;
    const int ic = NLC > 0 ? NLC : min(ich, inner - i0);
    const float2* g = boxes + (size_t)o * N + i0;
    int n = p.L * ic;
    // x planes that the sphere of this k-point does not reach are zero: not read
    const uint8_t* xpl = mk.xpl ? mk.xpl + (size_t)(o / mk.nbox_per_k) * gd.Nx : nullptr;
    if constexpr (NLC > 0)
    {
        // two adjacent columns per thread (one 16-byte load: the box, the chunk
        // start, the plane stride and the column pair are all even in points),
        // rows stepping by the rows a block covers
        static_assert(NLC % 2 == 0, "column pairs");
        constexpr int NP = NLC / 2, RP = 256 / NP;
        const int ip = threadIdx.x % NP, l0 = threadIdx.x / NP;
        if (l0 < RP)
        {
            const float2* gi = g + 2 * ip;
#pragma unroll 4
            for (int l = l0; l < CTL; l += RP)
                *reinterpret_cast<float4*>(a + l * NLC + 2 * ip) =
                    (xpl && !xpl[l]) ? make_float4(0.f, 0.f, 0.f, 0.f)
                                     : *reinterpret_cast<const float4*>(gi + (size_t)l * inner);
        }
    }
    else
    {
        const RecipDiv dc = recip_div(ic);
        for (int idx = threadIdx.x; idx < n; idx += blockDim.x)
        {
            int i;
            const int l = div_rem(idx, dc, i);
            a[l * ic + i] = (xpl && !xpl[l]) ? make_float2(0.f, 0.f) : g[(size_t)l * inner + i];
        }
    }
    __syncthreads();
    float2* r;
    if constexpr (CTL > 0)
        r = ct_fft<float2, float, CTL, 0, 1, true, NLC>(a, b, ic, ic, 1, nullptr, ic, 1, tws, sign);
    else
        r = fft_smem<float2, float>(a, b, ic, ic, 1, p, tws, sign);
    // box o -> (kslot, spin, band, spinor)
    int sp = o % gd.nspinor;
    int t = o / gd.nspinor;
    int band = t % gd.nbnds;
    t /= gd.nbnds;
    int spin = t % gd.nspin;
    int kslot = t / gd.nspin;
    int kbz = k0 + kslot;
    float sc = band_scale[((size_t)kbz * gd.nspin + spin) * gd.nbnds + band];
    // tile-major operands: one 32-point K block of all rows of a (k, spin, hi|lo)
    // group is contiguous (NT rows x 128 B), as is one 16-point block of the
    // FP32 rows of a (k, spin) (nbp rows x 128 B)
    const int NT = 2 * gd.nbp;
    const size_t nkb = (size_t)gd.nspinor * N / 32;
    const size_t npb = (size_t)gd.nspinor * N / 16;
    const size_t rg_hi = (size_t)(kbz * gd.nspin + spin) * 2;
    const size_t pg = (size_t)(kbz * gd.nspin + spin);
    // 64-bit bases of this box's rows; per element only 32-bit offsets: row
    // `band` (and nbp + band) of K block kb sits at kb*NT*32 + row*32 words
    uint32_t* const Bhi = reinterpret_cast<uint32_t*>(Bsplit) + rg_hi * nkb * NT * 32 + (size_t)band * 32;
    uint32_t* const Blo = Bhi + nkb * NT * 32;
    const uint32_t rot = (uint32_t)gd.nbp * 32;  // (-Im, Re) rows
    float2* const P = psi32 + pg * npb * gd.nbp * 16 + (size_t)band * 16;
    const uint32_t kbase = (uint32_t)((long long)sp * N) + (uint32_t)i0;  // K index of (x = 0, column 0)
    if constexpr (NLC > 0)
    {
        // two adjacent points per thread: kc is even, so both sit in one
        // 32-point K block (8-byte stores of the split rows) and one 16-point
        // psi block (a 16-byte store)
        constexpr int NP = NLC / 2, RP = 256 / NP;
        const int ip = threadIdx.x % NP, lr = threadIdx.x / NP;
        if (lr < RP)
        {
            for (int l = lr; l < CTL; l += RP)
            {
                const float4 w = *reinterpret_cast<const float4*>(r + l * NLC + 2 * ip);
                const float2 v0 = make_float2(w.x * sc, w.y * sc), v1 = make_float2(w.z * sc, w.w * sc);
                const uint32_t kc = kbase + (uint32_t)(l * inner + 2 * ip);
                uint32_t h0a, l0a, h1a, l1a, h0b, l0b, h1b, l1b;
                split2<BF16>(v0.x, v0.y, h0a, l0a);
                split2<BF16>(-v0.y, v0.x, h1a, l1a);
                split2<BF16>(v1.x, v1.y, h0b, l0b);
                split2<BF16>(-v1.y, v1.x, h1b, l1b);
                const uint32_t off = (kc >> 5) * (uint32_t)NT * 32u + (kc & 31u);
                *reinterpret_cast<uint2*>(Bhi + off) = make_uint2(h0a, h0b);
                *reinterpret_cast<uint2*>(Blo + off) = make_uint2(l0a, l0b);
                *reinterpret_cast<uint2*>(Bhi + off + rot) = make_uint2(h1a, h1b);
                *reinterpret_cast<uint2*>(Blo + off + rot) = make_uint2(l1a, l1b);
                *reinterpret_cast<float4*>(P + (kc >> 4) * (uint32_t)gd.nbp * 16u + (kc & 15u)) =
                    make_float4(v0.x, v0.y, v1.x, v1.y);
            }
        }
        return;
    }
    // one column per thread, rows (x) stepping by the columns a block covers
    const int rows_per = (int)blockDim.x / ic;
    const int i = threadIdx.x % ic;
    if (rows_per > 0 && threadIdx.x < rows_per * ic)
    {
        for (int l = threadIdx.x / ic; l < p.L; l += rows_per)
        {
            float2 v = r[l * ic + i];
            v.x *= sc;
            v.y *= sc;
            const uint32_t kc = kbase + (uint32_t)(l * inner + i);
            uint32_t h0, l0, h1, l1;
            split2<BF16>(v.x, v.y, h0, l0);
            split2<BF16>(-v.y, v.x, h1, l1);
            const uint32_t off = (kc >> 5) * (uint32_t)NT * 32u + (kc & 31u);
            Bhi[off] = h0;
            Blo[off] = l0;
            Bhi[off + rot] = h1;
            Blo[off + rot] = l1;
            // FP32 copy of the scaled psi(r) (rows (kbz, spin, band))
            P[(kc >> 4) * (uint32_t)gd.nbp * 16u + (kc & 15u)] = v;
        }
    }
    else
    {
        for (int idx = threadIdx.x; idx < n; idx += blockDim.x)
        {
            const int l = idx / ic, ii = idx - l * ic;
            float2 v = r[l * ic + ii];
            v.x *= sc;
            v.y *= sc;
            const uint32_t kc = kbase + (uint32_t)(l * inner + ii);
            uint32_t h0, l0, h1, l1;
            split2<BF16>(v.x, v.y, h0, l0);
            split2<BF16>(-v.y, v.x, h1, l1);
            const uint32_t off = (kc >> 5) * (uint32_t)NT * 32u + (kc & 31u);
            Bhi[off] = h0;
            Blo[off] = l0;
            Bhi[off + rot] = h1;
            Blo[off + rot] = l1;
            P[(kc >> 4) * (uint32_t)gd.nbp * 16u + (kc & 15u)] = v;
        }
    }
}

// ------------------------------------------------------- column lists

// one block per k: the occupied z-columns of its box as a list (any order)
__global__ void __launch_bounds__(256) k_col_lists(const uint8_t* __restrict__ col, int ncol, int* __restrict__ list,
                                                   int* __restrict__ cnt)
{
    __shared__ int n;
    const int k = blockIdx.x;
    if (threadIdx.x == 0) n = 0;
    __syncthreads();
    const uint8_t* ck = col + (size_t)k * ncol;
    for (int c = threadIdx.x; c < ncol; c += blockDim.x)
        if (ck[c]) list[(size_t)k * ncol + atomicAdd(&n, 1)] = c;
    __syncthreads();
    if (threadIdx.x == 0) cnt[k] = n;
}

// one block per box of a chunk: zero the occupied columns of its k (each warp
// one column at a time, lanes along z; 16-byte stores when Nz is even)
__global__ void __launch_bounds__(256) k_clear_cols(float2* __restrict__ boxes, int nbox_per_k, long long N, int Nz,
                                                    int ncol, const int* __restrict__ list,
                                                    const int* __restrict__ cnt)
{
    const int box = blockIdx.x;
    const int kslot = box / nbox_per_k;
    const int n = cnt[kslot];
    const int* lk = list + (size_t)kslot * ncol;
    float2* b = boxes + (size_t)box * N;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if ((Nz & 1) == 0)
    {
        const int h = Nz >> 1;
        for (int j = warp; j < n; j += nw)
        {
            float4* c4 = reinterpret_cast<float4*>(b + (size_t)lk[j] * Nz);
            for (int z = lane; z < h; z += 32) c4[z] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    else
        for (int j = warp; j < n; j += nw)
        {
            float2* c2 = b + (size_t)lk[j] * Nz;
            for (int z = lane; z < Nz; z += 32) c2[z] = make_float2(0.f, 0.f);
        }
}

void lelph_launch_col_lists(const uint8_t* col, int nk, int ncol, int* list, int* cnt, cudaStream_t st)
{
    if (nk > 0) k_col_lists<<<nk, 256, 0, st>>>(col, ncol, list, cnt);
}

void lelph_launch_clear_cols(float2* boxes, int nk, int nbox_per_k, long long N, int Nz, int ncol, const int* list,
                             const int* cnt, cudaStream_t st)
{
    const long long nbox = (long long)nk * nbox_per_k;
    if (nbox > 0) k_clear_cols<<<(unsigned)nbox, 256, 0, st>>>(boxes, nbox_per_k, N, Nz, ncol, list, cnt);
}

// ------------------------------------------------------------- scatter

// grid: (ceil(npw_max / 256), nk); one thread per plane wave G of a k-point:
// the box index and the phase e^{-i 2 pi G.tau} depend only on (k, G), so
// they are formed once and applied to every (spin, band) set.
template <typename T2>
__global__ void __launch_bounds__(256) k_scatter(int k0, const KPointSym* __restrict__ ks,
                                                 const int* __restrict__ miller, const long long* __restrict__ pw_off,
                                                 const int* __restrict__ npw_arr, const double2* __restrict__ coef,
                                                 const long long* __restrict__ coef_off, GeomDev gd,
                                                 T2* __restrict__ boxes, double2* __restrict__ chat,
                                                 float2* __restrict__ chat32, const long long* __restrict__ chat_off,
                                                 BoxMask mk)
{
    const int kslot = blockIdx.y;
    const int kbz = k0 + kslot;
    const KPointSym s = ks[kbz];
    const int npw = npw_arr[s.ik];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= npw) return;
    const int* mil = miller + 3 * pw_off[s.ik];
    const long long N = (long long)gd.Nx * gd.Ny * gd.Nz;
    const int nsets = gd.nspin * gd.nbnds;
    const int n0 = mil[3 * g], n1 = mil[3 * g + 1], n2 = mil[3 * g + 2];
    const int G0 = s.W[0] * n0 + s.W[1] * n1 + s.W[2] * n2;
    const int G1 = s.W[3] * n0 + s.W[4] * n1 + s.W[5] * n2;
    const int G2 = s.W[6] * n0 + s.W[7] * n1 + s.W[8] * n2;
    // e^{-i 2 pi G.tau} (the reference: cexp(-I*2*ELPH_PI*dot)); then kphase * gphase
    const double dot = (double)G0 * s.tau_crys[0] + (double)G1 * s.tau_crys[1] + (double)G2 * s.tau_crys[2];
    double sn, cs;
    sincos(2.0 * LELPH_PI_T * dot, &sn, &cs);
    const double2 ph = cmul(make_double2(s.kphase[0], s.kphase[1]), make_double2(cs, -sn));
    int ix = G0 % gd.Nx;
    if (ix < 0) ix += gd.Nx;
    int iy = G1 % gd.Ny;
    if (iy < 0) iy += gd.Ny;
    int iz = G2 % gd.Nz;
    if (iz < 0) iz += gd.Nz;
    const size_t bidx = ((size_t)ix * gd.Ny + iy) * gd.Nz + iz;
    if (mk.col)
    {
        mk.col[((size_t)kslot * gd.Nx + ix) * gd.Ny + iy] = 1;
        mk.xpl[(size_t)kslot * gd.Nx + ix] = 1;
    }
    const double2 u0 = make_double2(s.su2[0], s.su2[1]), u1 = make_double2(s.su2[2], s.su2[3]);
    const double2 u2 = make_double2(s.su2[4], s.su2[5]), u3 = make_double2(s.su2[6], s.su2[7]);
    const double2* cbase = coef + coef_off[s.ik];
    // the unfolded coefficients in FP64, or in FP32 (chat32) for the tensor-core projections
    double2* chb = chat32 ? nullptr : chat + chat_off[kbz];
    float2* chb32 = chat32 ? chat32 + chat_off[kbz] : nullptr;
    T2* bxb = boxes ? boxes + (size_t)kslot * nsets * gd.nspinor * N : nullptr;
    for (int set = 0; set < nsets; ++set)
    {
        const double2* c = cbase + (size_t)set * gd.nspinor * npw;
        double2 v[2];
        if (gd.nspinor == 2)
        {
            const double2 up = c[g], dw = c[npw + g];
            v[0] = cadd(cmul(up, u0), cmul(dw, u1));
            v[1] = cadd(cmul(up, u2), cmul(dw, u3));
        }
        else
        {
            v[0] = c[g];
        }
        const size_t co = (size_t)set * gd.nspinor * npw;
        for (int sp = 0; sp < gd.nspinor; ++sp)
        {
            double2 w = cmul(v[sp], ph);
            if (s.trev) w.y = -w.y;
            if (chb32) chb32[co + (size_t)sp * npw + g] = make_float2((float)w.x, (float)w.y);
            else chb[co + (size_t)sp * npw + g] = w;
            if (bxb) bxb[((size_t)set * gd.nspinor + sp) * N + bidx] = mk2<T2>(w.x, w.y);
        }
    }
}

__global__ void k_gmap(const KPointSym* __restrict__ ks, int kbz, const int* __restrict__ miller,
                       const long long* __restrict__ pw_off, const int* __restrict__ npw_arr, GeomDev gd,
                       const int* __restrict__ ulm, int* __restrict__ out)
{
    const KPointSym s = ks[kbz];
    const int npw = npw_arr[s.ik];
    const int* mil = miller + 3 * pw_off[s.ik];
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < npw; g += gridDim.x * blockDim.x)
    {
        int n0 = mil[3 * g], n1 = mil[3 * g + 1], n2 = mil[3 * g + 2];
        int G0 = s.W[0] * n0 + s.W[1] * n1 + s.W[2] * n2 + ulm[0];
        int G1 = s.W[3] * n0 + s.W[4] * n1 + s.W[5] * n2 + ulm[1];
        int G2 = s.W[6] * n0 + s.W[7] * n1 + s.W[8] * n2 + ulm[2];
        out[3 * g] = G0;
        out[3 * g + 1] = G1;
        out[3 * g + 2] = G2;
    }
}

// ---------------------------------------------------------------- launchers

static int ich_for(int L, int inner, int elems)
{
    int ich = elems / L;
    ich = ich >= 32 ? (ich / 16) * 16 : (ich < 1 ? 1 : ich);
    if (ich > inner) ich = inner;
    return ich;
}

// Line lengths with a compile-time FFT instance (FP32 passes of the mixed form)
#define LELPH_CT_SIZES(X) X(24) X(36) X(48) X(60) X(64) X(72) X(96)

template <typename T2, typename T, int CTL>
static void launch_contig_l(T2* data, long long nlines, const FftPlan1D& p, const T2* tw, int sign, cudaStream_t st,
                            const BoxMask& mk)
{
    const int elems = sizeof(T) == 8 ? 2048 : 4096;
    int lpc = elems / p.L;
    if (lpc < 1) lpc = 1;
    size_t smem = (size_t)(2 * lpc * p.L + p.L) * sizeof(T2) + sizeof(int) * lpc;
    static bool attr_set = false;
    if (!attr_set)
    {
        cudaFuncSetAttribute(k_fft_contig<T2, T, CTL>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    long long nb = (nlines + lpc - 1) / lpc;
    k_fft_contig<T2, T, CTL><<<(unsigned)nb, 256, smem, st>>>(data, nlines, p, tw, sign, lpc, mk);
}

template <typename T2, typename T, int CTL>
static void launch_strided_l(T2* data, long long nouter, int inner, const FftPlan1D& p, const T2* tw, int sign,
                             cudaStream_t st, const BoxMask& mk)
{
    const int elems = sizeof(T) == 8 ? 2048 : 4096;
    int ich = ich_for(p.L, inner, elems);
    int nchunk = (inner + ich - 1) / ich;
    size_t smem = (size_t)(2 * ich * p.L + p.L) * sizeof(T2);
    static bool attr_set = false;
    if (!attr_set)
    {
        cudaFuncSetAttribute(k_fft_strided<T2, T, CTL, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    long long nb = nouter * nchunk;
    if (CTL > 0 && inner == CTL && ich == CTL)
    {
        // cubic planes (inner = L): a compile-time line count
        constexpr int NLC = CTL;
        static bool attr_n = false;
        if (!attr_n)
        {
            cudaFuncSetAttribute(k_fft_strided<T2, T, CTL, NLC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 200 * 1024);
            attr_n = true;
        }
        k_fft_strided<T2, T, CTL, NLC><<<(unsigned)nb, 256, smem, st>>>(data, nouter, inner, ich, nchunk, p, tw, sign,
                                                                        mk);
        return;
    }
    k_fft_strided<T2, T, CTL, 0><<<(unsigned)nb, 256, smem, st>>>(data, nouter, inner, ich, nchunk, p, tw, sign, mk);
}

template <typename T2, typename T>
static void launch_contig(T2* data, long long nlines, const FftPlan1D& p, const T2* tw, int sign, cudaStream_t st,
                          const BoxMask& mk)
{
    if constexpr (sizeof(T) == 4)
    {
        switch (p.L)
        {
#define LELPH_CT_CASE(N) \
    case N: launch_contig_l<T2, T, N>(data, nlines, p, tw, sign, st, mk); return;
            LELPH_CT_SIZES(LELPH_CT_CASE)
#undef LELPH_CT_CASE
        default: break;
        }
    }
    launch_contig_l<T2, T, 0>(data, nlines, p, tw, sign, st, mk);
}

template <typename T2, typename T>
static void launch_strided(T2* data, long long nouter, int inner, const FftPlan1D& p, const T2* tw, int sign,
                           cudaStream_t st, const BoxMask& mk)
{
    if constexpr (sizeof(T) == 4)
    {
        switch (p.L)
        {
#define LELPH_CT_CASE(N) \
    case N: launch_strided_l<T2, T, N>(data, nouter, inner, p, tw, sign, st, mk); return;
            LELPH_CT_SIZES(LELPH_CT_CASE)
#undef LELPH_CT_CASE
        default: break;
        }
    }
    launch_strided_l<T2, T, 0>(data, nouter, inner, p, tw, sign, st, mk);
}

void lelph_launch_fft_contig_d(double2* data, long long nlines, const FftPlan1D& p, const double2* tw, int sign,
                               cudaStream_t st)
{
    launch_contig<double2, double>(data, nlines, p, tw, sign, st, BoxMask());
}
void lelph_launch_fft_contig_f(float2* data, long long nlines, const FftPlan1D& p, const float2* tw, int sign,
                               cudaStream_t st, const BoxMask& mk)
{
    launch_contig<float2, float>(data, nlines, p, tw, sign, st, mk);
}
void lelph_launch_fft_strided_d(double2* data, long long nouter, int inner, const FftPlan1D& p, const double2* tw,
                                int sign, cudaStream_t st)
{
    launch_strided<double2, double>(data, nouter, inner, p, tw, sign, st, BoxMask());
}
void lelph_launch_fft_strided_f(float2* data, long long nouter, int inner, const FftPlan1D& p, const float2* tw,
                                int sign, cudaStream_t st, const BoxMask& mk)
{
    launch_strided<float2, float>(data, nouter, inner, p, tw, sign, st, mk);
}

// columns per x-pass block for a compile-time length: ich_for(L, ., 2048)
// before it is clipped to the plane
__host__ __device__ constexpr int x_split_nlc(int L)
{
    return (2048 / L) >= 32 ? (2048 / L) / 16 * 16 : (2048 / L);
}

template <int BF16, int CTL, int NLC>
static void launch_x_split_n(unsigned nb, size_t smem, const float2* boxes, int nbox, int k0, int ich, int nchunk,
                             const FftPlan1D& p, const float2* tw, int sign, const GeomDev& g,
                             const float* band_scale, uint16_t* Bsplit, float2* psi32, cudaStream_t st,
                             const BoxMask& mk)
{
    static bool attr_set = false;
    if (!attr_set)
    {
        cudaFuncSetAttribute(k_fft_x_split<BF16, CTL, NLC>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    k_fft_x_split<BF16, CTL, NLC><<<nb, 256, smem, st>>>(boxes, nbox, k0, ich, nchunk, p, tw, sign, g, band_scale,
                                                         Bsplit, psi32, mk);
}

template <int BF16, int CTL>
static void launch_x_split_l(unsigned nb, size_t smem, const float2* boxes, int nbox, int k0, int ich, int nchunk,
                             const FftPlan1D& p, const float2* tw, int sign, const GeomDev& g,
                             const float* band_scale, uint16_t* Bsplit, float2* psi32, cudaStream_t st,
                             const BoxMask& mk)
{
    // an even count: the compile-time form works on column pairs
    constexpr int NLC = (CTL > 0 && x_split_nlc(CTL) % 2 == 0) ? x_split_nlc(CTL) : 0;
    const int inner = g.Ny * g.Nz;
    if (NLC > 0 && ich == NLC && inner % NLC == 0 && 256 / NLC >= 1)
        launch_x_split_n<BF16, CTL, NLC>(nb, smem, boxes, nbox, k0, ich, nchunk, p, tw, sign, g, band_scale, Bsplit,
                                         psi32, st, mk);
    else
        launch_x_split_n<BF16, CTL, 0>(nb, smem, boxes, nbox, k0, ich, nchunk, p, tw, sign, g, band_scale, Bsplit,
                                       psi32, st, mk);
}

template <int BF16>
static void launch_x_split(unsigned nb, size_t smem, const float2* boxes, int nbox, int k0, int ich, int nchunk,
                           const FftPlan1D& p, const float2* tw, int sign, const GeomDev& g, const float* band_scale,
                           uint16_t* Bsplit, float2* psi32, cudaStream_t st, const BoxMask& mk)
{
    switch (p.L)
    {
#define LELPH_CT_CASE(N)                                                                                         \
    case N:                                                                                                      \
        launch_x_split_l<BF16, N>(nb, smem, boxes, nbox, k0, ich, nchunk, p, tw, sign, g, band_scale, Bsplit, psi32, \
                                  st, mk);                                                                       \
        return;
        LELPH_CT_SIZES(LELPH_CT_CASE)
#undef LELPH_CT_CASE
    default: break;
    }
    launch_x_split_l<BF16, 0>(nb, smem, boxes, nbox, k0, ich, nchunk, p, tw, sign, g, band_scale, Bsplit, psi32, st,
                              mk);
}

void lelph_launch_fft_x_to_split(const float2* boxes, int nbox_k, int k0, const FftPlan1D& p, const float2* tw,
                                 int sign, const GeomDev& g, const float* band_scale, int ab_bf16, uint16_t* Bsplit,
                                 float2* psi32, cudaStream_t st, const BoxMask& mk)
{
    const int inner = g.Ny * g.Nz;
    // 2048 elements a block (half the other passes' chunk): more blocks per SM to
    // overlap one block's loads with another's transform and stores (measured
    // 5.7 -> 5.4 ms per bench step; 1024 is slower again)
    int ich = ich_for(p.L, inner, 2048);
    int nchunk = (inner + ich - 1) / ich;
    size_t smem = (size_t)(2 * ich * p.L + p.L) * sizeof(float2);
    long long nbox = (long long)nbox_k * g.nspin * g.nbnds * g.nspinor;
    unsigned nb = (unsigned)(nbox * nchunk);
    if (ab_bf16)
        launch_x_split<1>(nb, smem, boxes, (int)nbox, k0, ich, nchunk, p, tw, sign, g, band_scale, Bsplit, psi32, st,
                          mk);
    else
        launch_x_split<0>(nb, smem, boxes, (int)nbox, k0, ich, nchunk, p, tw, sign, g, band_scale, Bsplit, psi32, st,
                          mk);
}

void lelph_launch_scatter(int k0, int nk, const KPointSym* ksym_dev, const int* miller, const long long* pw_off,
                          const int* npw, int npw_max, const double2* coef, const long long* coef_off,
                          const GeomDev& g, int box_fp64, void* boxes, double2* chat, const long long* chat_off,
                          cudaStream_t st, const BoxMask& mk, float2* chat32)
{
    dim3 grid((unsigned)((npw_max + 255) / 256), nk);
    if (box_fp64)
        k_scatter<double2><<<grid, 256, 0, st>>>(k0, ksym_dev, miller, pw_off, npw, coef, coef_off, g,
                                                 (double2*)boxes, chat, chat32, chat_off, mk);
    else
        k_scatter<float2><<<grid, 256, 0, st>>>(k0, ksym_dev, miller, pw_off, npw, coef, coef_off, g,
                                                (float2*)boxes, chat, chat32, chat_off, mk);
}

void lelph_launch_gmap(const KPointSym* ks, int kbz, const int* miller, const long long* pw_off, const int* npw,
                       const GeomDev& g, const int* ulm, int* out, cudaStream_t st)
{
    k_gmap<<<16, 256, 0, st>>>(ks, kbz, miller, pw_off, npw, g, ulm, out);
}
