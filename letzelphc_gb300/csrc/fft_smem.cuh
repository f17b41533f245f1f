// Shared-memory FFT building blocks: radix-2/3/4/5 butterflies, exact
// division through an FP32 reciprocal, one Stockham pass over lines held in
// shared memory and the driver running every pass of a plan.  Used by the
// batched box FFTs (fft_gather.cu) and the G-space route (gspace.cu).
#pragma once
#include <cuda_runtime.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"

// ------------------------------------------------------------- butterflies

// The direction sign is a run-time +-1: it selects between constants and
// negations rather than multiplying (an int or double product would put a
// conversion or an FP64 multiply on GB300's slow FP64 pipe in every butterfly).
template <typename T2>
__device__ __forceinline__ T2 mul_i(T2 a, int sign)  // multiply by sign * i
{
    T2 r;
    if (sign > 0)
    {
        r.x = -a.y;
        r.y = a.x;
    }
    else
    {
        r.x = a.y;
        r.y = -a.x;
    }
    return r;
}

template <typename T2, typename T>
__device__ __forceinline__ void dft2(T2* v)
{
    T2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <typename T2, typename T>
__device__ __forceinline__ void dft4(T2* v, int sign)
{
    T2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    T2 s13 = cadd(v[1], v[3]), d13 = mul_i(csub(v[1], v[3]), sign);
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
}

template <typename T2, typename T>
__device__ __forceinline__ void dft3(T2* v, int sign)
{
    const T c = (T)-0.5;
    const T s = sign > 0 ? (T)0.86602540378443864676 : (T)-0.86602540378443864676;  // sign sin(2 pi / 3)
    T2 a = cadd(v[1], v[2]);
    T2 d = csub(v[1], v[2]);
    T2 t1;
    t1.x = v[0].x + c * a.x;
    t1.y = v[0].y + c * a.y;
    T2 t2;  // i s d
    t2.x = -s * d.y;
    t2.y = s * d.x;
    v[0] = cadd(v[0], a);
    v[1] = cadd(t1, t2);
    v[2] = csub(t1, t2);
}

template <typename T2, typename T>
__device__ __forceinline__ void dft5(T2* v, int sign)
{
    const T c1 = (T)0.30901699437494742410;   // cos(2 pi / 5)
    const T c2 = (T)-0.80901699437494742410;  // cos(4 pi / 5)
    const T s1 = sign > 0 ? (T)0.95105651629515357212 : (T)-0.95105651629515357212;  // sign sin(2 pi / 5)
    const T s2 = sign > 0 ? (T)0.58778525229247312917 : (T)-0.58778525229247312917;  // sign sin(4 pi / 5)
    T2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    T2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    T2 x0 = v[0];
    T2 r1, r2, i1, i2;
    r1.x = x0.x + c1 * a1.x + c2 * a2.x;
    r1.y = x0.y + c1 * a1.y + c2 * a2.y;
    r2.x = x0.x + c2 * a1.x + c1 * a2.x;
    r2.y = x0.y + c2 * a1.y + c1 * a2.y;
    // i (s1 b1 + s2 b2) and i (s2 b1 - s1 b2)
    T2 u, w;
    u.x = s1 * b1.x + s2 * b2.x;
    u.y = s1 * b1.y + s2 * b2.y;
    w.x = s2 * b1.x - s1 * b2.x;
    w.y = s2 * b1.y - s1 * b2.y;
    i1.x = -u.y;
    i1.y = u.x;
    i2.x = -w.y;
    i2.y = w.x;
    v[0] = cadd(x0, cadd(a1, a2));
    v[1] = cadd(r1, i1);
    v[4] = csub(r1, i1);
    v[2] = cadd(r2, i2);
    v[3] = csub(r2, i2);
}

// One Stockham pass of radix R over nlines lines held in shared memory;
// element e of line l lives at buf[l*ls + e*es].  Consecutive threads take
// consecutive elements of a line when elements are contiguous (es == 1) and
// consecutive lines otherwise (ls == 1), so that a warp's shared-memory
// accesses fall into distinct banks either way.
// Division by a run-time divisor d through its FP32 reciprocal: q = trunc(x/d)
// is at most one off for 0 <= x < 2^24 and is corrected from the remainder
// (the index arithmetic of the passes stays far below that bound).
struct RecipDiv
{
    float inv;
    int d;
};
__device__ __forceinline__ RecipDiv recip_div(int d) { return RecipDiv{__frcp_rn((float)d), d}; }
__device__ __forceinline__ int div_rem(int x, const RecipDiv& f, int& r)
{
    int q = __float2int_rz((float)x * f.inv);
    r = x - q * f.d;
    if (r < 0)
    {
        --q;
        r += f.d;
    }
    else if (r >= f.d)
    {
        ++q;
        r -= f.d;
    }
    return q;
}

template <typename T2, typename T, int R>
__device__ __forceinline__ void stockham_pass(const T2* __restrict__ src, T2* __restrict__ dst, int nlines, int L,
                                              int Ns, int es, int ls, const T2* tw, int sign)
{
    const int LR = L / R;
    const int nwork = nlines * LR;
    const int tstride = L / (Ns * R);
    const bool line_fast = es != 1;
    const RecipDiv dl = recip_div(line_fast ? nlines : LR), dn = recip_div(Ns);
    for (int w = threadIdx.x; w < nwork; w += blockDim.x)
    {
        int line, j;
        if (line_fast)
            j = div_rem(w, dl, line);
        else
            line = div_rem(w, dl, j);
        int k;
        const int jq = div_rem(j, dn, k);
        const T2* s = src + (size_t)line * ls;
        T2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = s[(size_t)(j + r * LR) * es];
        if (k != 0)
        {
#pragma unroll
            for (int r = 1; r < R; ++r)
            {
                T2 t = tw[r * k * tstride];
                if (sign < 0) t.y = -t.y;
                v[r] = cmul(v[r], t);
            }
        }
        if (R == 2) dft2<T2, T>(v);
        if (R == 3) dft3<T2, T>(v, sign);
        if (R == 4) dft4<T2, T>(v, sign);
        if (R == 5) dft5<T2, T>(v, sign);
        T2* d = dst + (size_t)line * ls;
        int base = jq * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) d[(size_t)(base + r * Ns) * es] = v[r];
    }
}

// Runs all passes; returns the buffer holding the result.
template <typename T2, typename T>
__device__ T2* fft_smem(T2* a, T2* b, int nlines, int es, int ls, const FftPlan1D& p, const T2* tw, int sign)
{
    int Ns = 1;
    for (int st = 0; st < p.nstage; ++st)
    {
        int R = p.radix[st];
        if (R == 4) stockham_pass<T2, T, 4>(a, b, nlines, p.L, Ns, es, ls, tw, sign);
        else if (R == 2) stockham_pass<T2, T, 2>(a, b, nlines, p.L, Ns, es, ls, tw, sign);
        else if (R == 3) stockham_pass<T2, T, 3>(a, b, nlines, p.L, Ns, es, ls, tw, sign);
        else stockham_pass<T2, T, 5>(a, b, nlines, p.L, Ns, es, ls, tw, sign);
        __syncthreads();
        T2* t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// ---------------------------------------------- compile-time line length
// Stockham FFT of lines whose length L is a compile-time constant: the radix
// schedule and the divisions of the index arithmetic are constants; each
// pass takes the largest radix up to 16 that divides what is left (two
// passes for the common grid sizes: 36 = 12 x 3, 48 = 16 x 3, 60 = 15 x 4,
// ...), composite radices being done in registers as two levels of
// radix-2/3/4/5 butterflies.
__host__ __device__ constexpr int ct_radix0(int L)
{
    return L % 16 == 0 ? 16 : L % 15 == 0 ? 15 : L % 12 == 0 ? 12 : L % 10 == 0 ? 10 : L % 9 == 0 ? 9
         : L % 8 == 0 ? 8 : L % 6 == 0 ? 6 : L % 5 == 0 ? 5 : L % 4 == 0 ? 4 : L % 3 == 0 ? 3 : 2;
}
__host__ __device__ constexpr int ct_nstage(int L) { return L <= 1 ? 0 : 1 + ct_nstage(L / ct_radix0(L)); }
__host__ __device__ constexpr int ct_radix_at(int L, int i) { return i == 0 ? ct_radix0(L) : ct_radix_at(L / ct_radix0(L), i - 1); }
__host__ __device__ constexpr bool ct_smooth(int L) { return L == 1 || ((L % 2 == 0 || L % 3 == 0 || L % 5 == 0) && ct_smooth(L / ct_radix0(L))); }
// first factor of a composite radix (the second is a radix-2/3/4/5)
__host__ __device__ constexpr int ct_split(int R) { return R == 16 ? 4 : R == 15 ? 3 : R == 12 ? 4 : R == 10 ? 2 : R == 9 ? 3 : R == 8 ? 4 : R == 6 ? 2 : R; }

template <typename T2, typename T, int R>
__device__ __forceinline__ void dft_base(T2* v, int sign)
{
    if constexpr (R == 2) dft2<T2, T>(v);
    if constexpr (R == 3) dft3<T2, T>(v, sign);
    if constexpr (R == 4) dft4<T2, T>(v, sign);
    if constexpr (R == 5) dft5<T2, T>(v, sign);
}

// DFT of R = R1 R2 points in registers: R2 DFTs of R1 points over the
// stride-R2 subsets, twiddles w_R^(n2 k1) (w_R^m = tw[m L / R], tw holding
// e^{+2 pi i t / L}), then R1 DFTs of R2 points; X[k1 + R1 k2].
template <typename T2, typename T, int R, int L>
__device__ __forceinline__ void dft_ct(T2* v, int sign, const T2* __restrict__ tw)
{
    constexpr int R1 = ct_split(R);
    if constexpr (R1 == R)
        dft_base<T2, T, R>(v, sign);
    else
    {
        constexpr int R2 = R / R1;
        T2 t[R];
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2)
        {
            T2 u[R1];
#pragma unroll
            for (int n1 = 0; n1 < R1; ++n1) u[n1] = v[R2 * n1 + n2];
            dft_base<T2, T, R1>(u, sign);
#pragma unroll
            for (int k1 = 0; k1 < R1; ++k1)
            {
                T2 x = u[k1];
                if (n2 * k1 != 0)
                {
                    T2 w = tw[n2 * k1 * (L / R)];
                    if (sign < 0) w.y = -w.y;
                    x = cmul(x, w);
                }
                t[n2 * R1 + k1] = x;
            }
        }
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1)
        {
            T2 w2[R2];
#pragma unroll
            for (int n2 = 0; n2 < R2; ++n2) w2[n2] = t[n2 * R1 + k1];
            dft_base<T2, T, R2>(w2, sign);
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) v[k1 + R1 * k2] = w2[k2];
        }
    }
}

// One Stockham pass of radix R (stage with NS = product of earlier radices).
// Element e of source line l sits at src[(loff ? loff[l] : l*ls_s) + e*es_s],
// of destination line l at dst[l*ls_d + e*es_d].  LINE_FAST: consecutive
// threads take consecutive lines (lines interleaved in memory), else
// consecutive elements of a line.
template <typename T2, typename T, int L, int R, int NS, bool LINE_FAST, int NLC>
__device__ __forceinline__ void ct_pass(const T2* __restrict__ src, T2* __restrict__ dst, int nlines, int es_s,
                                        int ls_s, const int* __restrict__ loff, int es_d, int ls_d,
                                        const T2* __restrict__ tw, int sign)
{
    constexpr int LR = L / R;
    constexpr int TS = L / (NS * R);
    if (NLC > 0) nlines = NLC;
    const int nwork = nlines * LR;
    const RecipDiv dl = recip_div(LINE_FAST && NLC == 0 ? nlines : 1);
    for (int w = threadIdx.x; w < nwork; w += blockDim.x)
    {
        int line, j;
        if constexpr (LINE_FAST && NLC > 0)
        {
            j = w / NLC;
            line = w - j * NLC;
        }
        else if constexpr (LINE_FAST)
            j = div_rem(w, dl, line);
        else
        {
            line = w / LR;
            j = w - line * LR;
        }
        const int k = j % NS, jq = j / NS;
        const T2* sp = src + (loff ? loff[line] : line * ls_s);
        T2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = sp[(j + r * LR) * es_s];
        if (NS > 1 && k != 0)
        {
#pragma unroll
            for (int r = 1; r < R; ++r)
            {
                T2 t = tw[r * k * TS];
                if (sign < 0) t.y = -t.y;
                v[r] = cmul(v[r], t);
            }
        }
        dft_ct<T2, T, R, L>(v, sign, tw);
        T2* dp = dst + line * ls_d;
        const int base = jq * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dp[(base + r * NS) * es_d] = v[r];
    }
}

// All passes; the first reads the source layout, the rest the destination
// layout.  Returns the buffer holding the result.
template <typename T2, typename T, int L, int STAGE, int NS, bool LINE_FAST, int NLC>
__device__ __forceinline__ T2* ct_fft(T2* a, T2* b, int nlines, int es_s, int ls_s, const int* loff, int es, int ls,
                                      const T2* tw, int sign)
{
    if constexpr (STAGE == ct_nstage(L))
        return a;
    else
    {
        constexpr int R = ct_radix_at(L, STAGE);
        ct_pass<T2, T, L, R, NS, LINE_FAST, NLC>(a, b, nlines, es_s, ls_s, loff, es, ls, tw, sign);
        __syncthreads();
        return ct_fft<T2, T, L, STAGE + 1, NS * R, LINE_FAST, NLC>(b, a, nlines, es, ls, nullptr, es, ls, tw, sign);
    }
}
