// q-star expansion of the matrix elements: the star loop of
// compute_and_write_elphq (src/elph/compute_elph_matq.c:159-217) with
// elph_q_rotate (src/symmetries/elphq_expand.c:16-73).  For a star member
// S q and a full-BZ k,
//   g(Sq, Sk)[i'][f'] = sum_{i,f} conj(Dr[i'][i]) g~(q,k)[i][f] Dl[f'][f],
// Dl = D[S][k+q], Dr = D[S][k], g~ = conj(g) for a time-reversed S, stored
// at S k.  One CTA per (star member, k, spin): Dl^T and Dr staged in shared
// memory once, then per mode the two nb x nb x nb products through shared
// memory (broadcast rows, consecutive columns: conflict-free).  Compute type
// C2 (FP64 in the plain form, FP32 in the mixed form), element type IO2 of
// the matrix elements in and out.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"

template <typename A, typename B> __device__ __forceinline__ A qs_cvt(B v) { return mk2<A>((double)v.x, (double)v.y); }

template <typename C2> __device__ __forceinline__ void qs_cfma(C2& acc, C2 a, C2 b)
{
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}

template <typename C2, typename IO2>
__global__ void __launch_bounds__(256) k_qstar(const QStarItem* __restrict__ items, int nb, int nspin, int nmodes,
                                               const double2* __restrict__ D, const IO2* __restrict__ g,
                                               IO2* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char qs_smem[];
    const int nn = nb * nb;
    C2* sDlT = reinterpret_cast<C2*>(qs_smem);
    C2* sDr = sDlT + nn;
    C2* sG = sDr + nn;
    C2* sT = sG + nn;
    const QStarItem it = items[blockIdx.x];
    const int spin = blockIdx.y;
    const int t = threadIdx.x;
    const double2* Dl = D + ((long long)it.dl * nspin + spin) * nn;
    const double2* Dr = D + ((long long)it.dr * nspin + spin) * nn;
    for (int e = t; e < nn; e += blockDim.x)
    {
        const int r = e / nb, c = e - r * nb;
        sDlT[c * nb + r] = qs_cvt<C2>(Dl[e]);
        sDr[e] = qs_cvt<C2>(Dr[e]);
    }
    const long long gsz = (long long)nmodes * nspin * nn;
    for (int mode = 0; mode < nmodes; ++mode)
    {
        const IO2* G = g + (long long)it.src * gsz + ((long long)mode * nspin + spin) * nn;
        __syncthreads();  // the previous mode's products are done with sG and sT
        for (int e = t; e < nn; e += blockDim.x)
        {
            C2 v = qs_cvt<C2>(G[e]);
            if (it.trev) v = cconj(v);
            sG[e] = v;
        }
        __syncthreads();
        // T = g~ Dl^T
        for (int e = t; e < nn; e += blockDim.x)
        {
            const int i = e / nb, fp = e - i * nb;
            C2 acc = mk2<C2>(0.0, 0.0);
            for (int f = 0; f < nb; ++f) qs_cfma(acc, sG[i * nb + f], sDlT[f * nb + fp]);
            sT[e] = acc;
        }
        __syncthreads();
        // out = conj(Dr) T
        IO2* O = out + (long long)it.dst * gsz + ((long long)mode * nspin + spin) * nn;
        for (int e = t; e < nn; e += blockDim.x)
        {
            const int ip = e / nb, fp = e - ip * nb;
            C2 acc = mk2<C2>(0.0, 0.0);
            for (int i = 0; i < nb; ++i) qs_cfma(acc, cconj(sDr[ip * nb + i]), sT[i * nb + fp]);
            O[e] = qs_cvt<IO2>(acc);
        }
    }
}

size_t lelph_qstar_smem_bytes(int nb, int fp64)
{
    return 4 * (size_t)nb * nb * (fp64 ? sizeof(double2) : sizeof(float2));
}

template <typename C2, typename IO2>
static int launch_qs(const QStarItem* items, long long nitems, int nb, int nspin, int nmodes, const double2* D,
                     const void* g, void* out, cudaStream_t st)
{
    const size_t smem = lelph_qstar_smem_bytes(nb, sizeof(C2) == sizeof(double2));
    if (cudaFuncSetAttribute(k_qstar<C2, IO2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    dim3 grid((unsigned)nitems, (unsigned)nspin);
    k_qstar<C2, IO2><<<grid, 256, smem, st>>>(items, nb, nspin, nmodes, D, (const IO2*)g, (IO2*)out);
    return 0;
}

int lelph_launch_qstar(const QStarItem* items, long long nitems, int nb, int nspin, int nmodes, const double2* D,
                       int fp64, int out_c64, const void* g, void* out, cudaStream_t st)
{
    if (nitems <= 0) return 0;
    if (nitems > 0x7fffffffLL || lelph_qstar_smem_bytes(nb, fp64) > 220 * 1024) return -1;
    if (fp64)
        return out_c64 ? launch_qs<double2, float2>(items, nitems, nb, nspin, nmodes, D, g, out, st)
                       : launch_qs<double2, double2>(items, nitems, nb, nspin, nmodes, D, g, out, st);
    return out_c64 ? launch_qs<float2, float2>(items, nitems, nb, nspin, nmodes, D, g, out, st)
                   : launch_qs<float2, double2>(items, nitems, nb, nspin, nmodes, D, g, out, st);
}
