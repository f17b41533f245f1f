// dV_scf ingest (read_dvscf_qe, src/io/qe/read_dvscf.c:15-172, after the file
// read): QE's dvscf holds (pattern, nmag, Nz, Ny, Nx) complex doubles in the
// pattern basis; the stage wants (mode, nmag, Nx, Ny, Nz) in the mode basis,
//   dV_nu = sum_p (eig pats^H)[nu][p] dV_p.
// One CTA per (16 x-points, y, 8 z-points, nmag component): every pattern's
// 16 x 8 tile is read along x (the file's fast axis) into shared memory, and
// each thread then forms all modes of one (x, z) point and writes them along
// z (the stage's fast axis).  FP64, HBM-bound: one read and one write of the
// array.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"

#define DVI_TX 16
#define DVI_TZ 8
#define DVI_THREADS (DVI_TX * DVI_TZ)

__global__ void __launch_bounds__(DVI_THREADS) k_dvscf_ingest(const double2* __restrict__ raw,
                                                              const double2* __restrict__ M, int nmodes, int nmag,
                                                              int Nx, int Ny, int Nz, double2* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char dvi_smem[];
    double2* sM = reinterpret_cast<double2*>(dvi_smem);     // nmodes x nmodes
    double2* tile = sM + nmodes * nmodes;                     // [pattern][z][x], x padded to 17
    const int t = threadIdx.x;
    const int x0 = blockIdx.x * DVI_TX, y = blockIdx.y;
    const int nzt = (Nz + DVI_TZ - 1) / DVI_TZ;
    const int z0 = (blockIdx.z % nzt) * DVI_TZ, m = blockIdx.z / nzt;
    const long long N = (long long)Nx * Ny * Nz;
    for (int e = t; e < nmodes * nmodes; e += DVI_THREADS) sM[e] = M[e];
    {
        const int xx = t % DVI_TX, zz = t / DVI_TX;
        const int x = x0 + xx, z = z0 + zz;
        const bool in = x < Nx && z < Nz;
        for (int p = 0; p < nmodes; ++p)
        {
            const long long src = ((long long)p * nmag + m) * N + ((long long)z * Ny + y) * Nx + x;
            tile[(p * DVI_TZ + zz) * (DVI_TX + 1) + xx] = in ? raw[src] : make_double2(0.0, 0.0);
        }
    }
    __syncthreads();
    const int zz = t % DVI_TZ, xx = t / DVI_TZ;
    const int x = x0 + xx, z = z0 + zz;
    if (x >= Nx || z >= Nz) return;
    for (int v = 0; v < nmodes; ++v)
    {
        double2 acc = make_double2(0.0, 0.0);
        for (int p = 0; p < nmodes; ++p)
        {
            const double2 a = sM[v * nmodes + p], b = tile[(p * DVI_TZ + zz) * (DVI_TX + 1) + xx];
            acc.x = fma(a.x, b.x, acc.x);
            acc.x = fma(-a.y, b.y, acc.x);
            acc.y = fma(a.x, b.y, acc.y);
            acc.y = fma(a.y, b.x, acc.y);
        }
        out[((long long)v * nmag + m) * N + ((long long)x * Ny + y) * Nz + z] = acc;
    }
}

int lelph_launch_dvscf_ingest(const double2* raw, const double2* M, int nmodes, int nmag, int Nx, int Ny, int Nz,
                              double2* out, cudaStream_t st)
{
    const size_t smem = sizeof(double2) * ((size_t)nmodes * nmodes + (size_t)nmodes * DVI_TZ * (DVI_TX + 1));
    if (smem > 200 * 1024 || Ny > 65535) return -1;
    if (cudaFuncSetAttribute(k_dvscf_ingest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    const int nzt = (Nz + DVI_TZ - 1) / DVI_TZ;
    dim3 grid((unsigned)((Nx + DVI_TX - 1) / DVI_TX), (unsigned)Ny, (unsigned)(nzt * nmag));
    k_dvscf_ingest<<<grid, DVI_THREADS, smem, st>>>(raw, M, nmodes, nmag, Nx, Ny, Nz, out);
    return 0;
}
