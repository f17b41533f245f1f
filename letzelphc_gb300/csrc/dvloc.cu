// Local bare potential per q: the change of the local pseudopotential under
// the phonon modes, added to the induced dV_scf before the sandwich (the
// reference does this in elph_driver ahead of compute_and_write_elphq,
// src/elph/elph_driver.c:234-252).
//
// * k_vloc_table: V_loc(|G|) on a uniform |G| grid per species, the radial
//   integral 4 pi / V int (sin(G r)/G) (r V_loc(r) + e2 Z erf(r)) dr by the
//   reference's Simpson weights (create_vlocg_table / Vloc_Gspace,
//   src/dvloc/vlocg_table.c:16-154, src/dvloc/VlocG_atom.c:10-57).  The
//   spline slopes of the table are solved on the host.
// * k_dvloc_g: for every point of the reference FFT box, V(|q+G|) from the
//   cubic spline, minus the long-range erf part (with the 2-D Coulomb cutoff
//   factor for slabs), times -i (q+G) e^{-i (q+G).tau_a} per atom and
//   direction, transformed to modes with eigVec (dVlocq,
//   src/dvloc/dVbare_loc.c:16-231).  The inverse FFT that follows uses the
//   FP64 Stockham passes of fft_gather.cu.
// * k_add_dvscf: dV_scf += dV_loc per magnetic component, and the nmag = 4
//   composite [V + Bz, Bx - i By, Bx + i By, V - Bz] (add_dvscf_qe,
//   src/dvloc/add_dvscf.c:12-92).
// Everything here is FP64.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"

#define LELPH_EPS_K 1e-5

// grid: (npts); 256 threads; one |G| point per block
__global__ void __launch_bounds__(256) k_vloc_table(const double* __restrict__ r, const double* __restrict__ wrab,
                                                    const double* __restrict__ vloc, int ngrid, double zval,
                                                    double volume, int cut3, double dg, double* __restrict__ out)
{
    __shared__ double red[256];
    const double G = (double)blockIdx.x * dg;
    const bool small = G < LELPH_EPS_K;
    double acc = 0.0;
    for (int i = threadIdx.x; i < ngrid; i += blockDim.x)
    {
        const double ri = r[i];
        const double fac = small ? ri : sin(ri * G) / G;
        const double body = (small && cut3) ? ri * vloc[i] + LELPH_E2 * zval : ri * vloc[i] + LELPH_E2 * zval * erf(ri);
        acc += fac * body * wrab[i];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1)
    {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = 4.0 * LELPH_PI_T * (red[0] / 3.0) / volume;
}

// grid: ceil(N / 256); one box point per thread; dynamic shared memory holds
// eigVec (nmodes x 3 natom complex), the atoms' positions and types.
__global__ void __launch_bounds__(256) k_dvloc_g(VlocDesc vd, const double2* __restrict__ eig, double2* __restrict__ out,
                                                 unsigned* __restrict__ status)
{
    extern __shared__ __align__(16) unsigned char dsm[];
    const int nj = 3 * vd.natom;
    double2* se = reinterpret_cast<double2*>(dsm);
    double* spos = reinterpret_cast<double*>(se + (size_t)vd.nmodes * nj);
    int* styp = reinterpret_cast<int*>(spos + 3 * vd.natom);
    for (int e = threadIdx.x; e < vd.nmodes * nj; e += blockDim.x) se[e] = eig[e];
    for (int e = threadIdx.x; e < 3 * vd.natom; e += blockDim.x) spos[e] = vd.atom_pos[e];
    for (int e = threadIdx.x; e < vd.natom; e += blockDim.x) styp[e] = vd.atom_type[e];
    __syncthreads();
    const long long N = (long long)vd.Nx * vd.Ny * vd.Nz;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    const int iz = (int)(p % vd.Nz);
    const int iy = (int)((p / vd.Nz) % vd.Ny);
    const int ix = (int)(p / ((long long)vd.Ny * vd.Nz));
    // Miller index of an FFT index: [-N/2, N/2) (get_miller_idx, src/common/numerical_func.c:436)
    const int n3[3] = {vd.Nx, vd.Ny, vd.Nz};
    const int i3[3] = {ix, iy, iz};
    double m[3];
    for (int x = 0; x < 3; ++x)
    {
        const int mid = (n3[x] - 1) / 2 + 1;
        m[x] = (double)(i3[x] < mid ? i3[x] : (i3[x] - mid) - n3[x] / 2) + vd.q[x];
    }
    // cartesian q + G, 2 pi included (blat . (m))
    double qG[3];
    for (int x = 0; x < 3; ++x) qG[x] = vd.blat[3 * x] * m[0] + vd.blat[3 * x + 1] * m[1] + vd.blat[3 * x + 2] * m[2];
    const double nrm = sqrt(qG[0] * qG[0] + qG[1] * qG[1] + qG[2] * qG[2]);
    const int gi = (int)floor(nrm / vd.dg);
    if (gi + 1 >= vd.npts)
    {
        atomicOr(status, LELPH_DEV_ERR_BOUNDS);
        for (int nu = 0; nu < vd.nmodes; ++nu) out[(size_t)nu * N + p] = make_double2(0.0, 0.0);
        return;
    }
    double cutf = 1.0;
    if (vd.dim2)
    {
        const double c = vd.alat_zz;
        const double gp = sqrt(qG[0] * qG[0] + qG[1] * qG[1]);
        double cs = cos(qG[2] * c * 0.5);
        if (gp > LELPH_EPS_K) cs = cs - sin(qG[2] * c * 0.5) * qG[2] / gp;
        cutf = 1.0 - exp(-c * gp * 0.5) * cs;
    }
    // V_loc(|q+G|) of every species: cubic Hermite form of the spline on
    // [x_gi, x_gi+1] with the table's slopes, then the long-range part removed
    double vt[LELPH_VLOC_MAXTYPE];
    const double x0 = gi * vd.dg, x1 = (gi + 1) * vd.dg;
    const double h = x1 - x0;
    const double t = (nrm - x0) / h;
    for (int it = 0; it < vd.ntype; ++it)
    {
        const double* y = vd.v + (size_t)it * vd.npts;
        const double* dy = vd.dv + (size_t)it * vd.npts;
        const double ax = dy[gi] * h - (y[gi + 1] - y[gi]);
        const double bx = -dy[gi + 1] * h + (y[gi + 1] - y[gi]);
        double val = (1 - t) * y[gi] + t * y[gi + 1] + t * (1 - t) * ((1 - t) * ax + t * bx);
        if (nrm >= LELPH_EPS_K)
            val -= (4 * LELPH_PI_T * LELPH_E2) * vd.zval[it] * exp(-nrm * nrm * 0.25) * cutf / (nrm * nrm * vd.volume);
        vt[it] = val;
    }
    // cartesian displacement components: -i e^{-i (q+G).tau_a} V_type(a) (q+G)_x,
    // then modes: out[nu] = sum_j eigVec[nu][j] cart[j]
    double2 acc[LELPH_VLOC_MAXMODES];
    for (int nu = 0; nu < vd.nmodes; ++nu) acc[nu] = make_double2(0.0, 0.0);
    for (int a = 0; a < vd.natom; ++a)
    {
        const double dot = qG[0] * spos[3 * a] + qG[1] * spos[3 * a + 1] + qG[2] * spos[3 * a + 2];
        double sn, cs;
        sincos(dot, &sn, &cs);
        // -i (cos - i sin) = -sin - i cos
        const double vv = vt[styp[a]];
        const double2 fac = make_double2(-sn * vv, -cs * vv);
        for (int x = 0; x < 3; ++x)
        {
            const double2 c = make_double2(fac.x * qG[x], fac.y * qG[x]);
            const int j = 3 * a + x;
            for (int nu = 0; nu < vd.nmodes; ++nu) acc[nu] = cadd(acc[nu], cmul(se[nu * nj + j], c));
        }
    }
    for (int nu = 0; nu < vd.nmodes; ++nu) out[(size_t)nu * N + p] = acc[nu];
}

// dv (nmodes, nmag, N) += vloc (nmodes, N) per add_dvscf_qe
__global__ void k_add_dvscf(double2* __restrict__ dv, const double2* __restrict__ vloc, int nmodes, int nmag,
                            long long N)
{
    const long long n = (long long)nmodes * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    {
        const int nu = (int)(e / N);
        const long long r = e - (long long)nu * N;
        double2* d = dv + (size_t)nu * nmag * N + r;
        const double2 v = vloc[e];
        if (nmag == 2)
        {
            d[0] = cadd(d[0], v);
            d[N] = cadd(d[N], v);
        }
        else if (nmag == 4)
        {
            const double2 V = cadd(d[0], v), Bx = d[N], By = d[2 * N], Bz = d[3 * N];
            const double2 iBy = make_double2(-By.y, By.x);
            d[0] = cadd(V, Bz);
            d[N] = csub(Bx, iBy);
            d[2 * N] = cadd(Bx, iBy);
            d[3 * N] = csub(V, Bz);
        }
        else
        {
            d[0] = cadd(d[0], v);
        }
    }
}

void lelph_launch_vloc_table(const double* r, const double* wrab, const double* vloc, int ngrid, double zval,
                             double volume, int cut3, double dg, int npts, double* out, cudaStream_t st)
{
    k_vloc_table<<<npts, 256, 0, st>>>(r, wrab, vloc, ngrid, zval, volume, cut3, dg, out);
}

int lelph_launch_dvloc_g(const VlocDesc& vd, const double2* eig, double2* out, unsigned* status, cudaStream_t st)
{
    if (vd.ntype > LELPH_VLOC_MAXTYPE || vd.nmodes > LELPH_VLOC_MAXMODES) return -1;
    const long long N = (long long)vd.Nx * vd.Ny * vd.Nz;
    const size_t smem = sizeof(double2) * (size_t)vd.nmodes * 3 * vd.natom + sizeof(double) * 3 * vd.natom +
                        sizeof(int) * vd.natom + 16;
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(k_dvloc_g, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    k_dvloc_g<<<(unsigned)((N + 255) / 256), 256, smem, st>>>(vd, eig, out, status);
    return 0;
}

void lelph_launch_add_dvscf(double2* dv, const double2* vloc, int nmodes, int nmag, long long N, cudaStream_t st)
{
    k_add_dvscf<<<1024, 256, 0, st>>>(dv, vloc, nmodes, nmag, N);
}
