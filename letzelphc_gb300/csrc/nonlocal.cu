// Kleinman-Bylander nonlocal term and the per-pair finish step.
//
// The reference builds, per (k, k+q) pair and atom, the projectors
// beta_x(K) = F(K) e^{-i 2pi K.tau_a} Y_lm(K) (1, K_x sign, K_y sign, K_z sign)
// on K = S(k+G) and projects both wavefunctions on them
// (src/nonloc/Vbare_nloc.c:147-459), then combines the projections
// (sum_VNL_KKp, src/nonloc/sum_VNL_KKp.c:8-58) and maps atom displacements
// to modes with -2 pi i e2 eigVec (src/nonloc/Vbare_nloc.c:543-560).
// The projections only depend on the full-BZ k-point, not on q, so here they
// are computed once per k (k_projections) and the per-pair work reduces to
// the small combination done in k_finish:
//   role k+q : Pi[k+q]                      (= bandbufferK)
//   role k   : conj(Pi[k]) for x = 0, -conj(Pi[k]) for x > 0   (= bandbufferKp)
// with Pi[k][a][p][x][set] = sum_G beta_x(G) conj(c^(G)), c^ the unfolded
// coefficients (SU(2), fractional-translation phase, time-reversal conj).
#include <cuda_runtime.h>
#include <stdint.h>

#include "lelph_common.cuh"
#include "lelph_internal.h"

__device__ __forceinline__ double ylm_legendre(int l, int m, double x)
{
    // associated Legendre function without the Condon-Shortley phase, m >= 0
    double val = 1.0;
    if (l == 0 && m == 0) return 1.0;
    if (m > l) return 0.0;
    double sq = sqrt(1.0 - x * x);
    for (int im = 1; im <= m; ++im) val *= (2 * im - 1) * sq;
    if (l == m) return val;
    double vmm = val;
    val *= (2 * m + 1) * x;
    if (l == m + 1) return val;
    for (int im = m + 2; im <= l; ++im)
    {
        double tmp = val;
        val = (2 * im - 1) * x * val - (im + m - 1) * vmm;
        val = val / (im - m);
        vmm = tmp;
    }
    return val;
}

// real spherical harmonics of Blanco, Florez and Bermejo (J. Mol. Struct.
// THEOCHEM 419, 19 (1997)), the convention of src/common/numerical_func.c:97-152
__device__ __forceinline__ double ylm_real(int l, int m, double vx, double vy, double vz)
{
    const double fact[8] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0};
    double norm = sqrt(vx * vx + vy * vy + vz * vz);
    if (norm < 1e-6) return (l != 0) ? 0.0 : 1.0 / sqrt(4 * LELPH_PI_T);
    double cost = vz / norm;
    double phi = atan2(vy, vx);
    double sh;
    int am = m < 0 ? -m : m;
    if (m > 0) sh = sqrt(2.0) * cos(m * phi);
    else if (m < 0) sh = sqrt(2.0) * sin(am * phi);
    else sh = 1.0;
    sh *= ylm_legendre(l, am, cost);
    sh *= sqrt(fact[l - am] * (2 * l + 1) / (4 * LELPH_PI_T * fact[l + am]));
    return sh;
}

#define PJ_G 32
#define PJ_MAXP 24

// grid: (nk, natom, nsb * npb); 256 threads.  A block covers nset_b <= 64
// consecutive coefficient sets (set-block sb) and 256/nset_b consecutive
// (projector, component) pairs (px-block pb); one output per thread.
// Pi layout: proj[(((kbz*natom + a)*nproj_max + p)*4 + x)*nsets + set],
// nsets = nspin*nbnds*nspinor, set = (spin*nbnds + band)*nspinor + spinor.
template <int F32ACC>
__global__ void __launch_bounds__(256) k_projections(int k0, const KPointSym* __restrict__ ks,
                                                     const double* __restrict__ gvec,
                                                     const long long* __restrict__ pw_off,
                                                     const int* __restrict__ npw_arr, const double* __restrict__ Fk,
                                                     const long long* __restrict__ fk_off,
                                                     const double2* __restrict__ chat,
                                                     const long long* __restrict__ chat_off, NonlocalDesc nl,
                                                     GeomDev gd, int nset_b, int nsb, double2* __restrict__ proj)
{
    __shared__ double2 base_s[PJ_MAXP][PJ_G];  // F e^{-i 2pi K.tau_a} Y_lm(K) per projector
    __shared__ double kx_s[3][PJ_G];
    __shared__ double2 ch_s[PJ_G][65];
    __shared__ int plist[PJ_MAXP][3];  // (lidx, l, m)
    __shared__ double psign[PJ_MAXP];
    __shared__ int nproj_s;
    const int kbz = k0 + blockIdx.x;
    const int a = blockIdx.y;
    const int sb = blockIdx.z % nsb, pb = blockIdx.z / nsb;
    const KPointSym S = ks[kbz];
    const int it = nl.atom_type[a];
    const int npw = npw_arr[S.ik];
    const int nsets = gd.nspin * gd.nbnds * gd.nspinor;
    if (threadIdx.x == 0)
    {
        int np = 0;
        for (int lidx = 0; lidx < nl.nltimesj; ++lidx)
        {
            int l = (int)rint(nl.PP_table[(lidx * nl.ntype + it) * 3] - 1.0);
            if (l < 0) continue;
            for (int im = 0; im <= 2 * l && np < PJ_MAXP; ++im, ++np)
            {
                plist[np][0] = lidx;
                plist[np][1] = l;
                plist[np][2] = im - l;
                psign[np] = nl.Fsign[lidx * nl.ntype + it];
            }
        }
        nproj_s = np;
    }
    __syncthreads();
    const int nproj = nproj_s;
    const int ppb = blockDim.x / nset_b;
    const int set_l = threadIdx.x % nset_b;
    const int px = pb * ppb + threadIdx.x / nset_b;
    const int p = px >> 2, x = px & 3;
    const int set0 = sb * nset_b;
    const int set = set0 + set_l;
    const int nset_here = min(nset_b, nsets - set0);
    const bool active = (threadIdx.x / nset_b) < ppb && p < nproj && set < nsets;
    const double* G = gvec + 3 * pw_off[S.ik];
    const double* F = Fk + fk_off[S.ik];
    const double2* C = chat + chat_off[kbz];
    const double tx = nl.atom_pos[3 * a], ty = nl.atom_pos[3 * a + 1], tz = nl.atom_pos[3 * a + 2];
    double2 acc = make_double2(0.0, 0.0);
    for (int g0 = 0; g0 < npw; g0 += PJ_G)
    {
        const int ng = min(PJ_G, npw - g0);
        __syncthreads();
        if (threadIdx.x < ng)
        {
            int g = g0 + threadIdx.x;
            // K = S (k + G), cartesian (src/nonloc/Vbare_nloc.c:148-168)
            double v0 = S.kcart[0] + G[3 * g], v1 = S.kcart[1] + G[3 * g + 1], v2 = S.kcart[2] + G[3 * g + 2];
            double K0 = S.R[0] * v0 + S.R[1] * v1 + S.R[2] * v2;
            double K1 = S.R[3] * v0 + S.R[4] * v1 + S.R[5] * v2;
            double K2 = S.R[6] * v0 + S.R[7] * v1 + S.R[8] * v2;
            kx_s[0][threadIdx.x] = K0;
            kx_s[1][threadIdx.x] = K1;
            kx_s[2][threadIdx.x] = K2;
            double dot = K0 * tx + K1 * ty + K2 * tz;
            double sn, cs;
            sincos(2.0 * LELPH_PI_T * dot, &sn, &cs);
            for (int pp = 0; pp < nproj; ++pp)
            {
                int lidx = plist[pp][0], l = plist[pp][1], m = plist[pp][2];
                double f = F[((size_t)lidx * nl.ntype + it) * npw + g];
                double y = ylm_real(l, m, K0, K1, K2);
                base_s[pp][threadIdx.x] = make_double2(f * cs * y, -f * sn * y);
            }
        }
        for (int e = threadIdx.x; e < ng * nset_here; e += blockDim.x)
        {
            int gg = e / nset_here, ss = e - gg * nset_here;
            ch_s[gg][ss] = C[(size_t)(set0 + ss) * npw + g0 + gg];
        }
        __syncthreads();
        if (active)
        {
            const double kk = (x > 0) ? psign[p] : 1.0;
            if (F32ACC)
            {
                float2 a32 = make_float2(0.f, 0.f);
                for (int gg = 0; gg < ng; ++gg)
                {
                    double2 b = base_s[p][gg];
                    double w = (x > 0) ? kx_s[x - 1][gg] * kk : 1.0;
                    float2 bf = make_float2((float)(b.x * w), (float)(b.y * w));
                    double2 c = ch_s[gg][set_l];
                    a32 = cadd(a32, cmul(bf, make_float2((float)c.x, (float)-c.y)));
                }
                acc.x += a32.x;
                acc.y += a32.y;
            }
            else
            {
                for (int gg = 0; gg < ng; ++gg)
                {
                    double2 b = base_s[p][gg];
                    if (x > 0)
                    {
                        double w = kx_s[x - 1][gg] * kk;
                        b.x *= w;
                        b.y *= w;
                    }
                    acc = cadd(acc, cmul(b, cconj(ch_s[gg][set_l])));
                }
            }
        }
    }
    if (active) proj[((((size_t)kbz * nl.natom + a) * nl.nproj_max + p) * 4 + x) * nsets + set] = acc;
}

void lelph_launch_projections(int k0, int nk, const KPointSym* ksym_dev, const double* gvec, const long long* pw_off,
                              const int* npw, const double* Fk, const long long* fk_off, const double2* chat,
                              const long long* chat_off, const NonlocalDesc& nl, const GeomDev& g, int f32acc,
                              double2* proj, cudaStream_t st)
{
    const int nsets = g.nspin * g.nbnds * g.nspinor;
    const int nset_b = nsets < 64 ? nsets : 64;
    const int nsb = (nsets + nset_b - 1) / nset_b;
    const int ppb = 256 / nset_b;
    const int npb = (nl.nproj_max * 4 + ppb - 1) / ppb;
    dim3 grid(nk, nl.natom, nsb * npb);
    if (f32acc)
        k_projections<1><<<grid, 256, 0, st>>>(k0, ksym_dev, gvec, pw_off, npw, Fk, fk_off, chat, chat_off, nl, g,
                                               nset_b, nsb, proj);
    else
        k_projections<0><<<grid, 256, 0, st>>>(k0, ksym_dev, gvec, pw_off, npw, Fk, fk_off, chat, chat_off, nl, g,
                                               nset_b, nsb, proj);
}

// ------------------------------------------------------------------ finish

#define FIN_MN 32
#define FIN_MAXJ 48  // 3 * natom

// grid: (ceil(nb*nb/32), npairs*nspin); 256 threads.
// gout layout per pair: (nmodes, nspin, nb_k, nb_kq) complex.
__global__ void __launch_bounds__(256) k_finish(const PairInfo* __restrict__ pairs, int mode_fp64,
                                                const double2* __restrict__ glocal,
                                                const float* __restrict__ partials, int nchunks,
                                                const float* __restrict__ mode_scale,
                                                const float* __restrict__ band_scale,
                                                const double2* __restrict__ proj, const double2* __restrict__ eig,
                                                int non_loc, NonlocalDesc nl, GeomDev gd, int out_c64,
                                                void* __restrict__ gout)
{
    __shared__ double2 out_s[FIN_MAXJ][FIN_MN];
    const int zp = blockIdx.y;
    const int pair = zp / gd.nspin, spin = zp - pair * gd.nspin;
    const PairInfo P = pairs[pair];
    const int nb = gd.nbnds, ns = gd.nspinor;
    const int nsets = gd.nspin * nb * ns;
    const int mn0 = blockIdx.x * FIN_MN;
    const int nj = 3 * nl.natom;
    if (non_loc)
    {
        for (int e = threadIdx.x; e < nj * FIN_MN; e += blockDim.x)
        {
            int j = e / FIN_MN, t = e - j * FIN_MN;
            int mn = mn0 + t;
            double2 acc = make_double2(0.0, 0.0);
            if (mn < nb * nb)
            {
                int m = mn / nb, n = mn - m * nb;  // m: band of k, n: band of k+q
                int a = j / 3, x = j - 3 * a;
                int it = nl.atom_type[a];
                const double2* PK = proj + (((size_t)P.kbz_kq * nl.natom + a) * nl.nproj_max) * 4 * nsets;
                const double2* PKp = proj + (((size_t)P.kbz_k * nl.natom + a) * nl.nproj_max) * 4 * nsets;
                int pbase = 0;
                for (int lidx = 0; lidx < nl.nltimesj; ++lidx)
                {
                    int l = (int)rint(nl.PP_table[(lidx * nl.ntype + it) * 3] - 1.0);
                    if (l < 0) continue;
                    int twoj = (int)rint(nl.PP_table[(lidx * nl.ntype + it) * 3 + 1]);
                    double soc_fac = 1.0;
                    if (twoj != 0 && !nl.is_soc) soc_fac = (twoj + 1.0) / (4.0 * l + 2.0);
                    int foff = nl.fcoef ? nl.fcoef_off[lidx * nl.ntype + it] : -1;
                    int tl = 2 * l + 1;
                    for (int im1 = 0; im1 < tl; ++im1)
                        for (int im2 = 0; im2 < tl; ++im2)
                        {
                            if (foff < 0 && im1 != im2) continue;
                            int p1 = pbase + im1, p2 = pbase + im2;
                            for (int s1 = 0; s1 < ns; ++s1)
                                for (int s2 = 0; s2 < ns; ++s2)
                                {
                                    double2 f;
                                    if (foff >= 0)
                                    {
                                        const double* fc = nl.fcoef + 2 * ((size_t)foff + (im1 * tl + im2) * ns * ns +
                                                                           s1 * ns + s2);
                                        f = make_double2(fc[0], fc[1]);
                                    }
                                    else
                                    {
                                        f = make_double2(s1 == s2 ? soc_fac : 0.0, 0.0);
                                    }
                                    if (f.x == 0.0 && f.y == 0.0) continue;
                                    int setK = (spin * nb + n) * ns + s1;
                                    int setKp = (spin * nb + m) * ns + s2;
                                    double2 K0 = PK[((size_t)p1 * 4 + 0) * nsets + setK];
                                    double2 Kx = PK[((size_t)p1 * 4 + 1 + x) * nsets + setK];
                                    double2 Kp0 = cconj(PKp[((size_t)p2 * 4 + 0) * nsets + setKp]);
                                    double2 Kpx = PKp[((size_t)p2 * 4 + 1 + x) * nsets + setKp];
                                    Kpx = make_double2(-Kpx.x, Kpx.y);  // -conj
                                    double2 t2 = cadd(cmul(Kx, Kp0), cmul(K0, Kpx));
                                    acc = cadd(acc, cmul(f, t2));
                                }
                        }
                    pbase += tl;
                }
            }
            out_s[j][t] = acc;
        }
        __syncthreads();
    }
    const double invN = 1.0 / ((double)gd.Nx * gd.Ny * gd.Nz);
    const int nrows = gd.nmodes * nb;
    const int mtiles = (gd.nmodes + gd.mt_modes - 1) / gd.mt_modes;
    const int NT = 2 * gd.nbp;
    // pre-factor -2 pi i e2 (src/nonloc/Vbare_nloc.c:547)
    const double2 pre = make_double2(0.0, -2.0 * LELPH_PI_T * LELPH_E2);
    const double2* E = eig + (size_t)P.qslot * gd.nmodes * gd.nmodes;
    for (int e = threadIdx.x; e < gd.nmodes * FIN_MN; e += blockDim.x)
    {
        int nu = e / FIN_MN, t = e - nu * FIN_MN;
        int mn = mn0 + t;
        if (mn >= nb * nb) continue;
        int m = mn / nb, n = mn - m * nb;
        int row = nu * nb + m;
        double2 v;
        if (mode_fp64)
        {
            v = glocal[((size_t)zp * nrows + row) * nb + n];
        }
        else
        {
            int mt = nu / gd.mt_modes, rr = (nu - mt * gd.mt_modes) * nb + m;
            const float* pp = partials + (((size_t)zp * mtiles + mt) * nchunks * 128 + rr) * NT;
            double re = 0.0, im = 0.0;
            for (int c = 0; c < nchunks; ++c)
            {
                re += (double)pp[(size_t)c * 128 * NT + n];
                im += (double)pp[(size_t)c * 128 * NT + gd.nbp + n];
            }
            double sc = (double)mode_scale[(size_t)P.dvslot * gd.nmodes + nu] *
                        (double)band_scale[((size_t)P.kbz_k * gd.nspin + spin) * nb + m] *
                        (double)band_scale[((size_t)P.kbz_kq * gd.nspin + spin) * nb + n];
            double f = invN / sc;
            v = make_double2(re * f, im * f);
        }
        if (non_loc)
        {
            double2 s = make_double2(0.0, 0.0);
            for (int j = 0; j < nj; ++j) s = cadd(s, cmul(E[(size_t)nu * gd.nmodes + j], out_s[j][t]));
            v = cadd(v, cmul(pre, s));
        }
        size_t oidx = ((((size_t)pair * gd.nmodes + nu) * gd.nspin + spin) * nb + m) * nb + n;
        if (out_c64)
            reinterpret_cast<float2*>(gout)[oidx] = make_float2((float)v.x, (float)v.y);
        else
            reinterpret_cast<double2*>(gout)[oidx] = v;
    }
}

void lelph_launch_finish(const PairInfo* pairs, int npairs, int mode_fp64, const double2* glocal,
                         const float* partials, int nchunks, const float* mode_scale, const float* band_scale,
                         const double2* proj, const double2* eig, int non_loc, const NonlocalDesc& nl,
                         const GeomDev& g, int out_c64, void* gout, cudaStream_t st)
{
    dim3 grid((g.nbnds * g.nbnds + FIN_MN - 1) / FIN_MN, npairs * g.nspin);
    k_finish<<<grid, 256, 0, st>>>(pairs, mode_fp64, glocal, partials, nchunks, mode_scale, band_scale, proj, eig,
                                   non_loc, nl, g, out_c64, gout);
}
