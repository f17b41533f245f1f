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

#include <algorithm>
#include <stdint.h>

#include <type_traits>

#include "lelph_common.cuh"
#include "lelph_internal.h"
#include "ylm.cuh"

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

#define PJ_MAXP 24
#define PJ_ROWS 64   // (atom, projector, component) rows per block
#define PJ_SETS 32   // coefficient sets per block

template <typename T> struct PjCfg;
template <> struct PjCfg<float> { static constexpr int G = 64; };
template <> struct PjCfg<double> { static constexpr int G = 32; };

template <typename T> static constexpr size_t pj_smem_bytes()
{
    typedef typename cplx_of<T>::type C2;
    constexpr int G = PjCfg<T>::G;
    return sizeof(C2) * (PJ_ROWS * (G + 1) + G * (PJ_SETS + 1) + 4 * G) + sizeof(T) * (16 * G + 3 * G);
}

// grid: (nk, row blocks, set blocks x gsplit); 256 threads, 4 rows x 2 sets per
// thread; with gsplit > 1 a block takes every gsplit-th chunk of the plane
// waves and adds its sums into the zeroed Pi entries.
// Rows r = (atom*nproj_max + p)*4 + x; Pi layout proj[((kbz*rows_tot) + r)*nsets + set],
// nsets = nspin*nbnds*nspinor, set = (spin*nbnds + band)*nspinor + spinor.
// T = float: beta, coefficients and products in FP32, each G chunk summed in
// FP32 and the chunk sums in FP64; the K vectors, Y_lm and the structure-factor
// phases e^{-i 2pi K.tau} are evaluated in FP64 (the mixed form reduces the
// phase angle to one turn in FP64 and takes sine and cosine in FP32).
template <typename T>
__global__ void __launch_bounds__(256) k_projections(int k0, const KPointSym* __restrict__ ks,
                                                     const double* __restrict__ gvec,
                                                     const long long* __restrict__ pw_off,
                                                     const int* __restrict__ npw_arr, const double* __restrict__ Fk,
                                                     const long long* __restrict__ fk_off,
                                                     const double2* __restrict__ chat,
                                                     const long long* __restrict__ chat_off, NonlocalDesc nl,
                                                     GeomDev gd, int gsplit, double2* __restrict__ proj)
{
    typedef typename cplx_of<T>::type C2;
    constexpr int PG = PjCfg<T>::G;
    constexpr int PARTS = 256 / PG;
    extern __shared__ __align__(16) unsigned char pj_smem[];
    C2* beta_s = reinterpret_cast<C2*>(pj_smem);   // [PJ_ROWS][PG + 1]
    C2* ch_s = beta_s + PJ_ROWS * (PG + 1);          // [PG][PJ_SETS + 1]
    C2* ph_s = ch_s + PG * (PJ_SETS + 1);            // [4][PG]
    T* ylm_s = reinterpret_cast<T*>(ph_s + 4 * PG);  // [16][PG]
    T* kx_s = ylm_s + 16 * PG;                       // [3][PG]
    __shared__ int rinfo[PJ_ROWS][4];  // atom slot, lm index, (lidx*ntype+type), x
    __shared__ T rsign[PJ_ROWS];
    const int kbz = k0 + blockIdx.x;
    const KPointSym S = ks[kbz];
    const int npw = npw_arr[S.ik];
    const int nsets = gd.nspin * gd.nbnds * gd.nspinor;
    const int rows_tot = nl.natom * nl.nproj_max * 4;
    const int r0 = blockIdx.y * PJ_ROWS;
    const int gs = blockIdx.z % gsplit;  // this block's share of the plane waves: chunks gs, gs + gsplit, ...
    const int s0 = (blockIdx.z / gsplit) * PJ_SETS;
    const int nr = min(PJ_ROWS, rows_tot - r0);
    const int ns = min(PJ_SETS, nsets - s0);
    const int a0 = r0 / (nl.nproj_max * 4);
    if (threadIdx.x < PJ_ROWS)
    {
        const int r = r0 + threadIdx.x;
        int info[4] = {-1, 0, 0, 0};
        double sg = 1.0;
        if (threadIdx.x < nr)
        {
            const int a = r / (nl.nproj_max * 4);
            const int p = (r / 4) % nl.nproj_max;
            const int x = r % 4;
            const int it = nl.atom_type[a];
            int np = 0;
            for (int lidx = 0; lidx < nl.nltimesj; ++lidx)
            {
                int l = (int)rint(nl.PP_table[(lidx * nl.ntype + it) * 3] - 1.0);
                if (l < 0) continue;
                if (p >= np && p < np + 2 * l + 1)
                {
                    info[0] = a - a0;
                    info[1] = l * l + (p - np);  // lm index: l*l + l + m with m = (p-np) - l
                    info[2] = lidx * nl.ntype + it;
                    info[3] = x;
                    sg = nl.Fsign[lidx * nl.ntype + it];
                }
                np += 2 * l + 1;
            }
        }
        for (int c = 0; c < 4; ++c) rinfo[threadIdx.x][c] = info[c];
        rsign[threadIdx.x] = (T)sg;
    }
    const int tr = threadIdx.x / 16, tsx = threadIdx.x % 16;  // rows tr*4.., sets tsx*2..
    C2 acc[4][2];
    double2 acc64[4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
        {
            acc[i][j].x = 0;
            acc[i][j].y = 0;
            acc64[i][j] = make_double2(0.0, 0.0);
        }
    const double* G = gvec + 3 * pw_off[S.ik];
    const double* F = Fk + fk_off[S.ik];
    const double2* Cc = chat + chat_off[kbz];
    const int natom_blk = min(4, nl.natom - a0);
    const int nlm = (nl.lmax + 1) * (nl.lmax + 1);
    for (int g0 = gs * PG; g0 < npw; g0 += gsplit * PG)
    {
        const int ng = min(PG, npw - g0);
        __syncthreads();
        {
            // K = S (k + G), cartesian (src/nonloc/Vbare_nloc.c:148-168); part 0
            // tabulates Y_lm and K, parts 0..3 one structure-factor phase each
            const int t = threadIdx.x % PG, part = threadIdx.x / PG;
            if (t < ng && (part == 0 || part < natom_blk))
            {
                const int g = g0 + t;
                double v0 = S.kcart[0] + G[3 * g], v1 = S.kcart[1] + G[3 * g + 1], v2 = S.kcart[2] + G[3 * g + 2];
                double K0 = S.R[0] * v0 + S.R[1] * v1 + S.R[2] * v2;
                double K1 = S.R[3] * v0 + S.R[4] * v1 + S.R[5] * v2;
                double K2 = S.R[6] * v0 + S.R[7] * v1 + S.R[8] * v2;
                if (part == 0)
                {
                    double y[16];
                    kx_s[0 * PG + t] = (T)K0;
                    kx_s[1 * PG + t] = (T)K1;
                    kx_s[2 * PG + t] = (T)K2;
                    ylm_all(nl.lmax, K0, K1, K2, y);
                    for (int i = 0; i < nlm; ++i) ylm_s[i * PG + t] = (T)y[i];
                }
                if (part < natom_blk)
                {
                    const double* tau = nl.atom_pos + 3 * (a0 + part);
                    double dot = K0 * tau[0] + K1 * tau[1] + K2 * tau[2];
                    if constexpr (std::is_same<T, float>::value)
                    {
                        // mixed form: the angle 2 pi_T dot is reduced to one turn in FP64
                        // (pi_T the reference's truncated pi) and the phase taken in FP32
                        const double turns = dot * (LELPH_PI_T / 3.14159265358979323846);
                        float sn, cs;
                        sincospif(2.0f * (float)(turns - rint(turns)), &sn, &cs);
                        ph_s[part * PG + t] = mk2<C2>(cs, -sn);
                    }
                    else
                    {
                        double sn, cs;
                        sincos(2.0 * LELPH_PI_T * dot, &sn, &cs);
                        ph_s[part * PG + t] = mk2<C2>(cs, -sn);
                    }
                }
            }
        }
        (void)PARTS;
        for (int e = threadIdx.x; e < ns * PG; e += blockDim.x)
        {
            const int ss = e / PG, gg = e - ss * PG;
            const double2 c = gg < ng ? Cc[(size_t)(s0 + ss) * npw + g0 + gg] : make_double2(0.0, 0.0);
            ch_s[gg * (PJ_SETS + 1) + ss] = mk2<C2>(c.x, -c.y);  // conj(c^)
        }
        __syncthreads();
        // beta_x(G) = F e^{-i 2pi K.tau} Y_lm (1 | K_x sign)  (src/nonloc/Vbare_nloc.c:318-363)
        for (int e = threadIdx.x; e < PJ_ROWS * PG; e += blockDim.x)
        {
            const int rr = e / PG, gg = e - rr * PG;
            C2 b;
            b.x = 0;
            b.y = 0;
            if (gg < ng && rinfo[rr][0] >= 0)
            {
                const T f = (T)F[(size_t)rinfo[rr][2] * npw + g0 + gg];
                const C2 ph = ph_s[rinfo[rr][0] * PG + gg];
                T fy = f * ylm_s[rinfo[rr][1] * PG + gg];
                const int x = rinfo[rr][3];
                if (x > 0) fy *= kx_s[(x - 1) * PG + gg] * rsign[rr];
                b.x = fy * ph.x;
                b.y = fy * ph.y;
            }
            beta_s[rr * (PG + 1) + gg] = b;
        }
        __syncthreads();
        // Pi += beta conj(c^) over the chunk
#pragma unroll 8
        for (int gg = 0; gg < PG; ++gg)
        {
            C2 bv[4], cv[2];
#pragma unroll
            for (int i = 0; i < 4; ++i) bv[i] = beta_s[(tr * 4 + i) * (PG + 1) + gg];
#pragma unroll
            for (int j = 0; j < 2; ++j) cv[j] = ch_s[gg * (PJ_SETS + 1) + tsx * 2 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) acc[i][j] = cadd(acc[i][j], cmul(bv[i], cv[j]));
        }
        if (std::is_same<T, float>::value)
        {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j)
                {
                    acc64[i][j].x += (double)acc[i][j].x;
                    acc64[i][j].y += (double)acc[i][j].y;
                    acc[i][j].x = 0;
                    acc[i][j].y = 0;
                }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
        {
            const int rr = tr * 4 + i, ss = tsx * 2 + j;
            if (rr < nr && ss < ns)
            {
                double2 v = std::is_same<T, float>::value ? acc64[i][j]
                                                          : make_double2((double)acc[i][j].x, (double)acc[i][j].y);
                double2* o = proj + ((size_t)kbz * rows_tot + r0 + rr) * nsets + s0 + ss;
                if (gsplit == 1)
                    *o = v;
                else
                {
                    // the plane-wave shares of one k add into the zeroed entry
                    atomicAdd(&o->x, v.x);
                    atomicAdd(&o->y, v.y);
                }
            }
        }
}

void lelph_launch_projections(int k0, int nk, const KPointSym* ksym_dev, const double* gvec, const long long* pw_off,
                              const int* npw, const double* Fk, const long long* fk_off, const double2* chat,
                              const long long* chat_off, const NonlocalDesc& nl, const GeomDev& g, int f32acc,
                              double2* proj, cudaStream_t st)
{
    const int nsets = g.nspin * g.nbnds * g.nspinor;
    const int rows = nl.natom * nl.nproj_max * 4;
    const int rb = (rows + PJ_ROWS - 1) / PJ_ROWS, sb = (nsets + PJ_SETS - 1) / PJ_SETS;
    // one block per (k, row block, set block) leaves most SMs idle for a few k:
    // the plane waves of a k are shared by up to 8 blocks (about 4 blocks per SM)
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const long long base = (long long)nk * rb * sb;
    const int gsplit = (int)std::max(1LL, std::min(8LL, (4LL * nsm + base - 1) / base));
    if (gsplit > 1)
        cudaMemsetAsync(proj + (size_t)k0 * rows * nsets, 0, sizeof(double2) * (size_t)nk * rows * nsets, st);
    dim3 grid(nk, rb, sb * gsplit);
    static bool attr = false;
    if (!attr)
    {
        cudaFuncSetAttribute(k_projections<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)pj_smem_bytes<float>());
        cudaFuncSetAttribute(k_projections<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)pj_smem_bytes<double>());
        attr = true;
    }
    if (f32acc)
        k_projections<float><<<grid, 256, pj_smem_bytes<float>(), st>>>(k0, ksym_dev, gvec, pw_off, npw, Fk, fk_off,
                                                                        chat, chat_off, nl, g, gsplit, proj);
    else
        k_projections<double><<<grid, 256, pj_smem_bytes<double>(), st>>>(k0, ksym_dev, gvec, pw_off, npw, Fk,
                                                                          fk_off, chat, chat_off, nl, g, gsplit,
                                                                          proj);
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
            const float* pp = partials + lelph_tc_partial_offset(gd, nchunks, zp, mt, 0, rr);
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

// Knuth's TwoSum: s + x is added into s, its rounding error into e.  The
// _rn intrinsics keep the compiler from contracting or reassociating.
__device__ __forceinline__ void ff_two_sum(float& s, float& e, float x)
{
    const float t = __fadd_rn(s, x), z = __fsub_rn(t, s);
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z)));
    s = t;
}

// (s + e) (fh + fl) + t rounded once to float.  The product's rounding error
// is recovered exactly with an FMA (the error-free product of Ogita, Rump and
// Oishi), the addition of t with TwoSum; the remaining terms are summed at
// the error's own scale, so the result carries about 2^-46 of |(s+e) fh| on
// top of its final rounding.
__device__ __forceinline__ float ff_scale_add(float s, float e, float fh, float fl, float t)
{
    const float p = __fmul_rn(s, fh);
    float pe = __fmaf_rn(s, fh, -p);
    pe = __fmaf_rn(s, fl, pe);
    pe = __fmaf_rn(e, fh, pe);
    pe = __fmaf_rn(e, fl, pe);
    const float u = __fadd_rn(p, t), z = __fsub_rn(u, p);
    const float ue = __fadd_rn(__fsub_rn(p, __fsub_rn(u, z)), __fsub_rn(t, z));
    return __fadd_rn(u, __fadd_rn(pe, ue));
}

// Finish, one block per (pair, spin): the two projection sets of the pair
// (this spin) and the pair's eigVec live in shared memory; each thread owns
// (m, n) elements and keeps the 3*natom displacement sums in registers.
// T is the arithmetic of the nonlocal combination and the mode transform
// (double in the plain form, float in the mixed form).  The plain form adds
// the FP64 local term in FP64; the mixed form sums the local sandwich's K-chunk
// partials and adds the nonlocal term with float error-free transformations
// (three blocks per SM: 80 registers).
template <int NJ, typename T>
__global__ void __launch_bounds__(NJ <= 12 ? 256 : 128, (NJ <= 12 && sizeof(T) == 4) ? 3 : 0) k_finish_pair(const PairInfo* __restrict__ pairs, int mode_fp64,
                                                     const double2* __restrict__ glocal,
                                                     const float* __restrict__ partials, int nchunks,
                                                     const float* __restrict__ mode_scale,
                                                     const float* __restrict__ band_scale,
                                                     const double2* __restrict__ proj,
                                                     const double2* __restrict__ eig, int non_loc, NonlocalDesc nl,
                                                     GeomDev gd, int out_c64, void* __restrict__ gout)
{
    typedef typename cplx_of<T>::type C2;
    extern __shared__ __align__(16) unsigned char fsm[];
    const int zp = blockIdx.x;
    const int pair = zp / gd.nspin, spin = zp - pair * gd.nspin;
    const PairInfo P = pairs[pair];
    const int nb = gd.nbnds, ns = gd.nspinor;
    const int nsets = gd.nspin * nb * ns;
    const int sets = nb * ns;  // this spin's sets
    const int rows = nl.natom * nl.nproj_max * 4;
    const int nj = 3 * nl.natom;
    C2* sK = reinterpret_cast<C2*>(fsm);                     // [rows][sets]  role k+q
    C2* sKp = sK + (size_t)rows * sets;                      // [rows][sets]  role k (raw Pi)
    C2* sE = sKp + (size_t)rows * sets;                      // [nmodes][nj]
    int* sch = reinterpret_cast<int*>(sE + (size_t)gd.nmodes * nj);  // channels: [type][8][4] = lidx, l, pbase, foff
    T* ssoc = reinterpret_cast<T*>(sch + nl.ntype * 8 * 4);
    int* snp = reinterpret_cast<int*>(ssoc + nl.ntype * 8);  // [type] projector slots in use
    int* styp = snp + nl.ntype;                               // [atom] type
    if (non_loc)
    {
        const double2* PK = proj + (size_t)P.kbz_kq * rows * nsets + (size_t)spin * sets;
        const double2* PKp = proj + (size_t)P.kbz_k * rows * nsets + (size_t)spin * sets;
        for (int e = threadIdx.x; e < rows * sets; e += blockDim.x)
        {
            const int r = e / sets, c = e - r * sets;
            const double2 k1 = PK[(size_t)r * nsets + c], k2 = PKp[(size_t)r * nsets + c];
            sK[e] = mk2<C2>(k1.x, k1.y);
            sKp[e] = mk2<C2>(k2.x, k2.y);
        }
        const double2* E = eig + (size_t)P.qslot * gd.nmodes * gd.nmodes;
        for (int e = threadIdx.x; e < gd.nmodes * nj; e += blockDim.x)
        {
            const double2 v = E[(e / nj) * gd.nmodes + (e % nj)];
            sE[e] = mk2<C2>(v.x, v.y);
        }
        for (int a = threadIdx.x; a < nl.natom; a += blockDim.x) styp[a] = nl.atom_type[a];
        if (threadIdx.x < nl.ntype)
        {
            const int it = threadIdx.x;
            int nc = 0, pb = 0;
            for (int lidx = 0; lidx < nl.nltimesj && nc < 8; ++lidx)
            {
                int l = (int)rint(nl.PP_table[(lidx * nl.ntype + it) * 3] - 1.0);
                if (l < 0) continue;
                int twoj = (int)rint(nl.PP_table[(lidx * nl.ntype + it) * 3 + 1]);
                int* ch = sch + (it * 8 + nc) * 4;
                ch[0] = lidx;
                ch[1] = l;
                ch[2] = pb;
                ch[3] = nl.fcoef ? nl.fcoef_off[lidx * nl.ntype + it] : -1;
                ssoc[it * 8 + nc] = (T)((twoj != 0 && !nl.is_soc) ? (twoj + 1.0) / (4.0 * l + 2.0) : 1.0);
                pb += 2 * l + 1;
                ++nc;
            }
            for (; nc < 8; ++nc) sch[(it * 8 + nc) * 4 + 1] = -1;
            snp[it] = pb;
        }
        __syncthreads();
        // The channel coefficients act on the k role alone, so they are folded
        // into its projections once per block, in place: for a channel of atom
        // a with slots pb .. pb + tl - 1,
        //   Z(p1, s1; m)   =  sum_{p2, s2} f(p1, p2, s1, s2) conj(Pi_0(p2, m, s2))
        //   W_x(p1, s1; m) = -sum_{p2, s2} f(p1, p2, s1, s2) conj(Pi_x(p2, m, s2))
        // (f diagonal, = the channel's weight, without SOC coefficients), so that
        //   out_{a,x}(m, n) = sum_{p1, s1} K_x(p1, n, s1) Z(p1, s1; m) + K_0(p1, n, s1) W_x(p1, s1; m)
        // with K the k+q role: the terms of src/nonloc/sum_VNL_KKp.c:8-58, regrouped.
        // One thread owns one (atom, channel, band, component) block, reads it
        // whole before writing it, and no other thread touches it.
        for (int w = threadIdx.x; w < nl.natom * 8 * nb * 4; w += blockDim.x)
        {
            const int comp = w & 3, r = w >> 2;
            const int a = r / (8 * nb), r2 = r - a * 8 * nb, c = r2 / nb, mm = r2 - c * nb;
            const int it = styp[a];
            const int* ch = sch + (it * 8 + c) * 4;
            const int l = ch[1];
            if (l < 0) continue;
            const int tl = 2 * l + 1, pb = ch[2], foff = ch[3];
            C2* blk = sKp + (size_t)(a * nl.nproj_max * 4 + pb * 4 + comp) * sets + mm * ns;  // slot stride 4 sets
            const T sg = comp ? (T)-1 : (T)1;
            if (foff < 0)
            {
                const T wgt = ssoc[it * 8 + c] * sg;
                for (int im = 0; im < tl; ++im)
                    for (int sp = 0; sp < ns; ++sp)
                    {
                        const C2 v = blk[(size_t)im * 4 * sets + sp];
                        blk[(size_t)im * 4 * sets + sp] = mk2<C2>(wgt * v.x, -wgt * v.y);
                    }
            }
            else
            {
                C2 vin[14];  // tl * ns <= 7 * 2 (l <= 3 is checked at context creation)
                for (int im = 0; im < tl; ++im)
                    for (int sp = 0; sp < ns; ++sp) vin[im * ns + sp] = cconj(blk[(size_t)im * 4 * sets + sp]);
                for (int im1 = 0; im1 < tl; ++im1)
                    for (int s1 = 0; s1 < ns; ++s1)
                    {
                        C2 acc = mk2<C2>(0.0, 0.0);
                        for (int im2 = 0; im2 < tl; ++im2)
                            for (int s2 = 0; s2 < ns; ++s2)
                            {
                                const double* fc = nl.fcoef + 2 * ((size_t)foff + (im1 * tl + im2) * ns * ns + s1 * ns + s2);
                                acc = cadd(acc, cmul(mk2<C2>(fc[0], fc[1]), vin[im2 * ns + s2]));
                            }
                        blk[(size_t)im1 * 4 * sets + s1] = mk2<C2>(sg * acc.x, sg * acc.y);
                    }
            }
        }
        __syncthreads();
    }
    const double invN = 1.0 / ((double)gd.Nx * gd.Ny * gd.Nz);
    const float invN_hi = (float)invN, invN_lo = (float)(invN - (double)invN_hi);  // 1/M as a float pair
    const int NT = 2 * gd.nbp;
    const double2 pre = make_double2(0.0, -2.0 * LELPH_PI_T * LELPH_E2);
    const C2 preT = mk2<C2>(0.0, -2.0 * LELPH_PI_T * LELPH_E2);
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x)
    {
        const int m = e / nb, n = e - m * nb;  // m: band of k, n: band of k+q
        C2 out[NJ];
#pragma unroll
        for (int j = 0; j < NJ; ++j) out[j] = mk2<C2>(0.0, 0.0);
        if (non_loc)
        {
#pragma unroll
            for (int a = 0; a < NJ / 3; ++a)
            {
                if (a >= nl.natom) break;
                const int np = snp[styp[a]];
                const C2* kq = sK + (size_t)a * nl.nproj_max * 4 * sets + n * ns;  // K(slot, comp; n)
                const C2* kk = sKp + (size_t)a * nl.nproj_max * 4 * sets + m * ns;  // Z, W_x(slot; m)
                C2 a0 = mk2<C2>(0.0, 0.0), a1 = a0, a2 = a0;
                for (int p = 0; p < np; ++p)
                    for (int sp = 0; sp < ns; ++sp)
                    {
                        const size_t o = (size_t)p * 4 * sets + sp;
                        const C2 K0 = kq[o], Z = kk[o];
                        a0 = cadd(a0, cadd(cmul(kq[o + sets], Z), cmul(K0, kk[o + sets])));
                        a1 = cadd(a1, cadd(cmul(kq[o + 2 * sets], Z), cmul(K0, kk[o + 2 * sets])));
                        a2 = cadd(a2, cadd(cmul(kq[o + 3 * sets], Z), cmul(K0, kk[o + 3 * sets])));
                    }
                out[3 * a] = a0;
                out[3 * a + 1] = a1;
                out[3 * a + 2] = a2;
            }
        }
        if (mode_fp64)
        {
            for (int nu = 0; nu < gd.nmodes; ++nu)
            {
                const size_t oidx = ((((size_t)pair * gd.nmodes + nu) * gd.nspin + spin) * nb + m) * nb + n;
                double2 v = glocal[((size_t)zp * gd.nmodes * nb + nu * nb + m) * nb + n];
                if (non_loc)
                {
                    C2 sacc = mk2<C2>(0.0, 0.0);
#pragma unroll
                    for (int j = 0; j < NJ; ++j)
                        if (j < nj) sacc = cadd(sacc, cmul(sE[nu * nj + j], out[j]));
                    v = cadd(v, cmul(pre, make_double2((double)sacc.x, (double)sacc.y)));
                }
                if (out_c64)
                    reinterpret_cast<float2*>(gout)[oidx] = make_float2((float)v.x, (float)v.y);
                else
                    reinterpret_cast<double2*>(gout)[oidx] = v;
            }
            continue;
        }
        // mixed form: the K-chunk partials are summed in FP32 with TwoSum
        // compensation (the pair (s, e) holds the sum to about twice FP32's
        // precision), two modes at a time so that 16 loads are in flight, then
        // unscaled (exact inverse of the power-of-two operand scales, 1/M as a
        // float pair) and added to the nonlocal term with error-free
        // transformations: the complex64 result is rounded once, without FP64
        // arithmetic (GB300's FP64 rate is 1/64 of FP32's)
        const float bsc = band_scale[((size_t)P.kbz_k * gd.nspin + spin) * nb + m] *
                          band_scale[((size_t)P.kbz_kq * gd.nspin + spin) * nb + n];
        const float* msc = mode_scale + (size_t)P.dvslot * gd.nmodes;
        const size_t CS = (size_t)128 * NT;  // stride of one K chunk
        for (int nu0 = 0; nu0 < gd.nmodes; nu0 += 2)
        {
            // an odd mode count reads the last mode twice and stores it once
            const int nu1 = min(nu0 + 1, gd.nmodes - 1);
            const int mt0 = nu0 / gd.mt_modes, mt1 = nu1 / gd.mt_modes;
            const float* pa = partials + lelph_tc_partial_offset(gd, nchunks, zp, mt0, 0, (nu0 - mt0 * gd.mt_modes) * nb + m);
            const float* pb = partials + lelph_tc_partial_offset(gd, nchunks, zp, mt1, 0, (nu1 - mt1 * gd.mt_modes) * nb + m);
            float sv[4] = {0.f, 0.f, 0.f, 0.f}, ev[4] = {0.f, 0.f, 0.f, 0.f};  // re, im of nu0; re, im of nu1
            int c = 0;
            for (; c + 4 <= nchunks; c += 4)
            {
                float x[4][4];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                {
                    x[u][0] = pa[(size_t)(c + u) * CS + n];
                    x[u][1] = pa[(size_t)(c + u) * CS + gd.nbp + n];
                    x[u][2] = pb[(size_t)(c + u) * CS + n];
                    x[u][3] = pb[(size_t)(c + u) * CS + gd.nbp + n];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int v = 0; v < 4; ++v) ff_two_sum(sv[v], ev[v], x[u][v]);
            }
            for (; c < nchunks; ++c)
            {
                ff_two_sum(sv[0], ev[0], pa[(size_t)c * CS + n]);
                ff_two_sum(sv[1], ev[1], pa[(size_t)c * CS + gd.nbp + n]);
                ff_two_sum(sv[2], ev[2], pb[(size_t)c * CS + n]);
                ff_two_sum(sv[3], ev[3], pb[(size_t)c * CS + gd.nbp + n]);
            }
#pragma unroll
            for (int hm = 0; hm < 2; ++hm)
            {
                const int nu = hm ? nu1 : nu0;
                if (hm && nu1 == nu0) break;
                const size_t oidx = ((((size_t)pair * gd.nmodes + nu) * gd.nspin + spin) * nb + m) * nb + n;
                float tr = 0.f, ti = 0.f;
                if (non_loc)
                {
                    C2 sacc = mk2<C2>(0.0, 0.0);
#pragma unroll
                    for (int j = 0; j < NJ; ++j)
                        if (j < nj) sacc = cadd(sacc, cmul(sE[nu * nj + j], out[j]));
                    const C2 t = cmul(preT, sacc);
                    tr = (float)t.x;
                    ti = (float)t.y;
                }
                const float p2 = 1.0f / (msc[nu] * bsc);  // a power of two: exact
                if (out_c64)
                {
                    const float fh = invN_hi * p2, fl = invN_lo * p2;  // exact scalings
                    reinterpret_cast<float2*>(gout)[oidx] =
                        make_float2(ff_scale_add(sv[2 * hm], ev[2 * hm], fh, fl, tr),
                                    ff_scale_add(sv[2 * hm + 1], ev[2 * hm + 1], fh, fl, ti));
                }
                else
                {
                    const double f = invN * (double)p2;
                    reinterpret_cast<double2*>(gout)[oidx] =
                        make_double2(((double)sv[2 * hm] + (double)ev[2 * hm]) * f + (double)tr,
                                     ((double)sv[2 * hm + 1] + (double)ev[2 * hm + 1]) * f + (double)ti);
                }
            }
        }
    }
}

static size_t finish_pair_smem(const NonlocalDesc& nl, const GeomDev& g, size_t csz)
{
    const size_t rows = (size_t)nl.natom * nl.nproj_max * 4;
    const size_t sets = (size_t)g.nbnds * g.nspinor;
    return 2 * rows * sets * csz + (size_t)g.nmodes * 3 * nl.natom * csz + (size_t)nl.ntype * 8 * 4 * sizeof(int) +
           (size_t)nl.ntype * 8 * sizeof(double) + (size_t)(nl.ntype + nl.natom) * sizeof(int);
}

// Finish for many displacement components (3 natom > 24, where the
// per-pair form's projection sets overflow shared memory): one CTA per
// (16 x 16 band tile, pair, spin); the projections of the tile's 16 bands
// of k and 16 bands of k+q, the pair's eigVec and the channel table sit in
// shared memory; each thread owns one (m, n) and keeps its NJ displacement
// sums in registers, then applies the mode transform.  glocal (FP64 local
// term) is added in FP64; T is the arithmetic of the nonlocal term.
#define FT_B 16
template <int NJ, typename T>
__global__ void __launch_bounds__(FT_B * FT_B) k_finish_tile(const PairInfo* __restrict__ pairs,
                                                             const double2* __restrict__ glocal,
                                                             const double2* __restrict__ proj,
                                                             const double2* __restrict__ eig, int non_loc,
                                                             NonlocalDesc nl, GeomDev gd, int out_c64,
                                                             void* __restrict__ gout)
{
    typedef typename cplx_of<T>::type C2;
    extern __shared__ __align__(16) unsigned char ftsm[];
    const int ntile = (gd.nbnds + FT_B - 1) / FT_B;
    const int tm = blockIdx.x / ntile, tn = blockIdx.x - tm * ntile;
    const int zp = blockIdx.y;
    const int pair = zp / gd.nspin, spin = zp - pair * gd.nspin;
    const PairInfo P = pairs[pair];
    const int nb = gd.nbnds, ns = gd.nspinor;
    const int nsets = gd.nspin * nb * ns;
    const int rows = nl.natom * nl.nproj_max * 4;
    const int nj = 3 * nl.natom;
    const int sets = FT_B * ns;                               // the tile's sets of one role
    C2* sK = reinterpret_cast<C2*>(ftsm);                    // [rows][sets]  role k+q (bands n0 ..)
    C2* sKp = sK + (size_t)rows * sets;                      // [rows][sets]  role k (bands m0 ..)
    C2* sE = sKp + (size_t)rows * sets;                      // [nmodes][nj]
    int* sch = reinterpret_cast<int*>(sE + (size_t)gd.nmodes * nj);
    T* ssoc = reinterpret_cast<T*>(sch + nl.ntype * 8 * 4);
    const int m0 = tm * FT_B, n0 = tn * FT_B;
    if (non_loc)
    {
        const double2* PK = proj + (size_t)P.kbz_kq * rows * nsets + (size_t)spin * nb * ns;
        const double2* PKp = proj + (size_t)P.kbz_k * rows * nsets + (size_t)spin * nb * ns;
        for (int e = threadIdx.x; e < rows * sets; e += blockDim.x)
        {
            const int r = e / sets, c = e - r * sets;
            const int bn = n0 * ns + c, bm = m0 * ns + c;
            const double2 k1 = bn < nb * ns ? PK[(size_t)r * nsets + bn] : make_double2(0.0, 0.0);
            const double2 k2 = bm < nb * ns ? PKp[(size_t)r * nsets + bm] : make_double2(0.0, 0.0);
            sK[e] = mk2<C2>(k1.x, k1.y);
            sKp[e] = mk2<C2>(k2.x, k2.y);
        }
        const double2* E = eig + (size_t)P.qslot * gd.nmodes * gd.nmodes;
        for (int e = threadIdx.x; e < gd.nmodes * nj; e += blockDim.x)
        {
            const double2 v = E[(e / nj) * gd.nmodes + (e % nj)];
            sE[e] = mk2<C2>(v.x, v.y);
        }
        if (threadIdx.x < nl.ntype)
        {
            const int it = threadIdx.x;
            int nc = 0, pb = 0;
            for (int lidx = 0; lidx < nl.nltimesj && nc < 8; ++lidx)
            {
                int l = (int)rint(nl.PP_table[(lidx * nl.ntype + it) * 3] - 1.0);
                if (l < 0) continue;
                int twoj = (int)rint(nl.PP_table[(lidx * nl.ntype + it) * 3 + 1]);
                int* ch = sch + (it * 8 + nc) * 4;
                ch[0] = lidx;
                ch[1] = l;
                ch[2] = pb;
                ch[3] = nl.fcoef ? nl.fcoef_off[lidx * nl.ntype + it] : -1;
                ssoc[it * 8 + nc] = (T)((twoj != 0 && !nl.is_soc) ? (twoj + 1.0) / (4.0 * l + 2.0) : 1.0);
                pb += 2 * l + 1;
                ++nc;
            }
            for (; nc < 8; ++nc) sch[(it * 8 + nc) * 4 + 1] = -1;
        }
    }
    __syncthreads();
    const int ml = threadIdx.x / FT_B, nlc = threadIdx.x - ml * FT_B;
    const int m = m0 + ml, n = n0 + nlc;  // m: band of k, n: band of k+q
    if (m >= nb || n >= nb) return;
    C2 out[NJ];
#pragma unroll
    for (int j = 0; j < NJ; ++j) out[j] = mk2<C2>(0.0, 0.0);
    if (non_loc)
    {
#pragma unroll
        for (int j = 0; j < NJ; ++j)
        {
            if (j >= nj) continue;
            const int a = j / 3, x = j - 3 * a;
            const int it = nl.atom_type[a];
            const int rb = a * nl.nproj_max * 4;
            C2 acc = mk2<C2>(0.0, 0.0);
            for (int c = 0; c < 8; ++c)
            {
                const int* ch = sch + (it * 8 + c) * 4;
                const int l = ch[1];
                if (l < 0) break;
                const int tl = 2 * l + 1, pb = ch[2], foff = ch[3];
                const T soc = ssoc[it * 8 + c];
                for (int im1 = 0; im1 < tl; ++im1)
                    for (int im2 = 0; im2 < tl; ++im2)
                    {
                        if (foff < 0 && im1 != im2) continue;
                        const int p1 = pb + im1, p2 = pb + im2;
                        for (int s1 = 0; s1 < ns; ++s1)
                            for (int s2 = 0; s2 < ns; ++s2)
                            {
                                C2 f;
                                if (foff >= 0)
                                {
                                    const double* fc = nl.fcoef + 2 * ((size_t)foff + (im1 * tl + im2) * ns * ns + s1 * ns + s2);
                                    f = mk2<C2>(fc[0], fc[1]);
                                }
                                else
                                {
                                    if (s1 != s2) continue;
                                    f.x = soc;
                                    f.y = 0;
                                }
                                const C2 K0 = sK[(size_t)(rb + p1 * 4 + 0) * sets + nlc * ns + s1];
                                const C2 Kx = sK[(size_t)(rb + p1 * 4 + 1 + x) * sets + nlc * ns + s1];
                                const C2 Kp0 = cconj(sKp[(size_t)(rb + p2 * 4 + 0) * sets + ml * ns + s2]);
                                C2 Kpx = sKp[(size_t)(rb + p2 * 4 + 1 + x) * sets + ml * ns + s2];
                                Kpx.x = -Kpx.x;  // -conj
                                acc = cadd(acc, cmul(f, cadd(cmul(Kx, Kp0), cmul(K0, Kpx))));
                            }
                    }
            }
            out[j] = acc;
        }
    }
    const double2 pre = make_double2(0.0, -2.0 * LELPH_PI_T * LELPH_E2);
    for (int nu = 0; nu < gd.nmodes; ++nu)
    {
        const size_t oidx = ((((size_t)pair * gd.nmodes + nu) * gd.nspin + spin) * nb + m) * nb + n;
        double2 v = glocal[((size_t)zp * gd.nmodes * nb + nu * nb + m) * nb + n];
        if (non_loc)
        {
            C2 sacc = mk2<C2>(0.0, 0.0);
#pragma unroll
            for (int j = 0; j < NJ; ++j)
                if (j < nj) sacc = cadd(sacc, cmul(sE[nu * nj + j], out[j]));
            v = cadd(v, cmul(pre, make_double2((double)sacc.x, (double)sacc.y)));
        }
        if (out_c64)
            reinterpret_cast<float2*>(gout)[oidx] = make_float2((float)v.x, (float)v.y);
        else
            reinterpret_cast<double2*>(gout)[oidx] = v;
    }
}

static size_t finish_tile_smem(const NonlocalDesc& nl, const GeomDev& g, size_t csz)
{
    const size_t rows = (size_t)nl.natom * nl.nproj_max * 4;
    const size_t sets = (size_t)FT_B * g.nspinor;
    return 2 * rows * sets * csz + (size_t)g.nmodes * 3 * nl.natom * csz + (size_t)nl.ntype * 8 * 4 * sizeof(int) +
           (size_t)nl.ntype * 8 * sizeof(double);
}

void lelph_launch_finish(const PairInfo* pairs, int npairs, int mode_fp64, const double2* glocal,
                         const float* partials, int nchunks, const float* mode_scale, const float* band_scale,
                         const double2* proj, const double2* eig, int non_loc, const NonlocalDesc& nl,
                         const GeomDev& g, int out_c64, void* gout, cudaStream_t st)
{
    // mode_fp64: 0 = K-chunk partials (mixed real-space route), 1 = FP64 local
    // term and FP64 nonlocal arithmetic (plain form), 2 = FP64 local term and
    // FP32 nonlocal arithmetic (mixed form on the G-space route)
    const bool t64 = mode_fp64 == 1;
    const size_t smem = finish_pair_smem(nl, g, t64 ? sizeof(double2) : sizeof(float2));
    const int nj = 3 * nl.natom;
    if (smem <= 160 * 1024 && nj <= 24)
    {
        static bool attr = false;
        if (!attr)
        {
            cudaFuncSetAttribute(k_finish_pair<12, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
            cudaFuncSetAttribute(k_finish_pair<24, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
            cudaFuncSetAttribute(k_finish_pair<12, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
            cudaFuncSetAttribute(k_finish_pair<24, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
            attr = true;
        }
        const int nz = npairs * g.nspin;
#define FINL(NJ, T)                                                                                              \
    k_finish_pair<NJ, T><<<nz, NJ <= 12 ? 256 : 128, smem, st>>>(pairs, mode_fp64, glocal, partials, nchunks,    \
                                                                  mode_scale, band_scale, proj, eig, non_loc, nl, g, \
                                                                  out_c64, gout)
        if (t64)
        {
            if (nj <= 12) FINL(12, double);
            else FINL(24, double);
        }
        else
        {
            if (nj <= 12) FINL(12, float);
            else FINL(24, float);
        }
#undef FINL
        return;
    }
    const size_t tsm = finish_tile_smem(nl, g, t64 ? sizeof(double2) : sizeof(float2));
    if (mode_fp64 && nj <= 48 && tsm <= 200 * 1024)
    {
        static bool tattr = false;
        if (!tattr)
        {
            cudaFuncSetAttribute(k_finish_tile<48, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            cudaFuncSetAttribute(k_finish_tile<48, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            tattr = true;
        }
        const int nt = (g.nbnds + FT_B - 1) / FT_B;
        dim3 tg((unsigned)(nt * nt), (unsigned)(npairs * g.nspin));
        if (t64)
            k_finish_tile<48, double><<<tg, FT_B * FT_B, tsm, st>>>(pairs, glocal, proj, eig, non_loc, nl, g, out_c64,
                                                                  gout);
        else
            k_finish_tile<48, float><<<tg, FT_B * FT_B, tsm, st>>>(pairs, glocal, proj, eig, non_loc, nl, g, out_c64,
                                                                 gout);
        return;
    }
    dim3 grid((g.nbnds * g.nbnds + FIN_MN - 1) / FIN_MN, npairs * g.nspin);
    k_finish<<<grid, 256, 0, st>>>(pairs, mode_fp64, glocal, partials, nchunks, mode_scale, band_scale, proj, eig,
                                   non_loc, nl, g, out_c64, gout);
}
