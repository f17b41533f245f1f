/* compute_and_write_elphq on the GB300 library: the binding a maintainer of
 * LetzElPhC compiles in place of src/elph/compute_elph_matq.c.
 *
 * Same symbol and signature as the reference's per-q stage
 * (src/elph/elph.h:10-17), the same inputs (struct WFC / Lattice / Pseudo /
 * Phonon, eigVec, dVscfq) and the same outputs: elph_mat[qpos + star member]
 * [k] slices written through nc_put_vara with the reference's start/count
 * (src/elph/compute_elph_matq.c:82-85,145-152,206-214), Dmats read through
 * nc_get_vara where the star expansion needs them.  The reference's callers
 * (elph_driver, src/elph/elph_driver.c:303-306) are unchanged.
 *
 * * The first call builds a device context from the wavefunctions, lattice and
 *   pseudopotential tables (they do not change between q-points) and keeps it
 *   for the following calls; a call with other wavefunction arrays rebuilds it.
 *   The context is released at exit.
 * * Precision follows the reference's build: with -DCOMPILE_ELPH_DOUBLE the
 *   arrays are handed over as they are and the library's FP64 form runs; in
 *   the default single-precision build every real and complex input is widened
 *   to double once (the library's ABI is double) and the library's mixed form
 *   runs (FP32 FFTs, split-f16 tensor cores), whose error against FP64 is below
 *   that of the reference's own single-precision build; the output is narrowed
 *   back to float complex.  LELPH_GPU_PRECISION=fp64|f16|bf16 overrides.
 * * k pools: this process computes the k-points of its pool, split as the
 *   reference splits them (distribute_to_grps, compute_elph_matq.c:51-54).
 *   With one pool the q-star expansion runs on the device with Dmats computed
 *   there (lelph_gpu_compute_elphq_star); with several, the pool's k-points
 *   are computed and rotated with the Dmats read from ndb.Dmats, as the
 *   reference does (compute_elph_matq.c:159-217).  Plane waves must not be
 *   split inside a pool (commK of one rank): one GPU holds a whole pair.
 * * Errors: a nonzero status of the library goes to error_msg (the reference's
 *   abort path, src/common/error.c:8-21) with the library's message.
 *
 * Build: add -I<repo>/include to CFLAGS and -L<repo>/letzelphc_gb300/_lib
 * -llelph_gpu (with an rpath) to the link, and compile this file instead of
 * src/elph/compute_elph_matq.c. */
#include <complex.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mpi.h>
#include <netcdf.h>

#include "common/dtypes.h"
#include "common/error.h"
#include "common/numerical_func.h"
#include "common/parallel.h"
#include "elph/elph.h"
#include "elphC.h"
#include "lelph_gpu.h"

static lelph_gpu* g_ctx = NULL;
static const struct WFC* g_wfcs = NULL;  /* the wavefunction array the context was built from */
static ELPH_cmplx* g_wfc0 = NULL;

static void gpu_check(int st)
{
    if (st == LELPH_GPU_OK) return;
    char msg[640];
    snprintf(msg, sizeof msg, "GB300 elph stage: %s (%s)", lelph_gpu_strerror(st),
             g_ctx ? lelph_gpu_last_error(g_ctx) : "no context");
    error_msg(msg);
}

static void* xmalloc(size_t n)
{
    void* p = malloc(n ? n : 1);
    if (!p) error_msg("GB300 elph stage: out of host memory");
    return p;
}

/* double copy of n reals (a fresh array; the caller frees it) */
static double* widen(const ELPH_float* x, size_t n)
{
    double* y = xmalloc(sizeof(double) * n);
    for (size_t i = 0; i < n; ++i) y[i] = (double)x[i];
    return y;
}

/* inputs in the library's (double) types: the arrays themselves in the double
 * build, widened copies in the single-precision build */
static const double* as_double(const ELPH_float* x, size_t n, double** own)
{
    if (sizeof(ELPH_float) == sizeof(double) || !x)
    {
        *own = NULL;
        return (const double*)x;
    }
    *own = widen(x, n);
    return *own;
}

static void release_context(void)
{
    if (g_ctx) lelph_gpu_destroy(g_ctx);
    g_ctx = NULL;
}

static int precision_of_build(void)
{
    const char* e = getenv("LELPH_GPU_PRECISION");
    if (e && !strcmp(e, "fp64")) return LELPH_GPU_FP64;
    if (e && !strcmp(e, "f16")) return LELPH_GPU_MIXED_F16;
    if (e && !strcmp(e, "bf16")) return LELPH_GPU_MIXED_BF16;
    return sizeof(ELPH_float) == sizeof(double) ? LELPH_GPU_FP64 : LELPH_GPU_MIXED_F16;
}

static void build_context(const struct WFC* wfcs, const struct Lattice* lat, const struct Pseudo* ps)
{
    release_context();
    const int nk = (int)lat->nkpts_iBZ, nsym = lat->nsym;
    const size_t nfc = (size_t)ps->nltimesj * ps->ntype;
    int* npw = xmalloc(sizeof(int) * nk);
    const double** gv = xmalloc(sizeof(double*) * nk);
    const double** wf = xmalloc(sizeof(double*) * nk);
    const double** fk = xmalloc(sizeof(double*) * nk);
    double** own = xmalloc(sizeof(double*) * (3 * (size_t)nk + nfc + 16));
    size_t nown = 0;
    for (int ik = 0; ik < nk; ++ik)
    {
        if (wfcs[ik].npw_loc != wfcs[ik].npw_total)
            error_msg("GB300 elph stage: plane waves split inside a k pool (one rank per pool is required)");
        const size_t n = (size_t)wfcs[ik].npw_total;
        npw[ik] = (int)n;
        const size_t nset = (size_t)lat->nspin * lat->nbnds * lat->nspinor;
        gv[ik] = as_double(wfcs[ik].gvec, 3 * n, &own[nown++]);
        wf[ik] = as_double((const ELPH_float*)wfcs[ik].wfc, 2 * nset * n, &own[nown++]);
        fk[ik] = as_double(wfcs[ik].Fk, nfc * n, &own[nown++]);
    }
    double* R = xmalloc(sizeof(double) * 9 * (size_t)nsym);
    double* tau = xmalloc(sizeof(double) * 3 * (size_t)nsym);
    int* trev = xmalloc(sizeof(int) * (size_t)nsym);
    for (int i = 0; i < nsym; ++i)
    {
        for (int x = 0; x < 9; ++x) R[9 * i + x] = lat->syms[i].Rmat[x];
        for (int x = 0; x < 3; ++x) tau[3 * i + x] = lat->syms[i].tau[x];
        trev[i] = lat->syms[i].time_rev;
    }
    double alat[9], blat[9];
    for (int x = 0; x < 9; ++x)
    {
        alat[x] = lat->alat_vec[x];
        blat[x] = lat->blat_vec[x];
    }
    const double** fc = NULL;
    if (ps->fCoeff)
    {
        fc = xmalloc(sizeof(double*) * nfc);
        for (size_t i = 0; i < nfc; ++i)
        {
            if (!ps->fCoeff[i])
            {
                fc[i] = NULL;
                continue;
            }
            /* (2l+1, 2l+1, nspinor, nspinor) complex, l from PP_table's l+1 */
            const int l = (int)(ps->PP_table[3 * i] - 1 + 0.5);
            const size_t n = 2 * (size_t)(2 * l + 1) * (2 * l + 1) * lat->nspinor * lat->nspinor;
            fc[i] = as_double((const ELPH_float*)ps->fCoeff[i], n, &own[nown++]);
        }
    }
    double *o1, *o2, *o3, *o4, *o5, *o6, *o7;
    lelph_gpu_desc d;
    memset(&d, 0, sizeof d);
    d.natom = lat->natom;
    d.nsym = nsym;
    d.timerev = lat->timerev;
    d.nspin = lat->nspin;
    d.nspinor = lat->nspinor;
    d.nbnds = lat->nbnds;
    d.nmag = (int)lat->nmag;
    d.nmodes = (int)lat->nmodes;
    d.nkpts_iBZ = nk;
    d.nkpts_BZ = (int)lat->nkpts_BZ;
    for (int x = 0; x < 3; ++x) d.fft_dims[x] = (int)lat->fft_dims[x];
    d.alat_vec = alat;
    d.blat_vec = blat;
    d.atomic_pos = as_double(lat->atomic_pos, 3 * (size_t)lat->natom, &o1);
    d.atom_type = lat->atom_type;
    d.kpt_iredBZ = as_double(lat->kpt_iredBZ, 3 * (size_t)nk, &o2);
    d.kpt_fullBZ_crys = as_double(lat->kpt_fullBZ_crys, 3 * (size_t)lat->nkpts_BZ, &o3);
    d.kmap = lat->kmap;
    d.sym_Rmat = R;
    d.sym_tau = tau;
    d.sym_time_rev = trev;
    d.is_soc_present = lat->is_soc_present;
    d.npw = npw;
    d.gvec = gv;
    d.wfc = wf;
    d.Fk = fk;
    d.ntype = (int)ps->ntype;
    d.nltimesj = (int)ps->nltimesj;
    d.lmax = ps->lmax;
    d.PP_table = as_double(ps->PP_table, 3 * nfc, &o4);
    d.Fsign = as_double(ps->Fsign, nfc, &o5);
    d.fCoeff = fc;
    d.precision = precision_of_build();
    d.device = 0;
    d.route = LELPH_GPU_ROUTE_AUTO;
    o6 = o7 = NULL;
    gpu_check(lelph_gpu_create(&d, &g_ctx));  /* the library copies every input to the device */
    double* tmp[] = {o1, o2, o3, o4, o5, o6, o7};
    for (size_t i = 0; i < sizeof tmp / sizeof tmp[0]; ++i) free(tmp[i]);
    for (size_t i = 0; i < nown; ++i) free(own[i]);
    free(own);
    free(fc);
    free(npw);
    free(gv);
    free(wf);
    free(fk);
    free(R);
    free(tau);
    free(trev);
    g_wfcs = wfcs;
    g_wfc0 = wfcs[0].wfc;
    static bool registered = false;
    if (!registered)
    {
        atexit(release_context);
        registered = true;
    }
}

/* one matrix-element slice (nmodes, nspin, nb, nb) from the library's complex128 into ELPH_cmplx */
static void narrow(const double* g, size_t n, ELPH_cmplx* out)
{
    for (size_t i = 0; i < n; ++i) out[i] = (ELPH_float)g[2 * i] + (ELPH_float)g[2 * i + 1] * I;
}

static void put_slice(int ncid, int varid, size_t q, size_t k, const struct Lattice* lat, const double* g,
                      ELPH_cmplx* buf)
{
    size_t startp[7] = {q, k, 0, 0, 0, 0, 0};
    size_t countp[7] = {1, 1, (size_t)lat->nmodes, (size_t)lat->nspin, (size_t)lat->nbnds, (size_t)lat->nbnds, 2};
    const size_t n = (size_t)lat->nmodes * lat->nspin * lat->nbnds * lat->nbnds;
    const void* src = g;
    if (sizeof(ELPH_float) != sizeof(double))
    {
        narrow(g, n, buf);
        src = buf;
    }
    int e = nc_put_vara(ncid, varid, startp, countp, src);
    if (e) ERR(e);
}

void compute_and_write_elphq(struct WFC* wfcs, struct Lattice* lattice, struct Pseudo* pseudo,
                             struct Phonon* phonon, const ND_int iqpt, ELPH_cmplx* eigVec, ELPH_cmplx* dVscfq,
                             const int ncid_elph, const int varid_elph, const int ncid_dmat, const int varid_dmat,
                             const bool non_loc, const bool kminusq, const struct ELPH_MPI_Comms* Comm)
{
    if (Comm->commK_size != 1)
        error_msg("GB300 elph stage: one rank per k pool (plane waves are not split across ranks)");
    if (!g_ctx || g_wfcs != wfcs || g_wfc0 != wfcs[0].wfc) build_context(wfcs, lattice, pseudo);

    const ND_int nk = lattice->nkpts_BZ;
    const size_t slice = (size_t)lattice->nmodes * lattice->nspin * lattice->nbnds * lattice->nbnds;
    ND_int qpos = 0;
    for (ND_int i = 0; i < iqpt; ++i) qpos += phonon->nqstar[i];
    if (phonon->qmap[2 * qpos] != iqpt || phonon->qmap[2 * qpos + 1] != 0)
        error_msg("Qpoint in iBZ cannot be traced in phonon qmap");
    ND_int kshift;
    const ND_int nk_pool = distribute_to_grps(nk, Comm->nkpools, Comm->commQ_rank / Comm->commK_size, &kshift);
    if (nk_pool < 1) error_msg("There are no kpoints in some cpus, Make sure nkpool < # of kpoints in full BZ.");

    const int nstar = (int)phonon->nqstar[iqpt];
    const size_t nv = (size_t)lattice->nmodes * lattice->nmag * lattice->fft_dims[0] * lattice->fft_dims[1] *
                      lattice->fft_dims[2];
    double q[3];
    for (int x = 0; x < 3; ++x) q[x] = phonon->qpts_iBZ[3 * iqpt + x];
    double *own_e, *own_v;
    const double* eig = as_double((const ELPH_float*)eigVec, 2 * (size_t)lattice->nmodes * lattice->nmodes, &own_e);
    const double* dv = as_double((const ELPH_float*)dVscfq, 2 * nv, &own_v);
    ELPH_cmplx* nbuf = sizeof(ELPH_float) != sizeof(double) ? xmalloc(sizeof(ELPH_cmplx) * slice) : NULL;

    if (Comm->nkpools == 1)
    {
        /* every k of the full BZ and every star member on the device */
        const int nps = (int)phonon->nph_sym;
        double* R = xmalloc(sizeof(double) * 9 * (size_t)nps);
        double* tau = xmalloc(sizeof(double) * 3 * (size_t)nps);
        int* trev = xmalloc(sizeof(int) * (size_t)nps);
        int* ssym = xmalloc(sizeof(int) * (size_t)nstar);
        for (int i = 0; i < nps; ++i)
        {
            for (int x = 0; x < 9; ++x) R[9 * i + x] = phonon->ph_syms[i].Rmat[x];
            for (int x = 0; x < 3; ++x) tau[3 * i + x] = phonon->ph_syms[i].tau[x];
            trev[i] = phonon->ph_syms[i].time_rev;
        }
        for (int s = 0; s < nstar; ++s) ssym[s] = phonon->qmap[2 * (qpos + s) + 1];
        double* g = xmalloc(sizeof(double) * 2 * slice * (size_t)nk * nstar);
        gpu_check(lelph_gpu_compute_elphq_star(g_ctx, q, eig, dv, non_loc, kminusq, nps, R, tau, trev, nstar, ssym,
                                               LELPH_GPU_OUT_C128, g));
        for (int s = 0; s < nstar; ++s)
            for (ND_int i = 0; i < nk; ++i)
                put_slice(ncid_elph, varid_elph, (size_t)(qpos + s), (size_t)i, lattice,
                          g + 2 * slice * ((size_t)s * nk + i), nbuf);
        free(g);
        free(R);
        free(tau);
        free(trev);
        free(ssym);
    }
    else
    {
        /* this pool's k-points; star members from the Dmats in ndb.Dmats */
        gpu_check(lelph_gpu_set_q(g_ctx, 0, q, eig, dv));
        int* qs = xmalloc(sizeof(int) * (size_t)nk_pool);
        int* ks = xmalloc(sizeof(int) * (size_t)nk_pool);
        for (ND_int i = 0; i < nk_pool; ++i)
        {
            qs[i] = 0;
            ks[i] = (int)(kshift + i);
        }
        double* g = xmalloc(sizeof(double) * 2 * slice * (size_t)nk_pool);
        gpu_check(lelph_gpu_run(g_ctx, (int)nk_pool, qs, ks, non_loc, kminusq, LELPH_GPU_OUT_C128, g));
        const size_t dsz = (size_t)lattice->nspin * lattice->nbnds * lattice->nbnds;
        ELPH_cmplx* Dl = nstar > 1 ? xmalloc(sizeof(ELPH_cmplx) * dsz) : NULL;
        ELPH_cmplx* Dr = nstar > 1 ? xmalloc(sizeof(ELPH_cmplx) * dsz) : NULL;
        double* Dld = nstar > 1 ? xmalloc(sizeof(double) * 2 * dsz) : NULL;
        double* Drd = nstar > 1 ? xmalloc(sizeof(double) * 2 * dsz) : NULL;
        double* gs = nstar > 1 ? xmalloc(sizeof(double) * 2 * slice) : NULL;
        int* kq = xmalloc(sizeof(int) * (size_t)nk);
        ELPH_float qt[3];
        for (int x = 0; x < 3; ++x) qt[x] = kminusq ? -phonon->qpts_iBZ[3 * iqpt + x] : phonon->qpts_iBZ[3 * iqpt + x];
        get_KplusQ_idxs(nk, lattice->kpt_fullBZ_crys, qt, kq);
        for (ND_int ii = 0; ii < nk_pool; ++ii)
        {
            const ND_int i = kshift + ii;
            const double* gi = g + 2 * slice * (size_t)ii;
            put_slice(ncid_elph, varid_elph, (size_t)qpos, (size_t)i, lattice, gi, nbuf);
            int idx_k = (int)i, idx_kq = kq[i];
            if (kminusq)
            {
                const int t = idx_k;
                idx_k = idx_kq;
                idx_kq = t;
            }
            for (int s = 1; s < nstar; ++s)
            {
                const int S = phonon->qmap[2 * (qpos + s) + 1];
                size_t sp[6] = {(size_t)S, (size_t)idx_kq, 0, 0, 0, 0};
                size_t cp[6] = {1, 1, (size_t)lattice->nspin, (size_t)lattice->nbnds, (size_t)lattice->nbnds, 2};
                int e = nc_get_vara(ncid_dmat, varid_dmat, sp, cp, Dl);
                if (e) ERR(e);
                sp[1] = (size_t)idx_k;
                e = nc_get_vara(ncid_dmat, varid_dmat, sp, cp, Dr);
                if (e) ERR(e);
                for (size_t j = 0; j < dsz; ++j)
                {
                    Dld[2 * j] = creal(Dl[j]);
                    Dld[2 * j + 1] = cimag(Dl[j]);
                    Drd[2 * j] = creal(Dr[j]);
                    Drd[2 * j + 1] = cimag(Dr[j]);
                }
                gpu_check(lelph_gpu_elph_q_rotate(g_ctx, Dld, gi, Drd, phonon->ph_syms[S].time_rev, gs));
                /* S k, as compute_elph_matq.c:190-205 finds it */
                ELPH_float Sk_cart[3], Sk_crys[3];
                MatVec3f(phonon->ph_syms[S].Rmat, lattice->kpt_fullBZ + 3 * i, false, Sk_cart);
                MatVec3f(lattice->alat_vec, Sk_cart, true, Sk_crys);
                const ND_int iSk = find_kidx_in_list(lattice->nkpts_BZ, lattice->kpt_fullBZ_crys, Sk_crys);
                if (iSk < 0) error_msg("Unable to to find S*k index This is due to incommenserate k and q grids.");
                put_slice(ncid_elph, varid_elph, (size_t)(qpos + s), (size_t)iSk, lattice, gs, nbuf);
            }
        }
        free(kq);
        free(gs);
        free(Dld);
        free(Drd);
        free(Dl);
        free(Dr);
        free(g);
        free(qs);
        free(ks);
    }
    free(nbuf);
    free(own_e);
    free(own_v);
}
