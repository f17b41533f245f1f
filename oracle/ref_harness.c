/* Oracle harness around the reference's own per-q stage.
 *
 * Loads a synthetic system written by letzelphc_gb300/synth.py:write_system,
 * fills the reference's boundary structs (struct WFC / Lattice / Pseudo /
 * Phonon / ELPH_MPI_Comms, src/common/dtypes.h) and calls the UNMODIFIED
 * compute_and_write_elphq (src/elph/compute_elph_matq.c:20) once per q, the
 * way elph_driver does (src/elph/elph_driver.c:303-306), with every q its own
 * star.  The netCDF writes of elph_mat are captured in memory and written out
 * as complex128 (nq, nk_BZ, nmodes, nspin, nb, nb).
 *
 * Timing samples: LELPH_REF_KPOOLS=P splits the full-BZ k-points into the
 * reference's P k pools and LELPH_REF_KPOOL=i makes this process pool i (pool
 * 0 by default); LELPH_REF_QPT=i runs only the i-th q of the file.
 *
 * usage: lelph_ref <system.bin> <g_out.bin> [rotate <D_in.bin> <g_rot_out.bin>]
 *        lelph_ref <system.bin> <g_out.bin> dvloc <v_out.bin>
 *        lelph_ref <system.bin> <unused> rotdv <spec.bin> <dv_out.bin>
 *        lelph_ref <system.bin> <unused> dmats <D_out.bin>
 *        lelph_ref <system.bin> <g_out.bin> star <star.bin>
 *        lelph_ref <system.bin> <unused> dvscf <spec.bin> <dvscf_file> <dv_out.bin>
 *
 * dvloc: the system's dVscf records are the induced part (QE's dvscf); the
 * harness builds the V_loc table (create_vlocg_table, src/dvloc/vlocg_table.c)
 * from the loc_* records, and per q runs dVlocq and add_dvscf_qe
 * (src/dvloc/dVbare_loc.c:16, src/dvloc/add_dvscf.c:12) the way elph_driver
 * does (src/elph/elph_driver.c:234-252) before compute_and_write_elphq.
 * v_out.bin receives, per q, Vlocr (nmodes, nfft) then the summed dV
 * (nmodes, nmag, nfft), complex128.
 *
 * rotdv: rotate_dvscf (src/symmetries/rotate_dvscf.c:22) of the spec's dV
 * (records rq, rR, rtau, rtrev, rcomp, rdv) on the system's lattice; the
 * matrix elements are not computed.
 *
 * dmats: electronic_reps (src/symmetries/elec_reps.c:16) for every symmetry of
 * the system and every full-BZ k, in the order of compute_and_write_dmats
 * (src/elph/compute_dmats.c:99-118); D_out.bin is complex128
 * (nsym, nk_BZ, nspin, nb, nb).  The matrix elements are not computed.
 *
 * star: q stars from star.bin (records nqstar: members per iBZ q, qsym: the
 * phonon symmetry of every member, identity first); the Dmats of every
 * (symmetry, k) are computed with electronic_reps and served to the stage's
 * reads, so compute_and_write_elphq expands each q over its star
 * (src/elph/compute_elph_matq.c:159-217); g_out.bin is (nq_BZ, nk_BZ, ...).
 *
 * dvscf: read_dvscf_qe (src/io/qe/read_dvscf.c:15-172) of dvscf_file (QE's
 * layout: (patterns, nmag, Nz, Ny, Nx) complex128) with the spec's eig and
 * pats records; dv_out.bin is the dV in the mode basis (nmodes, nmag, Nx, Ny, Nz).
 *
 * Built with -DCOMPILE_ELPH_DOUBLE (the parity build) every input is used as
 * written; built without it (the reference's default single-precision build,
 * src/elphC.h:21-31) every real and complex input is rounded once to float on
 * load, and g is widened back to complex128 on output.
 *
 * TEST INFRASTRUCTURE ONLY (the compiled reference is the checker's checker). */
#include <complex.h>
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "common/ELPH_timers.h"
#include "common/dtypes.h"
#include "dvloc/dvloc.h"
#include "elph/elph.h"
#include "io/qe/qe_io.h"
#include "netcdf.h"
#include "symmetries/symmetries.h"

struct rec
{
    char name[32];
    int code;
    unsigned ndim;
    long long dims[8];
    void* data;
    size_t nbytes;
};

static struct rec recs[4096];
static int nrec = 0;

static void die(const char* m)
{
    fprintf(stderr, "lelph_ref: %s\n", m);
    exit(2);
}

static void load(const char* path)
{
    FILE* f = fopen(path, "rb");
    if (!f) die("cannot open system file");
    char magic[8];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "LELPHSYS", 8)) die("bad magic");
    for (;;)
    {
        struct rec r;
        memset(&r, 0, sizeof(r));
        if (fread(r.name, 1, 32, f) != 32) die("truncated");
        if (!strcmp(r.name, "END")) break;
        if (fread(&r.code, 4, 1, f) != 1 || fread(&r.ndim, 4, 1, f) != 1) die("truncated");
        if (r.ndim > 8) die("ndim");
        if (fread(r.dims, 8, r.ndim, f) != r.ndim) die("truncated");
        size_t n = 1;
        for (unsigned i = 0; i < r.ndim; ++i) n *= (size_t)r.dims[i];
        size_t es = r.code == 0 ? 8 : (r.code == 1 ? 4 : 16);
        r.nbytes = n * es;
        r.data = malloc(r.nbytes ? r.nbytes : 1);
        if (fread(r.data, 1, r.nbytes, f) != r.nbytes) die("truncated data");
        if (sizeof(ELPH_float) == 4 && r.code != 1)
        {
            /* the reference's default build reads every real and complex
             * input in single precision: round each value once */
            const size_t nv = r.code == 0 ? n : 2 * n;
            const double* src = r.data;
            float* dst = malloc(nv * sizeof(float) + 1);
            if (!dst) die("out of memory");
            for (size_t i = 0; i < nv; ++i) dst[i] = (float)src[i];
            free(r.data);
            r.data = dst;
            r.nbytes = nv * sizeof(float);
        }
        if (nrec >= 4096) die("too many records");
        recs[nrec++] = r;
    }
    fclose(f);
}

static struct rec* get(const char* name, int required)
{
    for (int i = 0; i < nrec; ++i)
        if (!strcmp(recs[i].name, name)) return &recs[i];
    if (required)
    {
        fprintf(stderr, "missing record %s\n", name);
        exit(2);
    }
    return NULL;
}

/* elph_mat slices land here: (nq, nk, nmodes, nspin, nb, nb) */
static ELPH_cmplx* g_all = NULL;
static size_t g_slice = 0;
static size_t g_nk = 0;
/* Dmats served to nc_get_vara: (nsym, nk, nspin, nb, nb) */
static ELPH_cmplx* dmats = NULL;
static size_t dmat_slice = 0, dmat_nk = 0;

int nc_put_vara(int ncid, int varid, const size_t* startp, const size_t* countp, const void* op)
{
    (void)ncid; (void)varid; (void)countp;
    memcpy(g_all + (startp[0] * g_nk + startp[1]) * g_slice, op, sizeof(ELPH_cmplx) * g_slice);
    return 0;
}

int nc_get_vara(int ncid, int varid, const size_t* startp, const size_t* countp, void* ip)
{
    (void)ncid; (void)varid; (void)countp;
    if (!dmats) return 1;
    memcpy(ip, dmats + (startp[0] * dmat_nk + startp[1]) * dmat_slice, sizeof(ELPH_cmplx) * dmat_slice);
    return 0;
}

const char* nc_strerror(int e)
{
    (void)e;
    return "oracle netCDF stand-in error";
}

int main(int argc, char** argv)
{
    if (argc < 3) die("usage: lelph_ref <system.bin> <g_out.bin> [rotate <D.bin> <out.bin>]");
    load(argv[1]);
    init_ELPH_clocks();
    const int* h = (const int*)get("header", 1)->data;
    int natom = h[0], ntype = h[1], nsym = h[2], timerev = h[3], nspin = h[4], nspinor = h[5], nbnds = h[6];
    int nmag = h[7], nmodes = h[8], nkibz = h[9], nkbz = h[10];
    int Nx = h[11], Ny = h[12], Nz = h[13], nltimesj = h[14], lmax = h[15], soc = h[16], nq = h[17];
    int kminusq = h[18], non_loc = h[19];
    char dimension = (char)h[20];

    struct Lattice lat;
    memset(&lat, 0, sizeof(lat));
    lat.natom = natom;
    lat.nsym = nsym;
    lat.timerev = timerev;
    lat.nspin = nspin;
    lat.nspinor = nspinor;
    lat.total_bands = nbnds;
    lat.start_band = 1;
    lat.end_band = nbnds;
    lat.nbnds = nbnds;
    lat.dimension = dimension;
    lat.nmag = nmag;
    lat.nmodes = nmodes;
    lat.nkpts_iBZ = nkibz;
    lat.nkpts_BZ = nkbz;
    lat.fft_dims[0] = Nx;
    lat.fft_dims[1] = Ny;
    lat.fft_dims[2] = Nz;
    lat.nfftz_loc = Nz;
    lat.nfftz_loc_shift = 0;
    memcpy(lat.alat_vec, get("alat", 1)->data, 9 * sizeof(ELPH_float));
    memcpy(lat.blat_vec, get("blat", 1)->data, 9 * sizeof(ELPH_float));
    lat.volume = 0;
    lat.atomic_pos = get("atom_pos", 1)->data;
    lat.atom_type = get("atom_type", 1)->data;
    lat.kpt_iredBZ = get("kibz", 1)->data;
    lat.kpt_fullBZ_crys = get("kbz_crys", 1)->data;
    lat.kpt_fullBZ = malloc(sizeof(ELPH_float) * 3 * (size_t)nkbz);
    for (int i = 0; i < nkbz; ++i)
        for (int x = 0; x < 3; ++x)
        {
            double s = 0;
            for (int j = 0; j < 3; ++j) s += lat.blat_vec[3 * x + j] * lat.kpt_fullBZ_crys[3 * i + j];
            lat.kpt_fullBZ[3 * i + x] = s / (2 * 3.1415927);
        }
    lat.kmap = get("kmap", 1)->data;
    lat.is_soc_present = soc != 0;
    lat.syms = malloc(sizeof(struct symmetry) * (size_t)nsym);
    const ELPH_float* R = get("sym_R", 1)->data;
    const ELPH_float* T = get("sym_tau", 1)->data;
    const int* TR = get("sym_trev", 1)->data;
    for (int i = 0; i < nsym; ++i)
    {
        memcpy(lat.syms[i].Rmat, R + 9 * i, 9 * sizeof(ELPH_float));
        memcpy(lat.syms[i].tau, T + 3 * i, 3 * sizeof(ELPH_float));
        lat.syms[i].time_rev = TR[i] != 0;
    }

    struct WFC* wfcs = calloc((size_t)nkibz, sizeof(struct WFC));
    long long npw_max = 0;
    for (int ik = 0; ik < nkibz; ++ik)
    {
        char nm[32];
        snprintf(nm, 32, "gvec%d", ik);
        struct rec* g = get(nm, 1);
        snprintf(nm, 32, "wfc%d", ik);
        struct rec* w = get(nm, 1);
        snprintf(nm, 32, "Fk%d", ik);
        struct rec* fk = get(nm, 1);
        wfcs[ik].gvec = g->data;
        wfcs[ik].wfc = w->data;
        wfcs[ik].Fk = fk->data;
        wfcs[ik].npw_total = g->dims[0];
        wfcs[ik].npw_loc = g->dims[0];
        if (g->dims[0] > npw_max) npw_max = g->dims[0];
    }
    lat.npw_max = npw_max;

    struct Pseudo ps;
    memset(&ps, 0, sizeof(ps));
    ps.PP_table = get("PP_table", 1)->data;
    ps.Fsign = get("Fsign", 1)->data;
    ps.nltimesj = nltimesj;
    ps.ntype = ntype;
    ps.lmax = lmax;
    ps.fCoeff = NULL;
    if (soc && nspinor == 2)
    {
        ps.fCoeff = calloc((size_t)(nltimesj * ntype), sizeof(ELPH_cmplx*));
        for (int i = 0; i < nltimesj * ntype; ++i)
        {
            char nm[32];
            snprintf(nm, 32, "fCoeff%d", i);
            struct rec* r = get(nm, 0);
            ps.fCoeff[i] = r ? r->data : NULL;
        }
    }

    struct Phonon ph;
    memset(&ph, 0, sizeof(ph));
    ph.nq_iBZ = nq;
    ph.nq_BZ = nq;
    ph.nq_iBZ_loc = nq;
    ph.qpts_iBZ = get("qpts", 1)->data;
    ph.qpts_BZ = ph.qpts_iBZ;
    ph.nph_sym = nsym;
    ph.ph_syms = lat.syms;
    ph.qmap = malloc(sizeof(int) * 2 * (size_t)nq);
    ph.nqstar = malloc(sizeof(ND_int) * (size_t)nq);
    for (int i = 0; i < nq; ++i)
    {
        ph.qmap[2 * i] = i;
        ph.qmap[2 * i + 1] = 0;
        ph.nqstar[i] = 1;
    }

    struct ELPH_MPI_Comms comm;
    memset(&comm, 0, sizeof(comm));
    comm.commW = comm.commQ = comm.commK = comm.commR = comm.commRq = MPI_COMM_WORLD;
    comm.nqpools = comm.nkpools = 1;
    /* LELPH_REF_KPOOLS=n: the reference's own k-pool split (distribute_to_grps in
     * compute_elph_matq.c:50-58) with this process as pool 0, so that only the
     * first nk_BZ/n k-points of each q are computed (a timing sample) */
    if (getenv("LELPH_REF_KPOOLS")) comm.nkpools = atoi(getenv("LELPH_REF_KPOOLS"));
    if (comm.nkpools < 1) comm.nkpools = 1;
    /* LELPH_REF_KPOOL=i: this process is pool i instead (the pool index is
     * commQ_rank / commK_size, compute_elph_matq.c:52-54) */
    if (getenv("LELPH_REF_KPOOL")) comm.commQ_rank = atoi(getenv("LELPH_REF_KPOOL"));
    if (comm.commQ_rank < 0 || comm.commQ_rank >= comm.nkpools) die("LELPH_REF_KPOOL out of range");
    comm.commW_size = comm.commQ_size = comm.commK_size = comm.commR_size = comm.commRq_size = 1;

    if (sizeof(ELPH_float) == 4 && argc >= 4 && strcmp(argv[3], "star"))
        die("the single-precision build runs the matrix elements (and the star mode) only");
#ifdef COMPILE_ELPH_DOUBLE
    if (argc >= 6 && !strcmp(argv[3], "rotdv"))
    {
        nrec = 0;
        load(argv[4]);
        struct symmetry sy;
        memset(&sy, 0, sizeof(sy));
        memcpy(sy.Rmat, get("rR", 1)->data, 9 * sizeof(double));
        memcpy(sy.tau, get("rtau", 1)->data, 3 * sizeof(double));
        sy.time_rev = ((const int*)get("rtrev", 1)->data)[0] != 0;
        const int comp = ((const int*)get("rcomp", 1)->data)[0];
        struct rec* din = get("rdv", 1);
        double _Complex* out = malloc(din->nbytes);
        rotate_dvscf(get("rq", 1)->data, din->data, &sy, &lat, comp != 0, out, comm.commK);
        FILE* fr = fopen(argv[5], "wb");
        if (!fr) die("cannot write rotdv output");
        fwrite(out, 1, din->nbytes, fr);
        fclose(fr);
        return 0;
    }
    if (argc >= 7 && !strcmp(argv[3], "dvscf"))
    {
        /* read_dvscf_qe of a dvscf file in QE's layout, with the eig and pats
         * records of the spec (pattern -> mode basis) */
        load(argv[4]);
        const size_t n = (size_t)nmodes * nmag * Nx * Ny * Nz;
        double _Complex* dvo = malloc(sizeof(double _Complex) * n);
        if (!dvo) die("out of memory");
        read_dvscf_qe(argv[5], &lat, get("eig", 1)->data, get("pats", 1)->data, dvo, comm.commK);
        FILE* fo = fopen(argv[6], "wb");
        if (!fo) die("cannot write dvscf output");
        fwrite(dvo, sizeof(double _Complex), n, fo);
        fclose(fo);
        return 0;
    }
    if (argc >= 5 && !strcmp(argv[3], "dmats"))
    {
        /* every (symmetry, full-BZ k) Dmat, in compute_and_write_dmats' order */
        size_t ds = (size_t)nspin * nbnds * nbnds;
        double _Complex* D = malloc(sizeof(double _Complex) * ds);
        FILE* fd = fopen(argv[4], "wb");
        if (!D || !fd) die("cannot write dmats output");
        for (int is = 0; is < nsym; ++is)
            for (int ik = 0; ik < nkbz; ++ik)
            {
                electronic_reps(wfcs, &lat, lat.syms[is].Rmat, lat.syms[is].tau, lat.syms[is].time_rev, ik, D,
                                &comm);
                fwrite(D, sizeof(double _Complex), ds, fd);
            }
        fclose(fd);
        return 0;
    }
#endif
    g_slice = (size_t)nmodes * nspin * nbnds * nbnds;
    g_nk = (size_t)nkbz;
    size_t nq_bz = (size_t)nq;
    if (argc >= 5 && !strcmp(argv[3], "star"))
    {
        /* q stars: nqstar per iBZ q and the phonon symmetry of every member
         * (qmap), with the Dmats of every (symmetry, k) served to the stage's
         * nc_get_vara reads (compute_elph_matq.c:159-217) */
        load(argv[4]);
        const int* ns = get("nqstar", 1)->data;
        const int* qs = get("qsym", 1)->data;
        nq_bz = 0;
        for (int i = 0; i < nq; ++i) nq_bz += (size_t)ns[i];
        free(ph.qmap);
        ph.qmap = malloc(sizeof(int) * 2 * nq_bz);
        size_t pos = 0;
        for (int i = 0; i < nq; ++i)
        {
            ph.nqstar[i] = ns[i];
            for (int j = 0; j < ns[i]; ++j, ++pos)
            {
                ph.qmap[2 * pos] = i;
                ph.qmap[2 * pos + 1] = qs[pos];
            }
        }
        ph.nq_BZ = (ND_int)nq_bz;
        dmat_slice = (size_t)nspin * nbnds * nbnds;
        dmat_nk = (size_t)nkbz;
        dmats = malloc(sizeof(ELPH_cmplx) * (size_t)nsym * dmat_nk * dmat_slice);
        if (!dmats) die("out of memory for Dmats");
        for (int is = 0; is < nsym; ++is)
            for (int ik = 0; ik < nkbz; ++ik)
                electronic_reps(wfcs, &lat, lat.syms[is].Rmat, lat.syms[is].tau, lat.syms[is].time_rev, ik,
                                dmats + ((size_t)is * dmat_nk + ik) * dmat_slice, &comm);
    }
    g_all = calloc(nq_bz * g_nk * g_slice, sizeof(ELPH_cmplx));
    ELPH_cmplx* eig = get("eigVec", 1)->data;
    ELPH_cmplx* dv = get("dVscf", 1)->data;
    size_t nfft = (size_t)Nx * Ny * Nz;
#ifdef COMPILE_ELPH_DOUBLE
    if (argc >= 5 && !strcmp(argv[3], "dvloc"))
    {
        const double* A = lat.alat_vec;
        double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                     A[2] * (A[3] * A[7] - A[4] * A[6]);
        lat.volume = det < 0 ? -det : det;
        const double* zv = get("loc_zval", 1)->data;
        ps.loc_pseudo = calloc((size_t)ntype, sizeof(struct local_pseudo));
        ps.ngrid_max = 0;
        for (int t = 0; t < ntype; ++t)
        {
            char nm[32];
            snprintf(nm, 32, "loc_r%d", t);
            struct rec* rr = get(nm, 1);
            snprintf(nm, 32, "loc_rab%d", t);
            struct rec* ra = get(nm, 1);
            snprintf(nm, 32, "loc_v%d", t);
            struct rec* rv = get(nm, 1);
            ps.loc_pseudo[t].r_grid = rr->data;
            ps.loc_pseudo[t].rab_grid = ra->data;
            ps.loc_pseudo[t].Vloc_atomic = rv->data;
            ps.loc_pseudo[t].ngrid = rr->dims[0];
            ps.loc_pseudo[t].Zval = zv[t];
            if (rr->dims[0] > ps.ngrid_max) ps.ngrid_max = rr->dims[0];
        }
        /* qmax_abs as src/io/get_save_data.c:622-631 sets it */
        double qmax = 0;
        for (int i = 0; i < 3 * nq; ++i)
        {
            double a = ph.qpts_iBZ[i] < 0 ? -ph.qpts_iBZ[i] : ph.qpts_iBZ[i];
            if (a > qmax) qmax = a;
        }
        ps.vloc_table->qmax_abs = ceil(qmax) + 1;
        create_vlocg_table(&lat, &ps, &comm);
        FILE* fv = fopen(argv[4], "wb");
        if (!fv) die("cannot write dvloc output");
        double _Complex* vloc = malloc(sizeof(double _Complex) * (size_t)nmodes * nfft);
        for (int iq = 0; iq < nq; ++iq)
        {
            double _Complex* dvq = dv + (size_t)iq * nmodes * nmag * nfft;
            dVlocq(ph.qpts_iBZ + 3 * iq, &lat, &ps, eig + (size_t)iq * nmodes * nmodes, vloc, comm.commK);
            add_dvscf_qe(dvq, vloc, &lat);
            fwrite(vloc, sizeof(double _Complex), (size_t)nmodes * nfft, fv);
            fwrite(dvq, sizeof(double _Complex), (size_t)nmodes * nmag * nfft, fv);
        }
        fclose(fv);
        free(vloc);
    }
#endif
    /* LELPH_REF_QPT=i: only the i-th q of the file (a timing sample) */
    const int q_only = getenv("LELPH_REF_QPT") ? atoi(getenv("LELPH_REF_QPT")) : -1;
    if (q_only >= nq) die("LELPH_REF_QPT out of range");
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int iq = 0; iq < nq; ++iq)
    {
        if (q_only >= 0 && iq != q_only) continue;
        compute_and_write_elphq(wfcs, &lat, &ps, &ph, iq, eig + (size_t)iq * nmodes * nmodes,
                                dv + (size_t)iq * nmodes * nmag * nfft, 0, 0, 0, 0, non_loc != 0,
                                kminusq != 0, &comm);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    /* wall time of the stage calls alone (no input loading), for timing samples */
    fprintf(stderr, "lelph_ref: stage_seconds %.6f\n", (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec));
    FILE* fo = fopen(argv[2], "wb");
    if (!fo) die("cannot write output");
    for (size_t i = 0; i < nq_bz * g_nk * g_slice; ++i)
    {
        const double v[2] = {creal(g_all[i]), cimag(g_all[i])};  /* complex128 in either build */
        fwrite(v, sizeof(double), 2, fo);
    }
    fclose(fo);

#ifdef COMPILE_ELPH_DOUBLE
    if (argc >= 6 && !strcmp(argv[3], "rotate"))
    {
        /* elph_q_rotate on (g, Dl, Dr, time_rev) records of a separate file */
        nrec = 0;
        load(argv[4]);
        struct rec* gq = get("g", 1);
        struct rec* dl = get("Dl", 1);
        struct rec* dr = get("Dr", 1);
        const int* tr = get("trev", 1)->data;
        double _Complex* out = malloc(gq->nbytes);
        elph_q_rotate(dl->data, gq->data, dr->data, &lat, tr[0] != 0, out);
        FILE* fr = fopen(argv[5], "wb");
        fwrite(out, 1, gq->nbytes, fr);
        fclose(fr);
    }
#endif
    return 0;
}
