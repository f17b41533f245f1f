/*
 * lelph_gpu.h -- C ABI of the GB300 electron-phonon matrix-element stage.
 *
 * Drop-in for the per-q stage of LetzElPhC:
 *   void compute_and_write_elphq(struct WFC* wfcs, struct Lattice* lattice,
 *        struct Pseudo* pseudo, struct Phonon* phonon, const ND_int iqpt,
 *        ELPH_cmplx* eigVec, ELPH_cmplx* dVscfq, const int ncid_elph,
 *        const int varid_elph, const int ncid_dmat, const int varid_dmat,
 *        const bool non_loc, const bool kminusq, const struct ELPH_MPI_Comms* Comm)
 *   (src/elph/elph.h:10-17, src/elph/compute_elph_matq.c:20-234)
 * together with its inner units elphLocal (src/dvloc/dvloc.h:16-18) and
 * add_elphNonLocal (src/nonloc/Vnonloc.h:8-11).
 *
 * Plain pointers and sizes only.  Complex numbers are interleaved (re, im)
 * doubles unless stated.  The library copies every input to the device; the
 * caller owns all host buffers.  Functions return LELPH_GPU_OK (0) or a
 * negative status and never abort the process (the reference aborts through
 * error_msg -> MPI_Abort, src/common/error.c:8-21; a caller that wants that
 * behaviour maps a nonzero status to error_msg).  One context per host
 * thread; a context is not re-entrant.  Calls are synchronous: on return the
 * outputs are in the caller's buffer.
 */
#ifndef LELPH_GPU_H
#define LELPH_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LELPH_GPU_OK 0
#define LELPH_GPU_ERR_INVALID (-1)     /* bad argument or inconsistent sizes */
#define LELPH_GPU_ERR_ALLOC (-2)       /* device or host allocation failed */
#define LELPH_GPU_ERR_CUDA (-3)        /* CUDA runtime/driver error */
#define LELPH_GPU_ERR_TIMEOUT (-4)     /* a device-side wait ran out (kernel bailed out) */
#define LELPH_GPU_ERR_GEOMETRY (-5)    /* k+q not on the grid, non-integral symmetry, box too small */
#define LELPH_GPU_ERR_STATE (-6)       /* call order (e.g. run on an empty q slot) */
#define LELPH_GPU_ERR_UNSUPPORTED (-7) /* size outside what this build handles */

/* arithmetic of the path */
#define LELPH_GPU_FP64 0       /* FP64 throughout (the plain form) */
#define LELPH_GPU_MIXED_F16 1  /* FP32 FFTs, split-f16 (hi,lo) tensor-core sandwich, FP64 phases/reduction */
#define LELPH_GPU_MIXED_BF16 2 /* as above with split-bf16 */

/* lelph_gpu_desc.route: the order of work of the local sandwich.
 * REAL: psi(r) of every full-BZ k resident, one contraction over the grid per
 *       pair (tensor cores in the mixed form; at most 64 bands there).
 * GSPACE: the reference's order (elphLocal, src/dvloc/compute_Vbare_loc.c:264-310):
 *       forward FFT of dV psi_k per (mode, band), pruned to the k+q sphere,
 *       then a GEMM over the sphere; psi(r) is built per k when it is needed.
 * AUTO: REAL unless its resident operands exceed half of the device memory or
 *       the mixed form's tensor-core tile cannot hold the bands; when both fit,
 *       the mixed form takes the route a cost model per pair (rates measured on
 *       GB300) finds cheaper.  lelph_gpu_tune measures the candidates instead. */
#define LELPH_GPU_ROUTE_AUTO 0
#define LELPH_GPU_ROUTE_REAL 1
#define LELPH_GPU_ROUTE_GSPACE 2

/* element type of matrix-element outputs */
#define LELPH_GPU_OUT_C128 0 /* double complex (reference built with -DCOMPILE_ELPH_DOUBLE) */
#define LELPH_GPU_OUT_C64 1  /* float complex (reference default build, src/elphC.h:24-31) */

typedef struct lelph_gpu lelph_gpu;

/* The contents of struct Lattice / WFC / Pseudo (src/common/dtypes.h:80-266)
 * that the per-q stage reads.  Layouts are the reference's. */
typedef struct lelph_gpu_desc
{
    /* struct Lattice */
    int natom, nsym, timerev, nspin, nspinor, nbnds, nmag, nmodes;
    int nkpts_iBZ, nkpts_BZ;
    int fft_dims[3];
    const double* alat_vec;        /* [9]  a_i = alat[:, i], row-major */
    const double* blat_vec;        /* [9]  b_i = blat[:, i], includes 2 pi */
    const double* atomic_pos;      /* [natom*3] cartesian */
    const int* atom_type;          /* [natom] */
    const double* kpt_iredBZ;      /* [nkpts_iBZ*3] cartesian, no 2 pi */
    const double* kpt_fullBZ_crys; /* [nkpts_BZ*3] crystal */
    const int* kmap;               /* [nkpts_BZ*2] (iBZ k, symmetry) */
    const double* sym_Rmat;        /* [nsym*9] cartesian, row-major */
    const double* sym_tau;         /* [nsym*3] cartesian fractional translations */
    const int* sym_time_rev;       /* [nsym] */
    int is_soc_present;
    /* struct WFC, one per iBZ k-point */
    const int* npw;                /* [nkpts_iBZ] plane waves of each k */
    const double* const* gvec;     /* [ik] -> [npw*3] cartesian, no 2 pi */
    const double* const* wfc;      /* [ik] -> (nspin, nbnds, nspinor, npw) complex */
    const double* const* Fk;       /* [ik] -> (nltimesj, ntype, npw) KB form factors */
    /* struct Pseudo */
    int ntype, nltimesj, lmax;
    const double* PP_table;        /* (nltimesj, ntype, 3): l+1, 2j, spin */
    const double* Fsign;           /* (nltimesj, ntype) */
    const double* const* fCoeff;   /* [lidx*ntype+itype] -> (2l+1,2l+1,nspinor,nspinor) complex, or NULL */
    /* library options */
    int precision;                 /* LELPH_GPU_FP64 / LELPH_GPU_MIXED_F16 / LELPH_GPU_MIXED_BF16 */
    int device;                    /* CUDA device ordinal */
    int route;                     /* LELPH_GPU_ROUTE_* (0 = automatic) */
    int tile_points;               /* real-space route, mixed form: grid points per stage of the tensor-core
                                      pipeline, 64 or 32 (0 = the library's choice) */
    int gs_gemm;                   /* G-space route, mixed form: LELPH_GPU_GS_GEMM_* (0 = tensor cores where
                                      the band count allows) */
} lelph_gpu_desc;

#define LELPH_GPU_GS_GEMM_TENSOR 1 /* split-TF32 tcgen05 GEMM */
#define LELPH_GPU_GS_GEMM_SIMT 2   /* FP32 SIMT GEMM */

/* What lelph_gpu_tune measured and chose. */
typedef struct lelph_gpu_tuning
{
    int route;                     /* chosen LELPH_GPU_ROUTE_REAL / LELPH_GPU_ROUTE_GSPACE */
    int tile_points;               /* chosen stage size of the real-space route (0 on the G-space route) */
    int gs_gemm;                   /* chosen GEMM of the G-space route (0 on the real-space route) */
    int cached;                    /* 1: read from the cache file, nothing was measured */
    double ms_per_pair[4];         /* device time per (k, q) pair of each candidate: real-space with 64- and
                                      32-point stages, G-space with the tensor-core and the SIMT GEMM
                                      (negative: not a candidate for this system or form) */
} lelph_gpu_tuning;

typedef struct lelph_gpu_stats
{
    long long kernel_launches;   /* kernels launched by this context so far */
    long long local_launches;    /* launches of the local-sandwich kernel */
    double local_ms;             /* device time of those launches (profiling on) */
    double prepare_ms;           /* device time of the q-independent stage (profiling on) */
    double finish_ms;            /* device time of the finish kernel (profiling on) */
    long long pairs_done;        /* (k, q) pairs computed */
    size_t device_bytes;         /* device memory held by the context */
    int product_grid[3];         /* grid of the real-space sandwich and wavefunction FFTs */
    int chunk_points;            /* grid points per K chunk of the tensor-core sandwich (mixed form) */
    double dmats_ms;             /* device time of the Dmat kernels (index maps + contraction, profiling on) */
    double dmats_host_ms;        /* host time spent building Dmat jobs (always measured) */
    long long dmats_done;        /* Dmats computed */
    double qstar_ms;             /* device time of the q-star rotations (profiling on) */
    double dvscf_ms;             /* device time of the dV_scf ingest kernel (profiling on) */
    int route;                   /* route in use: LELPH_GPU_ROUTE_REAL or LELPH_GPU_ROUTE_GSPACE */
    double gs_plane_ms;          /* G-space route: device time of the plane, x-pass and GEMM kernels */
    double gs_xpass_ms;          /*   (profiling on; each launch timed with events on the library stream) */
    double gs_gemm_ms;
    double prep_scatter_ms;      /* real-space route, mixed form, profiling on: device time of the */
    double prep_fft_ms;          /*   preparation's roles -- sphere -> box scatter, z and y FFT passes, */
    double prep_xsplit_ms;       /*   x pass writing the tensor-core operands, KB projections, and the */
    double prep_proj_ms;         /*   dV windows (prepare) */
    double windows_ms;
    long long box_columns;       /* real-space route, mixed form: occupied z-columns of the wavefunction boxes
                                    summed over the full-BZ k (known after the first preparation; the later
                                    ones zero only these columns) */
    double local_live_ms;        /* device time of the local-sandwich launches of every run, from events recorded
                                    around them always (no profiling synchronisations), read after the run */
    long long local_live_launches;
} lelph_gpu_stats;

/* Create a context: validates the inputs, derives the integer symmetry maps,
 * uploads wavefunctions, form factors and projector tables.
 * Replaces the per-call setup of elphLocal / add_elphNonLocal
 * (src/dvloc/compute_Vbare_loc.c:93-205, src/nonloc/Vbare_nloc.c:96-245). */
int lelph_gpu_create(const lelph_gpu_desc* desc, lelph_gpu** out);

/* Measured choice of the route and the tile options for a system (no
 * counterpart in the reference, whose FFTW plans are measured per call with
 * FFTW_MEASURE, src/fft/planner.c:224-306): every candidate the system and
 * precision allow -- the real-space route with 64- and 32-point stages of the
 * tensor-core pipeline (when its resident operands fit in half of the device
 * memory), the G-space route with the tensor-core and the SIMT GEMM -- runs
 * as its own context on the caller's q (qpt_crys, eigVec, dVscf as in
 * lelph_gpu_set_q) and the first npairs full-BZ k-points, is timed after a
 * warm-up, and the fastest is returned; route, tile_points and gs_gemm of
 * *out fill the same fields of a descriptor.  desc->route, tile_points and
 * gs_gemm are ignored.  With cache_path (may be NULL) the result is looked up
 * in, and otherwise appended to, that text file under a key of the system's
 * sizes, precision and device name. */
int lelph_gpu_tune(const lelph_gpu_desc* desc, const double qpt_crys[3], const double* eigVec, const double* dVscf,
                   int npairs, const char* cache_path, lelph_gpu_tuning* out);

/* Replace the plane-wave coefficients of every iBZ k-point
 * ([ik] -> (nspin, nbnds, nspinor, npw) complex); invalidates lelph_gpu_prepare. */
int lelph_gpu_set_wavefunctions(lelph_gpu* h, const double* const* wfc);

/* q-independent work: unfold every full-BZ wavefunction (rotation, SU(2),
 * fractional translation, time reversal), inverse-FFT it to the grid and
 * project it on the KB projectors.  Runs implicitly on first use. */
int lelph_gpu_prepare(lelph_gpu* h);

/* Load one q-point into a slot: q in crystal coordinates, eigVec
 * (nmodes, 3*natom) complex, dVscf (nmodes, nmag, Nx, Ny, Nz) complex -- the
 * dVscfq / eigVec arguments of compute_and_write_elphq. */
int lelph_gpu_set_q(lelph_gpu* h, int slot, const double qpt_crys[3], const double* eigVec, const double* dVscf);

/* Matrix elements for n (q slot, full-BZ k) items, flags as in
 * compute_and_write_elphq (non_loc, kminusq).  g_out (host) receives
 * (n, nmodes, nspin, nbnds_k, nbnds_k+q) complex of out_type -- the
 * elph_mat[q][k] slice layout (src/elph/elph_driver.c:164-187). */
int lelph_gpu_run(lelph_gpu* h, int n, const int* qslot, const int* kbz, int non_loc, int kminusq, int out_type,
                  void* g_out);

/* Same, output left in device memory (g_out_dev, same layout). */
int lelph_gpu_run_device(lelph_gpu* h, int n, const int* qslot, const int* kbz, int non_loc, int kminusq,
                         int out_type, void* g_out_dev);

/* Allocation-free variant of lelph_gpu_run_device (no counterpart in the
 * reference).  For callers that cannot allocate device memory once set-up is
 * done: a host code whose device memory is entirely owned by another pool or
 * framework, or a service loop that must not meet an allocation failure or the
 * latency of cudaMalloc in the middle of a run.  The call makes no cudaMalloc,
 * cudaFree or other device-allocating call (and no host heap allocation on
 * its success path): its working storage (the
 * pair table and the local-sandwich partial sums) is a 64 MiB file-scope
 * static device array that every GPU loading the library holds until exit.
 * The context must already be prepared (lelph_gpu_prepare) and its q slots
 * loaded; g_out_dev is a caller-owned device buffer laid out as in
 * lelph_gpu_run.  Items are processed in batches that fit the array; a size
 * whose single (k, q) pair needs more than the array returns
 * LELPH_GPU_ERR_UNSUPPORTED.  The first call on a device looks the array up
 * (cudaGetSymbolAddress) with that device current, and so does the first call
 * after the device's context was destroyed and re-created (cudaDeviceReset
 * reloads the array elsewhere); such a first call should come before any
 * stream capture.  All calls share the one array and every
 * call overwrites what it uses, so calls that overlap on the GPU (several
 * contexts or threads at once on one device) race and must be serialised by
 * the caller. */
int lelph_gpu_run_device_noalloc(lelph_gpu* h, int n, const int* qslot, const int* kbz, int non_loc, int kminusq,
                                 int out_type, void* g_out_dev);

/* Local pseudopotential of every species on its radial mesh -- the fields of
 * struct local_pseudo (src/common/dtypes.h:204-217): ngrid[t] points r_grid[t],
 * mesh derivative rab_grid[t], V_loc in Ry, valence charge zval[t] -- and the
 * cell's periodicity ('3', or '2' for a slab with the Coulomb cutoff along z).
 * Builds the V_loc(|G|) interpolation table of create_vlocg_table
 * (src/dvloc/vlocg_table.c:16-154) on the device; qmax_abs bounds |q| in
 * crystal units as Vloc_table.qmax_abs does (ceil(max |q_i|) + 1). */
int lelph_gpu_set_local_pseudo(lelph_gpu* h, const int* ngrid, const double* const* r_grid,
                               const double* const* rab_grid, const double* const* vloc_atomic, const double* zval,
                               int dimension, double qmax_abs);

/* dVlocq (src/dvloc/dVbare_loc.c:16-231): the local bare potential change of
 * every mode of q in real space, Vlocr (nmodes, Nx, Ny, Nz) complex, on the
 * reference's FFT box.  Needs lelph_gpu_set_local_pseudo. */
int lelph_gpu_dvlocq(lelph_gpu* h, const double qpt_crys[3], const double* eigVec, double* Vlocr);

/* lelph_gpu_set_q from the induced potential alone: dVscf_induced
 * (nmodes, nmag, Nx, Ny, Nz) is QE's dvscf (dV_Ha + dV_xc), or NULL for the
 * bare kernels; the library adds dVlocq on the device with add_dvscf_qe's
 * rule (src/dvloc/add_dvscf.c:12-92), as elph_driver does before
 * compute_and_write_elphq (src/elph/elph_driver.c:234-252). */
int lelph_gpu_set_q_induced(lelph_gpu* h, int slot, const double qpt_crys[3], const double* eigVec,
                            const double* dVscf_induced);

/* read_dvscf_qe (src/io/qe/read_dvscf.c:15-172) after the file read, on the
 * device: dvscf_qe is the content of QE's dvscf file for this q, (nmodes
 * patterns, nmag, Nz, Ny, Nx) complex double in the pattern basis; it is
 * transposed to (Nx, Ny, Nz), taken to the mode basis (eigVec pats^H dV,
 * pats = the patterns (nmodes, natom, 3) of read_pattern_qe) and loaded into
 * q slot `slot`: as the induced part with dVlocq added when induced != 0
 * (like lelph_gpu_set_q_induced), else as the whole dV (like
 * lelph_gpu_set_q).  dvscf_out (may be NULL) receives the mode-basis dV
 * before any dVlocq, (nmodes, nmag, Nx, Ny, Nz) -- read_dvscf_qe's output. */
int lelph_gpu_set_q_dvscf_qe(lelph_gpu* h, int slot, const double qpt_crys[3], const double* eigVec,
                             const double* pats, const double* dvscf_qe, int induced, double* dvscf_out);

/* rotate_dvscf (src/symmetries/rotate_dvscf.c:22-368): dV_scf of S q from
 * dV_scf of q for the symmetry (Rmat cartesian row-major, tau cartesian,
 * time_rev) -- the box permutation S^-1 (r - tau), the phase e^{-i (Sq).tau},
 * the SU(2) rotation of the spin part for nmag = 4 (composite_form: inputs
 * already [V+Bz, Bx-iBy, Bx+iBy, V-Bz]) and the conjugate for time reversal.
 * dvscf_in, dvscf_out: (nmodes, nmag, Nx, Ny, Nz) complex on the reference box.
 * LELPH_GPU_ERR_GEOMETRY if the operation does not map the FFT grid onto itself. */
int lelph_gpu_rotate_dvscf(lelph_gpu* h, const double qpt_crys[3], const double Rmat[9], const double tau[3],
                           int time_rev, int composite_form, const double* dvscf_in, double* dvscf_out);

/* compute_and_write_elphq for one iBZ q without the netCDF writes: every
 * full-BZ k, output (nkpts_BZ, nmodes, nspin, nbnds, nbnds) complex double. */
int lelph_gpu_compute_elphq(lelph_gpu* h, const double qpt_crys[3], const double* eigVec, const double* dVscfq,
                            int non_loc, int kminusq, double* elph_out);

/* elph_q_rotate (src/symmetries/elphq_expand.c:16-73): g_Sq = (g^{T|C} D_r^H)^T D_l^T
 * per (mode, spin); g, out (nmodes, nspin, nb, nb), D (nspin, nb, nb) complex. */
int lelph_gpu_elph_q_rotate(lelph_gpu* h, const double* Dmats_l, const double* elph_q, const double* Dmats_r,
                            int time_rev, double* elph_Sq);

/* Dmats: the electronic representation matrices of compute_and_write_dmats
 * (src/elph/compute_dmats.c:20-131), one electronic_reps
 * (src/symmetries/elec_reps.c:16-413) per (symmetry, full-BZ k) pair
 * idmat = isym * nkpts_BZ + ikBZ, for idmat = first .. first + count - 1 (the
 * block distribute_to_grps gives a pool, compute_dmats.c:95-97).  Rmat
 * (nsym, 3, 3) cartesian row-major, tau (nsym, 3) cartesian, time_rev (nsym):
 * the phonon symmetries (struct symmetry).  Dmats (may be NULL): complex double
 * (count, nspin, nbnds, nbnds), D[., s, b, a] = <psi_{Rk,b}| U(R) |psi_{k,a}>,
 * the reference's ndb.Dmats slice layout.  The block also stays on the device.
 * LELPH_GPU_ERR_GEOMETRY if R k is not on the k grid ("Rotated k point not
 * found") or an operation is not integral on the lattice. */
int lelph_gpu_dmats(lelph_gpu* h, int nsym, const double* Rmat, const double* tau, const int* time_rev,
                    long long first, long long count, double* Dmats);

/* compute_and_write_elphq with its q-star expansion
 * (src/elph/compute_elph_matq.c:20-234) without the netCDF I/O: g of the
 * irreducible q (qpt_crys, eigVec, dVscfq, non_loc, kminusq as in
 * lelph_gpu_compute_elphq) at every full-BZ k, then for each star member
 * istar = 1 .. nstar-1 with phonon symmetry S = star_sym[istar] (the
 * reference's phonon->qmap[2*(qpos+istar)+1]):
 *   g(Sq, Sk) = elph_q_rotate(D[S][k+q], g(q, k), D[S][k], time_rev(S)),
 * stored at S k.  ph_Rmat (nph_sym, 3, 3), ph_tau (nph_sym, 3), ph_time_rev
 * (nph_sym): the phonon symmetries (phonon->ph_syms).  The Dmats come from the
 * block lelph_gpu_dmats left on the device when it was made for the same
 * symmetries and holds the star's rows; otherwise the needed rows are computed
 * here.  out: (nstar, nkpts_BZ, nmodes, nspin, nbnds, nbnds) of out_type, the
 * ndb.elph rows qpos .. qpos+nstar-1.  star_sym[0] must be 0 (the reference's
 * check "Qpoint in iBZ cannot be traced in phonon qmap"); LELPH_GPU_ERR_GEOMETRY
 * if S k is off the grid.  Rotations need 4 nbnds^2 complex in shared memory:
 * up to 83 bands (mixed form) or 58 (plain form) when nstar > 1. */
int lelph_gpu_compute_elphq_star(lelph_gpu* h, const double qpt_crys[3], const double* eigVec, const double* dVscfq,
                                 int non_loc, int kminusq, int nph_sym, const double* ph_Rmat, const double* ph_tau,
                                 const int* ph_time_rev, int nstar, const int* star_sym, int out_type, void* out);

/* Rotated (and umklapp-shifted) Miller indices of full-BZ k-point kbz, as the
 * device computes them: out[npw*3].  Parity check of the integer maps of
 * rotateGvecs + Sort_pw (src/wfc/rotate_Gvecs.c:15-81, src/wfc/sortpw.c:95-315). */
int lelph_gpu_debug_gvec_map(lelph_gpu* h, int kbz, const int ulm[3], int* out);

/* Layout check of the partial sums of the mixed form's real-space sandwich
 * (host arithmetic only, no device work; the output size nmodes * nspin *
 * nb^2 per pair of elphLocal, src/dvloc/compute_Vbare_loc.c:286-341, is
 * assembled from them): for nmodes, nbnds (<= 64), nspin and nchunks K chunks
 * per pair, out[0] = floats the library allocates for npairs pairs, out[1] =
 * one past the highest float the tensor-core sandwich writes, out[2] = one
 * past the highest float the finish kernel reads. */
int lelph_gpu_debug_partials_extent(int nmodes, int nbnds, int nspin, int nchunks, int npairs,
                                    unsigned long long out[3]);

int lelph_gpu_set_profiling(lelph_gpu* h, int on);
/* Limit, in nanoseconds, of every wait between the roles of the tensor-core
 * sandwich's pipeline (0: the default, 1.5 s).  A wait that runs out makes the
 * kernel stop, let its copies and MMAs in flight finish, release its tensor
 * memory and report LELPH_GPU_ERR_TIMEOUT; the context stays usable.  (No
 * counterpart in the reference, which has no device waits; a short limit lets
 * a test exercise that path.) */
int lelph_gpu_set_wait_limit(lelph_gpu* h, unsigned long long ns);
int lelph_gpu_stats_get(lelph_gpu* h, lelph_gpu_stats* s);
/* the CUDA stream (cudaStream_t) every kernel of the context runs on */
void* lelph_gpu_stream(lelph_gpu* h);
const char* lelph_gpu_strerror(int status);
const char* lelph_gpu_last_error(lelph_gpu* h);
void lelph_gpu_destroy(lelph_gpu* h);

#ifdef __cplusplus
}
#endif
#endif
