/*
 * lelph_ndb.h -- writer of the ndb.elph database of the elph stage.
 *
 * Holds every variable the reference puts into ndb.elph, with its names,
 * dimension names, shapes and element types:
 *   POLARIZATION_VECTORS (nq, nmodes, atom, pol, re_im), FREQ (nq, nmodes),
 *   elph_mat (nq, nk, nmodes, nspin, initial_band, final_band_PH_abs, re_im)
 *     -- src/elph/elph_driver.c:152-187;
 *   kpoints, qpoints, qpoints_iBZ, qmap, kmap, bands,
 *   number_of_phonon_symmetries, time_reversal_phonon, symmetry_matrices,
 *   fractional_translation, kernel, convention, epsilon, Born_charges,
 *   Quadrupole_tensor -- src/io/write_basic_data.c:15-215.
 * The reference creates the file as NetCDF-4 (HDF5 storage, elph_mat chunked
 * by k).  Without the netCDF/HDF5 libraries this writer emits the netCDF
 * classic 64-bit-offset format (CDF-2), which the netCDF library opens with
 * the same nc_open / nc_get_vara calls: readers see the same variables; only
 * the storage (contiguous, big-endian, elph_mat last so it may exceed 4 GiB)
 * differs.  Host code only, no device calls.
 */
#ifndef LELPH_NDB_H
#define LELPH_NDB_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lelph_ndb lelph_ndb;

typedef struct lelph_ndb_desc
{
    int nq_BZ, nq_iBZ, nkpts_BZ, nmodes, natom, nspin, nbnds, nph_sym;
    int start_band, end_band;    /* lattice->start_band, end_band (1-based) */
    int io_double;               /* element type of the real variables: 1 NC_DOUBLE (COMPILE_ELPH_DOUBLE), 0 NC_FLOAT */
    const double* kpoints;       /* (nkpts_BZ, 3) crystal: lattice->kpt_fullBZ_crys */
    const double* qpoints;       /* (nq_BZ, 3): phonon->qpts_BZ */
    const double* qpoints_iBZ;   /* (nq_iBZ, 3): phonon->qpts_iBZ */
    const int* qmap;             /* (nq_BZ, 2): phonon->qmap */
    const int* kmap;             /* (nkpts_BZ, 2): lattice->kmap */
    const double* sym_Rmat;      /* (nph_sym, 3, 3): phonon->ph_syms[].Rmat */
    const double* sym_tau;       /* (nph_sym, 3): phonon->ph_syms[].tau */
    const int* sym_time_rev;     /* (nph_sym): phonon->ph_syms[].time_rev */
    const char* kernel;          /* the kernel string of the input (kernel_str) */
    int kminusq;                 /* convention: "yambo" if nonzero, else "standard" */
    const double* epsilon;       /* (3, 3) or NULL (zeros) */
    const double* Zborn;         /* (natom, 3, 3) or NULL (zeros) */
    const double* Qpole;         /* (natom, 3, 3, 3) or NULL (zeros) */
} lelph_ndb_desc;

/* Create (overwrite, as NC_CLOBBER) the file, define every variable and write
 * the basic data; elph_mat, POLARIZATION_VECTORS and FREQ are filled by the
 * calls below (unwritten parts read as zeros).  Returns 0 or a negative
 * status (-1 invalid argument, -2 allocation, -8 I/O). */
int lelph_ndb_create(const char* path, const lelph_ndb_desc* desc, lelph_ndb** out);

/* elph_mat[iq_BZ][k0 .. k0 + nk) from g (nk, nmodes, nspin, nbnds, nbnds)
 * complex, interleaved doubles (c64 = 0) or floats (c64 = 1): the
 * nc_put_vara of compute_elph_matq.c:145-152 and :206-214. */
int lelph_ndb_put_elph(lelph_ndb* f, int iq_BZ, int k0, int nk, const void* g, int c64);

/* POLARIZATION_VECTORS[iq_BZ] (nmodes, natom, 3) complex and FREQ[iq_BZ]
 * (nmodes): the nc_put_vara of elph_driver.c:262-300 (either may be NULL). */
int lelph_ndb_put_phonon(lelph_ndb* f, int iq_BZ, const double* eig, const double* omega);

/* Flush and close; frees f. */
int lelph_ndb_close(lelph_ndb* f);

#ifdef __cplusplus
}
#endif
#endif
