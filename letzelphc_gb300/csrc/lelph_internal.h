// Internal launch interface shared by the .cu translation units of the
// electron-phonon library (not part of the public C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define LELPH_MAX_RADIX_STAGES 12
#define TC_KPTS_MAX 64  // largest pipeline stage of the tensor-core sandwich (grid points)

// One 1-D transform length L = prod(radix[0..nstage)), radices in {2,3,4,5}.
struct FftPlan1D
{
    int L;
    int nstage;
    int radix[LELPH_MAX_RADIX_STAGES];
};

// Per full-BZ k-point symmetry data (host-computed, FP64).
struct KPointSym
{
    int ik;          // iBZ index
    int isym;        // symmetry index
    int trev;        // time-reversal symmetry
    int W[9];        // integer action on Miller indices (row-major)
    double R[9];     // cartesian rotation (row-major, v' = R v)
    double tau_crys[3];
    double tau_cart[3];
    double kphase[2];  // exp(-i 2 pi kvec_crys . tau_crys), kvec_crys = alat^T R k_iBZ
    double kcart[3];   // k_iBZ (cart)
    double su2[8];     // 2x2 complex spinor rotation (re, im interleaved)
};

// One (k, k+q) pair of a run.
struct PairInfo
{
    int kbz_k;   // full-BZ index of the k wavefunction
    int kbz_kq;  // full-BZ index of the k+q wavefunction
    int ulm[3];  // umklapp G0 (crystal) applied to the k+q wavefunction
    int qslot;   // q slot (eigVec)
    int dvslot;  // dV window of (q slot, G0) on the product grid
};

struct GeomDev
{
    int Nx, Ny, Nz;
    int nspin, nspinor, nbnds, nbp, nmag, nmodes;
    int mt_modes;  // whole modes per 128-row tile of the tensor-core sandwich: min(nmodes, max(1, 128/nbnds))
    int kpts;      // grid points per pipeline stage of the tensor-core sandwich (64, or 32 for wide tiles)
};

// Partial sums of the tensor-core sandwich, laid out
// [pair * nspin + spin][mode tile][K chunk][128 rows][2 nbp] (FP32).  A mode
// tile holds mt_modes whole modes, so there are ceil(nmodes / mt_modes) tiles
// per (pair, spin) -- more than ceil(nmodes * nbnds / 128) whenever 128 is not
// a multiple of nbnds.  The kernel that writes the partials, the finish that
// reads them and every allocation of them use these helpers.
inline int lelph_tc_tile_modes(int nmodes, int nbnds)  // mt_modes; a tile row is one (mode, band of k)
{
    const int m = 128 / nbnds > 1 ? 128 / nbnds : 1;
    return nmodes < m ? nmodes : m;
}
__host__ __device__ inline int lelph_tc_mode_tiles(const GeomDev& g)
{
    return (g.nmodes + g.mt_modes - 1) / g.mt_modes;
}
__host__ __device__ inline size_t lelph_tc_partial_offset(const GeomDev& g, int nchunks, long long zp, int mt,
                                                          int chunk, int row)
{
    return ((((size_t)zp * lelph_tc_mode_tiles(g) + mt) * nchunks + chunk) * 128 + row) * (size_t)(2 * g.nbp);
}
inline size_t lelph_tc_partials_per_pair(const GeomDev& g, int nchunks)
{
    return (size_t)g.nspin * lelph_tc_mode_tiles(g) * nchunks * 128 * (size_t)(2 * g.nbp);
}

// Occupancy of the boxes of a chunk of k-points after the sphere -> box
// scatter: col[(kslot*Nx + x)*Ny + y] != 0 when the z-column (x, y) holds a
// plane wave of k, xpl[kslot*Nx + x] != 0 when the plane x does.  Every band
// of a k-point shares its sphere.  col == nullptr: no masking.  With masks the
// passes never read a point outside the sphere's columns and planes: the z
// pass reads the occupied columns, the y pass reads unoccupied columns as
// zero, the x pass unoccupied planes; only the occupied columns need zeros
// (off the sphere) before a scatter.
struct BoxMask
{
    uint8_t* col = nullptr;
    uint8_t* xpl = nullptr;
    int Nx = 0, Ny = 0, nbox_per_k = 1;
};

// FFT (fft_gather.cu)
void lelph_launch_fft_contig_d(double2* data, long long nlines, const FftPlan1D& p, const double2* tw, int sign,
                               cudaStream_t st);
void lelph_launch_fft_contig_f(float2* data, long long nlines, const FftPlan1D& p, const float2* tw, int sign,
                               cudaStream_t st, const BoxMask& mk = BoxMask());
void lelph_launch_fft_strided_d(double2* data, long long nouter, int inner, const FftPlan1D& p, const double2* tw,
                                int sign, cudaStream_t st);
void lelph_launch_fft_strided_f(float2* data, long long nouter, int inner, const FftPlan1D& p, const float2* tw,
                                int sign, cudaStream_t st, const BoxMask& mk = BoxMask());
// x-pass of the mixed form writing the split tensor-core operand directly
void lelph_launch_fft_x_to_split(const float2* boxes, int nbox_k, int k0, const FftPlan1D& p, const float2* tw,
                                 int sign, const GeomDev& g, const float* band_scale, int ab_bf16, uint16_t* Bsplit,
                                 float2* psi32, cudaStream_t st, const BoxMask& mk = BoxMask());

// occupied columns of each k as a list (col[k*ncol + c] != 0 -> list[k*ncol + i] = c,
// i < cnt[k], any order), and the zeroing of those columns in a chunk's boxes
void lelph_launch_col_lists(const uint8_t* col, int nk, int ncol, int* list, int* cnt, cudaStream_t st);
void lelph_launch_clear_cols(float2* boxes, int nk, int nbox_per_k, long long N, int Nz, int ncol, const int* list,
                             const int* cnt, cudaStream_t st);

// sphere -> box scatter with su2, fractional-translation phase and conj
void lelph_launch_scatter(int k0, int nk, const KPointSym* ksym_dev, const int* miller, const long long* pw_off,
                          const int* npw, int npw_max, const double2* coef, const long long* coef_off,
                          const GeomDev& g, int box_fp64, void* boxes, double2* chat, const long long* chat_off,
                          cudaStream_t st, const BoxMask& mk = BoxMask(), float2* chat32 = nullptr);

// debugging / parity: box index of each rotated plane wave of one full-BZ k
void lelph_launch_gmap(const KPointSym* ks, int kbz, const int* miller, const long long* pw_off, const int* npw,
                       const GeomDev& g, const int* ulm, int* out, cudaStream_t st);

// G-space route of the local sandwich (gspace.cu)
struct GsGeom
{
    int Nx, Ny, Nz;  // product grid
    int nb, nspinor, nmag, spin;
};
size_t lelph_gs_plane_smem(const GsGeom& gg, int fp64);
size_t lelph_gs_xpass_smem(const GsGeom& gg, int fp64);
// plane pass of modes nu0 .. nu0+nub-1: out [(nu - nu0) nb + m][s][x][ncol]; square planes of the
// sizes lelph_gs_plane_fixed accepts run the compile-time kernel (cols2, zl: pruned y transform)
bool lelph_gs_plane_fixed(const GsGeom& gg, int fp64);
int lelph_launch_gs_plane(const GsGeom& gg, int fp64, const void* psi, const void* win, int nu0, int nub,
                          const FftPlan1D& py, const FftPlan1D& pz, const void* twy, const void* twz, const int* cols,
                          int ncol, const int* cols2, const int* zl, int nzl, void* out, cudaStream_t st);
// x pass: A [rb][npad] (rb = row-box index of the block) in the sphere's sorted order;
// with A_lo (FP32 only) A receives the TF32-rounded values and A_lo the rounded remainders
int lelph_launch_gs_xpass(const GsGeom& gg, int fp64, const void* in, int nrb, int ncol, const FftPlan1D& px,
                          const void* twx, const int* cst, const int* kcx, int npad, void* A, cudaStream_t st,
                          void* A_lo = nullptr);
// tensor-core GEMM of the mixed form (gspace_tc.cu): tmaps = CUtensorMap[4] of
// A hi, A lo (nrows x 2 Ktot FP32, box 32 x 128), B hi, B lo (2 nb x 2 Ktot,
// box 32 x NT); B from lelph_launch_gs_bsplit
int lelph_gs_tc_ntile(int nb, int* ntiles);
int lelph_gs_tc_supported(int nb);
size_t lelph_gs_tc_smem(int nb);
void lelph_launch_gs_bsplit(const float2* Bp, int nb, int Ktot, float* Bq, cudaStream_t st);
int lelph_launch_gs_gemm_tc(const void* tmaps, int nrows, int nb, int Ktot, int kchunk, int rowoff,
                            int nrows_total, float2* part, unsigned* status, unsigned long long wait_ns,
                            cudaStream_t st);
int lelph_launch_gs_gemm(int fp64, const void* A, const void* B, int nrows, int nb, int Ktot, int kchunk,
                         int rowoff, int nrows_total, void* part, cudaStream_t st);
void lelph_launch_gs_reduce(int fp64, const void* part, long long nel, int nchunks, double invM, double2* glocal,
                            cudaStream_t st);
int lelph_launch_gs_bperm(int fp64, const double2* chat, const long long* chat_off, const int* npw_k,
                          const int* npad_k, const long long* perm_off, const int* perm, const long long* bp_off,
                          int k0, int nk, int rows_per_k, int npad_max, void* Bp, cudaStream_t st);

// local sandwich (sandwich.cu)
void lelph_launch_local_fp64(const PairInfo* pairs, int npairs, const double2* psi, const double2* dV,
                             const GeomDev& g, double2* glocal, unsigned* status, cudaStream_t st);
int lelph_local_tc_smem_bytes(const GeomDev& g);
int lelph_local_tc_stages(const GeomDev& g);
int lelph_local_tc_tile_modes(const GeomDev& g);
int lelph_local_tc_supported(const GeomDev& g);
void lelph_launch_local_tc(const PairInfo* pairs, int npairs, const void* tmapB, const void* tmapP,
                           const void* tmapV, const GeomDev& g, int ab_bf16, int chunk_pts, int nchunks,
                           float* partials, unsigned* status, cudaStream_t st,
                           unsigned long long wait_ns = 0);  // limit of each pipeline wait (0: the default)

// nonlocal + finish (nonlocal.cu)
struct NonlocalDesc
{
    int natom, ntype, nltimesj, lmax, nproj_max, is_soc;
    const int* atom_type;    // natom
    const double* atom_pos;  // natom*3 cart
    const double* PP_table;  // nltimesj*ntype*3
    const double* Fsign;     // nltimesj*ntype
    const double* fcoef;     // packed (see host), may be null
    const int* fcoef_off;    // per lidx*ntype+itype, -1 if none
};
void lelph_launch_projections(int k0, int nk, const KPointSym* ksym_dev, const double* gvec, const long long* pw_off,
                              const int* npw, const double* Fk, const long long* fk_off, const double2* chat,
                              const long long* chat_off, const NonlocalDesc& nl, const GeomDev& g, int f32acc,
                              double2* proj, cudaStream_t st);
// the same projections on the tensor cores (mixed form; projections_tc.cu):
// TF32 split operands built in shared memory, FP64 sums; proj is overwritten
// (chat: the unfolded coefficients as double2, or as float2 with chat_f32)
int lelph_projections_tc_supported(const NonlocalDesc& nl);
int lelph_launch_projections_tc(int k0, int nk, const KPointSym* ksym_dev, const double* gvec,
                                const long long* pw_off, const int* npw, const double* Fk, const long long* fk_off,
                                const void* chat, int chat_f32, const long long* chat_off, const NonlocalDesc& nl,
                                const GeomDev& g, double2* proj, unsigned* status, unsigned long long wait_ns,
                                cudaStream_t st);
void lelph_launch_finish(const PairInfo* pairs, int npairs, int mode_fp64, const double2* glocal,
                         const float* partials, int nchunks, const float* mode_scale, const float* band_scale,
                         const double2* proj, const double2* eig, int non_loc, const NonlocalDesc& nl,
                         const GeomDev& g, int out_c64, void* gout, cudaStream_t st);

// ---------------------------------------------------------- local bare potential
#define LELPH_VLOC_MAXTYPE 16
#define LELPH_VLOC_MAXMODES 48
struct VlocDesc
{
    int Nx, Ny, Nz;             // the reference's FFT box
    int natom, ntype, nmodes;
    int npts;                   // |G| table points, spacing dg
    int dim2;                   // 2-D Coulomb cutoff (slab along z)
    double q[3];                // crystal coordinates
    double blat[9];             // b_i = blat[:, i], 2 pi included
    double alat_zz;             // alat_vec[2][2], the slab period used by the cutoff
    double dg, volume;
    double zval[LELPH_VLOC_MAXTYPE];
    const double* v;            // (ntype, npts) V_loc(|G|)
    const double* dv;           // (ntype, npts) spline slopes
    const double* atom_pos;     // (natom, 3) cartesian
    const int* atom_type;       // (natom)
};
void lelph_launch_vloc_table(const double* r, const double* wrab, const double* vloc, int ngrid, double zval,
                             double volume, int cut3, double dg, int npts, double* out, cudaStream_t st);
int lelph_launch_dvloc_g(const VlocDesc& vd, const double2* eig, double2* out, unsigned* status, cudaStream_t st);
void lelph_launch_add_dvscf(double2* dv, const double2* vloc, int nmodes, int nmag, long long N, cudaStream_t st);

// ------------------------------------------------------------ dV rotation
struct RotDvDesc
{
    int Nx, Ny, Nz, nmodes, nmag;
    int trev, composite;
    double sym_red[9];   // crystal action on box coordinates (rows), sign of time reversal included
    double tau_red[3];   // fractional translation in box (crystal) units
    double2 ph;          // e^{-i (S q).tau}
    double2 su2[4];      // SU(2) matrix of the operation (nmag = 4)
};
void lelph_launch_rotate_dvscf(const RotDvDesc& rd, const double2* in, double2* out, unsigned* status,
                               cudaStream_t st);

// ------------------------------------------------------------ Dmats
struct DmatGeom
{
    int nb, nspin, nspinor;
    int Nx, Ny, Nz;  // the reference's FFT box (Miller range of the plane-wave lists)
    int ntab;        // Nx + Ny + Nz + 3 per-axis phase factors
};
// One (symmetry R, full-BZ k) job: k = S1 k1, Rk = S2 k2 (irreducible k1, k2).
// D[b][a] = sum_{p,t} v_{b,t}(p) y~_{a,t}(p): y~ = psi_k1 (conjugated when
// conj_w), v = C e^{-i 2 pi m.t} M x~ with x~ = psi_k2 at the matched plane
// wave (conjugated when conj_v), m the Miller index of plane wave p of k1.
struct DmatJob
{
    int ik1, ik2;
    int WRS1[9];     // R S1 on Miller indices (row-major)
    int W2inv[9];    // S2^-1 on Miller indices
    int ulm[3];      // G0 = S2 k2 - R S1 k1 (crystal)
    int conj_w, conj_v;
    double t[3];     // phase vector
    double2 C;       // constant phase
    double2 M[4];    // 2x2 spinor matrix (row-major)
};
static_assert(sizeof(DmatJob) == 208, "DmatJob layout");
// jobs perm[first .. first + count) share ik1 and conj_w (tensor-core form)
struct DmatGroup
{
    int first, count, ik1, conj_w;
};
// tensor-core form of the mixed Dmats (dmats.cu): jobs grouped by (ik1, conj_w)
// into groups of at most JB (lelph_dmats_tc_config); out is overwritten
void lelph_dmats_tc_config(int nb, int* JB, int* nbt, int* NT, int* ntiles);
int lelph_dmats_tc_supported(const DmatGeom& dg);
// coef32t: the FP32 coefficients in the plane-wave-major order of lelph_launch_dm_c64t
void lelph_launch_dm_c64t(const double2* in, const long long* coef_off, const int* npw, int nk, int nspin, int nb,
                          int ns, float2* out, cudaStream_t st);
int lelph_launch_dmats_tc(const DmatJob* jobs, long long njobs, const DmatGroup* groups, const int* perm,
                          int ngroups, const DmatGeom& dg, const float2* coef32, const float2* coef32t,
                          const long long* coef_off, const int* miller, const long long* pw_off, const int* npw,
                          const int* gtab, int npw_max, int* map, double2* out, unsigned* status,
                          unsigned long long wait_ns, cudaStream_t st);
size_t lelph_dmats_smem_bytes(const DmatGeom& dg, int fp64);
void lelph_launch_dm_gtab(const int* miller, const long long* pw_off, const int* npw, int nk, int npw_max, int Nx,
                          int Ny, int Nz, int* gtab, cudaStream_t st);
void lelph_launch_dm_c64(const double2* in, long long n, float2* out, cudaStream_t st);
// index maps (njobs x npw_max ints in `map`) then the contraction: FP32
// operands from coef32 when it is given (mixed form), else FP64 from coef64
int lelph_launch_dmats(const DmatJob* jobs, long long njobs, const DmatGeom& dg, const double2* coef64,
                       const float2* coef32,
                       const long long* coef_off, const int* miller, const long long* pw_off, const int* npw,
                       const int* gtab, int npw_max, int* map, double2* out, cudaStream_t st);

// ------------------------------------------------------------ q-star expansion
// One (star member, k) item: g of row src (the irreducible q at k) rotated
// with Dl = D[dl] (k+q) and Dr = D[dr] (k) into row dst (the member at S k).
struct QStarItem
{
    int src, dst;
    long long dl, dr;  // matrix indices in the Dmats array (each nspin x nb x nb)
    int trev;
    int pad;
};
size_t lelph_qstar_smem_bytes(int nb, int fp64);
int lelph_launch_qstar(const QStarItem* items, long long nitems, int nb, int nspin, int nmodes, const double2* D,
                       int fp64, int out_c64, const void* g, void* out, cudaStream_t st);

// ------------------------------------------------------------ dV_scf ingest
// raw (pattern, nmag, Nz, Ny, Nx) -> out (mode, nmag, Nx, Ny, Nz) = M raw, M = eig pats^H
int lelph_launch_dvscf_ingest(const double2* raw, const double2* M, int nmodes, int nmag, int Nx, int Ny, int Nz,
                              double2* out, cudaStream_t st);
