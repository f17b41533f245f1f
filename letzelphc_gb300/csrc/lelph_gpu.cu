// Host side of the C ABI declared in include/lelph_gpu.h.
//
// Owns the device state of one context: the iBZ wavefunctions and form
// factors, the unfolded full-BZ wavefunctions on the FFT grid (FP64 boxes for
// the plain form, split 16-bit tensor-core operands for the mixed form), the
// KB projections, the q slots (dV_scf, eigVec) and the run workspaces.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/lelph_gpu.h"
#include "lelph_common.cuh"
#include "lelph_internal.h"

namespace
{
const double PI_T = 3.1415927;  // src/common/constants.h:11
const double EPS_K = 1e-5;      // ELPH_EPS, src/common/constants.h:9

struct DevBuf
{
    void* p = nullptr;
    size_t n = 0;
};
}  // namespace

struct QSlot
{
    bool set = false;
    double q[3];
    std::vector<int> ulms;  // distinct umklapp vectors (3 ints each) of every k+q and k-q pair of this q
    int dmin[3];            // first G' - G1 of the window of differences this q needs
};

struct lelph_gpu
{
    lelph_gpu_desc d;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaStream_t st_copy = nullptr;    // copies of finished output batches to the host (run)
    cudaEvent_t evc[2] = {nullptr, nullptr};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t evg0 = nullptr, evg1 = nullptr;  // per-kernel timing of the G-space route (profiling on)
    // always-on events around each local-sandwich launch of a run (one pair per
    // batch), read after the run's own synchronisation: the kernel's time in
    // back-to-back work, without the synchronisations of the profiling mode
    std::vector<cudaEvent_t> evlive;
    bool profiling = false;
    std::string err;
    lelph_gpu_stats stats;
    GeomDev g;
    int nltimesj = 0, ntype = 0;
    int nproj_max = 0;
    int ab_bf16 = 0;
    unsigned long long wait_ns = 0;  // limit of each pipeline wait of the tensor-core sandwich (0: default)
    bool mixed = false;
    bool prepared = false;
    bool gspace = false;  // G-space route of the local sandwich
    bool proj_tc = false;  // KB projections on the tensor cores (mixed form)
    // host copies
    std::vector<double> alat, blat, kibz, kbz_crys, symR, symtau, atom_pos, PP, Fsign;
    std::vector<int> kmap, symtr, atom_type, npw;
    std::vector<long long> pw_off, coef_off, fk_off, chat_off;
    std::vector<KPointSym> ksym;
    std::vector<float> band_scale;  // (nk_bz, nspin, nb)
    std::vector<int> miller;        // concatenated (npw*3)
    std::vector<QSlot> qslots;
    long long total_pw = 0;
    // device buffers
    std::vector<DevBuf*> owned;
    DevBuf d_miller, d_pwoff, d_npw, d_coef, d_coefoff, d_gvec, d_fk, d_fkoff, d_ksym, d_chat, d_chatoff;
    DevBuf d_psi64, d_boxes32, d_bsplit, d_psi32, d_band_scale, d_proj;
    DevBuf d_atype, d_apos, d_pp, d_fsign, d_fcoef, d_fcoefoff;
    DevBuf d_tw64[3], d_tw32[3], d_twN[3], d_twN32[3];
    DevBuf d_dvr, d_eig, d_maxabs;                 // per q slot: dV_scf on the reference box (FP64), eigVec
    DevBuf d_win64, d_win32, d_winscale, d_wtmpN, d_wtmpM;  // dV windows on the product grid, per (slot, umklapp)
    DevBuf d_pairs, d_glocal, d_partials, d_gout, d_status, d_tmp;
    std::vector<int> ulms_all;  // every q slot's umklapp list, the host side of one upload
    FftPlan1D plan[3];   // product grid (g.Nx, g.Ny, g.Nz)
    FftPlan1D planN[3];  // the reference's FFT box
    int Nbox[3] = {0, 0, 0};
    double Rc[3] = {0, 0, 0};  // largest |k+G| component (crystal units) over every rotated sphere
    std::vector<int> win_base;  // first window entry of each q slot
    int nwin = 0;
    bool windows_ok = false;
    CUtensorMap tmapB, tmapP, tmapV;
    void* tmapV_base = nullptr;
    int tmapV_rows = 0;
    int nslots_alloc = 0;
    int chunk_pts = 0, nchunks = 0;
    // local bare potential: V_loc(|G|) table and its spline slopes per species
    DevBuf d_vl_v, d_vl_dv, d_vl_in, d_vloc;
    DevBuf d_colmask;  // box occupancy of every full-BZ k (z-columns of all k, then x planes of all k)
    DevBuf d_collist, d_colcnt;  // occupied z-columns of every k as lists
    bool boxmask_ready = false;  // occupancy and lists built (geometry only: they stay valid)
    // Dmats: Miller -> position tables of the iBZ lists, the job table and the
    // last block of representation matrices (jobs dm_first .. dm_first + dm_count - 1)
    DevBuf d_dmgtab, d_dmjobs, d_dmats, d_dmmap, d_dmcoef32, d_dmstar, d_gstar, d_qsitems;
    DevBuf d_dmgroups, d_dmperm, d_dmcoefT;  // job groups, plane-wave-major FP32 coefficients (tensor-core Dmats)
    bool dm_coefT_ready = false;
    DevBuf d_dvraw;  // QE-layout dV_scf of the last ingest and eig pats^H
    bool dm_coef32_ready = false;
    long long coef_total = 0;  // complex coefficients of every iBZ k
    std::unordered_map<long long, int> khash;  // full-BZ k-points by wrapped, quantised coordinates
    bool dm_gtab_ready = false;
    long long dm_first = 0, dm_count = 0;
    int dm_nsym = 0;
    std::vector<double> dm_R, dm_tau;  // the symmetries of the resident block
    std::vector<int> dm_trev;
    bool vl_ready = false;
    int vl_npts = 0, vl_dim2 = 0;
    double vl_dg = 0, vl_volume = 0;
    std::vector<double> vl_zval;
    // G-space route: every full-BZ k's sphere (its k+q role) sorted by
    // ((y, z) column, x) on the product grid, and the k+q coefficients stored
    // in that order (Bp); psi(r) of one k at a time and the pass buffers
    std::vector<int> gs_npad, gs_ncol, gs_nzl;
    std::vector<long long> gs_perm_off, gs_col_off, gs_cst_off, gs_bp_off, gs_zl_off;
    int gs_npad_max = 0, gs_ncol_max = 0;
    long long gs_bp_total = 0;
    DevBuf d_gs_perm, d_gs_kcx, d_gs_cols, d_gs_cst, d_gs_npw, d_gs_npad, d_gs_permoff, d_gs_bpoff, d_gs_bp;
    DevBuf d_gs_psi, d_gs_out1, d_gs_A, d_gs_part;
    DevBuf d_gs_bq;      // mixed form on the tensor cores: the pair's k+q operand split into TF32 hi / lo
    bool gs_tc = false;  // mixed G-space GEMM on the tensor cores (gspace_tc.cu)
    DevBuf d_gs_zl, d_gs_cols2;  // z lines holding a column of the sphere; column index into the pruned plane
};

namespace
{
int fail(lelph_gpu* h, int code, const std::string& msg)
{
    if (h) h->err = msg;
    return code;
}

#define CUDA_TRY(h, call)                                                                                  \
    do                                                                                                     \
    {                                                                                                      \
        cudaError_t e__ = (call);                                                                          \
        if (e__ != cudaSuccess)                                                                            \
            return fail((h), e__ == cudaErrorMemoryAllocation ? LELPH_GPU_ERR_ALLOC : LELPH_GPU_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e__));                              \
    } while (0)

// Runs work(w) for every w in [0, nthr): worker 0 on the calling thread, the
// others on new threads.  A worker whose thread cannot be started (a limit on
// threads) runs on the calling thread instead, so the limit costs time, not
// the call.
template <typename F>
void run_workers(int nthr, F&& work)
{
    std::vector<std::thread> pool;
    std::vector<int> here;
    for (int w = 1; w < nthr; ++w)
    {
        try
        {
            pool.emplace_back(work, w);
        }
        catch (const std::system_error&)
        {
            here.push_back(w);
        }
    }
    work(0);
    for (int w : here) work(w);
    for (auto& t : pool) t.join();
}

int ensure(lelph_gpu* h, DevBuf& b, size_t bytes)
{
    if (b.n >= bytes && b.p) return LELPH_GPU_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return fail(h, LELPH_GPU_ERR_ALLOC, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    b.n = bytes;
    return LELPH_GPU_OK;
}

int upload(lelph_gpu* h, DevBuf& b, const void* src, size_t bytes)
{
    int rc = ensure(h, b, bytes);
    if (rc) return rc;
    if (bytes) CUDA_TRY(h, cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, h->st));
    return LELPH_GPU_OK;
}

void mat_vec3(const double* M, const double* v, bool trans, double* out)
{
    if (trans)
    {
        out[0] = M[0] * v[0] + M[3] * v[1] + M[6] * v[2];
        out[1] = M[1] * v[0] + M[4] * v[1] + M[7] * v[2];
        out[2] = M[2] * v[0] + M[5] * v[1] + M[8] * v[2];
    }
    else
    {
        out[0] = M[0] * v[0] + M[1] * v[1] + M[2] * v[2];
        out[1] = M[3] * v[0] + M[4] * v[1] + M[5] * v[2];
        out[2] = M[6] * v[0] + M[7] * v[1] + M[8] * v[2];
    }
}

double det3(const double* m)
{
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
           m[2] * (m[7] * m[3] - m[4] * m[6]);
}

// SU(2) matrix of a rotation (Euler angles), -i sigma_y for time reversal:
// the construction of SU2mat, src/wfc/su2mat.c:16-117
bool su2mat(const double* sym_in, int nspinor, bool time_rev, std::complex<double>* u)
{
    typedef std::complex<double> C;
    if (nspinor == 1)
    {
        u[0] = 1.0;
        u[1] = u[2] = 0.0;
        u[3] = 1.0;
        return true;
    }
    double det = det3(sym_in);
    if (std::fabs(std::fabs(det) - 1) > 1e-4) return false;
    double s[9];
    for (int i = 0; i < 9; ++i) s[i] = sym_in[i] / det;
    double alpha, beta, delta;
    if (std::fabs(s[6] + 1) < EPS_K)
    {
        alpha = 0;
        beta = PI_T / 2.0;
        delta = std::atan2(s[1], s[2]);
    }
    else if (std::fabs(s[6] - 1) < EPS_K)
    {
        alpha = 0;
        beta = -PI_T / 2.0;
        delta = std::atan2(-s[1], -s[2]);
    }
    else
    {
        beta = -std::asin(s[6]);
        alpha = std::atan2(s[3] / std::cos(beta), s[0] / std::cos(beta));
        delta = std::atan2(s[7] / std::cos(beta), s[8] / std::cos(beta));
    }
    alpha /= 2;
    beta /= 2;
    delta /= 2;
    const C I(0, 1);
    C p0[4] = {1, 0, 0, 1}, px[4] = {0, 1, 1, 0}, py[4] = {0, -I, I, 0}, pz[4] = {1, 0, 0, -1};
    C sd[4], sb[4], sa[4], t[4];
    for (int i = 0; i < 4; ++i)
    {
        sd[i] = std::cos(delta) * p0[i] - I * std::sin(delta) * px[i];
        sb[i] = std::cos(beta) * p0[i] - I * std::sin(beta) * py[i];
        sa[i] = std::cos(alpha) * p0[i] - I * std::sin(alpha) * pz[i];
    }
    auto mm = [](const C* a, const C* b, C* o) {
        o[0] = a[0] * b[0] + a[1] * b[2];
        o[1] = a[0] * b[1] + a[1] * b[3];
        o[2] = a[2] * b[0] + a[3] * b[2];
        o[3] = a[2] * b[1] + a[3] * b[3];
    };
    mm(sb, sd, t);
    mm(sa, t, u);
    if (time_rev)
    {
        C a1 = u[0], b1 = u[1], c1 = u[2], d1 = u[3];
        u[0] = -c1;
        u[1] = -d1;
        u[2] = a1;
        u[3] = b1;
    }
    return true;
}

bool plan_1d(int L, FftPlan1D& p)
{
    p.L = L;
    p.nstage = 0;
    int n = L;
    while (n % 4 == 0 && p.nstage < LELPH_MAX_RADIX_STAGES)
    {
        p.radix[p.nstage++] = 4;
        n /= 4;
    }
    const int rs[3] = {2, 3, 5};
    for (int r : rs)
        while (n % r == 0 && p.nstage < LELPH_MAX_RADIX_STAGES)
        {
            p.radix[p.nstage++] = r;
            n /= r;
        }
    return n == 1;
}

float pow2_scale(double bound, double target)
{
    if (!(bound > 0)) return 1.0f;
    int e = (int)std::floor(std::log2(target / bound));
    if (e > 100) e = 100;
    if (e < -100) e = -100;
    return std::ldexp(1.0f, e);
}

// -------------------------------------------------------------- small kernels

// scaled FP32 copy of nwin windows (rows (mode, component) of M points) into the
// tile-major window array: 32-point blocks of all ncomp rows of a window contiguous
template <typename T2>
__global__ void k_dv_convert(const T2* __restrict__ in, float2* __restrict__ out, int nwin, int ncomp,
                             long long M, int wbase, int nmag, const float* __restrict__ scale)
{
    const long long nkb = M / 32;
    const long long n = (long long)nwin * ncomp * M;
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n; o += (long long)gridDim.x * blockDim.x)
    {
        const int p = (int)(o & 31);
        long long t = o >> 5;
        const int row = (int)(t % ncomp);
        t /= ncomp;
        const long long kb = t % nkb;
        const int w = (int)(t / nkb);
        const T2 v = in[((size_t)w * ncomp + row) * M + kb * 32 + p];
        const float sc = scale[(size_t)w * (ncomp / nmag) + row / nmag];  // a power of two: exact in either type
        out[(((size_t)(wbase + w) * nkb + kb) * ncomp + row) * 32 + p] = make_float2((float)(v.x * sc), (float)(v.y * sc));
    }
}

// max over r (and spin rows s) of sum_{s'} |dV^{s s'}(r)| per mode -> atomicMax on float bits
template <typename T2>
__global__ void k_dv_maxabs(const T2* __restrict__ dv, int nmodes, int nmag, long long N,
                            unsigned* __restrict__ maxbits)
{
    const int nu = blockIdx.y;
    const T2* d = dv + (size_t)nu * nmag * N;
    // in the operand type: the result only picks a power-of-two scale with a margin
    typedef decltype(T2().x) R;
    float m = 0.f;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < N; r += (long long)gridDim.x * blockDim.x)
    {
        R v;
        if (nmag == 4)
        {
            const R a0 = hypot(d[r].x, d[r].y) + hypot(d[N + r].x, d[N + r].y);
            const R a1 = hypot(d[2 * N + r].x, d[2 * N + r].y) + hypot(d[3 * N + r].x, d[3 * N + r].y);
            v = a0 > a1 ? a0 : a1;
        }
        else
        {
            v = 0;
            for (int c = 0; c < nmag; ++c)
            {
                const R h = hypot(d[c * N + r].x, d[c * N + r].y);
                v = h > v ? h : v;
            }
        }
        m = fmaxf(m, (float)v);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&maxbits[nu], __float_as_uint(m));
}

__global__ void k_mode_scale(const unsigned* __restrict__ maxbits, int nmodes, float* __restrict__ scale)
{
    int nu = blockIdx.x * blockDim.x + threadIdx.x;
    if (nu < nmodes)
    {
        float m = __uint_as_float(maxbits[nu]) * 1.0001f;
        // |dV s_nu| <= 2: together with |psi s_m| <= 2^14 the operand stays below 2^15
        int e = m > 0.f ? (int)floorf(log2f(2.0f / m)) : 0;
        scale[nu] = ldexpf(1.0f, e);
    }
}

// tmp[a][b] = sum_c op(g)[a][c] conj(Dr[b][c]), op(g)[a][c] = g[c][a] (conj if trev)
__global__ void k_qrot1(const double2* g, const double2* Dr, int nb, int nspin, int trev, double2* tmp)
{
    int mode = blockIdx.y, s = blockIdx.z;
    const double2* gq = g + ((size_t)mode * nspin + s) * nb * nb;
    const double2* D = Dr + (size_t)s * nb * nb;
    double2* t = tmp + ((size_t)mode * nspin + s) * nb * nb;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nb * nb; e += gridDim.x * blockDim.x)
    {
        int a = e / nb, b = e - a * nb;
        double2 acc = make_double2(0, 0);
        for (int c = 0; c < nb; ++c)
        {
            double2 x = gq[(size_t)c * nb + a];
            if (trev) x.y = -x.y;
            acc = cadd(acc, cmul(x, cconj(D[(size_t)b * nb + c])));
        }
        t[e] = acc;
    }
}

// out[i][j] = sum_k tmp[k][i] Dl[j][k]
__global__ void k_qrot2(const double2* tmp, const double2* Dl, int nb, int nspin, double2* out)
{
    int mode = blockIdx.y, s = blockIdx.z;
    const double2* t = tmp + ((size_t)mode * nspin + s) * nb * nb;
    const double2* D = Dl + (size_t)s * nb * nb;
    double2* o = out + ((size_t)mode * nspin + s) * nb * nb;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nb * nb; e += gridDim.x * blockDim.x)
    {
        int i = e / nb, j = e - i * nb;
        double2 acc = make_double2(0, 0);
        for (int k = 0; k < nb; ++k) acc = cadd(acc, cmul(t[(size_t)k * nb + i], D[(size_t)j * nb + k]));
        o[e] = acc;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn)
    {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

int make_tmap(lelph_gpu* h, CUtensorMap* m, void* base, unsigned long long inner, unsigned long long rows,
              unsigned box_rows, bool swz, bool f32 = false, unsigned box_inner = 64)
{
    auto enc = get_encode();
    if (!enc) return fail(h, LELPH_GPU_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    const unsigned long long es_bytes = f32 ? 4 : 2;
    cuuint64_t dims[2] = {inner, rows};
    cuuint64_t strides[1] = {inner * es_bytes};
    cuuint32_t box[2] = {box_inner, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(m, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, base, dims, strides,
                     box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     swz ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(h, LELPH_GPU_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string(r));
    return LELPH_GPU_OK;
}

// 3-D tile-major tensor: dims {inner, rows, blocks}, rows packed (stride inner
// elements), blocks packed (stride rows * inner elements)
int make_tmap3(lelph_gpu* h, CUtensorMap* m, void* base, bool f32, unsigned long long inner, unsigned long long rows,
               unsigned long long blocks, unsigned box_rows, unsigned box_blocks, bool swz)
{
    auto enc = get_encode();
    if (!enc) return fail(h, LELPH_GPU_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    const unsigned long long es_bytes = f32 ? 4 : 2;
    cuuint64_t dims[3] = {inner, rows, blocks};
    cuuint64_t strides[2] = {inner * es_bytes, rows * inner * es_bytes};
    cuuint32_t box[3] = {(cuuint32_t)inner, box_rows, box_blocks};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(m, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, base, dims, strides,
                     box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     swz ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(h, LELPH_GPU_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string(r));
    return LELPH_GPU_OK;
}

// key of a k-point on a 2^-20 lattice of its coordinates wrapped into [0, 1)
long long k_hash_key(const double* k)
{
    long long key = 0;
    for (int x = 0; x < 3; ++x)
    {
        const double f = k[x] - std::floor(k[x]);
        long long q = std::llround(f * 1048576.0) & 1048575;
        key = (key << 20) | q;
    }
    return key;
}

int find_k(const lelph_gpu* h, const double* kpt);

// find_k through a hash of the full-BZ list; a miss, or a hit that fails the
// reference's tolerance test, falls back to the linear search
int find_k_fast(lelph_gpu* h, const double* kpt)
{
    if (h->khash.empty())
        for (int i = 0; i < h->d.nkpts_BZ; ++i) h->khash.emplace(k_hash_key(&h->kbz_crys[3 * i]), i);
    auto it = h->khash.find(k_hash_key(kpt));
    if (it != h->khash.end())
    {
        const int i = it->second;
        double s = 0;
        for (int x = 0; x < 3; ++x)
        {
            double dd = h->kbz_crys[3 * i + x] - kpt[x];
            dd -= std::rint(dd);
            s += dd * dd;
        }
        // grid points lie far more than 2 EPS_K apart, so a point within
        // EPS_K is the one the linear search would return
        if (std::sqrt(s) < EPS_K) return i;
    }
    return find_k(h, kpt);
}

int find_k(const lelph_gpu* h, const double* kpt)
{
    const int nk = h->d.nkpts_BZ;
    for (int i = 0; i < nk; ++i)
    {
        double s = 0;
        for (int x = 0; x < 3; ++x)
        {
            double dd = h->kbz_crys[3 * i + x] - kpt[x];
            dd -= std::rint(dd);
            s += dd * dd;
        }
        if (std::sqrt(s) < EPS_K) return i;
    }
    return -1;
}

// umklapp G0 = S_kq k_kq - S_k k - q in crystal units for the pair
// (idx_k, idx_kq) (src/dvloc/compute_Vbare_loc.c:93-144); nonzero if not integral
int umklapp(const lelph_gpu* h, int idx_k, int idx_kq, const double* q, int* u)
{
    const KPointSym& sk = h->ksym[idx_k];
    const KPointSym& skq = h->ksym[idx_kq];
    double tkq[3], tk[3], qc[3], ulm[3], uc[3];
    mat_vec3(skq.R, &h->kibz[3 * skq.ik], false, tkq);
    mat_vec3(sk.R, &h->kibz[3 * sk.ik], false, tk);
    mat_vec3(h->blat.data(), q, false, qc);
    for (int x = 0; x < 3; ++x) ulm[x] = (tkq[x] - tk[x]) - qc[x] / (2 * PI_T);
    mat_vec3(h->alat.data(), ulm, true, uc);
    for (int x = 0; x < 3; ++x)
    {
        double r = std::rint(uc[x]);
        if (std::fabs(uc[x] - r) > 1e-3) return 1;
        u[x] = (int)r;
    }
    return 0;
}

// window entry of (q slot, umklapp vector), -1 if absent
int window_of(const lelph_gpu* h, int slot, const int* u)
{
    const std::vector<int>& L = h->qslots[slot].ulms;
    for (size_t e = 0; e < L.size(); e += 3)
        if (L[e] == u[0] && L[e + 1] == u[1] && L[e + 2] == u[2]) return h->win_base[slot] + (int)(e / 3);
    return -1;
}

int check_status(lelph_gpu* h)
{
    unsigned st = 0;
    CUDA_TRY(h, cudaMemcpyAsync(&st, h->d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    if (st & LELPH_DEV_ERR_TIMEOUT) return fail(h, LELPH_GPU_ERR_TIMEOUT, "a device-side wait ran out");
    if (st) return fail(h, LELPH_GPU_ERR_CUDA, "device status " + std::to_string(st));
    return LELPH_GPU_OK;
}

// Per-kernel device time while profiling (the G-space route's kernels, the
// preparation's roles): gs_tick marks
// the start, each gs_tock returns the time since the last mark and re-marks.
static void gs_tick(lelph_gpu* h)
{
    if (h->profiling) cudaEventRecord(h->evg0, h->st);
}
static double gs_tock(lelph_gpu* h)
{
    if (!h->profiling) return 0.0;
    cudaEventRecord(h->evg1, h->st);
    cudaEventSynchronize(h->evg1);
    float ms = 0;
    cudaEventElapsedTime(&ms, h->evg0, h->evg1);
    std::swap(h->evg0, h->evg1);
    return ms;
}

void tstart(lelph_gpu* h)
{
    if (h->profiling) cudaEventRecord(h->ev0, h->st);
}
double tstop(lelph_gpu* h)
{
    if (!h->profiling) return 0.0;
    cudaEventRecord(h->ev1, h->st);
    cudaEventSynchronize(h->ev1);
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    return ms;
}

NonlocalDesc nl_desc(lelph_gpu* h)
{
    NonlocalDesc nl;
    nl.natom = h->d.natom;
    nl.ntype = h->ntype;
    nl.nltimesj = h->nltimesj;
    nl.lmax = h->d.lmax;
    nl.nproj_max = h->nproj_max;
    nl.is_soc = h->d.is_soc_present;
    nl.atom_type = (const int*)h->d_atype.p;
    nl.atom_pos = (const double*)h->d_apos.p;
    nl.PP_table = (const double*)h->d_pp.p;
    nl.Fsign = (const double*)h->d_fsign.p;
    nl.fcoef = h->d_fcoef.n > 16 ? (const double*)h->d_fcoef.p : nullptr;
    nl.fcoef_off = (const int*)h->d_fcoefoff.p;
    return nl;
}
}  // namespace

// ====================================================================== API

extern "C" const char* lelph_gpu_strerror(int s)
{
    switch (s)
    {
        case LELPH_GPU_OK: return "ok";
        case LELPH_GPU_ERR_INVALID: return "invalid argument";
        case LELPH_GPU_ERR_ALLOC: return "allocation failed";
        case LELPH_GPU_ERR_CUDA: return "CUDA error";
        case LELPH_GPU_ERR_TIMEOUT: return "device wait timed out";
        case LELPH_GPU_ERR_GEOMETRY: return "inconsistent geometry (k+q, symmetry or FFT box)";
        case LELPH_GPU_ERR_STATE: return "call order";
        case LELPH_GPU_ERR_UNSUPPORTED: return "unsupported size";
        default: return "unknown status";
    }
}

extern "C" const char* lelph_gpu_last_error(lelph_gpu* h) { return h ? h->err.c_str() : "null context"; }

extern "C" void* lelph_gpu_stream(lelph_gpu* h) { return h ? (void*)h->st : nullptr; }

extern "C" int lelph_gpu_set_profiling(lelph_gpu* h, int on)
{
    if (!h) return LELPH_GPU_ERR_INVALID;
    h->profiling = on != 0;
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_set_wait_limit(lelph_gpu* h, unsigned long long ns)
{
    if (!h) return LELPH_GPU_ERR_INVALID;
    h->wait_ns = ns;
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_stats_get(lelph_gpu* h, lelph_gpu_stats* s)
{
    if (!h || !s) return LELPH_GPU_ERR_INVALID;
    *s = h->stats;
    size_t tot = 0;
    for (DevBuf* b : h->owned) tot += b->n;
    s->device_bytes = tot;
    s->product_grid[0] = h->g.Nx;
    s->product_grid[1] = h->g.Ny;
    s->product_grid[2] = h->g.Nz;
    s->chunk_points = h->chunk_pts;
    return LELPH_GPU_OK;
}

extern "C" void lelph_gpu_destroy(lelph_gpu* h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->st) cudaStreamSynchronize(h->st);
    for (DevBuf* b : h->owned)
        if (b->p) cudaFree(b->p);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->evg0) cudaEventDestroy(h->evg0);
    if (h->evg1) cudaEventDestroy(h->evg1);
    if (h->st_copy) cudaStreamSynchronize(h->st_copy);
    for (cudaEvent_t e : h->evc)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : h->evlive)
        if (e) cudaEventDestroy(e);
    if (h->st_copy) cudaStreamDestroy(h->st_copy);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
}

static int upload_wfc(lelph_gpu* h, const double* const* wfc)
{
    const lelph_gpu_desc& d = h->d;
    const int nsets = d.nspin * d.nbnds * d.nspinor;
    for (int ik = 0; ik < d.nkpts_iBZ; ++ik)
    {
        if (!wfc[ik]) return fail(h, LELPH_GPU_ERR_INVALID, "null wavefunction pointer");
        size_t bytes = sizeof(double2) * (size_t)nsets * h->npw[ik];
        CUDA_TRY(h, cudaMemcpyAsync((char*)h->d_coef.p + sizeof(double2) * h->coef_off[ik], wfc[ik], bytes,
                                    cudaMemcpyHostToDevice, h->st));
    }
    // power-of-two operand scales: |psi_b(r)| <= sum_G sum_s |c_b,s(G)| (L1 bound)
    const int nb = d.nbnds;
    // (the 1.0001 margin covers the rounding of the sum; the host cores share the k-points)
    std::vector<float> sc_ibz((size_t)d.nkpts_iBZ * d.nspin * nb);
    auto scales_of = [&](int ik) {
        for (int s = 0; s < d.nspin; ++s)
            for (int b = 0; b < nb; ++b)
            {
                const double* c = wfc[ik] + 2 * ((size_t)(s * nb + b) * d.nspinor * h->npw[ik]);
                double l1 = 0;
                for (long long i = 0; i < (long long)d.nspinor * h->npw[ik]; ++i)
                    l1 += std::sqrt(c[2 * i] * c[2 * i] + c[2 * i + 1] * c[2 * i + 1]);
                sc_ibz[((size_t)ik * d.nspin + s) * nb + b] = pow2_scale(l1 * 1.0001, 16384.0);
            }
    };
    {
        const int nthr = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), d.nkpts_iBZ));
        run_workers(nthr, [&](int w) {
            for (int ik = w; ik < d.nkpts_iBZ; ik += nthr) scales_of(ik);
        });
    }
    h->band_scale.resize((size_t)d.nkpts_BZ * d.nspin * nb);
    for (int i = 0; i < d.nkpts_BZ; ++i)
        for (int s = 0; s < d.nspin; ++s)
            for (int b = 0; b < nb; ++b)
                h->band_scale[((size_t)i * d.nspin + s) * nb + b] = sc_ibz[((size_t)h->ksym[i].ik * d.nspin + s) * nb + b];
    int rc = upload(h, h->d_band_scale, h->band_scale.data(), sizeof(float) * h->band_scale.size());
    if (rc) return rc;
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    h->prepared = false;
    h->dm_coef32_ready = false;
    h->dm_coefT_ready = false;
    return LELPH_GPU_OK;
}

// G-space route: the sphere of every full-BZ k (as the k+q wavefunction of a
// pair) on the product grid, sorted by ((y, z) column, x).  The sort order is
// the K order of the route's GEMM: the x pass then writes each column's
// sphere points as one contiguous run, and the k+q coefficients are stored
// permuted to it once (k_gs_bperm).  The box position of a plane wave is the
// one the scatter uses (W n modulo the grid), so no two plane waves of a
// sphere share one (the product grid spans more than the sphere's diameter).
static int gs_tables(lelph_gpu* h)
{
    const lelph_gpu_desc& d = h->d;
    const GeomDev& g = h->g;
    const int nk = d.nkpts_BZ;
    std::vector<std::vector<int>> perm(nk), kcx(nk), cols(nk), cst(nk), zls(nk), cols2(nk);
    std::vector<int> bad(nk, 0);
    auto one = [&](int k) {
        const KPointSym& ks = h->ksym[k];
        const int npw = h->npw[ks.ik];
        const int* mil = &h->miller[3 * h->pw_off[ks.ik]];
        std::vector<std::pair<long long, int>> v(npw);
        for (int p = 0; p < npw; ++p)
        {
            const int* n = mil + 3 * p;
            int G[3], N3[3] = {g.Nx, g.Ny, g.Nz};
            for (int r = 0; r < 3; ++r)
            {
                G[r] = (ks.W[3 * r] * n[0] + ks.W[3 * r + 1] * n[1] + ks.W[3 * r + 2] * n[2]) % N3[r];
                if (G[r] < 0) G[r] += N3[r];
            }
            v[p] = {((long long)G[1] * g.Nz + G[2]) * g.Nx + G[0], p};
        }
        std::sort(v.begin(), v.end());
        std::vector<int>& pm = perm[k];
        std::vector<int>& kc = kcx[k];
        std::vector<int>& cl = cols[k];
        std::vector<int>& cs = cst[k];
        pm.resize(npw);
        kc.resize(npw);
        long long last_col = -1;
        for (int K = 0; K < npw; ++K)
        {
            if (K > 0 && v[K].first == v[K - 1].first) bad[k] = 1;
            const long long col = v[K].first / g.Nx;
            const int x = (int)(v[K].first - col * g.Nx);
            if (col != last_col)
            {
                cl.push_back((int)col);
                cs.push_back(K);
                last_col = col;
            }
            pm[K] = v[K].second;
            kc[K] = (int)(cl.size() - 1) * g.Nx + x;
        }
        cs.push_back(npw);
        // z lines of the sphere's columns, and each column's place in the
        // result of the y transform run on those lines only
        std::vector<int>& zl = zls[k];
        std::vector<int> zpos(g.Nz, -1);
        for (int c : cl) zpos[c % g.Nz] = 1;
        for (int z = 0; z < g.Nz; ++z)
            if (zpos[z] > 0)
            {
                zpos[z] = (int)zl.size();
                zl.push_back(z);
            }
        std::vector<int>& c2 = cols2[k];
        c2.resize(cl.size());
        for (size_t c = 0; c < cl.size(); ++c) c2[c] = (cl[c] / g.Nz) * (int)zl.size() + zpos[cl[c] % g.Nz];
    };
    {
        const int nthr = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), nk));
        run_workers(nthr, [&](int w) {
            for (int k = w; k < nk; k += nthr) one(k);
        });
    }
    for (int k = 0; k < nk; ++k)
        if (bad[k]) return fail(h, LELPH_GPU_ERR_GEOMETRY, "G-space route: two plane waves share a product-grid point");
    const int nrowk = d.nspin * d.nbnds * d.nspinor;
    h->gs_npad.resize(nk);
    h->gs_ncol.resize(nk);
    h->gs_perm_off.resize(nk);
    h->gs_col_off.resize(nk);
    h->gs_cst_off.resize(nk);
    h->gs_bp_off.resize(nk);
    h->gs_nzl.resize(nk);
    h->gs_zl_off.resize(nk);
    std::vector<int> npw_k(nk);
    long long po = 0, co = 0, so = 0, bo = 0, zo = 0;
    h->gs_npad_max = h->gs_ncol_max = 0;
    for (int k = 0; k < nk; ++k)
    {
        npw_k[k] = (int)perm[k].size();
        h->gs_npad[k] = (npw_k[k] + 7) / 8 * 8;
        h->gs_ncol[k] = (int)cols[k].size();
        h->gs_perm_off[k] = po;
        h->gs_col_off[k] = co;
        h->gs_cst_off[k] = so;
        h->gs_bp_off[k] = bo;
        po += h->gs_npad[k];
        co += h->gs_ncol[k];
        so += h->gs_ncol[k] + 1;
        bo += (long long)nrowk * h->gs_npad[k];
        h->gs_nzl[k] = (int)zls[k].size();
        h->gs_zl_off[k] = zo;
        zo += h->gs_nzl[k];
        h->gs_npad_max = std::max(h->gs_npad_max, h->gs_npad[k]);
        h->gs_ncol_max = std::max(h->gs_ncol_max, h->gs_ncol[k]);
    }
    h->gs_bp_total = bo;
    std::vector<int> pall(po, 0), kall(po, 0), call(co), sall(so), c2all(co), zall(std::max(1LL, zo));
    for (int k = 0; k < nk; ++k)
    {
        std::copy(perm[k].begin(), perm[k].end(), pall.begin() + h->gs_perm_off[k]);
        std::copy(kcx[k].begin(), kcx[k].end(), kall.begin() + h->gs_perm_off[k]);
        std::copy(cols[k].begin(), cols[k].end(), call.begin() + h->gs_col_off[k]);
        std::copy(cst[k].begin(), cst[k].end(), sall.begin() + h->gs_cst_off[k]);
        std::copy(cols2[k].begin(), cols2[k].end(), c2all.begin() + h->gs_col_off[k]);
        std::copy(zls[k].begin(), zls[k].end(), zall.begin() + h->gs_zl_off[k]);
    }
    int rc;
    if ((rc = upload(h, h->d_gs_perm, pall.data(), sizeof(int) * pall.size()))) return rc;
    if ((rc = upload(h, h->d_gs_kcx, kall.data(), sizeof(int) * kall.size()))) return rc;
    if ((rc = upload(h, h->d_gs_cols, call.data(), sizeof(int) * call.size()))) return rc;
    if ((rc = upload(h, h->d_gs_cst, sall.data(), sizeof(int) * sall.size()))) return rc;
    if ((rc = upload(h, h->d_gs_cols2, c2all.data(), sizeof(int) * c2all.size()))) return rc;
    if ((rc = upload(h, h->d_gs_zl, zall.data(), sizeof(int) * zall.size()))) return rc;
    if ((rc = upload(h, h->d_gs_npw, npw_k.data(), sizeof(int) * nk))) return rc;
    if ((rc = upload(h, h->d_gs_npad, h->gs_npad.data(), sizeof(int) * nk))) return rc;
    if ((rc = upload(h, h->d_gs_permoff, h->gs_perm_off.data(), sizeof(long long) * nk))) return rc;
    if ((rc = upload(h, h->d_gs_bpoff, h->gs_bp_off.data(), sizeof(long long) * nk))) return rc;
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_create(const lelph_gpu_desc* desc, lelph_gpu** out)
{
    if (!desc || !out) return LELPH_GPU_ERR_INVALID;
    *out = nullptr;
    lelph_gpu* h = new (std::nothrow) lelph_gpu();
    if (!h) return LELPH_GPU_ERR_ALLOC;
    memset(&h->stats, 0, sizeof(h->stats));
    h->d = *desc;
    const lelph_gpu_desc& d = h->d;
    auto bad = [&](int code, const std::string& m) {
        fprintf(stderr, "lelph_gpu_create: %s\n", m.c_str());
        lelph_gpu_destroy(h);
        return code;
    };
    if (d.natom <= 0 || d.nsym <= 0 || d.nbnds <= 0 || d.nkpts_iBZ <= 0 || d.nkpts_BZ <= 0 || d.ntype <= 0 ||
        d.nltimesj < 0 || d.lmax < 0 || d.lmax > 3)
        return bad(LELPH_GPU_ERR_INVALID, "non-positive size");
    if (d.nspin < 1 || d.nspin > 2 || d.nspinor < 1 || d.nspinor > 2) return bad(LELPH_GPU_ERR_INVALID, "nspin/nspinor");
    if (!(d.nmag == 1 || d.nmag == 2 || d.nmag == 4)) return bad(LELPH_GPU_ERR_INVALID, "nmag");
    if (d.nmag == 2 && (d.nspin != 2 || d.nspinor != 1)) return bad(LELPH_GPU_ERR_INVALID, "Incompatible dvscf");
    if (d.nmag == 4 && d.nspinor != 2) return bad(LELPH_GPU_ERR_INVALID, "nmag 4 needs spinors");
    if (d.nspin == 2 && d.nmag != 2) return bad(LELPH_GPU_ERR_INVALID, "nspin 2 needs nmag 2");
    if (d.nmodes != 3 * d.natom) return bad(LELPH_GPU_ERR_INVALID, "nmodes != 3 natom");
    if (3 * d.natom > 48) return bad(LELPH_GPU_ERR_UNSUPPORTED, "more than 16 atoms");
    if (!d.alat_vec || !d.blat_vec || !d.atomic_pos || !d.atom_type || !d.kpt_iredBZ || !d.kpt_fullBZ_crys ||
        !d.kmap || !d.sym_Rmat || !d.sym_tau || !d.sym_time_rev || !d.npw || !d.gvec || !d.wfc || !d.Fk ||
        !d.PP_table || !d.Fsign)
        return bad(LELPH_GPU_ERR_INVALID, "null input pointer");
    if (d.precision < 0 || d.precision > 2) return bad(LELPH_GPU_ERR_INVALID, "precision");
    h->mixed = d.precision != LELPH_GPU_FP64;
    h->ab_bf16 = d.precision == LELPH_GPU_MIXED_BF16;
    h->device = d.device;
    for (int x = 0; x < 3; ++x)
    {
        if (d.fft_dims[x] <= 0 || !plan_1d(d.fft_dims[x], h->planN[x]))
            return bad(LELPH_GPU_ERR_UNSUPPORTED, "FFT dimension must factor into 2, 3, 5");
        h->Nbox[x] = d.fft_dims[x];
    }
    h->g.nspin = d.nspin;
    h->g.nspinor = d.nspinor;
    h->g.nbnds = d.nbnds;
    h->g.nbp = (d.nbnds + 7) / 8 * 8;
    h->g.nmag = d.nmag;
    h->g.nmodes = d.nmodes;
    h->g.mt_modes = lelph_tc_tile_modes(d.nmodes, d.nbnds);
    // 64-point pipeline stages when three stages and two A slots fit, else 32
    h->g.kpts = 64;
    if (!lelph_local_tc_supported(h->g)) h->g.kpts = 32;
    {
        GeomDev g3 = h->g;
        if (h->g.kpts == 64 && lelph_local_tc_smem_bytes(g3) > 0)
        {
            // a 64-point ring shallower than three stages loses to 32-point stages
            g3.kpts = 64;
            if (lelph_local_tc_stages(g3) < 3) h->g.kpts = 32;
        }
    }
    if (d.route < LELPH_GPU_ROUTE_AUTO || d.route > LELPH_GPU_ROUTE_GSPACE) return bad(LELPH_GPU_ERR_INVALID, "route");
    const bool tc_ok = !h->mixed || (2 * h->g.nbp <= 128 && lelph_local_tc_supported(h->g));
    if (d.route == LELPH_GPU_ROUTE_REAL && !tc_ok)
        return bad(LELPH_GPU_ERR_UNSUPPORTED, "the real-space route of the mixed form supports up to 64 bands");
    h->gspace = d.route == LELPH_GPU_ROUTE_GSPACE || !tc_ok;
    {
        // the mixed G-space GEMM on the tensor cores unless the descriptor asks for
        // the SIMT GEMM (or LELPH_GS_TC=0)
        if (d.gs_gemm < 0 || d.gs_gemm > LELPH_GPU_GS_GEMM_SIMT) return bad(LELPH_GPU_ERR_INVALID, "gs_gemm");
        if (d.gs_gemm == LELPH_GPU_GS_GEMM_TENSOR && h->mixed && !lelph_gs_tc_supported(d.nbnds))
            return bad(LELPH_GPU_ERR_UNSUPPORTED, "the tensor-core G-space GEMM does not take this band count");
        const char* e = std::getenv("LELPH_GS_TC");
        h->gs_tc = h->mixed && lelph_gs_tc_supported(d.nbnds) && d.gs_gemm != LELPH_GPU_GS_GEMM_SIMT &&
                   !(e && e[0] == '0');
        // the mixed form's KB projections on the tensor cores unless LELPH_PROJ_TC=0
        const char* ep = std::getenv("LELPH_PROJ_TC");
        h->proj_tc = h->mixed && !(ep && ep[0] == '0');
    }
    h->ntype = d.ntype;
    h->nltimesj = d.nltimesj;
    // host copies
    h->alat.assign(d.alat_vec, d.alat_vec + 9);
    h->blat.assign(d.blat_vec, d.blat_vec + 9);
    h->kibz.assign(d.kpt_iredBZ, d.kpt_iredBZ + 3 * d.nkpts_iBZ);
    h->kbz_crys.assign(d.kpt_fullBZ_crys, d.kpt_fullBZ_crys + 3 * d.nkpts_BZ);
    h->kmap.assign(d.kmap, d.kmap + 2 * d.nkpts_BZ);
    h->symR.assign(d.sym_Rmat, d.sym_Rmat + 9 * d.nsym);
    h->symtau.assign(d.sym_tau, d.sym_tau + 3 * d.nsym);
    h->symtr.assign(d.sym_time_rev, d.sym_time_rev + d.nsym);
    h->atom_pos.assign(d.atomic_pos, d.atomic_pos + 3 * d.natom);
    h->atom_type.assign(d.atom_type, d.atom_type + d.natom);
    h->PP.assign(d.PP_table, d.PP_table + 3 * d.nltimesj * d.ntype);
    h->Fsign.assign(d.Fsign, d.Fsign + d.nltimesj * d.ntype);
    h->npw.assign(d.npw, d.npw + d.nkpts_iBZ);
    for (int a = 0; a < d.natom; ++a)
        if (h->atom_type[a] < 0 || h->atom_type[a] >= d.ntype) return bad(LELPH_GPU_ERR_INVALID, "atom_type");
    // projectors per type
    h->nproj_max = 0;
    for (int t = 0; t < d.ntype; ++t)
    {
        int np = 0;
        for (int l = 0; l < d.nltimesj; ++l)
        {
            int ll = (int)std::rint(h->PP[3 * (l * d.ntype + t)] - 1);
            if (ll > 3) return bad(LELPH_GPU_ERR_UNSUPPORTED, "l > 3");
            if (ll >= 0) np += 2 * ll + 1;
        }
        h->nproj_max = std::max(h->nproj_max, np);
    }
    if (h->nproj_max > 24) return bad(LELPH_GPU_ERR_UNSUPPORTED, "more than 24 projectors per atom");
    if (h->nproj_max == 0) h->nproj_max = 1;
    // Miller indices of every iBZ plane wave: n = rint(alat^T G)
    h->pw_off.resize(d.nkpts_iBZ);
    h->coef_off.resize(d.nkpts_iBZ);
    h->fk_off.resize(d.nkpts_iBZ);
    long long tot = 0, ctot = 0, ftot = 0;
    const int nsets = d.nspin * d.nbnds * d.nspinor;
    for (int ik = 0; ik < d.nkpts_iBZ; ++ik)
    {
        if (h->npw[ik] <= 0 || !d.gvec[ik] || !d.Fk[ik]) return bad(LELPH_GPU_ERR_INVALID, "npw / gvec / Fk");
        h->pw_off[ik] = tot;
        h->coef_off[ik] = ctot;
        h->fk_off[ik] = ftot;
        tot += h->npw[ik];
        ctot += (long long)nsets * h->npw[ik];
        ftot += (long long)d.nltimesj * d.ntype * h->npw[ik];
    }
    h->total_pw = tot;
    h->miller.resize(3 * tot);
    std::vector<double> gall(3 * tot), fall(ftot);
    for (int ik = 0; ik < d.nkpts_iBZ; ++ik)
    {
        for (int g = 0; g < h->npw[ik]; ++g)
        {
            double c[3];
            mat_vec3(d.alat_vec, d.gvec[ik] + 3 * g, true, c);
            for (int x = 0; x < 3; ++x)
            {
                double r = std::rint(c[x]);
                if (std::fabs(c[x] - r) > 1e-4) return bad(LELPH_GPU_ERR_GEOMETRY, "G vector not on the reciprocal lattice");
                h->miller[3 * (h->pw_off[ik] + g) + x] = (int)r;
                gall[3 * (h->pw_off[ik] + g) + x] = d.gvec[ik][3 * g + x];
            }
        }
        memcpy(fall.data() + h->fk_off[ik], d.Fk[ik], sizeof(double) * d.nltimesj * d.ntype * h->npw[ik]);
    }
    // per full-BZ k symmetry data
    double B[9];
    for (int i = 0; i < 9; ++i) B[i] = d.blat_vec[i] / (2 * PI_T);
    h->ksym.resize(d.nkpts_BZ);
    int ext[3] = {0, 0, 0};  // largest extent (max - min) of a rotated sphere on each axis
    for (int i = 0; i < d.nkpts_BZ; ++i)
    {
        KPointSym& ks = h->ksym[i];
        memset(&ks, 0, sizeof(ks));
        ks.ik = h->kmap[2 * i];
        ks.isym = h->kmap[2 * i + 1];
        if (ks.ik < 0 || ks.ik >= d.nkpts_iBZ || ks.isym < 0 || ks.isym >= d.nsym)
            return bad(LELPH_GPU_ERR_INVALID, "kmap out of range");
        const double* R = &h->symR[9 * ks.isym];
        const double* tau = &h->symtau[3 * ks.isym];
        ks.trev = h->symtr[ks.isym] != 0;
        memcpy(ks.R, R, sizeof(ks.R));
        memcpy(ks.tau_cart, tau, sizeof(ks.tau_cart));
        // W = alat^T R A^{-T},  A^{-T} = blat / (2 pi)
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
            {
                double acc = 0;
                for (int k = 0; k < 3; ++k)
                    for (int l = 0; l < 3; ++l) acc += d.alat_vec[3 * k + r] * R[3 * k + l] * B[3 * l + c];
                double w = std::rint(acc);
                if (std::fabs(acc - w) > 1e-6) return bad(LELPH_GPU_ERR_GEOMETRY, "symmetry not integral on the reciprocal lattice");
                ks.W[3 * r + c] = (int)w;
            }
        double tc[3];
        mat_vec3(d.blat_vec, tau, true, tc);
        for (int x = 0; x < 3; ++x) ks.tau_crys[x] = tc[x] / (2 * PI_T);
        double kr[3], kc[3];
        mat_vec3(R, &h->kibz[3 * ks.ik], false, kr);
        mat_vec3(d.alat_vec, kr, true, kc);
        double dot = kc[0] * ks.tau_crys[0] + kc[1] * ks.tau_crys[1] + kc[2] * ks.tau_crys[2];
        std::complex<double> kp = std::exp(std::complex<double>(0, -2 * PI_T * dot));
        ks.kphase[0] = kp.real();
        ks.kphase[1] = kp.imag();
        memcpy(ks.kcart, &h->kibz[3 * ks.ik], sizeof(ks.kcart));
        std::complex<double> u[4];
        if (!su2mat(R, d.nspinor, ks.trev, u)) return bad(LELPH_GPU_ERR_GEOMETRY, "Wrong symmetric matrices");
        for (int e = 0; e < 4; ++e)
        {
            ks.su2[2 * e] = u[e].real();
            ks.su2[2 * e + 1] = u[e].imag();
        }
        // extent of the rotated sphere on each axis
        int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
        for (int g = 0; g < h->npw[ks.ik]; ++g)
        {
            const int* n = &h->miller[3 * (h->pw_off[ks.ik] + g)];
            for (int r = 0; r < 3; ++r)
            {
                int v = ks.W[3 * r] * n[0] + ks.W[3 * r + 1] * n[1] + ks.W[3 * r + 2] * n[2];
                lo[r] = std::min(lo[r], v);
                hi[r] = std::max(hi[r], v);
            }
        }
        for (int r = 0; r < 3; ++r) ext[r] = std::max(ext[r], hi[r] - lo[r]);
        // |S(k+G)| in crystal units: S(k+G) = W n + alat^T R k
        double krot[3];
        mat_vec3(d.alat_vec, kr, true, krot);
        for (int g = 0; g < h->npw[ks.ik]; ++g)
        {
            const int* n = &h->miller[3 * (h->pw_off[ks.ik] + g)];
            for (int r = 0; r < 3; ++r)
            {
                double u = (double)(ks.W[3 * r] * n[0] + ks.W[3 * r + 1] * n[1] + ks.W[3 * r + 2] * n[2]) + krot[r];
                h->Rc[r] = std::max(h->Rc[r], std::fabs(u));
            }
        }
    }
    for (int r = 0; r < 3; ++r)
        if (ext[r] >= d.fft_dims[r]) return bad(LELPH_GPU_ERR_GEOMETRY, "FFT box too small for the plane-wave sphere");
    // Product grid.  For a pair, D = G' - G1 (k+q sphere, shift G0 included,
    // minus k sphere) satisfies D + q = S'(k'+G') - S(k+G), so every component
    // of D lies in [-q - 2Rc, -q + 2Rc]: floor(4 Rc) + 3 consecutive integers
    // cover it for any q.  On a grid of at least that many points per axis the
    // real-space sandwich with the dV window of each q (k_dv_window) gives the
    // reference's sum over G exactly.  Smallest 2^a 3^b 5^c sizes, never above
    // the reference's box (which is always exact); the mixed form also wants
    // a multiple of 32 points.
    {
        auto friendly = [](int n) {
            for (int p : {2, 3, 5})
                while (n % p == 0) n /= p;
            return n == 1;
        };
        std::vector<int> cand[3];
        for (int r = 0; r < 3; ++r)
        {
            for (int n = (int)std::floor(4.0 * h->Rc[r] + 1e-9) + 3; n < d.fft_dims[r]; ++n)
                if (friendly(n)) cand[r].push_back(n);
            cand[r].push_back(d.fft_dims[r]);
        }
        long long best = -1;
        int bm[3] = {d.fft_dims[0], d.fft_dims[1], d.fft_dims[2]};
        for (int a : cand[0])
            for (int b : cand[1])
                for (int c : cand[2])
                {
                    long long p = (long long)a * b * c;
                    if (h->mixed && !h->gspace && p % 32 != 0) continue;
                    if (best < 0 || p < best)
                    {
                        best = p;
                        bm[0] = a;
                        bm[1] = b;
                        bm[2] = c;
                    }
                }
        if (const char* e = getenv("LELPH_FULL_BOX"))
            if (atoi(e) != 0) bm[0] = d.fft_dims[0], bm[1] = d.fft_dims[1], bm[2] = d.fft_dims[2];
        h->g.Nx = bm[0];
        h->g.Ny = bm[1];
        h->g.Nz = bm[2];
        for (int r = 0; r < 3; ++r)
            if (!plan_1d(bm[r], h->plan[r])) return bad(LELPH_GPU_ERR_UNSUPPORTED, "product grid");
    }
    const long long N = (long long)h->g.Nx * h->g.Ny * h->g.Nz;
    if (d.route == LELPH_GPU_ROUTE_AUTO && !h->gspace)
    {
        // the real-space route keeps psi(r) of every full-BZ k resident (split
        // k+q rows and FP32 psi in the mixed form, FP64 boxes in the plain form)
        const double per_kpt = h->mixed ? 24.0 * h->g.nbp * d.nspin * d.nspinor
                                        : 16.0 * d.nspin * d.nbnds * d.nspinor;
        const double resident = per_kpt * (double)N * d.nkpts_BZ;
        size_t fr = 0, tot = 0;
        if (cudaSetDevice(d.device) == cudaSuccess && cudaMemGetInfo(&fr, &tot) == cudaSuccess &&
            resident > 0.5 * (double)tot)
            h->gspace = true;
        // Mixed form, both routes fit: the cheaper per pair by a cost model with
        // rates measured on GB300 (one pair and spin; rows = modes x bands x
        // spinors): real-space, the split sandwich, 12 rows (2 nbp) M tensor flops
        // at 7.6e14/s; G-space, the pruned plane and x passes at 3.6e-12 s per grid
        // point of a row plus the GEMM over the sphere, 8 rows nb npw flops at
        // 1.8e14/s (the tensor-core GEMM; 4.7e13/s with the SIMT one).
        // lelph_gpu_tune measures instead of modelling.
        if (!h->gspace && h->mixed)
        {
            double npw_avg = 0;
            for (int ik = 0; ik < d.nkpts_iBZ; ++ik) npw_avg += h->npw[ik];
            npw_avg /= d.nkpts_iBZ;
            const double rows = (double)d.nmodes * d.nbnds * d.nspinor;
            const double gemm_rate = lelph_gs_tc_supported(d.nbnds) ? 1.8e14 : 4.7e13;
            const double t_real = 12.0 * rows * (2.0 * h->g.nbp) * (double)N / 7.6e14;
            const double t_gs = rows * (double)N * 3.6e-12 + 8.0 * rows * d.nbnds * npw_avg / gemm_rate;
            if (t_gs < t_real) h->gspace = true;
        }
        // (The plain form stays on the real-space route when it fits: it is the
        // validation form, and the allocation-free entry point runs only that
        // route; which FP64 route is faster depends on the system, and
        // lelph_gpu_tune measures it.)
    }
    if (h->gspace)
    {
        GsGeom gg{h->g.Nx, h->g.Ny, h->g.Nz, d.nbnds, d.nspinor, d.nmag, 0};
        if (lelph_gs_plane_smem(gg, !h->mixed) > 220 * 1024 || lelph_gs_xpass_smem(gg, !h->mixed) > 220 * 1024)
            return bad(LELPH_GPU_ERR_UNSUPPORTED, "G-space route: a (y, z) plane of the product grid exceeds shared memory");
    }
    if (h->mixed && !h->gspace)
    {
        if (N % 32 != 0) return bad(LELPH_GPU_ERR_UNSUPPORTED, "grid size must be a multiple of 32");
        if (N % h->g.kpts != 0) h->g.kpts = 32;
        // the descriptor's stage size (a tuned choice), or LELPH_TC_STAGE = 32 (tests)
        if (d.tile_points == 32) h->g.kpts = 32;
        else if (d.tile_points == 64 && h->g.kpts != 64)
            return bad(LELPH_GPU_ERR_UNSUPPORTED, "64-point stages do not fit this tile");
        else if (d.tile_points != 0 && d.tile_points != 64)
            return bad(LELPH_GPU_ERR_INVALID, "tile_points must be 0, 32 or 64");
        if (const char* e = getenv("LELPH_TC_STAGE"))
            if (atoi(e) == 32) h->g.kpts = 32;
        if (lelph_local_tc_smem_bytes(h->g) > 227 * 1024) return bad(LELPH_GPU_ERR_UNSUPPORTED, "shared memory");
    }
    // chat offsets per full-BZ k
    h->chat_off.resize(d.nkpts_BZ);
    long long chtot = 0;
    for (int i = 0; i < d.nkpts_BZ; ++i)
    {
        h->chat_off[i] = chtot;
        chtot += (long long)nsets * h->npw[h->ksym[i].ik];
    }

    // ---- device
    if (cudaSetDevice(h->device) != cudaSuccess) return bad(LELPH_GPU_ERR_CUDA, "cudaSetDevice");
    if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->st_copy, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->evc[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->evc[1], cudaEventDisableTiming) != cudaSuccess)
        return bad(LELPH_GPU_ERR_CUDA, "stream");
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    cudaEventCreate(&h->evg0);
    cudaEventCreate(&h->evg1);
    DevBuf* bufs[] = {&h->d_miller, &h->d_pwoff, &h->d_npw, &h->d_coef, &h->d_coefoff, &h->d_gvec, &h->d_fk,
                      &h->d_fkoff, &h->d_ksym, &h->d_chat, &h->d_chatoff, &h->d_psi64, &h->d_boxes32, &h->d_bsplit,
                      &h->d_psi32, &h->d_band_scale, &h->d_proj, &h->d_atype, &h->d_apos, &h->d_pp, &h->d_fsign, &h->d_fcoef,
                      &h->d_fcoefoff, &h->d_tw64[0], &h->d_tw64[1], &h->d_tw64[2], &h->d_tw32[0], &h->d_tw32[1],
                      &h->d_tw32[2], &h->d_twN[0], &h->d_twN[1], &h->d_twN[2], &h->d_twN32[0], &h->d_twN32[1],
                      &h->d_twN32[2], &h->d_dvr, &h->d_eig,
                      &h->d_maxabs, &h->d_win64, &h->d_win32, &h->d_winscale, &h->d_wtmpN, &h->d_wtmpM,
                      &h->d_pairs, &h->d_glocal, &h->d_partials, &h->d_gout, &h->d_status, &h->d_tmp,
                      &h->d_vl_v, &h->d_vl_dv, &h->d_vl_in, &h->d_vloc, &h->d_colmask, &h->d_collist, &h->d_colcnt,
                      &h->d_dmgtab,
                      &h->d_dmjobs, &h->d_dmats, &h->d_dmmap, &h->d_dmcoef32, &h->d_dmstar, &h->d_gstar,
                      &h->d_dmgroups, &h->d_dmperm, &h->d_dmcoefT,
                      &h->d_qsitems, &h->d_dvraw, &h->d_gs_perm, &h->d_gs_kcx, &h->d_gs_cols, &h->d_gs_cst,
                      &h->d_gs_npw, &h->d_gs_npad, &h->d_gs_permoff, &h->d_gs_bpoff, &h->d_gs_bp, &h->d_gs_psi,
                      &h->d_gs_out1, &h->d_gs_A, &h->d_gs_part, &h->d_gs_zl, &h->d_gs_cols2, &h->d_gs_bq};
    for (DevBuf* b : bufs) h->owned.push_back(b);
    int rc = 0;
#define UP(buf, ptr, bytes)                              \
    do                                                   \
    {                                                    \
        rc = upload(h, buf, ptr, bytes);                 \
        if (rc) return bad(rc, h->err);                  \
    } while (0)
    UP(h->d_miller, h->miller.data(), sizeof(int) * h->miller.size());
    UP(h->d_pwoff, h->pw_off.data(), sizeof(long long) * h->pw_off.size());
    UP(h->d_npw, h->npw.data(), sizeof(int) * h->npw.size());
    UP(h->d_coefoff, h->coef_off.data(), sizeof(long long) * h->coef_off.size());
    UP(h->d_gvec, gall.data(), sizeof(double) * gall.size());
    UP(h->d_fk, fall.data(), sizeof(double) * fall.size());
    UP(h->d_fkoff, h->fk_off.data(), sizeof(long long) * h->fk_off.size());
    UP(h->d_ksym, h->ksym.data(), sizeof(KPointSym) * h->ksym.size());
    UP(h->d_chatoff, h->chat_off.data(), sizeof(long long) * h->chat_off.size());
    UP(h->d_atype, h->atom_type.data(), sizeof(int) * h->atom_type.size());
    UP(h->d_apos, h->atom_pos.data(), sizeof(double) * h->atom_pos.size());
    UP(h->d_pp, h->PP.data(), sizeof(double) * h->PP.size());
    UP(h->d_fsign, h->Fsign.data(), sizeof(double) * h->Fsign.size());
    // fCoeff packing: offsets in complex units, -1 where absent
    {
        std::vector<int> off(std::max(1, d.nltimesj * d.ntype), -1);
        std::vector<double> pack;
        if (d.fCoeff)
        {
            for (int i = 0; i < d.nltimesj * d.ntype; ++i)
            {
                if (!d.fCoeff[i]) continue;
                int lidx = i / d.ntype, t = i % d.ntype;
                int l = (int)std::rint(h->PP[3 * (lidx * d.ntype + t)] - 1);
                if (l < 0) continue;
                size_t n = (size_t)(2 * l + 1) * (2 * l + 1) * d.nspinor * d.nspinor;
                off[i] = (int)(pack.size() / 2);
                pack.insert(pack.end(), d.fCoeff[i], d.fCoeff[i] + 2 * n);
            }
        }
        if (pack.empty()) pack.assign(2, 0.0);
        UP(h->d_fcoef, pack.data(), sizeof(double) * pack.size());
        if (pack.size() == 2) h->d_fcoef.n = 16;  // marks "no coefficients"
        UP(h->d_fcoefoff, off.data(), sizeof(int) * off.size());
    }
    // twiddles e^{+2 pi i t / L}: product grid and reference box, FP64 and FP32
    for (int x = 0; x < 6; ++x)
    {
        int L = x < 3 ? (x == 0 ? h->g.Nx : (x == 1 ? h->g.Ny : h->g.Nz)) : d.fft_dims[x - 3];
        std::vector<double2> t64(L);
        std::vector<float2> t32(L);
        for (int t = 0; t < L; ++t)
        {
            long double ang = 6.283185307179586476925286766559005768L * (long double)t / (long double)L;
            t64[t] = make_double2((double)cosl(ang), (double)sinl(ang));
            t32[t] = make_float2((float)cosl(ang), (float)sinl(ang));
        }
        if (x < 3)
        {
            UP(h->d_tw64[x], t64.data(), sizeof(double2) * L);
            UP(h->d_tw32[x], t32.data(), sizeof(float2) * L);
        }
        else
        {
            UP(h->d_twN[x - 3], t64.data(), sizeof(double2) * L);
            UP(h->d_twN32[x - 3], t32.data(), sizeof(float2) * L);
        }
    }
    rc = ensure(h, h->d_coef, sizeof(double2) * (size_t)ctot);
    if (rc) return bad(rc, h->err);
    h->coef_total = ctot;
    rc = ensure(h, h->d_chat, sizeof(double2) * (size_t)chtot);
    if (rc) return bad(rc, h->err);
    rc = ensure(h, h->d_proj, sizeof(double2) * (size_t)d.nkpts_BZ * d.natom * h->nproj_max * 4 * nsets);
    if (rc) return bad(rc, h->err);
    rc = ensure(h, h->d_status, 64);
    if (rc) return bad(rc, h->err);
    if (cudaMemsetAsync(h->d_status.p, 0, 64, h->st) != cudaSuccess) return bad(LELPH_GPU_ERR_CUDA, "memset");
    if (h->gspace)
    {
        rc = gs_tables(h);
        if (rc) return bad(rc, h->err);
    }
    if (h->mixed && !h->gspace)
    {
        const size_t Kr = 2 * (size_t)d.nspinor * N;
        const size_t rows = (size_t)d.nkpts_BZ * d.nspin * 2 * 2 * h->g.nbp;
        rc = ensure(h, h->d_bsplit, sizeof(uint16_t) * Kr * rows);
        if (rc) return bad(rc, h->err);
        if (cudaMemsetAsync(h->d_bsplit.p, 0, h->d_bsplit.n, h->st) != cudaSuccess) return bad(LELPH_GPU_ERR_CUDA, "memset");
        // split rows, tile-major: blocks (k, spin, hi|lo, 32-point K block) of 2*nbp rows x 64 halves
        rc = make_tmap3(h, &h->tmapB, h->d_bsplit.p, false, 64, 2 * h->g.nbp, rows / (2 * h->g.nbp) * (Kr / 64),
                        2 * h->g.nbp, 1, true);
        if (rc) return bad(rc, h->err);
        // FP32 psi(r) of the k role, tile-major: blocks (k, spin, 16-point block) of nbp rows x 32 floats,
        // four blocks (one 64-point stage) per box, 128-byte swizzled
        const size_t prow = (size_t)d.nkpts_BZ * d.nspin * h->g.nbp;
        rc = ensure(h, h->d_psi32, sizeof(float) * Kr * prow);
        if (rc) return bad(rc, h->err);
        if (cudaMemsetAsync(h->d_psi32.p, 0, h->d_psi32.n, h->st) != cudaSuccess) return bad(LELPH_GPU_ERR_CUDA, "memset");
        rc = make_tmap3(h, &h->tmapP, h->d_psi32.p, true, 32, h->g.nbp, (size_t)d.nkpts_BZ * d.nspin * (Kr / 32),
                        h->g.nbp, (unsigned)(h->g.kpts / 16), true);
        if (rc) return bad(rc, h->err);
        // K chunk per work unit: a multiple of the stage dividing N (so a chunk stays
        // within one spinor component), as large as possible up to 8192 points: each
        // chunk's FP32 sum is one FP64 term of the finish kernel
        const int kp = h->g.kpts;
        long long Ktot = (long long)d.nspinor * N;
        long long units = N / kp;
        long long best = 1;
        for (long long c = 1; c <= units; ++c)
            if (units % c == 0 && c * kp <= 8192) best = c;
        h->chunk_pts = (int)(best * kp);
        // tuning override: LELPH_TC_CHUNK = grid points per K chunk (multiple of the stage dividing N)
        if (const char* e = getenv("LELPH_TC_CHUNK"))
        {
            long long c = atoll(e);
            if (c > 0 && c % kp == 0 && N % c == 0) h->chunk_pts = (int)c;
        }
        h->nchunks = (int)(Ktot / h->chunk_pts);
    }
    rc = upload_wfc(h, d.wfc);
    if (rc) return bad(rc, h->err);
    if (cudaStreamSynchronize(h->st) != cudaSuccess) return bad(LELPH_GPU_ERR_CUDA, "sync");
    h->stats.route = h->gspace ? LELPH_GPU_ROUTE_GSPACE : LELPH_GPU_ROUTE_REAL;
    *out = h;
    return LELPH_GPU_OK;
#undef UP
}

extern "C" int lelph_gpu_set_wavefunctions(lelph_gpu* h, const double* const* wfc)
{
    if (!h || !wfc) return LELPH_GPU_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    return upload_wfc(h, wfc);
}

static int build_windows(lelph_gpu* h);

extern "C" int lelph_gpu_prepare(lelph_gpu* h)
{
    if (!h) return LELPH_GPU_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    const lelph_gpu_desc& d = h->d;
    const GeomDev& g = h->g;
    const long long N = (long long)g.Nx * g.Ny * g.Nz;
    const int nbox_per_k = d.nspin * d.nbnds * d.nspinor;
    const int npw_max = *std::max_element(h->npw.begin(), h->npw.end());
    tstart(h);
    int rc;
    // KB projections on the tensor cores (mixed form); on the real-space route they
    // read an FP32 copy of the unfolded coefficients, which nothing else uses there
    const bool proj_tc = h->proj_tc && lelph_projections_tc_supported(nl_desc(h));
    const bool chat_f32 = proj_tc && !h->gspace;
    if (h->gspace)
    {
        // G-space route: the unfolded coefficients of every full-BZ k (no
        // boxes: psi(r) is made per k when its pairs run) and their copy in
        // each sphere's sorted order, the GEMM operand of the k+q role
        lelph_launch_scatter(0, d.nkpts_BZ, (const KPointSym*)h->d_ksym.p, (const int*)h->d_miller.p,
                             (const long long*)h->d_pwoff.p, (const int*)h->d_npw.p, npw_max,
                             (const double2*)h->d_coef.p, (const long long*)h->d_coefoff.p, g, !h->mixed, nullptr,
                             (double2*)h->d_chat.p, (const long long*)h->d_chatoff.p, h->st);
        const size_t e = h->mixed ? sizeof(float2) : sizeof(double2);
        rc = ensure(h, h->d_gs_bp, e * (size_t)h->gs_bp_total);
        if (rc) return rc;
        if (lelph_launch_gs_bperm(!h->mixed, (const double2*)h->d_chat.p, (const long long*)h->d_chatoff.p,
                                  (const int*)h->d_gs_npw.p, (const int*)h->d_gs_npad.p,
                                  (const long long*)h->d_gs_permoff.p, (const int*)h->d_gs_perm.p,
                                  (const long long*)h->d_gs_bpoff.p, 0, d.nkpts_BZ, nbox_per_k, h->gs_npad_max,
                                  h->d_gs_bp.p, h->st))
            return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "G-space route: coefficient permutation grid");
        h->stats.kernel_launches += 2;
    }
    else if (!h->mixed)
    {
        size_t bytes = sizeof(double2) * (size_t)d.nkpts_BZ * nbox_per_k * N;
        rc = ensure(h, h->d_psi64, bytes);
        if (rc) return rc;
        CUDA_TRY(h, cudaMemsetAsync(h->d_psi64.p, 0, bytes, h->st));
        lelph_launch_scatter(0, d.nkpts_BZ, (const KPointSym*)h->d_ksym.p, (const int*)h->d_miller.p,
                             (const long long*)h->d_pwoff.p, (const int*)h->d_npw.p, npw_max,
                             (const double2*)h->d_coef.p, (const long long*)h->d_coefoff.p, g, 1, h->d_psi64.p, (double2*)h->d_chat.p,
                             (const long long*)h->d_chatoff.p, h->st);
        const long long nbox = (long long)d.nkpts_BZ * nbox_per_k;
        double2* psi = (double2*)h->d_psi64.p;
        lelph_launch_fft_contig_d(psi, nbox * g.Nx * g.Ny, h->plan[2], (const double2*)h->d_tw64[2].p, +1, h->st);
        lelph_launch_fft_strided_d(psi, nbox * g.Nx, g.Nz, h->plan[1], (const double2*)h->d_tw64[1].p, +1, h->st);
        lelph_launch_fft_strided_d(psi, nbox, g.Ny * g.Nz, h->plan[0], (const double2*)h->d_tw64[0].p, +1, h->st);
        h->stats.kernel_launches += 4;
    }
    else
    {
        // FP32 boxes in chunks of k-points (<= ~4 GB of boxes)
        const size_t per_k = sizeof(float2) * (size_t)nbox_per_k * N;
        int nkc = (int)std::max<size_t>(1, std::min<size_t>((size_t)d.nkpts_BZ, (4ull << 30) / per_k));
        // testing override: LELPH_PREP_CHUNK_K = at most this many k-points per chunk of boxes
        if (const char* e = getenv("LELPH_PREP_CHUNK_K"))
            if (atoi(e) > 0) nkc = std::min(nkc, atoi(e));
        rc = ensure(h, h->d_boxes32, per_k * nkc);
        if (rc) return rc;
        // occupancy of every k (geometry only), built by the first preparation's
        // scatters; afterwards a chunk's boxes need zeros only in their k's
        // occupied columns (see BoxMask), not a clear of the whole box
        const size_t ncol = (size_t)g.Nx * g.Ny;
        rc = ensure(h, h->d_colmask, (ncol + g.Nx) * d.nkpts_BZ);
        if (rc) return rc;
        rc = ensure(h, h->d_collist, sizeof(int) * ncol * d.nkpts_BZ);
        if (rc) return rc;
        rc = ensure(h, h->d_colcnt, sizeof(int) * d.nkpts_BZ);
        if (rc) return rc;
        uint8_t* col_all = (uint8_t*)h->d_colmask.p;
        uint8_t* xpl_all = col_all + ncol * d.nkpts_BZ;
        const bool masks = h->boxmask_ready;
        if (!masks) CUDA_TRY(h, cudaMemsetAsync(h->d_colmask.p, 0, (ncol + g.Nx) * d.nkpts_BZ, h->st));
        for (int k0 = 0; k0 < d.nkpts_BZ; k0 += nkc)
        {
            int nk = std::min(nkc, d.nkpts_BZ - k0);
            BoxMask mk;
            mk.col = col_all + (size_t)k0 * ncol;
            mk.xpl = xpl_all + (size_t)k0 * g.Nx;
            mk.Nx = g.Nx;
            mk.Ny = g.Ny;
            mk.nbox_per_k = nbox_per_k;
            gs_tick(h);
            if (masks)
                lelph_launch_clear_cols((float2*)h->d_boxes32.p, nk, nbox_per_k, N, g.Nz, (int)ncol,
                                        (const int*)h->d_collist.p + (size_t)k0 * ncol,
                                        (const int*)h->d_colcnt.p + k0, h->st);
            else
                CUDA_TRY(h, cudaMemsetAsync(h->d_boxes32.p, 0, per_k * nk, h->st));
            lelph_launch_scatter(k0, nk, (const KPointSym*)h->d_ksym.p, (const int*)h->d_miller.p,
                                 (const long long*)h->d_pwoff.p, (const int*)h->d_npw.p, npw_max,
                                 (const double2*)h->d_coef.p, (const long long*)h->d_coefoff.p, g, 0, h->d_boxes32.p,
                                 (double2*)h->d_chat.p, (const long long*)h->d_chatoff.p, h->st, mk,
                                 proj_tc ? (float2*)h->d_chat.p : nullptr);
            h->stats.prep_scatter_ms += gs_tock(h);
            const long long nbox = (long long)nk * nbox_per_k;
            float2* bx = (float2*)h->d_boxes32.p;
            // z pass on the occupied columns, y pass on the occupied x planes, x pass
            // reading only those planes (the rest of every box is zero)
            lelph_launch_fft_contig_f(bx, nbox * g.Nx * g.Ny, h->plan[2], (const float2*)h->d_tw32[2].p, +1, h->st,
                                      mk);
            lelph_launch_fft_strided_f(bx, nbox * g.Nx, g.Nz, h->plan[1], (const float2*)h->d_tw32[1].p, +1, h->st,
                                       mk);
            h->stats.prep_fft_ms += gs_tock(h);
            lelph_launch_fft_x_to_split(bx, nk, k0, h->plan[0], (const float2*)h->d_tw32[0].p, +1, g,
                                        (const float*)h->d_band_scale.p, h->ab_bf16, (uint16_t*)h->d_bsplit.p,
                                        (float2*)h->d_psi32.p, h->st, mk);
            h->stats.prep_xsplit_ms += gs_tock(h);
            h->stats.kernel_launches += masks ? 5 : 4;
        }
        if (!masks)
        {
            lelph_launch_col_lists(col_all, d.nkpts_BZ, (int)ncol, (int*)h->d_collist.p, (int*)h->d_colcnt.p, h->st);
            CUDA_TRY(h, cudaGetLastError());
            std::vector<int> cnt(d.nkpts_BZ);
            CUDA_TRY(h, cudaMemcpyAsync(cnt.data(), h->d_colcnt.p, sizeof(int) * cnt.size(), cudaMemcpyDeviceToHost,
                                        h->st));
            CUDA_TRY(h, cudaStreamSynchronize(h->st));
            h->stats.box_columns = 0;
            for (int c : cnt) h->stats.box_columns += c;
            h->boxmask_ready = true;
            h->stats.kernel_launches += 1;
        }
    }
    NonlocalDesc nl = nl_desc(h);
    gs_tick(h);
    if (proj_tc)
    {
        CUDA_TRY(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned), h->st));
        if (lelph_launch_projections_tc(0, d.nkpts_BZ, (const KPointSym*)h->d_ksym.p, (const double*)h->d_gvec.p,
                                        (const long long*)h->d_pwoff.p, (const int*)h->d_npw.p,
                                        (const double*)h->d_fk.p, (const long long*)h->d_fkoff.p, h->d_chat.p,
                                        chat_f32 ? 1 : 0, (const long long*)h->d_chatoff.p, nl, g,
                                        (double2*)h->d_proj.p, (unsigned*)h->d_status.p, h->wait_ns, h->st))
            return fail(h, LELPH_GPU_ERR_CUDA, "projection launch failed");
        // its status is read with the preparation's final synchronisation, so
        // that the dV windows' launches queue behind it without a host round trip
    }
    else
        lelph_launch_projections(0, d.nkpts_BZ, (const KPointSym*)h->d_ksym.p, (const double*)h->d_gvec.p,
                                 (const long long*)h->d_pwoff.p, (const int*)h->d_npw.p, (const double*)h->d_fk.p,
                                 (const long long*)h->d_fkoff.p, (const double2*)h->d_chat.p,
                                 (const long long*)h->d_chatoff.p, nl, g, h->mixed ? 1 : 0, (double2*)h->d_proj.p,
                                 h->st);
    h->stats.prep_proj_ms += gs_tock(h);
    h->stats.kernel_launches += 1;
    CUDA_TRY(h, cudaGetLastError());
    int wr = build_windows(h);
    if (wr) return wr;
    h->stats.windows_ms += gs_tock(h);
    h->stats.prepare_ms += tstop(h);
    if (proj_tc)
    {
        const int rs = check_status(h);  // synchronises the stream
        if (rs) return rs;
    }
    else
        CUDA_TRY(h, cudaStreamSynchronize(h->st));
    h->prepared = true;
    return LELPH_GPU_OK;
}

// dV on the product grid for one (q slot, umklapp G0): with dVhat the
// normalised forward transform of dV on the reference box,
//   dV_G0(r') = sum_d dVhat(d + G0) e^{i d.r'},  d over one period of the product grid
// (signed representatives), so that (1/M) sum_r' dV_G0 psi_k conj(psi_kq) equals
// the reference's sum_{G1,G'} c_k(G1) conj(c_kq(G')) dVhat(G' - G1) exactly.
template <typename T2>
__global__ void k_dv_window(const T2* __restrict__ dvhat, int ncomp, int Nx, int Ny, int Nz,
                            const int* __restrict__ ulms, int nu, int3 dmin, GeomDev g, double invN,
                            T2* __restrict__ out)
{
    const long long M = (long long)g.Nx * g.Ny * g.Nz;
    const int c = blockIdx.y;   // (mode, component)
    const int u = blockIdx.z;   // umklapp index
    const int ux = ulms[3 * u], uy = ulms[3 * u + 1], uz = ulms[3 * u + 2];
    const T2* src = dvhat + (size_t)c * ((size_t)Nx * Ny * Nz);
    T2* dst = out + ((size_t)u * ncomp + c) * M;
    // grid residue x stands for the difference D' = G'' - G1 in [dmin - G0, dmin - G0 + M); value dVhat(D' + G0)
    const int lx = dmin.x - ux, ly = dmin.y - uy, lz = dmin.z - uz;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < M; r += (long long)gridDim.x * blockDim.x)
    {
        int x = (int)(r / ((long long)g.Ny * g.Nz));
        int rem = (int)(r - (long long)x * g.Ny * g.Nz);
        int y = rem / g.Nz, z = rem - (rem / g.Nz) * g.Nz;
        int dx = lx + (((x - lx) % g.Nx) + g.Nx) % g.Nx;
        int dy = ly + (((y - ly) % g.Ny) + g.Ny) % g.Ny;
        int dz = lz + (((z - lz) % g.Nz) + g.Nz) % g.Nz;
        int ix = ((dx + ux) % Nx + Nx) % Nx;
        int iy = ((dy + uy) % Ny + Ny) % Ny;
        int iz = ((dz + uz) % Nz + Nz) % Nz;
        const T2 v = src[((size_t)ix * Ny + iy) * Nz + iz];
        const decltype(v.x) s = (decltype(v.x))invN;  // the operand type's 1/N
        dst[r] = mk2<T2>(v.x * s, v.y * s);
    }
}

// Load q slot `slot`: eigVec and dV (host); dVscf == nullptr loads zeros.
static int set_q_common(lelph_gpu* h, int slot, const double qpt_crys[3], const double* eigVec,
                        const double* dVscf)
{
    if (!h || slot < 0 || !qpt_crys || !eigVec) return LELPH_GPU_ERR_INVALID;
    if (slot > 4096) return fail(h, LELPH_GPU_ERR_INVALID, "slot index too large");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const lelph_gpu_desc& d = h->d;
    const long long NN = (long long)h->Nbox[0] * h->Nbox[1] * h->Nbox[2];
    const size_t dvn = (size_t)d.nmodes * d.nmag * NN;
    if (slot >= h->nslots_alloc)
    {
        // grow the slot arrays, keeping the loaded slots
        int ns = std::max(slot + 1, 2 * h->nslots_alloc);
        DevBuf ndv, neig;
        int rc = ensure(h, ndv, sizeof(double2) * dvn * ns);
        if (rc) return rc;
        rc = ensure(h, neig, sizeof(double2) * d.nmodes * d.nmodes * ns);
        if (rc) return rc;
        if (h->d_dvr.p)
            CUDA_TRY(h, cudaMemcpyAsync(ndv.p, h->d_dvr.p, sizeof(double2) * dvn * h->nslots_alloc,
                                        cudaMemcpyDeviceToDevice, h->st));
        if (h->d_eig.p)
            CUDA_TRY(h, cudaMemcpyAsync(neig.p, h->d_eig.p, sizeof(double2) * d.nmodes * d.nmodes * h->nslots_alloc,
                                        cudaMemcpyDeviceToDevice, h->st));
        CUDA_TRY(h, cudaStreamSynchronize(h->st));
        for (DevBuf* b : {&h->d_dvr, &h->d_eig})
            if (b->p) cudaFree(b->p);
        h->d_dvr = ndv;
        h->d_eig = neig;
        h->nslots_alloc = ns;
        h->qslots.resize(ns);
    }
    QSlot& q = h->qslots[slot];
    memcpy(q.q, qpt_crys, sizeof(q.q));
    for (int x = 0; x < 3; ++x) q.dmin[x] = (int)std::floor(-qpt_crys[x] - 2.0 * h->Rc[x] - 1e-9);
    // every umklapp vector a k+q (or, yambo convention, k-q) pair of this q can need
    q.ulms.clear();
    for (int conv = 0; conv < 2; ++conv)
        for (int k = 0; k < d.nkpts_BZ; ++k)
        {
            double kq[3];
            for (int x = 0; x < 3; ++x) kq[x] = h->kbz_crys[3 * k + x] + (conv ? -qpt_crys[x] : qpt_crys[x]);
            int o = find_k_fast(h, kq);
            if (o < 0) continue;  // the run reports non-commensurate grids
            int ik = conv ? o : k, ikq = conv ? k : o;
            int u[3];
            if (umklapp(h, ik, ikq, qpt_crys, u)) continue;
            bool seen = false;
            for (size_t e = 0; e < q.ulms.size(); e += 3)
                if (q.ulms[e] == u[0] && q.ulms[e + 1] == u[1] && q.ulms[e + 2] == u[2]) seen = true;
            if (!seen) q.ulms.insert(q.ulms.end(), u, u + 3);
        }
    CUDA_TRY(h, cudaMemcpyAsync((double2*)h->d_eig.p + (size_t)slot * d.nmodes * d.nmodes, eigVec,
                                sizeof(double2) * d.nmodes * d.nmodes, cudaMemcpyHostToDevice, h->st));
    if (dVscf)
        CUDA_TRY(h, cudaMemcpyAsync((double2*)h->d_dvr.p + (size_t)slot * dvn, dVscf, sizeof(double2) * dvn,
                                    cudaMemcpyHostToDevice, h->st));
    else
        CUDA_TRY(h, cudaMemsetAsync((double2*)h->d_dvr.p + (size_t)slot * dvn, 0, sizeof(double2) * dvn, h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    q.set = true;
    h->windows_ok = false;
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_set_q(lelph_gpu* h, int slot, const double qpt_crys[3], const double* eigVec,
                               const double* dVscf)
{
    if (!h || !dVscf) return LELPH_GPU_ERR_INVALID;
    return set_q_common(h, slot, qpt_crys, eigVec, dVscf);
}

// ------------------------------------------------------------ dV rotation

extern "C" int lelph_gpu_rotate_dvscf(lelph_gpu* h, const double qpt_crys[3], const double Rmat[9],
                                      const double tau[3], int time_rev, int composite_form, const double* dvscf_in,
                                      double* dvscf_out)
{
    if (!h || !qpt_crys || !Rmat || !tau || !dvscf_in || !dvscf_out) return LELPH_GPU_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    const lelph_gpu_desc& d = h->d;
    RotDvDesc rd;
    rd.Nx = h->Nbox[0];
    rd.Ny = h->Nbox[1];
    rd.Nz = h->Nbox[2];
    rd.nmodes = d.nmodes;
    rd.nmag = d.nmag;
    rd.trev = time_rev != 0;
    rd.composite = composite_form != 0;
    // box coordinates of S^-1 (r - tau): tau_red = blat^T tau / 2pi and
    // sym_red = blat^T (R^T alat) / 2pi, both negated for time reversal
    // (src/symmetries/rotate_dvscf.c:118-143)
    const double* A = h->alat.data();
    const double* B = h->blat.data();
    mat_vec3(B, tau, true, rd.tau_red);
    double tmp[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
        {
            double v = 0;
            for (int k = 0; k < 3; ++k) v += Rmat[3 * k + i] * A[3 * k + j];
            tmp[3 * i + j] = v / (2 * PI_T);
        }
    for (int i = 0; i < 3; ++i)
    {
        rd.tau_red[i] /= (2 * PI_T);
        if (rd.trev) rd.tau_red[i] = -rd.tau_red[i];
    }
    if (rd.trev)
        for (double& v : tmp) v = -v;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
        {
            double v = 0;
            for (int k = 0; k < 3; ++k) v += B[3 * k + i] * tmp[3 * k + j];
            rd.sym_red[3 * i + j] = v;
        }
    double qc[3], Rq[3];
    mat_vec3(B, qpt_crys, false, qc);
    mat_vec3(Rmat, qc, false, Rq);
    const double ang = Rq[0] * tau[0] + Rq[1] * tau[1] + Rq[2] * tau[2];
    rd.ph = make_double2(std::cos(ang), -std::sin(ang));
    std::complex<double> u[4];
    if (!su2mat(Rmat, d.nspinor, rd.trev, u)) return fail(h, LELPH_GPU_ERR_GEOMETRY, "improper symmetry matrix");
    for (int i = 0; i < 4; ++i) rd.su2[i] = make_double2(u[i].real(), u[i].imag());
    const long long NN = (long long)rd.Nx * rd.Ny * rd.Nz;
    const size_t n = (size_t)d.nmodes * d.nmag * NN;
    int rc = ensure(h, h->d_wtmpN, std::max(h->d_wtmpN.n, sizeof(double2) * 2 * n));
    if (rc) return rc;
    double2* din = (double2*)h->d_wtmpN.p;
    double2* dout = din + n;
    CUDA_TRY(h, cudaMemcpyAsync(din, dvscf_in, sizeof(double2) * n, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned), h->st));
    lelph_launch_rotate_dvscf(rd, din, dout, (unsigned*)h->d_status.p, h->st);
    h->stats.kernel_launches += 1;
    CUDA_TRY(h, cudaGetLastError());
    unsigned st = 0;
    CUDA_TRY(h, cudaMemcpyAsync(&st, h->d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(dvscf_out, dout, sizeof(double2) * n, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    if (st) return fail(h, LELPH_GPU_ERR_GEOMETRY, "symmetry operation is incompatible with the FFT grid");
    return LELPH_GPU_OK;
}

// ------------------------------------------------------ local bare potential

// Slopes of the not-a-knot cubic spline through (i*dg, y_i): the usual
// tridiagonal system for the slopes with third-derivative continuity at the
// second and next-to-last knots, the two extra entries removed by one row
// operation each, solved by the Thomas algorithm.
static std::vector<double> spline_slopes(const std::vector<double>& y, double dg)
{
    const int n = (int)y.size();
    std::vector<double> lo(n), di(n), up(n), rh(n), d(n);
    auto sl = [&](int i) { return (y[i + 1] - y[i]) / dg; };
    for (int i = 1; i < n - 1; ++i)
    {
        lo[i] = dg;
        di[i] = 4.0 * dg;
        up[i] = dg;
        rh[i] = 3.0 * (sl(i - 1) * dg + sl(i) * dg);
    }
    // first row (not-a-knot at x_1): dx^2 d0 + 0 d1 - dx^2 d2 = 2 (s0 - s1) dx^2, its
    // d2 entry removed against row 1
    {
        const double h2 = dg * dg;
        double a0 = h2, b0 = 0.0, c0 = -h2, r0 = 2.0 * (sl(0) - sl(1)) * h2;
        const double al = -c0 / up[1];
        a0 += al * lo[1];
        b0 += al * di[1];
        r0 += al * rh[1];
        di[0] = a0;
        up[0] = b0;
        rh[0] = r0;
    }
    {
        // last row: dx^2 d_{n-3} + 0 d_{n-2} - dx^2 d_{n-1} = 2 (s_{n-3} - s_{n-2}) dx^2,
        // its d_{n-3} entry removed against row n-2
        const double h2 = dg * dg;
        const double cm3 = h2, cm2 = 0.0, cm1 = -h2;
        const double al = -cm3 / lo[n - 2];
        lo[n - 1] = cm2 + al * di[n - 2];
        di[n - 1] = cm1 + al * up[n - 2];
        rh[n - 1] = 2.0 * (sl(n - 3) - sl(n - 2)) * h2 + al * rh[n - 2];
    }
    for (int i = 1; i < n; ++i)
    {
        const double w = lo[i] / di[i - 1];
        di[i] -= w * up[i - 1];
        rh[i] -= w * rh[i - 1];
    }
    d[n - 1] = rh[n - 1] / di[n - 1];
    for (int i = n - 2; i >= 0; --i) d[i] = (rh[i] - up[i] * d[i + 1]) / di[i];
    return d;
}

extern "C" int lelph_gpu_set_local_pseudo(lelph_gpu* h, const int* ngrid, const double* const* r_grid,
                                          const double* const* rab_grid, const double* const* vloc_atomic,
                                          const double* zval, int dimension, double qmax_abs)
{
    if (!h || !ngrid || !r_grid || !rab_grid || !vloc_atomic || !zval) return LELPH_GPU_ERR_INVALID;
    if (dimension != '3' && dimension != '2') return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "dimension must be '3' or '2'");
    if (h->ntype > LELPH_VLOC_MAXTYPE) return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "too many species");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const double* A = h->alat.data();
    const double* B = h->blat.data();
    const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                       A[2] * (A[3] * A[7] - A[4] * A[6]);
    h->vl_volume = std::fabs(det);
    // |G| range of the table: |q + G| <= b_max (1.7 (N_max + 4) + 3 |q|_max), spacing
    // b_min capped at 0.01 (src/dvloc/vlocg_table.c:29-95)
    double bmin = 1e300, bmax = 0;
    int nmax = 0;
    for (int i = 0; i < 3; ++i)
    {
        const double b = std::sqrt(B[i] * B[i] + B[3 + i] * B[3 + i] + B[6 + i] * B[6 + i]);
        bmin = std::min(bmin, b);
        bmax = std::max(bmax, b);
        nmax = std::max(nmax, h->Nbox[i]);
    }
    if (bmin > 0.01) bmin = 0.01;
    const double gmax = (1.7 * (nmax + 4.0) + 3 * std::fabs(qmax_abs)) * bmax;
    const int npts = (int)std::ceil(gmax / bmin);
    if (npts < 3) return fail(h, LELPH_GPU_ERR_INVALID, "V_loc table too short");
    h->vl_npts = npts;
    h->vl_dg = gmax / (npts - 1.0);
    h->vl_dim2 = dimension == '2';
    h->vl_zval.assign(zval, zval + h->ntype);
    int rc = ensure(h, h->d_vl_v, sizeof(double) * (size_t)h->ntype * npts);
    if (rc) return rc;
    rc = ensure(h, h->d_vl_dv, sizeof(double) * (size_t)h->ntype * npts);
    if (rc) return rc;
    int ngmax = 0;
    for (int t = 0; t < h->ntype; ++t)
    {
        if (ngrid[t] < 3 || !r_grid[t] || !rab_grid[t] || !vloc_atomic[t])
            return fail(h, LELPH_GPU_ERR_INVALID, "radial mesh of a species");
        ngmax = std::max(ngmax, ngrid[t]);
    }
    rc = ensure(h, h->d_vl_in, sizeof(double) * 3 * (size_t)ngmax);
    if (rc) return rc;
    std::vector<double> in(3 * (size_t)ngmax), table((size_t)h->ntype * npts), slopes((size_t)h->ntype * npts);
    for (int t = 0; t < h->ntype; ++t)
    {
        const int n = ngrid[t];
        // Simpson weights of the reference's rule (src/common/numerical_func.c:155-192)
        // times the mesh derivative; the kernel divides the sum by 3
        std::vector<double> w(n, 0.0);
        w[0] = 1.0;
        for (int i = 1; i < n - 1; i += 2) w[i] += 4.0;
        for (int i = 2; i < n - 1; i += 2) w[i] += 2.0;
        if (n % 2)
            w[n - 1] += 1.0;
        else
        {
            w[n - 3] -= 0.25;
            w[n - 2] += 1.0;
            w[n - 1] += 1.25;
        }
        for (int i = 0; i < n; ++i)
        {
            in[i] = r_grid[t][i];
            in[ngmax + i] = w[i] * rab_grid[t][i];
            in[2 * (size_t)ngmax + i] = vloc_atomic[t][i];
        }
        CUDA_TRY(h, cudaMemcpyAsync(h->d_vl_in.p, in.data(), sizeof(double) * 3 * ngmax, cudaMemcpyHostToDevice,
                                    h->st));
        const double* din = (const double*)h->d_vl_in.p;
        lelph_launch_vloc_table(din, din + ngmax, din + 2 * ngmax, n, zval[t], h->vl_volume, dimension == '3',
                                h->vl_dg, npts, (double*)h->d_vl_v.p + (size_t)t * npts, h->st);
        h->stats.kernel_launches += 1;
        CUDA_TRY(h, cudaGetLastError());
        CUDA_TRY(h, cudaMemcpyAsync(table.data() + (size_t)t * npts, (double*)h->d_vl_v.p + (size_t)t * npts,
                                    sizeof(double) * npts, cudaMemcpyDeviceToHost, h->st));
        CUDA_TRY(h, cudaStreamSynchronize(h->st));
    }
    for (int t = 0; t < h->ntype; ++t)
    {
        std::vector<double> y(table.begin() + (size_t)t * npts, table.begin() + (size_t)(t + 1) * npts);
        std::vector<double> d = spline_slopes(y, h->vl_dg);
        std::copy(d.begin(), d.end(), slopes.begin() + (size_t)t * npts);
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->d_vl_dv.p, slopes.data(), sizeof(double) * slopes.size(), cudaMemcpyHostToDevice,
                                h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    h->vl_ready = true;
    return LELPH_GPU_OK;
}

// dV_loc (nmodes, N) of q into h->d_vloc (device, reference box)
static int dvloc_device(lelph_gpu* h, const double qpt_crys[3], const double2* eig_dev)
{
    if (!h->vl_ready) return fail(h, LELPH_GPU_ERR_STATE, "lelph_gpu_set_local_pseudo was not called");
    const lelph_gpu_desc& d = h->d;
    const long long NN = (long long)h->Nbox[0] * h->Nbox[1] * h->Nbox[2];
    int rc = ensure(h, h->d_vloc, sizeof(double2) * (size_t)d.nmodes * NN);
    if (rc) return rc;
    VlocDesc vd;
    vd.Nx = h->Nbox[0];
    vd.Ny = h->Nbox[1];
    vd.Nz = h->Nbox[2];
    vd.natom = d.natom;
    vd.ntype = h->ntype;
    vd.nmodes = d.nmodes;
    vd.npts = h->vl_npts;
    vd.dim2 = h->vl_dim2;
    for (int x = 0; x < 3; ++x) vd.q[x] = qpt_crys[x];
    for (int i = 0; i < 9; ++i) vd.blat[i] = h->blat[i];
    vd.alat_zz = h->alat[8];
    vd.dg = h->vl_dg;
    vd.volume = h->vl_volume;
    for (int t = 0; t < LELPH_VLOC_MAXTYPE; ++t) vd.zval[t] = t < h->ntype ? h->vl_zval[t] : 0.0;
    vd.v = (const double*)h->d_vl_v.p;
    vd.dv = (const double*)h->d_vl_dv.p;
    vd.atom_pos = (const double*)h->d_apos.p;
    vd.atom_type = (const int*)h->d_atype.p;
    CUDA_TRY(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned), h->st));
    if (lelph_launch_dvloc_g(vd, eig_dev, (double2*)h->d_vloc.p, (unsigned*)h->d_status.p, h->st))
        return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "too many species or modes for the local potential");
    double2* v = (double2*)h->d_vloc.p;
    // unnormalised inverse transform on the reference box (FFTW_BACKWARD)
    lelph_launch_fft_contig_d(v, (long long)d.nmodes * h->Nbox[0] * h->Nbox[1], h->planN[2],
                              (const double2*)h->d_twN[2].p, +1, h->st);
    lelph_launch_fft_strided_d(v, (long long)d.nmodes * h->Nbox[0], h->Nbox[2], h->planN[1],
                               (const double2*)h->d_twN[1].p, +1, h->st);
    lelph_launch_fft_strided_d(v, (long long)d.nmodes, h->Nbox[1] * h->Nbox[2], h->planN[0],
                               (const double2*)h->d_twN[0].p, +1, h->st);
    h->stats.kernel_launches += 4;
    CUDA_TRY(h, cudaGetLastError());
    unsigned st = 0;
    CUDA_TRY(h, cudaMemcpyAsync(&st, h->d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    if (st) return fail(h, LELPH_GPU_ERR_GEOMETRY, "|q+G| beyond the V_loc table");
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_dvlocq(lelph_gpu* h, const double qpt_crys[3], const double* eigVec, double* Vlocr)
{
    if (!h || !qpt_crys || !eigVec || !Vlocr) return LELPH_GPU_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    const lelph_gpu_desc& d = h->d;
    int rc = ensure(h, h->d_tmp, std::max(h->d_tmp.n, sizeof(double2) * (size_t)d.nmodes * d.nmodes));
    if (rc) return rc;
    CUDA_TRY(h, cudaMemcpyAsync(h->d_tmp.p, eigVec, sizeof(double2) * d.nmodes * d.nmodes, cudaMemcpyHostToDevice,
                                h->st));
    rc = dvloc_device(h, qpt_crys, (const double2*)h->d_tmp.p);
    if (rc) return rc;
    const long long NN = (long long)h->Nbox[0] * h->Nbox[1] * h->Nbox[2];
    CUDA_TRY(h, cudaMemcpyAsync(Vlocr, h->d_vloc.p, sizeof(double2) * (size_t)d.nmodes * NN, cudaMemcpyDeviceToHost,
                                h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_set_q_induced(lelph_gpu* h, int slot, const double qpt_crys[3], const double* eigVec,
                                       const double* dVscf_induced)
{
    if (!h) return LELPH_GPU_ERR_INVALID;
    if (!h->vl_ready) return fail(h, LELPH_GPU_ERR_STATE, "lelph_gpu_set_local_pseudo was not called");
    int rc = set_q_common(h, slot, qpt_crys, eigVec, dVscf_induced);
    if (rc) return rc;
    const lelph_gpu_desc& d = h->d;
    rc = dvloc_device(h, qpt_crys, (const double2*)h->d_eig.p + (size_t)slot * d.nmodes * d.nmodes);
    if (rc) return rc;
    const long long NN = (long long)h->Nbox[0] * h->Nbox[1] * h->Nbox[2];
    const size_t dvn = (size_t)d.nmodes * d.nmag * NN;
    lelph_launch_add_dvscf((double2*)h->d_dvr.p + (size_t)slot * dvn, (const double2*)h->d_vloc.p, d.nmodes, d.nmag,
                           NN, h->st);
    h->stats.kernel_launches += 1;
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    h->windows_ok = false;
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_set_q_dvscf_qe(lelph_gpu* h, int slot, const double qpt_crys[3], const double* eigVec,
                                        const double* pats, const double* dvscf_qe, int induced, double* dvscf_out)
{
    if (!h || !pats || !dvscf_qe) return LELPH_GPU_ERR_INVALID;
    if (induced && !h->vl_ready) return fail(h, LELPH_GPU_ERR_STATE, "lelph_gpu_set_local_pseudo was not called");
    int rc = set_q_common(h, slot, qpt_crys, eigVec, nullptr);
    if (rc) return rc;
    const lelph_gpu_desc& d = h->d;
    const int nm = d.nmodes;
    const long long NN = (long long)h->Nbox[0] * h->Nbox[1] * h->Nbox[2];
    const size_t dvn = (size_t)nm * d.nmag * NN;
    // eig pats^H (read_dvscf.c:113-128), host
    std::vector<double2> M((size_t)nm * nm);
    for (int v = 0; v < nm; ++v)
        for (int p = 0; p < nm; ++p)
        {
            std::complex<double> acc = 0;
            for (int a = 0; a < nm; ++a)
                acc += std::complex<double>(eigVec[2 * (v * nm + a)], eigVec[2 * (v * nm + a) + 1]) *
                       std::conj(std::complex<double>(pats[2 * (p * nm + a)], pats[2 * (p * nm + a) + 1]));
            M[(size_t)v * nm + p] = make_double2(acc.real(), acc.imag());
        }
    rc = ensure(h, h->d_dvraw, sizeof(double2) * (dvn + (size_t)nm * nm));
    if (rc) return rc;
    double2* raw = (double2*)h->d_dvraw.p;
    double2* dM = raw + dvn;
    CUDA_TRY(h, cudaMemcpyAsync(raw, dvscf_qe, sizeof(double2) * dvn, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(dM, M.data(), sizeof(double2) * M.size(), cudaMemcpyHostToDevice, h->st));
    double2* slot_dv = (double2*)h->d_dvr.p + (size_t)slot * dvn;
    tstart(h);
    if (lelph_launch_dvscf_ingest(raw, dM, nm, d.nmag, h->Nbox[0], h->Nbox[1], h->Nbox[2], slot_dv, h->st))
        return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "dvscf ingest launch configuration");
    h->stats.kernel_launches += 1;
    CUDA_TRY(h, cudaGetLastError());
    h->stats.dvscf_ms += tstop(h);
    if (dvscf_out)
        CUDA_TRY(h, cudaMemcpyAsync(dvscf_out, slot_dv, sizeof(double2) * dvn, cudaMemcpyDeviceToHost, h->st));
    if (induced)
    {
        rc = dvloc_device(h, qpt_crys, (const double2*)h->d_eig.p + (size_t)slot * nm * nm);
        if (rc) return rc;
        lelph_launch_add_dvscf(slot_dv, (const double2*)h->d_vloc.p, nm, d.nmag, NN, h->st);
        h->stats.kernel_launches += 1;
        CUDA_TRY(h, cudaGetLastError());
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    h->windows_ok = false;
    return LELPH_GPU_OK;
}

// dV windows of every loaded q slot on the product grid (FP64 plain form;
// FP32 scaled by a per-mode power of two in the mixed form)
static int build_windows(lelph_gpu* h)
{
    const lelph_gpu_desc& d = h->d;
    const GeomDev& g = h->g;
    const long long NN = (long long)h->Nbox[0] * h->Nbox[1] * h->Nbox[2];
    const long long M = (long long)g.Nx * g.Ny * g.Nz;
    const int ncomp = d.nmodes * d.nmag;
    h->win_base.assign(h->qslots.size(), -1);
    int nwin = 0, umax = 0;
    for (size_t s = 0; s < h->qslots.size(); ++s)
        if (h->qslots[s].set)
        {
            h->win_base[s] = nwin;
            int nu = (int)h->qslots[s].ulms.size() / 3;
            nwin += nu;
            umax = std::max(umax, nu);
        }
    h->nwin = nwin;
    if (nwin == 0)
    {
        h->windows_ok = true;
        return LELPH_GPU_OK;
    }
    int rc = ensure(h, h->d_wtmpN, sizeof(double2) * ncomp * NN);
    if (rc) return rc;
    rc = ensure(h, h->d_wtmpM, sizeof(double2) * (size_t)umax * ncomp * M);
    if (rc) return rc;
    // the umklapp lists of every slot, uploaded in one copy (a pageable copy
    // may wait for the stream, so one per slot would stall the queue per slot)
    h->ulms_all.clear();
    std::vector<size_t> uoff(h->qslots.size(), 0);
    for (size_t s = 0; s < h->qslots.size(); ++s)
        if (h->qslots[s].set)
        {
            uoff[s] = h->ulms_all.size();
            h->ulms_all.insert(h->ulms_all.end(), h->qslots[s].ulms.begin(), h->qslots[s].ulms.end());
        }
    rc = ensure(h, h->d_tmp, sizeof(int) * h->ulms_all.size() + 16);
    if (rc) return rc;
    if (!h->ulms_all.empty())
        CUDA_TRY(h, cudaMemcpyAsync(h->d_tmp.p, h->ulms_all.data(), sizeof(int) * h->ulms_all.size(),
                                    cudaMemcpyHostToDevice, h->st));
    if (!h->mixed)
    {
        rc = ensure(h, h->d_win64, sizeof(double2) * (size_t)nwin * ncomp * M);
        if (rc) return rc;
    }
    else
    {
        rc = ensure(h, h->d_win32, sizeof(float2) * (size_t)nwin * ncomp * M);
        if (rc) return rc;
        rc = ensure(h, h->d_winscale, sizeof(float) * (size_t)nwin * d.nmodes);
        if (rc) return rc;
        rc = ensure(h, h->d_maxabs, sizeof(unsigned) * (size_t)umax * d.nmodes);
        if (rc) return rc;
    }
    for (size_t s = 0; s < h->qslots.size(); ++s)
    {
        if (!h->qslots[s].set) continue;
        const int nu = (int)h->qslots[s].ulms.size() / 3;
        if (nu == 0) continue;
        if (h->mixed)
        {
            // mixed form: FP32 transforms (the windows end up as FP32 tiles);
            // the scratch arrays of the FP64 path hold the FP32 data
            float2* tN = (float2*)h->d_wtmpN.p;
            float2* tM = (float2*)h->d_wtmpM.p;
            lelph_launch_dm_c64((const double2*)h->d_dvr.p + (size_t)s * ncomp * NN, (long long)ncomp * NN, tN, h->st);
            lelph_launch_fft_contig_f(tN, (long long)ncomp * h->Nbox[0] * h->Nbox[1], h->planN[2],
                                      (const float2*)h->d_twN32[2].p, -1, h->st);
            lelph_launch_fft_strided_f(tN, (long long)ncomp * h->Nbox[0], h->Nbox[2], h->planN[1],
                                       (const float2*)h->d_twN32[1].p, -1, h->st);
            lelph_launch_fft_strided_f(tN, (long long)ncomp, h->Nbox[1] * h->Nbox[2], h->planN[0],
                                       (const float2*)h->d_twN32[0].p, -1, h->st);
            const int3 dm = make_int3(h->qslots[s].dmin[0], h->qslots[s].dmin[1], h->qslots[s].dmin[2]);
            k_dv_window<float2><<<dim3(64, ncomp, nu), 256, 0, h->st>>>(tN, ncomp, h->Nbox[0], h->Nbox[1], h->Nbox[2],
                                                                        (const int*)h->d_tmp.p + uoff[s], nu, dm, g,
                                                                        1.0 / (double)NN, tM);
            lelph_launch_fft_contig_f(tM, (long long)nu * ncomp * g.Nx * g.Ny, h->plan[2],
                                      (const float2*)h->d_tw32[2].p, +1, h->st);
            lelph_launch_fft_strided_f(tM, (long long)nu * ncomp * g.Nx, g.Nz, h->plan[1],
                                       (const float2*)h->d_tw32[1].p, +1, h->st);
            lelph_launch_fft_strided_f(tM, (long long)nu * ncomp, g.Ny * g.Nz, h->plan[0],
                                       (const float2*)h->d_tw32[0].p, +1, h->st);
            if (h->gspace)
            {
                // the G-space route reads the windows as plain FP32 boxes
                CUDA_TRY(h, cudaMemcpyAsync((float2*)h->d_win32.p + (size_t)h->win_base[s] * ncomp * M, tM,
                                            sizeof(float2) * (size_t)nu * ncomp * M, cudaMemcpyDeviceToDevice, h->st));
                h->stats.kernel_launches += 7;
                CUDA_TRY(h, cudaGetLastError());
                continue;
            }
            unsigned* mx = (unsigned*)h->d_maxabs.p;
            float* sc = (float*)h->d_winscale.p + (size_t)h->win_base[s] * d.nmodes;
            CUDA_TRY(h, cudaMemsetAsync(mx, 0, sizeof(unsigned) * nu * d.nmodes, h->st));
            k_dv_maxabs<float2><<<dim3(64, nu * d.nmodes), 256, 0, h->st>>>(tM, nu * d.nmodes, d.nmag, M, mx);
            k_mode_scale<<<(nu * d.nmodes + 63) / 64, 64, 0, h->st>>>(mx, nu * d.nmodes, sc);
            k_dv_convert<float2><<<1024, 256, 0, h->st>>>(tM, (float2*)h->d_win32.p, nu, (int)ncomp, M,
                                                          h->win_base[s], d.nmag, sc);
            h->stats.kernel_launches += 11;
            CUDA_TRY(h, cudaGetLastError());
            continue;
        }
        // plain form: FP64 transforms
        double2* tN = (double2*)h->d_wtmpN.p;
        double2* tM = (double2*)h->d_wtmpM.p;
        CUDA_TRY(h, cudaMemcpyAsync(tN, (const double2*)h->d_dvr.p + (size_t)s * ncomp * NN,
                                    sizeof(double2) * ncomp * NN, cudaMemcpyDeviceToDevice, h->st));
        // forward transform on the reference box (FFTW_FORWARD, unnormalised)
        lelph_launch_fft_contig_d(tN, (long long)ncomp * h->Nbox[0] * h->Nbox[1], h->planN[2],
                                  (const double2*)h->d_twN[2].p, -1, h->st);
        lelph_launch_fft_strided_d(tN, (long long)ncomp * h->Nbox[0], h->Nbox[2], h->planN[1],
                                   (const double2*)h->d_twN[1].p, -1, h->st);
        lelph_launch_fft_strided_d(tN, (long long)ncomp, h->Nbox[1] * h->Nbox[2], h->planN[0],
                                   (const double2*)h->d_twN[0].p, -1, h->st);
        const int3 dm = make_int3(h->qslots[s].dmin[0], h->qslots[s].dmin[1], h->qslots[s].dmin[2]);
        k_dv_window<double2><<<dim3(64, ncomp, nu), 256, 0, h->st>>>(tN, ncomp, h->Nbox[0], h->Nbox[1], h->Nbox[2],
                                                             (const int*)h->d_tmp.p + uoff[s], nu, dm, g,
                                                             1.0 / (double)NN, tM);
        // inverse transform on the product grid
        lelph_launch_fft_contig_d(tM, (long long)nu * ncomp * g.Nx * g.Ny, h->plan[2], (const double2*)h->d_tw64[2].p,
                                  +1, h->st);
        lelph_launch_fft_strided_d(tM, (long long)nu * ncomp * g.Nx, g.Nz, h->plan[1], (const double2*)h->d_tw64[1].p,
                                   +1, h->st);
        lelph_launch_fft_strided_d(tM, (long long)nu * ncomp, g.Ny * g.Nz, h->plan[0], (const double2*)h->d_tw64[0].p,
                                   +1, h->st);
        const size_t base = (size_t)h->win_base[s] * ncomp * M;
        CUDA_TRY(h, cudaMemcpyAsync((double2*)h->d_win64.p + base, tM, sizeof(double2) * (size_t)nu * ncomp * M,
                                    cudaMemcpyDeviceToDevice, h->st));
        h->stats.kernel_launches += 7;
        CUDA_TRY(h, cudaGetLastError());
    }
    h->windows_ok = true;
    return LELPH_GPU_OK;
}


// Local term of pairs[0 .. n) on the G-space route, into glocal
// (pair, spin, mode x band of k, band of k+q), FP64, 1/M applied.  Pairs are
// visited grouped by their k so that psi(r) of a k is built once per group:
// scatter of the unfolded coefficients and the inverse FFT (the reference's
// invfft3D of the k wavefunction, src/dvloc/compute_Vbare_loc.c:206-238).
static int gs_local(lelph_gpu* h, const PairInfo* pairs, int n, double2* glocal)
{
    const lelph_gpu_desc& d = h->d;
    const GeomDev& g = h->g;
    const bool f64 = !h->mixed;
    const size_t e = f64 ? sizeof(double2) : sizeof(float2);
    const long long M = (long long)g.Nx * g.Ny * g.Nz;
    const int nb = d.nbnds, ns = d.nspinor, nm = d.nmodes;
    const int nbox = d.nspin * nb * ns;
    const int nrows = nm * nb;
    const int npw_max = *std::max_element(h->npw.begin(), h->npw.end());
    int rc = ensure(h, h->d_gs_psi, e * (size_t)nbox * M);
    if (rc) return rc;
    // modes per pass: the plane-pass output and the GEMM operand of a block of
    // modes stay within ~2 GB
    // (the tensor-core GEMM of the mixed form takes the sphere values as two
    // arrays, TF32 hi and lo, and the k+q coefficients split the same way)
    const bool tc = !f64 && h->gs_tc;
    const size_t na = tc ? 2 : 1;
    const size_t per_mode = e * (size_t)nb * ns * ((size_t)g.Nx * h->gs_ncol_max + na * h->gs_npad_max);
    const int nub = (int)std::max<size_t>(1, std::min<size_t>((size_t)nm, (2ull << 30) / per_mode));
    rc = ensure(h, h->d_gs_out1, e * (size_t)nub * nb * ns * g.Nx * h->gs_ncol_max);
    if (rc) return rc;
    const size_t a_cap = (size_t)nub * nb * ns * h->gs_npad_max;  // complex elements of one A array
    void* prev_A = h->d_gs_A.p;
    rc = ensure(h, h->d_gs_A, e * na * a_cap);
    if (rc) return rc;
    // a row's positions past its sphere (npw .. npad) meet zero k+q coefficients
    // and must hold finite values: clear a fresh buffer once
    if (h->d_gs_A.p != prev_A) CUDA_TRY(h, cudaMemsetAsync(h->d_gs_A.p, 0, h->d_gs_A.n, h->st));
    int ntile_count = 0;
    const int NT = tc ? lelph_gs_tc_ntile(nb, &ntile_count) : 0;
    if (tc)
    {
        rc = ensure(h, h->d_gs_bq, sizeof(float) * 2 * (size_t)(2 * nb) * (2 * (size_t)ns * h->gs_npad_max));
        if (rc) return rc;
    }
    void* A_lo = tc ? (void*)((float2*)h->d_gs_A.p + a_cap) : nullptr;
    const int kchunk = 1024;
    const int nch_max = (ns * h->gs_npad_max + kchunk - 1) / kchunk;
    rc = ensure(h, h->d_gs_part, e * (size_t)nch_max * nrows * nb);
    if (rc) return rc;
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return pairs[a].kbz_k < pairs[b].kbz_k; });
    const void* tw[3];
    for (int x = 0; x < 3; ++x) tw[x] = f64 ? h->d_tw64[x].p : h->d_tw32[x].p;
    const void* winb = f64 ? h->d_win64.p : h->d_win32.p;
    GsGeom gg{g.Nx, g.Ny, g.Nz, nb, ns, d.nmag, 0};
    int cur = -1;
    for (int oi = 0; oi < n; ++oi)
    {
        const int i = order[oi];
        const PairInfo& P = pairs[i];
        if (P.kbz_k != cur)
        {
            cur = P.kbz_k;
            CUDA_TRY(h, cudaMemsetAsync(h->d_gs_psi.p, 0, e * (size_t)nbox * M, h->st));
            lelph_launch_scatter(cur, 1, (const KPointSym*)h->d_ksym.p, (const int*)h->d_miller.p,
                                 (const long long*)h->d_pwoff.p, (const int*)h->d_npw.p, npw_max,
                                 (const double2*)h->d_coef.p, (const long long*)h->d_coefoff.p, g, f64, h->d_gs_psi.p,
                                 (double2*)h->d_chat.p, (const long long*)h->d_chatoff.p, h->st);
            if (f64)
            {
                double2* bx = (double2*)h->d_gs_psi.p;
                lelph_launch_fft_contig_d(bx, (long long)nbox * g.Nx * g.Ny, h->plan[2], (const double2*)tw[2], +1, h->st);
                lelph_launch_fft_strided_d(bx, (long long)nbox * g.Nx, g.Nz, h->plan[1], (const double2*)tw[1], +1, h->st);
                lelph_launch_fft_strided_d(bx, nbox, g.Ny * g.Nz, h->plan[0], (const double2*)tw[0], +1, h->st);
            }
            else
            {
                float2* bx = (float2*)h->d_gs_psi.p;
                lelph_launch_fft_contig_f(bx, (long long)nbox * g.Nx * g.Ny, h->plan[2], (const float2*)tw[2], +1, h->st);
                lelph_launch_fft_strided_f(bx, (long long)nbox * g.Nx, g.Nz, h->plan[1], (const float2*)tw[1], +1, h->st);
                lelph_launch_fft_strided_f(bx, nbox, g.Ny * g.Nz, h->plan[0], (const float2*)tw[0], +1, h->st);
            }
            h->stats.kernel_launches += 4;
        }
        const int kq = P.kbz_kq;
        const int npad = h->gs_npad[kq], ncol = h->gs_ncol[kq];
        const int Ktot = ns * npad;
        const int nch = (Ktot + kchunk - 1) / kchunk;
        const void* win = (const char*)winb + e * (size_t)P.dvslot * nm * d.nmag * M;
        for (int spin = 0; spin < d.nspin; ++spin)
        {
            gg.spin = spin;
            const void* psi = (const char*)h->d_gs_psi.p + e * (size_t)spin * nb * ns * M;
            const void* B = (const char*)h->d_gs_bp.p + e * ((size_t)h->gs_bp_off[kq] + (size_t)spin * nb * ns * npad);
            CUtensorMap tm[4];
            if (tc)
            {
                // B rows 2n = (br, bi), 2n + 1 = (-bi, br) over K = 2 Ktot, hi plane then lo plane
                float* bq = (float*)h->d_gs_bq.p;
                lelph_launch_gs_bsplit((const float2*)B, nb, Ktot, bq, h->st);
                h->stats.kernel_launches += 1;
                const size_t plane = (size_t)(2 * nb) * 2 * Ktot;
                rc = make_tmap(h, &tm[2], bq, 2ull * Ktot, 2ull * nb, (unsigned)NT, true, true, 32);
                if (!rc) rc = make_tmap(h, &tm[3], bq + plane, 2ull * Ktot, 2ull * nb, (unsigned)NT, true, true, 32);
                if (rc) return rc;
            }
            for (int nu0 = 0; nu0 < nm; nu0 += nub)
            {
                const int nmb = std::min(nub, nm - nu0);
                int bad = 0;
                if (tc)
                {
                    rc = make_tmap(h, &tm[0], h->d_gs_A.p, 2ull * Ktot, (unsigned long long)nmb * nb, 128, true, true,
                                   32);
                    if (!rc) rc = make_tmap(h, &tm[1], A_lo, 2ull * Ktot, (unsigned long long)nmb * nb, 128, true, true, 32);
                    if (rc) return rc;
                }
                gs_tick(h);
                bad |= lelph_launch_gs_plane(gg, f64, psi, win, nu0, nmb, h->plan[1], h->plan[2], tw[1], tw[2],
                                             (const int*)h->d_gs_cols.p + h->gs_col_off[kq], ncol,
                                             (const int*)h->d_gs_cols2.p + h->gs_col_off[kq],
                                             (const int*)h->d_gs_zl.p + h->gs_zl_off[kq], h->gs_nzl[kq],
                                             h->d_gs_out1.p, h->st);
                h->stats.gs_plane_ms += gs_tock(h);
                bad |= lelph_launch_gs_xpass(gg, f64, h->d_gs_out1.p, nmb * nb * ns, ncol, h->plan[0], tw[0],
                                             (const int*)h->d_gs_cst.p + h->gs_cst_off[kq],
                                             (const int*)h->d_gs_kcx.p + h->gs_perm_off[kq], npad, h->d_gs_A.p,
                                             h->st, A_lo);
                h->stats.gs_xpass_ms += gs_tock(h);
                if (tc)
                    bad |= lelph_launch_gs_gemm_tc(tm, nmb * nb, nb, Ktot, kchunk, nu0 * nb, nrows,
                                                   (float2*)h->d_gs_part.p, (unsigned*)h->d_status.p, h->wait_ns,
                                                   h->st);
                else
                    bad |= lelph_launch_gs_gemm(f64, h->d_gs_A.p, B, nmb * nb, nb, Ktot, kchunk, nu0 * nb, nrows,
                                                h->d_gs_part.p, h->st);
                h->stats.gs_gemm_ms += gs_tock(h);
                if (bad) return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "G-space route: launch configuration");
                h->stats.kernel_launches += 3;
            }
            lelph_launch_gs_reduce(f64, h->d_gs_part.p, (long long)nrows * nb, nch, 1.0 / (double)M,
                                   glocal + ((size_t)i * d.nspin + spin) * nrows * nb, h->st);
            h->stats.kernel_launches += 1;
        }
        CUDA_TRY(h, cudaGetLastError());
    }
    return LELPH_GPU_OK;
}

static int run_impl(lelph_gpu* h, int n, const int* qslot, const int* kbz, int non_loc, int kminusq, int out_type,
                    void* g_out, bool out_device)
{
    if (!h || n < 0 || (n > 0 && (!qslot || !kbz || !g_out))) return LELPH_GPU_ERR_INVALID;
    if (out_type != LELPH_GPU_OUT_C128 && out_type != LELPH_GPU_OUT_C64) return fail(h, LELPH_GPU_ERR_INVALID, "out_type");
    if (n == 0) return LELPH_GPU_OK;
    CUDA_TRY(h, cudaSetDevice(h->device));
    if (!h->prepared)
    {
        int rc = lelph_gpu_prepare(h);
        if (rc) return rc;
    }
    if (!h->windows_ok)
    {
        int rc = build_windows(h);
        if (rc) return rc;
    }
    const lelph_gpu_desc& d = h->d;
    const GeomDev& g = h->g;
    // pairs (src/elph/compute_elph_matq.c:65-128): per pair the k+q search, the
    // umklapp vector and the dV window; large batches are split over the host
    // cores (the GPU waits for this table), and the error reported is that of
    // the first failing pair, as in a serial loop
    std::vector<PairInfo> pairs(n);
    if (h->khash.empty())
        for (int i = 0; i < d.nkpts_BZ; ++i) h->khash.emplace(k_hash_key(&h->kbz_crys[3 * i]), i);
    struct PairErr
    {
        int at = -1, code = 0;
        const char* msg = "";
    };
    auto make_pairs = [&](int i0, int i1, PairErr& e) {
        for (int i = i0; i < i1; ++i)
        {
            auto bad = [&](int code, const char* msg) {
                e.at = i;
                e.code = code;
                e.msg = msg;
            };
            if (qslot[i] < 0 || qslot[i] >= (int)h->qslots.size() || !h->qslots[qslot[i]].set)
                return bad(LELPH_GPU_ERR_STATE, "q slot not loaded");
            if (kbz[i] < 0 || kbz[i] >= d.nkpts_BZ) return bad(LELPH_GPU_ERR_INVALID, "k index out of range");
            const double* q = h->qslots[qslot[i]].q;
            double qt[3], kq[3];
            for (int x = 0; x < 3; ++x) qt[x] = kminusq ? -q[x] : q[x];
            for (int x = 0; x < 3; ++x) kq[x] = h->kbz_crys[3 * kbz[i] + x] + qt[x];
            int ikq = find_k_fast(h, kq);
            if (ikq < 0) return bad(LELPH_GPU_ERR_GEOMETRY, "K+Q point cannot be found in kgrid");
            int idx_k = kbz[i], idx_kq = ikq;
            if (kminusq) std::swap(idx_k, idx_kq);
            PairInfo& P = pairs[i];
            P.kbz_k = idx_k;
            P.kbz_kq = idx_kq;
            P.qslot = qslot[i];
            if (umklapp(h, idx_k, idx_kq, q, P.ulm)) return bad(LELPH_GPU_ERR_GEOMETRY, "non-integral umklapp vector");
            P.dvslot = window_of(h, qslot[i], P.ulm);
            if (P.dvslot < 0) return bad(LELPH_GPU_ERR_GEOMETRY, "umklapp vector outside the q slot's set");
        }
    };
    {
        const int nthr = n >= 1024 ? std::max(1, std::min<int>(8, (int)std::thread::hardware_concurrency())) : 1;
        std::vector<PairErr> errs(nthr);
        const int per = (n + nthr - 1) / nthr;
        run_workers(nthr, [&](int t) { make_pairs(std::min(n, t * per), std::min(n, (t + 1) * per), errs[t]); });
        for (const PairErr& e : errs)
            if (e.at >= 0) return fail(h, e.code, e.msg);  // ranges are in order: the first is the earliest pair
    }
    int rc = upload(h, h->d_pairs, pairs.data(), sizeof(PairInfo) * n);
    if (rc) return rc;
    const size_t gsz = (size_t)d.nmodes * d.nspin * d.nbnds * d.nbnds;
    const size_t esz = out_type == LELPH_GPU_OUT_C64 ? sizeof(float2) : sizeof(double2);
    void* gdev = g_out;
    if (!out_device)
    {
        rc = ensure(h, h->d_gout, esz * gsz * n);
        if (rc) return rc;
        gdev = h->d_gout.p;
    }
    NonlocalDesc nl = nl_desc(h);
    if (h->mixed && !h->gspace && (h->tmapV_base != h->d_win32.p || h->tmapV_rows != h->nwin))
    {
        // dV windows, tile-major: blocks (window, 32-point block) of (mode, component) rows x 64 floats
        const long long M = (long long)g.Nx * g.Ny * g.Nz;
        rc = make_tmap3(h, &h->tmapV, h->d_win32.p, true, 64, (unsigned long long)d.nmodes * d.nmag,
                        (unsigned long long)h->nwin * (M / 32), (unsigned)(g.mt_modes * d.nmag),
                        (unsigned)(g.kpts / 32), false);
        if (rc) return rc;
        h->tmapV_base = h->d_win32.p;
        h->tmapV_rows = h->nwin;
    }
    CUDA_TRY(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned), h->st));
    const int nrows = d.nmodes * d.nbnds;
    // batch the pairs so the local workspace stays bounded (~4 GB)
    size_t per_pair;
    const bool fp64_local = !h->mixed || h->gspace;  // the local term arrives as FP64 sums (glocal)
    if (fp64_local) per_pair = sizeof(double2) * (size_t)d.nspin * nrows * d.nbnds;
    else per_pair = sizeof(float) * lelph_tc_partials_per_pair(g, h->nchunks);
    int batch = (int)std::max<size_t>(1, std::min<size_t>((size_t)n, (4ull << 30) / per_pair));
    // Output to host memory: the pairs go in four or more batches, and each
    // batch's result is copied on the copy stream while the next one computes
    // (the copy of batch i is issued after batch i + 1 is launched, so a
    // pageable destination, whose copy blocks the host, still overlaps).
    const bool overlap = !out_device && n >= 256;
    if (overlap) batch = std::min(batch, (n + 3) / 4);
    rc = ensure(h, fp64_local ? h->d_glocal : h->d_partials, per_pair * batch);
    if (rc) return rc;
    auto copy_batch = [&](int q0, int qn, int ev) -> int {
        CUDA_TRY(h, cudaStreamWaitEvent(h->st_copy, h->evc[ev], 0));
        CUDA_TRY(h, cudaMemcpyAsync((char*)g_out + esz * gsz * q0, (const char*)gdev + esz * gsz * q0,
                                    esz * gsz * qn, cudaMemcpyDeviceToHost, h->st_copy));
        return LELPH_GPU_OK;
    };
    int prev0 = -1, prevn = 0, ib = 0;
    for (int p0 = 0; p0 < n; p0 += batch, ++ib)
    {
        int nb = std::min(batch, n - p0);
        const PairInfo* dp = (const PairInfo*)h->d_pairs.p + p0;
        while ((int)h->evlive.size() < 2 * (ib + 1))
        {
            cudaEvent_t e = nullptr;
            CUDA_TRY(h, cudaEventCreate(&e));
            h->evlive.push_back(e);
        }
        CUDA_TRY(h, cudaEventRecord(h->evlive[2 * ib], h->st));
        tstart(h);
        if (h->gspace)
        {
            rc = gs_local(h, pairs.data() + p0, nb, (double2*)h->d_glocal.p);
            if (rc) return rc;
        }
        else if (!h->mixed)
            lelph_launch_local_fp64(dp, nb, (const double2*)h->d_psi64.p, (const double2*)h->d_win64.p, g,
                                    (double2*)h->d_glocal.p, (unsigned*)h->d_status.p, h->st);
        else
            lelph_launch_local_tc(dp, nb, &h->tmapB, &h->tmapP, &h->tmapV, g, h->ab_bf16, h->chunk_pts, h->nchunks,
                                  (float*)h->d_partials.p, (unsigned*)h->d_status.p, h->st, h->wait_ns);
        CUDA_TRY(h, cudaEventRecord(h->evlive[2 * ib + 1], h->st));
        h->stats.local_ms += tstop(h);
        h->stats.local_launches += 1;
        tstart(h);
        lelph_launch_finish(dp, nb, !fp64_local ? 0 : (h->mixed ? 2 : 1), (const double2*)h->d_glocal.p,
                            (const float*)h->d_partials.p,
                            h->nchunks, (const float*)h->d_winscale.p, (const float*)h->d_band_scale.p,
                            (const double2*)h->d_proj.p, (const double2*)h->d_eig.p, non_loc, nl, g,
                            out_type == LELPH_GPU_OUT_C64, (char*)gdev + esz * gsz * p0, h->st);
        h->stats.finish_ms += tstop(h);
        h->stats.kernel_launches += h->gspace ? 1 : 2;  // gs_local counts its own launches
        CUDA_TRY(h, cudaGetLastError());
        if (overlap)
        {
            CUDA_TRY(h, cudaEventRecord(h->evc[ib & 1], h->st));
            if (prev0 >= 0)
            {
                rc = copy_batch(prev0, prevn, (ib - 1) & 1);
                if (rc) return rc;
            }
            prev0 = p0;
            prevn = nb;
        }
    }
    if (overlap)
    {
        rc = copy_batch(prev0, prevn, (ib - 1) & 1);
        if (rc) return rc;
        CUDA_TRY(h, cudaStreamSynchronize(h->st_copy));
    }
    else if (!out_device)
        CUDA_TRY(h, cudaMemcpyAsync(g_out, gdev, esz * gsz * n, cudaMemcpyDeviceToHost, h->st));
    rc = check_status(h);
    if (rc) return rc;
    for (int b = 0; b < ib; ++b)
    {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, h->evlive[2 * b], h->evlive[2 * b + 1]) == cudaSuccess)
        {
            h->stats.local_live_ms += ms;
            h->stats.local_live_launches += 1;
        }
    }
    h->stats.pairs_done += n;
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_run(lelph_gpu* h, int n, const int* qslot, const int* kbz, int non_loc, int kminusq,
                             int out_type, void* g_out)
{
    return run_impl(h, n, qslot, kbz, non_loc, kminusq, out_type, g_out, false);
}

extern "C" int lelph_gpu_run_device(lelph_gpu* h, int n, const int* qslot, const int* kbz, int non_loc, int kminusq,
                                    int out_type, void* g_out_dev)
{
    return run_impl(h, n, qslot, kbz, non_loc, kminusq, out_type, g_out_dev, true);
}

extern "C" int lelph_gpu_compute_elphq(lelph_gpu* h, const double qpt_crys[3], const double* eigVec,
                                       const double* dVscfq, int non_loc, int kminusq, double* elph_out)
{
    if (!h) return LELPH_GPU_ERR_INVALID;
    int rc = lelph_gpu_set_q(h, 0, qpt_crys, eigVec, dVscfq);
    if (rc) return rc;
    std::vector<int> qs(h->d.nkpts_BZ, 0), ks(h->d.nkpts_BZ);
    for (int i = 0; i < h->d.nkpts_BZ; ++i) ks[i] = i;
    return lelph_gpu_run(h, h->d.nkpts_BZ, qs.data(), ks.data(), non_loc, kminusq, LELPH_GPU_OUT_C128, elph_out);
}

extern "C" int lelph_gpu_elph_q_rotate(lelph_gpu* h, const double* Dl, const double* g, const double* Dr,
                                       int time_rev, double* out)
{
    if (!h || !Dl || !g || !Dr || !out) return LELPH_GPU_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    const int nb = h->d.nbnds, ns = h->d.nspin, nm = h->d.nmodes;
    const size_t gs = (size_t)nm * ns * nb * nb, ds = (size_t)ns * nb * nb;
    int rc = ensure(h, h->d_tmp, sizeof(double2) * (3 * gs + 2 * ds));
    if (rc) return rc;
    double2* dg = (double2*)h->d_tmp.p;
    double2* dt = dg + gs;
    double2* dout = dt + gs;
    double2* ddl = dout + gs;
    double2* ddr = ddl + ds;
    CUDA_TRY(h, cudaMemcpyAsync(dg, g, sizeof(double2) * gs, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(ddl, Dl, sizeof(double2) * ds, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(h, cudaMemcpyAsync(ddr, Dr, sizeof(double2) * ds, cudaMemcpyHostToDevice, h->st));
    dim3 grid((nb * nb + 255) / 256, nm, ns);
    k_qrot1<<<grid, 256, 0, h->st>>>(dg, ddr, nb, ns, time_rev != 0, dt);
    k_qrot2<<<grid, 256, 0, h->st>>>(dt, ddl, nb, ns, dout);
    h->stats.kernel_launches += 2;
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaMemcpyAsync(out, dout, sizeof(double2) * gs, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    return LELPH_GPU_OK;
}

// ============================================ Dmats (electronic representations)

namespace
{
typedef std::complex<double> cd;

// integer action alat^T R A^-T of a cartesian rotation on Miller indices
int miller_action(const lelph_gpu* h, const double* R, int* W)
{
    double B[9];
    for (int i = 0; i < 9; ++i) B[i] = h->blat[i] / (2 * PI_T);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
        {
            double acc = 0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) acc += h->alat[3 * k + r] * R[3 * k + l] * B[3 * l + c];
            double w = std::rint(acc);
            if (std::fabs(acc - w) > 1e-6) return -1;
            W[3 * r + c] = (int)w;
        }
    return 0;
}

// inverse of a unimodular integer matrix (adjugate / determinant)
int int_inverse3(const int* m, int* inv)
{
    const long long det = (long long)m[0] * (m[4] * m[8] - m[5] * m[7]) - (long long)m[1] * (m[3] * m[8] - m[5] * m[6]) +
                          (long long)m[2] * (m[3] * m[7] - m[4] * m[6]);
    if (det != 1 && det != -1) return -1;
    const int d = (int)det;
    inv[0] = d * (m[4] * m[8] - m[5] * m[7]);
    inv[1] = d * (m[2] * m[7] - m[1] * m[8]);
    inv[2] = d * (m[1] * m[5] - m[2] * m[4]);
    inv[3] = d * (m[5] * m[6] - m[3] * m[8]);
    inv[4] = d * (m[0] * m[8] - m[2] * m[6]);
    inv[5] = d * (m[2] * m[3] - m[0] * m[5]);
    inv[6] = d * (m[3] * m[7] - m[4] * m[6]);
    inv[7] = d * (m[1] * m[6] - m[0] * m[7]);
    inv[8] = d * (m[0] * m[4] - m[1] * m[3]);
    return 0;
}

inline cd conj_if(cd z, bool c) { return c ? std::conj(z) : z; }

// Job of the pair (symmetry isym, full-BZ k ikBZ): the reference's sequence
// (src/symmetries/elec_reps.c:33-372) folded onto the k2 side.  With x^(c)
// the conjugate of x when c holds, the two sides of the reference are
//   right: w = phR^(trR) ph1^(x1) e^{-i 2 pi m.tw} UR^(trR) U1^(x1) psi_k1^(x1),  x1 = tr1 xor trR,
//          tw = s1 W1^T tau1 + sR W_RS1^T tauR  (s = -1 where conjugated)
//   left:  v = ph2^(!tr2) e^{-i 2 pi m.tv} U2^(!tr2) psi_k2^(!tr2),  tv = s2 W_RS1^T tau2
// with ph1 = e^{-i 2 pi (S1 k1).tau1}, phR = e^{-i 2 pi (R S1 k1).tauR},
// ph2 = e^{-i 2 pi (R S1 k1).tau2}; D = sum_p v . w moves every factor of w
// but psi_k1^(x1) onto v: t = tw + tv, C = phR^(trR) ph1^(x1) ph2^(!tr2),
// M = (UR^(trR) U1^(x1))^T U2^(!tr2).
int dmat_job(lelph_gpu* h, const double* R, const int* WR, const double* tauR_crys, const cd* UR, bool trR,
             int ikBZ, DmatJob& J, const char** why)
{
    const lelph_gpu_desc& d = h->d;
    double kc[3], Rk[3], Rkc[3];
    for (int x = 0; x < 3; ++x)
        kc[x] = (h->blat[3 * x] * h->kbz_crys[3 * ikBZ] + h->blat[3 * x + 1] * h->kbz_crys[3 * ikBZ + 1] +
                 h->blat[3 * x + 2] * h->kbz_crys[3 * ikBZ + 2]) /
                (2 * PI_T);
    mat_vec3(R, kc, false, Rk);
    mat_vec3(d.alat_vec, Rk, true, Rkc);
    const int iRk = find_k_fast(h, Rkc);
    if (iRk < 0)
    {
        *why = "Rotated k point not found. Either Wrong Phonon symmetry or using non-uniform kgrid";
        return LELPH_GPU_ERR_GEOMETRY;
    }
    const KPointSym& s1 = h->ksym[ikBZ];
    const KPointSym& s2 = h->ksym[iRk];
    memset(&J, 0, sizeof(J));
    J.ik1 = s1.ik;
    J.ik2 = s2.ik;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            J.WRS1[3 * r + c] = WR[3 * r] * s1.W[c] + WR[3 * r + 1] * s1.W[3 + c] + WR[3 * r + 2] * s1.W[6 + c];
    if (int_inverse3(s2.W, J.W2inv))
    {
        *why = "symmetry not unimodular on the lattice";
        return LELPH_GPU_ERR_GEOMETRY;
    }
    const double* S1 = &h->symR[9 * s1.isym];
    const double* S2 = &h->symR[9 * s2.isym];
    double RS1[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) RS1[3 * r + c] = R[3 * r] * S1[c] + R[3 * r + 1] * S1[3 + c] + R[3 * r + 2] * S1[6 + c];
    double RS1k1[3], S2k2[3], u[3], uc[3], Rkcrys[3];
    mat_vec3(RS1, &h->kibz[3 * s1.ik], false, RS1k1);
    mat_vec3(S2, &h->kibz[3 * s2.ik], false, S2k2);
    for (int x = 0; x < 3; ++x) u[x] = S2k2[x] - RS1k1[x];
    mat_vec3(d.alat_vec, u, true, uc);
    for (int x = 0; x < 3; ++x)
    {
        J.ulm[x] = (int)std::rint(uc[x]);
        if (std::fabs(uc[x] - J.ulm[x]) > 1e-4)
        {
            *why = "S2 k2 - R S1 k1 not a G vector";
            return LELPH_GPU_ERR_GEOMETRY;
        }
    }
    mat_vec3(d.alat_vec, RS1k1, true, Rkcrys);
    const bool tr1 = s1.trev != 0, tr2 = s2.trev != 0, x1 = tr1 != trR, nt2 = !tr2;
    auto kph = [](const double* k, const double* t) {
        return std::exp(cd(0, -2 * PI_T * (k[0] * t[0] + k[1] * t[1] + k[2] * t[2])));
    };
    const cd ph1(s1.kphase[0], s1.kphase[1]);
    const cd phR = kph(Rkcrys, tauR_crys), ph2 = kph(Rkcrys, s2.tau_crys);
    cd U1[4], U2[4], Mw[4];
    for (int e = 0; e < 4; ++e)
    {
        U1[e] = conj_if(cd(s1.su2[2 * e], s1.su2[2 * e + 1]), x1);
        U2[e] = conj_if(cd(s2.su2[2 * e], s2.su2[2 * e + 1]), nt2);
    }
    cd URc[4];
    for (int e = 0; e < 4; ++e) URc[e] = conj_if(UR[e], trR);
    Mw[0] = URc[0] * U1[0] + URc[1] * U1[2];
    Mw[1] = URc[0] * U1[1] + URc[1] * U1[3];
    Mw[2] = URc[2] * U1[0] + URc[3] * U1[2];
    Mw[3] = URc[2] * U1[1] + URc[3] * U1[3];
    // M = Mw^T U2
    const cd M[4] = {Mw[0] * U2[0] + Mw[2] * U2[2], Mw[0] * U2[1] + Mw[2] * U2[3], Mw[1] * U2[0] + Mw[3] * U2[2],
                     Mw[1] * U2[1] + Mw[3] * U2[3]};
    const cd C = conj_if(phR, trR) * conj_if(ph1, x1) * conj_if(ph2, nt2);
    const double sg1 = x1 ? -1.0 : 1.0, sgR = trR ? -1.0 : 1.0, sg2 = nt2 ? -1.0 : 1.0;
    for (int c = 0; c < 3; ++c)
    {
        double a = 0, b = 0, e = 0;
        for (int r = 0; r < 3; ++r)
        {
            a += s1.W[3 * r + c] * s1.tau_crys[r];
            b += J.WRS1[3 * r + c] * tauR_crys[r];
            e += J.WRS1[3 * r + c] * s2.tau_crys[r];
        }
        J.t[c] = sg1 * a + sgR * b + sg2 * e;
    }
    J.conj_w = x1;
    J.conj_v = nt2;
    J.C = make_double2(C.real(), C.imag());
    for (int e = 0; e < 4; ++e) J.M[e] = make_double2(M[e].real(), M[e].imag());
    return LELPH_GPU_OK;
}
}  // namespace

// Dmats of the (symmetry, full-BZ k) pairs id = isym * nk_BZ + ik, for
// id = first + i (ids == NULL) or id = ids[i], i < count, into the device
// array out (count, nspin, nb, nb).
static int dmats_run(lelph_gpu* h, int nsym, const double* Rmat, const double* tau, const int* time_rev,
                     long long first, long long count, const long long* ids, double2* out)
{
    const lelph_gpu_desc& d = h->d;
    const long long nkbz = d.nkpts_BZ;
    // per-symmetry integer action, crystal translation and SU(2) matrix
    std::vector<int> WR(9 * (size_t)nsym);
    std::vector<double> tauc(3 * (size_t)nsym);
    std::vector<cd> UR(4 * (size_t)nsym);
    for (int is = 0; is < nsym; ++is)
    {
        if (miller_action(h, Rmat + 9 * is, &WR[9 * is]))
            return fail(h, LELPH_GPU_ERR_GEOMETRY, "symmetry not integral on the reciprocal lattice");
        double tc[3];
        mat_vec3(d.blat_vec, tau + 3 * is, true, tc);
        for (int x = 0; x < 3; ++x) tauc[3 * is + x] = tc[x] / (2 * PI_T);
        if (!su2mat(Rmat + 9 * is, d.nspinor, time_rev[is] != 0, &UR[4 * is]))
            return fail(h, LELPH_GPU_ERR_GEOMETRY, "Wrong symmetric matrices");
    }
    const auto th0 = std::chrono::steady_clock::now();
    std::vector<DmatJob> jobs((size_t)count);
    if (h->khash.empty())
        for (int i = 0; i < d.nkpts_BZ; ++i) h->khash.emplace(k_hash_key(&h->kbz_crys[3 * i]), i);
    auto build = [&](long long i) {
        const long long id = ids ? ids[i] : first + i;
        const int is = (int)(id / nkbz), ik = (int)(id % nkbz);
        const char* why = "";
        int rc = dmat_job(h, Rmat + 9 * is, &WR[9 * is], &tauc[3 * is], &UR[4 * is], time_rev[is] != 0, ik,
                          jobs[(size_t)i], &why);
        return std::make_pair(rc, why);
    };
    // job construction on the host cores: every worker records its first
    // failing job; the lowest one is rebuilt alone to report its error
    const int nthr = (int)std::min<long long>(std::max(1u, std::thread::hardware_concurrency()), (count + 1023) / 1024);
    std::vector<long long> bad_job((size_t)std::max(1, nthr), -1);
    if (nthr <= 1)
    {
        for (long long i = 0; i < count; ++i)
        {
            auto r = build(i);
            if (r.first) return fail(h, r.first, r.second);
        }
    }
    else
    {
        run_workers(nthr, [&](int w) {
            for (long long i = count * w / nthr; i < count * (w + 1) / nthr; ++i)
                if (build(i).first != 0)
                {
                    bad_job[(size_t)w] = i;
                    return;
                }
        });
        for (long long b : bad_job)
            if (b >= 0)
            {
                auto r = build(b);
                return fail(h, r.first, r.second);
            }
    }
    h->stats.dmats_host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - th0).count();
    // Miller -> position tables of the iBZ lists on the reference's box, built once
    DmatGeom dg;
    dg.nb = d.nbnds;
    dg.nspin = d.nspin;
    dg.nspinor = d.nspinor;
    dg.Nx = h->Nbox[0];
    dg.Ny = h->Nbox[1];
    dg.Nz = h->Nbox[2];
    dg.ntab = dg.Nx + dg.Ny + dg.Nz + 3;
    if (!h->dm_gtab_ready)
    {
        for (long long i = 0; i < 3 * h->total_pw; ++i)
            if (2 * std::abs(h->miller[i]) > h->Nbox[i % 3])
                return fail(h, LELPH_GPU_ERR_GEOMETRY, "plane wave outside the FFT box");
        const size_t nbox = (size_t)dg.Nx * dg.Ny * dg.Nz;
        int rc = ensure(h, h->d_dmgtab, sizeof(int) * nbox * d.nkpts_iBZ);
        if (rc) return rc;
        CUDA_TRY(h, cudaMemsetAsync(h->d_dmgtab.p, 0xff, sizeof(int) * nbox * d.nkpts_iBZ, h->st));
        int npw_max = *std::max_element(h->npw.begin(), h->npw.end());
        lelph_launch_dm_gtab((const int*)h->d_miller.p, (const long long*)h->d_pwoff.p, (const int*)h->d_npw.p,
                             d.nkpts_iBZ, npw_max, dg.Nx, dg.Ny, dg.Nz, (int*)h->d_dmgtab.p, h->st);
        h->stats.kernel_launches += 1;
        CUDA_TRY(h, cudaGetLastError());
        h->dm_gtab_ready = true;
    }
    const int fp64 = h->mixed ? 0 : 1;
    if (lelph_dmats_smem_bytes(dg, fp64) > 200 * 1024) return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "FFT box too large for the Dmat phase tables");
    int rc = upload(h, h->d_dmjobs, jobs.data(), sizeof(DmatJob) * jobs.size());
    if (rc) return rc;
    const int npw_max = *std::max_element(h->npw.begin(), h->npw.end());
    rc = ensure(h, h->d_dmmap, sizeof(int) * (size_t)count * npw_max);
    if (rc) return rc;
    if (!fp64 && !h->dm_coef32_ready)
    {
        const long long n = h->coef_total;
        rc = ensure(h, h->d_dmcoef32, sizeof(float2) * (size_t)n);
        if (rc) return rc;
        lelph_launch_dm_c64((const double2*)h->d_coef.p, n, (float2*)h->d_dmcoef32.p, h->st);
        h->stats.kernel_launches += 1;
        CUDA_TRY(h, cudaGetLastError());
        h->dm_coef32_ready = true;
    }
    // mixed form on the tensor cores with LELPH_DMATS_TC=1: about four times more
    // accurate than the SIMT kernel, but slower at every band count measured
    // (operand formation, not the contraction, bounds it), so not the default
    const char* etc = std::getenv("LELPH_DMATS_TC");
    if (!fp64 && etc && etc[0] == '1' && lelph_dmats_tc_supported(dg))
    {
        // groups of jobs sharing (ik1, conj_w), at most JB each
        int JB, nbt, NT, ntiles;
        lelph_dmats_tc_config(dg.nb, &JB, &nbt, &NT, &ntiles);
        std::vector<int> perm((size_t)count);
        for (long long i = 0; i < count; ++i) perm[(size_t)i] = (int)i;
        std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) {
            const DmatJob &a = jobs[(size_t)x], &b = jobs[(size_t)y];
            return a.ik1 != b.ik1 ? a.ik1 < b.ik1 : a.conj_w < b.conj_w;
        });
        std::vector<DmatGroup> groups;
        for (long long i = 0; i < count;)
        {
            const DmatJob& J = jobs[(size_t)perm[(size_t)i]];
            DmatGroup gr{(int)i, 0, J.ik1, J.conj_w};
            while (i < count && gr.count < JB && jobs[(size_t)perm[(size_t)i]].ik1 == J.ik1 &&
                   jobs[(size_t)perm[(size_t)i]].conj_w == J.conj_w)
            {
                ++gr.count;
                ++i;
            }
            groups.push_back(gr);
        }
        if (!h->dm_coefT_ready)
        {
            rc = ensure(h, h->d_dmcoefT, sizeof(float2) * (size_t)h->coef_total);
            if (rc) return rc;
            lelph_launch_dm_c64t((const double2*)h->d_coef.p, (const long long*)h->d_coefoff.p,
                                 (const int*)h->d_npw.p, d.nkpts_iBZ, d.nspin, d.nbnds, d.nspinor,
                                 (float2*)h->d_dmcoefT.p, h->st);
            h->stats.kernel_launches += 1;
            CUDA_TRY(h, cudaGetLastError());
            h->dm_coefT_ready = true;
        }
        rc = upload(h, h->d_dmperm, perm.data(), sizeof(int) * perm.size());
        if (rc) return rc;
        rc = upload(h, h->d_dmgroups, groups.data(), sizeof(DmatGroup) * groups.size());
        if (rc) return rc;
        CUDA_TRY(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned), h->st));
        tstart(h);
        if (lelph_launch_dmats_tc((const DmatJob*)h->d_dmjobs.p, count, (const DmatGroup*)h->d_dmgroups.p,
                                  (const int*)h->d_dmperm.p, (int)groups.size(), dg, (const float2*)h->d_dmcoef32.p,
                                  (const float2*)h->d_dmcoefT.p, (const long long*)h->d_coefoff.p,
                                  (const int*)h->d_miller.p,
                                  (const long long*)h->d_pwoff.p, (const int*)h->d_npw.p, (const int*)h->d_dmgtab.p,
                                  npw_max, (int*)h->d_dmmap.p, out, (unsigned*)h->d_status.p, h->wait_ns, h->st))
            return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "Dmat launch configuration");
        h->stats.kernel_launches += 2;
        CUDA_TRY(h, cudaGetLastError());
        h->stats.dmats_ms += tstop(h);
        rc = check_status(h);
        if (rc) return rc;
        h->stats.dmats_done += count;
        return LELPH_GPU_OK;
    }
    tstart(h);
    if (lelph_launch_dmats((const DmatJob*)h->d_dmjobs.p, count, dg, (const double2*)h->d_coef.p,
                           fp64 ? nullptr : (const float2*)h->d_dmcoef32.p,
                           (const long long*)h->d_coefoff.p, (const int*)h->d_miller.p, (const long long*)h->d_pwoff.p,
                           (const int*)h->d_npw.p, (const int*)h->d_dmgtab.p, npw_max, (int*)h->d_dmmap.p,
                           out, h->st))
        return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "Dmat launch configuration");
    h->stats.kernel_launches += 2;
    CUDA_TRY(h, cudaGetLastError());
    h->stats.dmats_ms += tstop(h);
    h->stats.dmats_done += count;
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_dmats(lelph_gpu* h, int nsym, const double* Rmat, const double* tau, const int* time_rev,
                               long long first, long long count, double* Dmats)
{
    if (!h || nsym <= 0 || !Rmat || !tau || !time_rev || first < 0 || count < 0) return LELPH_GPU_ERR_INVALID;
    const lelph_gpu_desc& d = h->d;
    if (first + count > (long long)nsym * d.nkpts_BZ)
        return fail(h, LELPH_GPU_ERR_INVALID, "Dmat range beyond nsym * nk_BZ");
    if (count == 0) return LELPH_GPU_OK;
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t dbytes = sizeof(double2) * (size_t)count * d.nspin * d.nbnds * d.nbnds;
    int rc = ensure(h, h->d_dmats, dbytes);
    if (rc) return rc;
    h->dm_count = 0;
    rc = dmats_run(h, nsym, Rmat, tau, time_rev, first, count, nullptr, (double2*)h->d_dmats.p);
    if (rc) return rc;
    // the resident block and the symmetries it belongs to
    h->dm_first = first;
    h->dm_count = count;
    h->dm_nsym = nsym;
    h->dm_R.assign(Rmat, Rmat + 9 * (size_t)nsym);
    h->dm_tau.assign(tau, tau + 3 * (size_t)nsym);
    h->dm_trev.assign(time_rev, time_rev + nsym);
    if (Dmats) CUDA_TRY(h, cudaMemcpyAsync(Dmats, h->d_dmats.p, dbytes, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    return LELPH_GPU_OK;
}

// ============================================ q-star expansion of one irreducible q

extern "C" int lelph_gpu_compute_elphq_star(lelph_gpu* h, const double qpt_crys[3], const double* eigVec,
                                            const double* dVscfq, int non_loc, int kminusq, int nph_sym,
                                            const double* ph_Rmat, const double* ph_tau, const int* ph_time_rev,
                                            int nstar, const int* star_sym, int out_type, void* out)
{
    if (!h || !qpt_crys || !eigVec || !out || nstar < 1 || !star_sym || nph_sym < 1 || !ph_Rmat || !ph_tau ||
        !ph_time_rev)
        return LELPH_GPU_ERR_INVALID;
    if (out_type != LELPH_GPU_OUT_C128 && out_type != LELPH_GPU_OUT_C64) return fail(h, LELPH_GPU_ERR_INVALID, "out_type");
    for (int i = 0; i < nstar; ++i)
        if (star_sym[i] < 0 || star_sym[i] >= nph_sym) return fail(h, LELPH_GPU_ERR_INVALID, "star symmetry index");
    // the first member is the irreducible q itself (compute_elph_matq.c:45-49)
    if (star_sym[0] != 0) return fail(h, LELPH_GPU_ERR_INVALID, "Qpoint in iBZ cannot be traced in phonon qmap");
    const lelph_gpu_desc& d = h->d;
    CUDA_TRY(h, cudaSetDevice(h->device));
    const int nk = d.nkpts_BZ, nb = d.nbnds;
    const int fp64 = h->mixed ? 0 : 1;
    if (nstar > 1 && lelph_qstar_smem_bytes(nb, fp64) > 220 * 1024)
        return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "too many bands for the q-star rotation");
    int rc = lelph_gpu_set_q(h, 0, qpt_crys, eigVec, dVscfq);
    if (rc) return rc;
    const size_t gsz = (size_t)d.nmodes * d.nspin * nb * nb;
    const size_t esz = out_type == LELPH_GPU_OUT_C64 ? sizeof(float2) : sizeof(double2);
    const size_t total = esz * gsz * (size_t)nk * nstar;
    rc = ensure(h, h->d_gstar, total);
    if (rc) return rc;
    // row 0: the irreducible q at every k
    {
        std::vector<int> qs(nk, 0), ks(nk);
        for (int i = 0; i < nk; ++i) ks[i] = i;
        rc = run_impl(h, nk, qs.data(), ks.data(), non_loc, kminusq, out_type, h->d_gstar.p, true);
        if (rc) return rc;
    }
    if (nstar > 1)
    {
        // Dmats of the star's symmetries: the resident block when it was made
        // for these symmetries and holds their rows, else computed here
        std::vector<int> uniq(star_sym + 1, star_sym + nstar);
        std::sort(uniq.begin(), uniq.end());
        uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
        bool resident = h->dm_count > 0 && h->dm_nsym == nph_sym &&
                        std::equal(h->dm_R.begin(), h->dm_R.end(), ph_Rmat) &&
                        std::equal(h->dm_tau.begin(), h->dm_tau.end(), ph_tau) &&
                        std::equal(h->dm_trev.begin(), h->dm_trev.end(), ph_time_rev);
        for (int S : uniq)
            resident = resident && (long long)S * nk >= h->dm_first &&
                       (long long)(S + 1) * nk <= h->dm_first + h->dm_count;
        std::vector<long long> rowbase(nph_sym, -1);
        const double2* Dbase = nullptr;
        if (resident)
        {
            for (int S : uniq) rowbase[S] = (long long)S * nk - h->dm_first;
            Dbase = (const double2*)h->d_dmats.p;
        }
        else
        {
            std::vector<long long> ids;
            ids.reserve(uniq.size() * nk);
            for (size_t j = 0; j < uniq.size(); ++j)
            {
                rowbase[uniq[j]] = (long long)j * nk;
                for (int k = 0; k < nk; ++k) ids.push_back((long long)uniq[j] * nk + k);
            }
            rc = ensure(h, h->d_dmstar, sizeof(double2) * ids.size() * d.nspin * nb * nb);
            if (rc) return rc;
            rc = dmats_run(h, nph_sym, ph_Rmat, ph_tau, ph_time_rev, 0, (long long)ids.size(), ids.data(),
                           (double2*)h->d_dmstar.p);
            if (rc) return rc;
            Dbase = (const double2*)h->d_dmstar.p;
        }
        // (member, k) items: k+q as the stage finds it (compute_elph_matq.c:65-128),
        // S k in the full-BZ list (:186-205)
        if (h->khash.empty())
            for (int i = 0; i < nk; ++i) h->khash.emplace(k_hash_key(&h->kbz_crys[3 * i]), i);
        std::vector<int> kq_of(nk);
        for (int i = 0; i < nk; ++i)
        {
            double kq[3];
            for (int x = 0; x < 3; ++x) kq[x] = h->kbz_crys[3 * i + x] + (kminusq ? -qpt_crys[x] : qpt_crys[x]);
            kq_of[i] = find_k_fast(h, kq);
            if (kq_of[i] < 0) return fail(h, LELPH_GPU_ERR_GEOMETRY, "K+Q point cannot be found in kgrid");
        }
        std::vector<QStarItem> items((size_t)(nstar - 1) * nk);
        for (int m = 1; m < nstar; ++m)
        {
            const int S = star_sym[m];
            const double* R = ph_Rmat + 9 * S;
            for (int i = 0; i < nk; ++i)
            {
                int idx_k = i, idx_kq = kq_of[i];
                if (kminusq) std::swap(idx_k, idx_kq);
                double kc[3], Sk[3], Skc[3];
                for (int x = 0; x < 3; ++x)
                    kc[x] = (h->blat[3 * x] * h->kbz_crys[3 * i] + h->blat[3 * x + 1] * h->kbz_crys[3 * i + 1] +
                             h->blat[3 * x + 2] * h->kbz_crys[3 * i + 2]) /
                            (2 * PI_T);
                mat_vec3(R, kc, false, Sk);
                mat_vec3(d.alat_vec, Sk, true, Skc);
                const int isk = find_k_fast(h, Skc);
                if (isk < 0)
                    return fail(h, LELPH_GPU_ERR_GEOMETRY,
                                "Unable to to find S*k index This is due to incommenserate k and q grids.");
                QStarItem& it = items[(size_t)(m - 1) * nk + i];
                it.src = i;
                it.dst = m * nk + isk;
                it.dl = rowbase[S] + idx_kq;
                it.dr = rowbase[S] + idx_k;
                it.trev = ph_time_rev[S] != 0;
                it.pad = 0;
            }
        }
        rc = upload(h, h->d_qsitems, items.data(), sizeof(QStarItem) * items.size());
        if (rc) return rc;
        tstart(h);
        if (lelph_launch_qstar((const QStarItem*)h->d_qsitems.p, (long long)items.size(), nb, d.nspin, d.nmodes, Dbase,
                               fp64, out_type == LELPH_GPU_OUT_C64, h->d_gstar.p, h->d_gstar.p, h->st))
            return fail(h, LELPH_GPU_ERR_UNSUPPORTED, "q-star launch configuration");
        h->stats.kernel_launches += 1;
        CUDA_TRY(h, cudaGetLastError());
        h->stats.qstar_ms += tstop(h);
    }
    CUDA_TRY(h, cudaMemcpyAsync(out, h->d_gstar.p, total, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_debug_gvec_map(lelph_gpu* h, int kbz, const int ulm[3], int* out)
{
    if (!h || !out || kbz < 0 || kbz >= h->d.nkpts_BZ) return LELPH_GPU_ERR_INVALID;
    CUDA_TRY(h, cudaSetDevice(h->device));
    int npw = h->npw[h->ksym[kbz].ik];
    int rc = ensure(h, h->d_tmp, sizeof(int) * (3 * (size_t)npw + 4));
    if (rc) return rc;
    int u[3] = {ulm ? ulm[0] : 0, ulm ? ulm[1] : 0, ulm ? ulm[2] : 0};
    int* dt = (int*)h->d_tmp.p;
    CUDA_TRY(h, cudaMemcpyAsync(dt, u, sizeof(u), cudaMemcpyHostToDevice, h->st));
    lelph_launch_gmap((const KPointSym*)h->d_ksym.p, kbz, (const int*)h->d_miller.p, (const long long*)h->d_pwoff.p,
                      (const int*)h->d_npw.p, h->g, dt, dt + 4, h->st);
    h->stats.kernel_launches += 1;
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaMemcpyAsync(out, dt + 4, sizeof(int) * 3 * npw, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    return LELPH_GPU_OK;
}

extern "C" int lelph_gpu_debug_partials_extent(int nmodes, int nbnds, int nspin, int nchunks, int npairs,
                                               unsigned long long out[3])
{
    if (!out || nmodes < 1 || nbnds < 1 || nbnds > 64 || nspin < 1 || nchunks < 1 || npairs < 1)
        return LELPH_GPU_ERR_INVALID;
    GeomDev g{};
    g.nmodes = nmodes;
    g.nbnds = nbnds;
    g.nbp = (nbnds + 7) / 8 * 8;
    g.nspin = nspin;
    g.mt_modes = lelph_tc_tile_modes(nmodes, nbnds);
    const long long zlast = (long long)npairs * nspin - 1;
    // the sandwich writes 128 rows x 2 nbp columns of every (pair, spin, mode tile, K chunk)
    const size_t wr = lelph_tc_partial_offset(g, nchunks, zlast, lelph_tc_mode_tiles(g) - 1, nchunks - 1, 127) +
                      2 * (size_t)g.nbp;
    // the finish reads row (nu - mt mt_modes) nb + m of tile mt = nu / mt_modes, columns n and nbp + n
    size_t rd = 0;
    for (int nu = 0; nu < nmodes; ++nu)
    {
        const int mt = nu / g.mt_modes, rr = (nu - mt * g.mt_modes) * nbnds + (nbnds - 1);
        rd = std::max(rd, lelph_tc_partial_offset(g, nchunks, zlast, mt, nchunks - 1, rr) + g.nbp + nbnds);
    }
    out[0] = lelph_tc_partials_per_pair(g, nchunks) * (size_t)npairs;
    out[1] = wr;
    out[2] = rd;
    return LELPH_GPU_OK;
}

// ============================================================== tuning

namespace
{
// device time per pair of one candidate context: a warm-up call (preparation,
// dV windows, kernels loaded), then two timed calls; negative on failure
double tune_candidate(const lelph_gpu_desc& dc, const double* q, const double* eig, const double* dv, int n)
{
    lelph_gpu* h = nullptr;
    if (lelph_gpu_create(&dc, &h) != LELPH_GPU_OK)
    {
        lelph_gpu_destroy(h);
        return -1.0;
    }
    double ms = -1.0;
    void* gout = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<int> qs(n, 0), ks(n);
    for (int i = 0; i < n; ++i) ks[i] = i;
    const size_t bytes = sizeof(float2) * (size_t)n * dc.nmodes * dc.nspin * dc.nbnds * dc.nbnds;
    if (!h->gspace)
    {
        // the real-space route keeps psi(r) of every full-BZ k resident: skip it where
        // that would take more than half of the device memory (as the automatic route does)
        const double per_kpt = h->mixed ? 24.0 * h->g.nbp * dc.nspin * dc.nspinor
                                        : 16.0 * dc.nspin * dc.nbnds * dc.nspinor;
        const double resident = per_kpt * (double)h->g.Nx * h->g.Ny * h->g.Nz * dc.nkpts_BZ;
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess || resident > 0.5 * (double)tot) goto done;
    }
    if (lelph_gpu_set_q(h, 0, q, eig, dv) != LELPH_GPU_OK) goto done;
    if (cudaMalloc(&gout, bytes) != cudaSuccess)
    {
        cudaGetLastError();
        goto done;
    }
    if (run_impl(h, n, qs.data(), ks.data(), 1, 0, LELPH_GPU_OUT_C64, gout, true) != LELPH_GPU_OK) goto done;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) goto done;
    cudaEventRecord(e0, h->st);
    for (int r = 0; r < 2; ++r)
        if (run_impl(h, n, qs.data(), ks.data(), 1, 0, LELPH_GPU_OUT_C64, gout, true) != LELPH_GPU_OK) goto done;
    cudaEventRecord(e1, h->st);
    if (cudaEventSynchronize(e1) == cudaSuccess)
    {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, e0, e1) == cudaSuccess) ms = (double)t / (2.0 * n);
    }
done:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (gout) cudaFree(gout);
    cudaGetLastError();
    lelph_gpu_destroy(h);
    return ms;
}

std::string tune_key(const lelph_gpu_desc& d)
{
    long long npw = 0;
    for (int i = 0; i < d.nkpts_iBZ; ++i) npw += d.npw[i];
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, d.device);
    char buf[512];
    snprintf(buf, sizeof buf, "prec=%d spin=%d spinor=%d mag=%d bands=%d modes=%d fft=%dx%dx%d kBZ=%d npw=%lld dev=%s",
             d.precision, d.nspin, d.nspinor, d.nmag, d.nbnds, d.nmodes, d.fft_dims[0], d.fft_dims[1],
             d.fft_dims[2], d.nkpts_BZ, d.nkpts_iBZ ? npw / d.nkpts_iBZ : 0, prop.name);
    for (char* c = buf; *c; ++c)
        if (*c == '|' || *c == '\n') *c = '_';
    return buf;
}
}  // namespace

extern "C" int lelph_gpu_tune(const lelph_gpu_desc* desc, const double qpt_crys[3], const double* eigVec,
                              const double* dVscf, int npairs, const char* cache_path, lelph_gpu_tuning* out)
{
    if (!desc || !qpt_crys || !eigVec || !dVscf || !out || npairs < 1) return LELPH_GPU_ERR_INVALID;
    lelph_gpu_desc d = *desc;
    if (cudaSetDevice(d.device) != cudaSuccess) return LELPH_GPU_ERR_CUDA;
    npairs = std::min(npairs, d.nkpts_BZ);
    memset(out, 0, sizeof(*out));
    const std::string key = tune_key(d);
    if (cache_path)
        if (FILE* f = fopen(cache_path, "r"))
        {
            char line[1024];
            bool hit = false;
            while (!hit && fgets(line, sizeof line, f))
            {
                char* bar = strchr(line, '|');
                if (!bar || std::string(line, bar - line) != key) continue;
                hit = sscanf(bar + 1, "%d %d %d %lf %lf %lf %lf", &out->route, &out->tile_points, &out->gs_gemm,
                             &out->ms_per_pair[0], &out->ms_per_pair[1], &out->ms_per_pair[2],
                             &out->ms_per_pair[3]) == 7;
            }
            fclose(f);
            if (hit)
            {
                out->cached = 1;
                return LELPH_GPU_OK;
            }
        }
    struct Cand
    {
        int route, tile, gemm;
    };
    const bool mixed = d.precision != LELPH_GPU_FP64;
    const Cand cands[4] = {{LELPH_GPU_ROUTE_REAL, 64, 0},
                           {LELPH_GPU_ROUTE_REAL, 32, 0},
                           {LELPH_GPU_ROUTE_GSPACE, 0, LELPH_GPU_GS_GEMM_TENSOR},
                           {LELPH_GPU_ROUTE_GSPACE, 0, LELPH_GPU_GS_GEMM_SIMT}};
    int best = -1;
    for (int c = 0; c < 4; ++c)
    {
        out->ms_per_pair[c] = -1.0;
        // the plain form has one real-space kernel and one G-space GEMM
        if (!mixed && (c == 1 || c == 2)) continue;
        d.route = cands[c].route;
        d.tile_points = mixed ? cands[c].tile : 0;
        d.gs_gemm = mixed ? cands[c].gemm : 0;
        out->ms_per_pair[c] = tune_candidate(d, qpt_crys, eigVec, dVscf, npairs);
        if (out->ms_per_pair[c] > 0 && (best < 0 || out->ms_per_pair[c] < out->ms_per_pair[best])) best = c;
    }
    if (best < 0) return LELPH_GPU_ERR_UNSUPPORTED;
    out->route = cands[best].route;
    out->tile_points = mixed ? cands[best].tile : 0;
    out->gs_gemm = mixed ? cands[best].gemm : 0;
    if (cache_path)
        if (FILE* f = fopen(cache_path, "a"))
        {
            fprintf(f, "%s|%d %d %d %.6g %.6g %.6g %.6g\n", key.c_str(), out->route, out->tile_points, out->gs_gemm,
                    out->ms_per_pair[0], out->ms_per_pair[1], out->ms_per_pair[2], out->ms_per_pair[3]);
            fclose(f);
        }
    return LELPH_GPU_OK;
}

// ============================================ allocation-free variant of run

// Callers that cannot allocate device memory once set-up is over -- a host
// code whose device memory is all owned by another pool or framework, or a
// service loop that must not meet an allocation failure (or the latency of
// cudaMalloc) in the middle of a run -- can compute matrix elements through
// lelph_gpu_run_device_noalloc.  Its only working storage is this file-scope
// array: the (k, k+q) pair table in the first LELPH_NOALLOC_PAIR_BYTES and the
// local-sandwich partial sums (mixed form) or FP64 local blocks (plain form)
// after it.  Every GPU that loads the library holds the array until exit.
#define LELPH_NOALLOC_BYTES (64ull << 20)
#define LELPH_NOALLOC_PAIR_BYTES (256ull << 10)
static __device__ __align__(256) unsigned char lelph_noalloc_scratch[LELPH_NOALLOC_BYTES];

namespace
{
std::mutex g_noalloc_mu;
struct NoallocAddr
{
    unsigned long long ctx_id;  // unique id of the context the address belongs to (0: none yet)
    void* p;
};
NoallocAddr g_noalloc_addr[256] = {};

// Unique id of the calling thread's current context (cuCtxGetId, reached
// through the runtime's driver entry points); 0 if the driver cannot say.
unsigned long long current_ctx_id()
{
    using PFN_cur = CUresult (*)(CUcontext*);
    using PFN_id = CUresult (*)(CUcontext, unsigned long long*);
    static PFN_cur cur = nullptr;
    static PFN_id cid = nullptr;
    static bool looked = false;
    if (!looked)
    {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            cur = reinterpret_cast<PFN_cur>(p);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            cid = reinterpret_cast<PFN_id>(p);
        looked = true;
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!cur || !cid || cur(&c) != CUDA_SUCCESS || !c || cid(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array on h->device (current when this runs),
// looked up once per device and context: the first call on a device does this
// set-up, and so does the first call after the device's context was destroyed
// and re-created (cudaDeviceReset), when the module and its array are loaded
// anew at another address.
int noalloc_scratch(lelph_gpu* h, unsigned char** out)
{
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (h->device < 0 || h->device >= 256) return fail(h, LELPH_GPU_ERR_INVALID, "device ordinal");
    NoallocAddr& a = g_noalloc_addr[h->device];
    const unsigned long long id = current_ctx_id();
    if (!a.p || id == 0 || id != a.ctx_id)
    {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, lelph_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(h, LELPH_GPU_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        a.p = p;
        a.ctx_id = id;
    }
    *out = static_cast<unsigned char*>(a.p);
    return LELPH_GPU_OK;
}

// (k, k+q) pair of one item: k+q search and umklapp vector, as run does it
int noalloc_pair(lelph_gpu* h, int qs, int k, int kminusq, PairInfo& P)
{
    const lelph_gpu_desc& d = h->d;
    if (qs < 0 || qs >= (int)h->qslots.size() || !h->qslots[qs].set)
        return fail(h, LELPH_GPU_ERR_STATE, "q slot not loaded");
    if (k < 0 || k >= d.nkpts_BZ) return fail(h, LELPH_GPU_ERR_INVALID, "k index out of range");
    const double* q = h->qslots[qs].q;
    double kq[3];
    for (int x = 0; x < 3; ++x) kq[x] = h->kbz_crys[3 * k + x] + (kminusq ? -q[x] : q[x]);
    int ikq = find_k(h, kq);
    if (ikq < 0) return fail(h, LELPH_GPU_ERR_GEOMETRY, "K+Q point cannot be found in kgrid");
    int idx_k = k, idx_kq = ikq;
    if (kminusq) std::swap(idx_k, idx_kq);
    P.kbz_k = idx_k;
    P.kbz_kq = idx_kq;
    P.qslot = qs;
    if (umklapp(h, idx_k, idx_kq, q, P.ulm)) return fail(h, LELPH_GPU_ERR_GEOMETRY, "non-integral umklapp vector");
    P.dvslot = window_of(h, qs, P.ulm);
    if (P.dvslot < 0) return fail(h, LELPH_GPU_ERR_GEOMETRY, "umklapp vector outside the q slot's set");
    return LELPH_GPU_OK;
}
}  // namespace

extern "C" int lelph_gpu_run_device_noalloc(lelph_gpu* h, int n, const int* qslot, const int* kbz, int non_loc,
                                            int kminusq, int out_type, void* g_out_dev)
{
    if (!h || n < 0 || (n > 0 && (!qslot || !kbz || !g_out_dev))) return LELPH_GPU_ERR_INVALID;
    if (out_type != LELPH_GPU_OUT_C128 && out_type != LELPH_GPU_OUT_C64) return fail(h, LELPH_GPU_ERR_INVALID, "out_type");
    if (n == 0) return LELPH_GPU_OK;
    CUDA_TRY(h, cudaSetDevice(h->device));
    if (!h->prepared || !h->windows_ok)
        return fail(h, LELPH_GPU_ERR_STATE, "lelph_gpu_prepare must run (after the last set_q) before the allocation-free call");
    if (h->gspace)
        return fail(h, LELPH_GPU_ERR_UNSUPPORTED,
                    "the G-space route builds psi(r) per k in device buffers; it has no allocation-free form");
    unsigned char* scratch = nullptr;
    int rc = noalloc_scratch(h, &scratch);
    if (rc) return rc;
    const lelph_gpu_desc& d = h->d;
    const GeomDev& g = h->g;
    const int nrows = d.nmodes * d.nbnds;
    size_t per_pair;
    if (!h->mixed) per_pair = sizeof(double2) * (size_t)d.nspin * nrows * d.nbnds;
    else per_pair = sizeof(float) * lelph_tc_partials_per_pair(g, h->nchunks);
    const size_t room = LELPH_NOALLOC_BYTES - LELPH_NOALLOC_PAIR_BYTES;
    if (per_pair > room)
        return fail(h, LELPH_GPU_ERR_UNSUPPORTED,
                    "one (k, q) pair needs " + std::to_string(per_pair) + " bytes of scratch; the static scratch of "
                    "lelph_gpu_run_device_noalloc holds " + std::to_string(room));
    const int max_pairs = (int)(LELPH_NOALLOC_PAIR_BYTES / sizeof(PairInfo));
    const int batch = (int)std::min<size_t>({(size_t)n, room / per_pair, (size_t)max_pairs});
    if (h->mixed && (h->tmapV_base != h->d_win32.p || h->tmapV_rows != h->nwin))
    {
        const long long M = (long long)g.Nx * g.Ny * g.Nz;
        rc = make_tmap3(h, &h->tmapV, h->d_win32.p, true, 64, (unsigned long long)d.nmodes * d.nmag,
                        (unsigned long long)h->nwin * (M / 32), (unsigned)(g.mt_modes * d.nmag),
                        (unsigned)(g.kpts / 32), false);
        if (rc) return rc;
        h->tmapV_base = h->d_win32.p;
        h->tmapV_rows = h->nwin;
    }
    PairInfo* dpairs = reinterpret_cast<PairInfo*>(scratch);
    unsigned char* work = scratch + LELPH_NOALLOC_PAIR_BYTES;
    const size_t gsz = (size_t)d.nmodes * d.nspin * d.nbnds * d.nbnds;
    const size_t esz = out_type == LELPH_GPU_OUT_C64 ? sizeof(float2) : sizeof(double2);
    NonlocalDesc nl = nl_desc(h);
    CUDA_TRY(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned), h->st));
    PairInfo stage[256];  // host staging on the stack: no heap allocation either
    for (int p0 = 0; p0 < n; p0 += batch)
    {
        const int nb = std::min(batch, n - p0);
        for (int c0 = 0; c0 < nb; c0 += 256)
        {
            const int nc = std::min(256, nb - c0);
            for (int i = 0; i < nc; ++i)
            {
                rc = noalloc_pair(h, qslot[p0 + c0 + i], kbz[p0 + c0 + i], kminusq, stage[i]);
                if (rc) return rc;
            }
            // pageable source: the call returns once the staging buffer has been consumed
            CUDA_TRY(h, cudaMemcpyAsync(dpairs + c0, stage, sizeof(PairInfo) * nc, cudaMemcpyHostToDevice, h->st));
        }
        if (!h->mixed)
            lelph_launch_local_fp64(dpairs, nb, (const double2*)h->d_psi64.p, (const double2*)h->d_win64.p, g,
                                    (double2*)work, (unsigned*)h->d_status.p, h->st);
        else
            lelph_launch_local_tc(dpairs, nb, &h->tmapB, &h->tmapP, &h->tmapV, g, h->ab_bf16, h->chunk_pts,
                                  h->nchunks, (float*)work, (unsigned*)h->d_status.p, h->st, h->wait_ns);
        lelph_launch_finish(dpairs, nb, h->mixed ? 0 : 1, (const double2*)work, (const float*)work, h->nchunks,
                            (const float*)h->d_winscale.p, (const float*)h->d_band_scale.p,
                            (const double2*)h->d_proj.p, (const double2*)h->d_eig.p, non_loc, nl, g,
                            out_type == LELPH_GPU_OUT_C64, (char*)g_out_dev + esz * gsz * p0, h->st);
        h->stats.kernel_launches += 2;
        h->stats.local_launches += 1;
        CUDA_TRY(h, cudaGetLastError());
    }
    rc = check_status(h);
    if (rc) return rc;
    h->stats.pairs_done += n;
    return LELPH_GPU_OK;
}
