"""Python host binding of the C ABI in include/lelph_gpu.h (ctypes).

Mirrors the reference's per-q stage: ``compute_elphq`` corresponds to
``compute_and_write_elphq`` (src/elph/compute_elph_matq.c:20-234) with the
same argument meaning (q in crystal units, eigVec (nmodes, 3*natom), dVscfq
(nmodes, nmag, Nx, Ny, Nz), ``non_loc``, ``kminusq``) and returns the
elph_mat[q] slice (nk_BZ, nmodes, nspin, nb_k, nb_k+q) instead of writing it
through netCDF.  There is no CPU fallback: without the compiled library every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "liblelph_gpu.so")

FP64, MIXED_F16, MIXED_BF16 = 0, 1, 2
OUT_C128, OUT_C64 = 0, 1
PRECISIONS = {"fp64": FP64, "mixed": MIXED_F16, "mixed_f16": MIXED_F16, "mixed_bf16": MIXED_BF16}
ROUTE_AUTO, ROUTE_REAL, ROUTE_GSPACE = 0, 1, 2  # LELPH_GPU_ROUTE_*
ROUTES = {"auto": ROUTE_AUTO, "real": ROUTE_REAL, "gspace": ROUTE_GSPACE}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Desc(C.Structure):
    _fields_ = [
        ("natom", C.c_int), ("nsym", C.c_int), ("timerev", C.c_int), ("nspin", C.c_int), ("nspinor", C.c_int),
        ("nbnds", C.c_int), ("nmag", C.c_int), ("nmodes", C.c_int),
        ("nkpts_iBZ", C.c_int), ("nkpts_BZ", C.c_int),
        ("fft_dims", C.c_int * 3),
        ("alat_vec", _dp), ("blat_vec", _dp), ("atomic_pos", _dp), ("atom_type", _ip),
        ("kpt_iredBZ", _dp), ("kpt_fullBZ_crys", _dp), ("kmap", _ip),
        ("sym_Rmat", _dp), ("sym_tau", _dp), ("sym_time_rev", _ip),
        ("is_soc_present", C.c_int),
        ("npw", _ip), ("gvec", C.POINTER(_dp)), ("wfc", C.POINTER(_dp)), ("Fk", C.POINTER(_dp)),
        ("ntype", C.c_int), ("nltimesj", C.c_int), ("lmax", C.c_int),
        ("PP_table", _dp), ("Fsign", _dp), ("fCoeff", C.POINTER(_dp)),
        ("precision", C.c_int), ("device", C.c_int), ("route", C.c_int),
        ("tile_points", C.c_int), ("gs_gemm", C.c_int),
    ]


class Tuning(C.Structure):
    _fields_ = [("route", C.c_int), ("tile_points", C.c_int), ("gs_gemm", C.c_int), ("cached", C.c_int),
                ("ms_per_pair", C.c_double * 4)]


GS_GEMMS = {"auto": 0, "tensor": 1, "simt": 2}


class Stats(C.Structure):
    _fields_ = [
        ("kernel_launches", C.c_longlong), ("local_launches", C.c_longlong), ("local_ms", C.c_double),
        ("prepare_ms", C.c_double), ("finish_ms", C.c_double), ("pairs_done", C.c_longlong),
        ("device_bytes", C.c_size_t), ("product_grid", C.c_int * 3), ("chunk_points", C.c_int),
        ("dmats_ms", C.c_double), ("dmats_host_ms", C.c_double), ("dmats_done", C.c_longlong),
        ("qstar_ms", C.c_double), ("dvscf_ms", C.c_double), ("route", C.c_int),
        ("gs_plane_ms", C.c_double), ("gs_xpass_ms", C.c_double), ("gs_gemm_ms", C.c_double),
        ("prep_scatter_ms", C.c_double), ("prep_fft_ms", C.c_double), ("prep_xsplit_ms", C.c_double),
        ("prep_proj_ms", C.c_double), ("windows_ms", C.c_double), ("box_columns", C.c_longlong),
        ("local_live_ms", C.c_double), ("local_live_launches", C.c_longlong),
    ]


EXPORTS = [
    "lelph_gpu_create", "lelph_gpu_set_wavefunctions", "lelph_gpu_prepare", "lelph_gpu_set_q", "lelph_gpu_run",
    "lelph_gpu_run_device", "lelph_gpu_compute_elphq", "lelph_gpu_elph_q_rotate", "lelph_gpu_debug_gvec_map",
    "lelph_gpu_set_profiling", "lelph_gpu_stats_get", "lelph_gpu_stream", "lelph_gpu_strerror",
    "lelph_gpu_last_error", "lelph_gpu_destroy", "lelph_gpu_run_device_noalloc",
    "lelph_gpu_set_local_pseudo", "lelph_gpu_dvlocq", "lelph_gpu_set_q_induced", "lelph_gpu_rotate_dvscf",
    "lelph_gpu_dmats", "lelph_gpu_compute_elphq_star", "lelph_gpu_set_q_dvscf_qe",
    "lelph_gpu_debug_partials_extent", "lelph_gpu_set_wait_limit", "lelph_gpu_tune",
]

_lib = None


def load_library(path: str = LIB_PATH):
    """Load liblelph_gpu.so and declare the C signatures.  Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library {path} is missing: run __graft_entry__.build() first")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.lelph_gpu_create.argtypes = [C.POINTER(Desc), C.POINTER(vp)]
    L.lelph_gpu_set_wavefunctions.argtypes = [vp, C.POINTER(_dp)]
    L.lelph_gpu_prepare.argtypes = [vp]
    L.lelph_gpu_set_q.argtypes = [vp, C.c_int, _dp, _dp, _dp]
    L.lelph_gpu_set_local_pseudo.argtypes = [vp, _ip, C.POINTER(_dp), C.POINTER(_dp), C.POINTER(_dp), _dp,
                                             C.c_int, C.c_double]
    L.lelph_gpu_dvlocq.argtypes = [vp, _dp, _dp, _dp]
    L.lelph_gpu_set_q_induced.argtypes = [vp, C.c_int, _dp, _dp, _dp]
    L.lelph_gpu_rotate_dvscf.argtypes = [vp, _dp, _dp, _dp, C.c_int, C.c_int, _dp, _dp]
    L.lelph_gpu_dmats.argtypes = [vp, C.c_int, _dp, _dp, _ip, C.c_longlong, C.c_longlong, _dp]
    L.lelph_gpu_debug_partials_extent.argtypes = [C.c_int] * 5 + [C.POINTER(C.c_ulonglong)]
    L.lelph_gpu_set_wait_limit.argtypes = [vp, C.c_ulonglong]
    L.lelph_gpu_tune.argtypes = [C.POINTER(Desc), _dp, _dp, _dp, C.c_int, C.c_char_p, C.POINTER(Tuning)]
    L.lelph_gpu_set_q_dvscf_qe.argtypes = [vp, C.c_int, _dp, _dp, _dp, _dp, C.c_int, _dp]
    L.lelph_gpu_compute_elphq_star.argtypes = [vp, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, C.c_int,
                                               _ip, C.c_int, vp]
    L.lelph_gpu_run.argtypes = [vp, C.c_int, _ip, _ip, C.c_int, C.c_int, C.c_int, vp]
    L.lelph_gpu_run_device.argtypes = [vp, C.c_int, _ip, _ip, C.c_int, C.c_int, C.c_int, vp]
    L.lelph_gpu_run_device_noalloc.argtypes = [vp, C.c_int, _ip, _ip, C.c_int, C.c_int, C.c_int, vp]
    L.lelph_gpu_compute_elphq.argtypes = [vp, _dp, _dp, _dp, C.c_int, C.c_int, _dp]
    L.lelph_gpu_elph_q_rotate.argtypes = [vp, _dp, _dp, _dp, C.c_int, _dp]
    L.lelph_gpu_debug_gvec_map.argtypes = [vp, C.c_int, _ip, _ip]
    L.lelph_gpu_set_profiling.argtypes = [vp, C.c_int]
    L.lelph_gpu_stats_get.argtypes = [vp, C.POINTER(Stats)]
    L.lelph_gpu_stream.argtypes = [vp]
    L.lelph_gpu_stream.restype = vp
    L.lelph_gpu_strerror.argtypes = [C.c_int]
    L.lelph_gpu_strerror.restype = C.c_char_p
    L.lelph_gpu_last_error.argtypes = [vp]
    L.lelph_gpu_last_error.restype = C.c_char_p
    L.lelph_gpu_destroy.argtypes = [vp]
    L.lelph_gpu_destroy.restype = None
    for name in EXPORTS:
        if name not in ("lelph_gpu_stream", "lelph_gpu_strerror", "lelph_gpu_last_error", "lelph_gpu_destroy"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


class LelphError(RuntimeError):
    def __init__(self, status, detail):
        super().__init__(f"lelph_gpu status {status}: {detail}")
        self.status = status


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def describe(s, precision="fp64", device=0, route="auto", tile_points=0, gs_gemm="auto", keep=None):
    """lelph_gpu_desc of a system (the fields of the reference's Lattice, WFC[]
    and Pseudo under their own names); every array it points to is appended
    to `keep`, which must outlive the descriptor's use."""
    keep = [] if keep is None else keep
    d = Desc()

    def arr(x, dt):
        a = np.ascontiguousarray(x, dtype=dt)
        keep.append(a)
        return a

    d.natom, d.nsym, d.timerev = s.natom, len(s.sym_R), int(s.timerev)
    d.nspin, d.nspinor, d.nbnds, d.nmag, d.nmodes = s.nspin, s.nspinor, s.nbnds, s.nmag, s.nmodes
    d.nkpts_iBZ, d.nkpts_BZ = s.nk_ibz, s.nk_bz
    d.fft_dims[:] = list(s.fft_dims)
    d.alat_vec = _ptr(arr(s.alat, np.float64))
    d.blat_vec = _ptr(arr(s.blat, np.float64))
    d.atomic_pos = _ptr(arr(s.atom_pos, np.float64))
    d.atom_type = _ptr(arr(s.atom_type, np.int32), _ip)
    d.kpt_iredBZ = _ptr(arr(s.kibz, np.float64))
    d.kpt_fullBZ_crys = _ptr(arr(s.kbz_crys, np.float64))
    d.kmap = _ptr(arr(s.kmap, np.int32), _ip)
    d.sym_Rmat = _ptr(arr(s.sym_R, np.float64))
    d.sym_tau = _ptr(arr(s.sym_tau, np.float64))
    d.sym_time_rev = _ptr(arr(s.sym_trev, np.int32), _ip)
    d.is_soc_present = int(s.is_soc_present)
    d.npw = _ptr(arr([len(g) for g in s.gvec], np.int32), _ip)
    gv = (_dp * s.nk_ibz)(*[_ptr(arr(g, np.float64)) for g in s.gvec])
    fk = (_dp * s.nk_ibz)(*[_ptr(arr(f, np.float64)) for f in s.Fk])
    keep += [gv, fk]
    d.gvec, d.Fk = gv, fk
    wf = (_dp * s.nk_ibz)(*[_ptr(arr(w, np.complex128)) for w in s.wfc])
    keep.append(wf)
    d.wfc = wf
    d.ntype, d.nltimesj, d.lmax = s.ntype, s.nltimesj, s.lmax
    d.PP_table = _ptr(arr(s.PP_table, np.float64))
    d.Fsign = _ptr(arr(s.Fsign, np.float64))
    if s.fCoeff is not None:
        fc = (_dp * len(s.fCoeff))(*[(_ptr(arr(f, np.complex128)) if f is not None else _dp()) for f in s.fCoeff])
        keep.append(fc)
        d.fCoeff = fc
    else:
        d.fCoeff = C.POINTER(_dp)()
    d.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    d.device = device
    d.route = ROUTES[route] if isinstance(route, str) else int(route)
    d.tile_points = int(tile_points)
    d.gs_gemm = GS_GEMMS[gs_gemm] if isinstance(gs_gemm, str) else int(gs_gemm)
    return d


def tune(s, precision="mixed", iq=0, npairs=4, device=0, cache_path=None):
    """lelph_gpu_tune on the system's q-point iq and its first npairs full-BZ
    k-points: {"route", "tile_points", "gs_gemm", "cached", "ms_per_pair"}
    (route as a name; pass the three to LelphGPU)."""
    L = load_library()
    keep = []
    d = describe(s, precision, device, keep=keep)
    q = np.ascontiguousarray(s.qpts[iq], dtype=np.float64)
    e = np.ascontiguousarray(s.eigVec[iq], dtype=np.complex128)
    v = np.ascontiguousarray(s.dVscf[iq], dtype=np.complex128)
    t = Tuning()
    rc = L.lelph_gpu_tune(C.byref(d), _ptr(q), _ptr(e), _ptr(v), int(npairs),
                          cache_path.encode() if cache_path else None, C.byref(t))
    if rc != 0:
        raise LelphError(rc, L.lelph_gpu_strerror(rc).decode())
    names = {v: k for k, v in ROUTES.items()}
    return {"route": names[t.route], "tile_points": t.tile_points, "gs_gemm": t.gs_gemm, "cached": bool(t.cached),
            "ms_per_pair": {"real-space, 64-point stages": t.ms_per_pair[0],
                            "real-space, 32-point stages": t.ms_per_pair[1],
                            "G-space, tensor-core GEMM": t.ms_per_pair[2],
                            "G-space, SIMT GEMM": t.ms_per_pair[3]}}


class LelphGPU:
    """One device context holding a system (the reference's Lattice, WFC[],
    Pseudo) and any number of q slots."""

    def __init__(self, s, precision="fp64", device=0, route="auto", tile_points=0, gs_gemm="auto"):
        L = load_library()
        self._L = L
        self._keep = []
        d = self.desc = describe(s, precision, device, route, tile_points, gs_gemm, self._keep)
        h = C.c_void_p()
        rc = L.lelph_gpu_create(C.byref(d), C.byref(h))
        if rc != 0:
            raise LelphError(rc, L.lelph_gpu_strerror(rc).decode())
        self.h = h
        self.sys = s
        self.precision = precision

    def _check(self, rc):
        if rc != 0:
            raise LelphError(rc, self._L.lelph_gpu_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self._L.lelph_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- reference-shaped entry points
    def set_wavefunctions(self, wfc_list):
        arrs = [np.ascontiguousarray(w, dtype=np.complex128) for w in wfc_list]
        ptrs = (_dp * len(arrs))(*[_ptr(a) for a in arrs])
        self._check(self._L.lelph_gpu_set_wavefunctions(self.h, ptrs))

    def prepare(self):
        self._check(self._L.lelph_gpu_prepare(self.h))

    def set_q(self, slot, qpt, eigVec, dVscf):
        q = np.ascontiguousarray(qpt, dtype=np.float64)
        e = np.ascontiguousarray(eigVec, dtype=np.complex128)
        v = np.ascontiguousarray(dVscf, dtype=np.complex128)
        self._check(self._L.lelph_gpu_set_q(self.h, slot, _ptr(q), _ptr(e), _ptr(v)))

    def set_local_pseudo(self, qmax_abs=None):
        """Local pseudopotentials of the system's species (loc_r, loc_rab,
        loc_v, loc_zval) -> the device V_loc(|G|) table.  qmax_abs defaults to
        ceil(max |q_i|) + 1 over the system's q-points."""
        s = self.sys
        if qmax_abs is None:
            qmax_abs = float(np.ceil(np.abs(np.asarray(s.qpts)).max()) + 1)
        keep = [[np.ascontiguousarray(a, dtype=np.float64) for a in arrs]
                for arrs in (s.loc_r, s.loc_rab, s.loc_v)]
        self._keep_vloc = keep
        ngrid = np.array([len(r) for r in keep[0]], dtype=np.int32)
        tabs = [(_dp * s.ntype)(*[_ptr(a) for a in arrs]) for arrs in keep]
        z = np.ascontiguousarray(s.loc_zval, dtype=np.float64)
        self._check(self._L.lelph_gpu_set_local_pseudo(self.h, _ptr(ngrid, _ip), tabs[0], tabs[1], tabs[2], _ptr(z),
                                                       ord(s.dimension), qmax_abs))

    def dvlocq(self, qpt, eigVec):
        """dVlocq: (nmodes, Nx, Ny, Nz) complex on the reference box."""
        s = self.sys
        q = np.ascontiguousarray(qpt, dtype=np.float64)
        e = np.ascontiguousarray(eigVec, dtype=np.complex128)
        out = np.empty((s.nmodes, *s.fft_dims), dtype=np.complex128)
        self._check(self._L.lelph_gpu_dvlocq(self.h, _ptr(q), _ptr(e), _ptr(out)))
        return out

    def set_q_induced(self, slot, qpt, eigVec, dVscf_induced=None):
        """Load a q slot from the induced dV (None: the bare kernels); the
        local bare potential is added on the device."""
        q = np.ascontiguousarray(qpt, dtype=np.float64)
        e = np.ascontiguousarray(eigVec, dtype=np.complex128)
        if dVscf_induced is None:
            vp = None
        else:
            v = np.ascontiguousarray(dVscf_induced, dtype=np.complex128)
            vp = _ptr(v)
        self._check(self._L.lelph_gpu_set_q_induced(self.h, slot, _ptr(q), _ptr(e), vp))

    def set_q_dvscf_qe(self, slot, qpt, eigVec, pats, dvscf_qe, induced=False, want_dv=False):
        """Load a q slot from QE's dvscf layout (patterns, nmag, Nz, Ny, Nx)
        through the device ingest; with want_dv, return the mode-basis dV
        (nmodes, nmag, Nx, Ny, Nz)."""
        q = np.ascontiguousarray(qpt, dtype=np.float64)
        e = np.ascontiguousarray(eigVec, dtype=np.complex128)
        p = np.ascontiguousarray(pats, dtype=np.complex128)
        raw = np.ascontiguousarray(dvscf_qe, dtype=np.complex128)
        s = self.sys
        out = np.empty((s.nmodes, s.nmag) + tuple(s.fft_dims), np.complex128) if want_dv else None
        self._check(self._L.lelph_gpu_set_q_dvscf_qe(self.h, slot, _ptr(q), _ptr(e), _ptr(p), _ptr(raw),
                                                     int(induced), _ptr(out) if want_dv else None))
        return out

    def rotate_dvscf(self, qpt, R, tau, time_rev, composite, dv_in):
        """rotate_dvscf on the device: dV of S q, same shape as dv_in
        (nmodes, nmag, Nx, Ny, Nz)."""
        q = np.ascontiguousarray(qpt, dtype=np.float64)
        Rm = np.ascontiguousarray(R, dtype=np.float64)
        t = np.ascontiguousarray(tau, dtype=np.float64)
        v = np.ascontiguousarray(dv_in, dtype=np.complex128)
        out = np.empty_like(v)
        self._check(self._L.lelph_gpu_rotate_dvscf(self.h, _ptr(q), _ptr(Rm), _ptr(t), int(time_rev), int(composite),
                                                   _ptr(v), _ptr(out)))
        return out

    def dmats(self, sym_R, sym_tau, sym_trev, first=0, count=None, host=True):
        """Dmats of compute_and_write_dmats for the (symmetry, full-BZ k) pairs
        first .. first + count - 1 (pair = isym * nk_BZ + ik): complex
        (count, nspin, nb, nb), or None with ``host=False`` (the block then
        only stays on the device)."""
        R = np.ascontiguousarray(sym_R, dtype=np.float64).reshape(-1, 3, 3)
        t = np.ascontiguousarray(sym_tau, dtype=np.float64).reshape(-1, 3)
        tr = np.ascontiguousarray(np.asarray(sym_trev).astype(np.int32))
        nsym = R.shape[0]
        nk = self.sys.nk_bz
        if count is None:
            count = nsym * nk - first
        out = np.empty((count, self.sys.nspin, self.sys.nbnds, self.sys.nbnds), np.complex128) if host else None
        self._check(self._L.lelph_gpu_dmats(self.h, nsym, _ptr(R), _ptr(t), tr.ctypes.data_as(_ip), int(first),
                                            int(count), _ptr(out) if host else None))
        return out

    def compute_elphq_star(self, qpt, eigVec, dVscfq, star_syms, sym_R=None, sym_tau=None, sym_trev=None,
                           non_loc=True, kminusq=False, out=OUT_C128):
        """compute_and_write_elphq with its q-star expansion: (nstar, nk_BZ,
        nmodes, nspin, nb, nb); row istar belongs to the star member of
        symmetry star_syms[istar] (star_syms[0] = 0, the irreducible q).  The
        phonon symmetries default to the system's."""
        s = self.sys
        R = np.ascontiguousarray(s.sym_R if sym_R is None else sym_R, dtype=np.float64).reshape(-1, 3, 3)
        t = np.ascontiguousarray(s.sym_tau if sym_tau is None else sym_tau, dtype=np.float64).reshape(-1, 3)
        tr = np.ascontiguousarray(np.asarray(s.sym_trev if sym_trev is None else sym_trev).astype(np.int32))
        st = np.ascontiguousarray(star_syms, dtype=np.int32)
        q = np.ascontiguousarray(qpt, dtype=np.float64)
        e = np.ascontiguousarray(eigVec, dtype=np.complex128)
        v = np.ascontiguousarray(dVscfq, dtype=np.complex128)
        dt = np.complex64 if out == OUT_C64 else np.complex128
        g = np.empty((len(st), s.nk_bz, s.nmodes, s.nspin, s.nbnds, s.nbnds), dt)
        self._check(self._L.lelph_gpu_compute_elphq_star(
            self.h, _ptr(q), _ptr(e), _ptr(v), int(non_loc), int(kminusq), R.shape[0], _ptr(R), _ptr(t),
            tr.ctypes.data_as(_ip), len(st), st.ctypes.data_as(_ip), int(out), g.ctypes.data_as(C.c_void_p)))
        return g

    def run(self, qslots, kbz, non_loc=True, kminusq=False, out=OUT_C128, g_out=None):
        qs = np.ascontiguousarray(qslots, dtype=np.int32)
        ks = np.ascontiguousarray(kbz, dtype=np.int32)
        s = self.sys
        shape = (len(ks), s.nmodes, s.nspin, s.nbnds, s.nbnds)
        if g_out is None:
            g_out = np.empty(shape, dtype=np.complex64 if out == OUT_C64 else np.complex128)
        self._check(self._L.lelph_gpu_run(self.h, len(ks), _ptr(qs, _ip), _ptr(ks, _ip), int(non_loc), int(kminusq),
                                          out, g_out.ctypes.data_as(C.c_void_p)))
        return g_out

    def run_device(self, qslots, kbz, dev_ptr, non_loc=True, kminusq=False, out=OUT_C128):
        qs = np.ascontiguousarray(qslots, dtype=np.int32)
        ks = np.ascontiguousarray(kbz, dtype=np.int32)
        self._check(self._L.lelph_gpu_run_device(self.h, len(ks), _ptr(qs, _ip), _ptr(ks, _ip), int(non_loc),
                                                 int(kminusq), out, C.c_void_p(dev_ptr)))

    def compute_elphq(self, qpt, eigVec, dVscfq, non_loc=True, kminusq=False):
        """compute_and_write_elphq for one q: (nk_BZ, nmodes, nspin, nb, nb) complex128."""
        s = self.sys
        out = np.empty((s.nk_bz, s.nmodes, s.nspin, s.nbnds, s.nbnds), np.complex128)
        q = np.ascontiguousarray(qpt, dtype=np.float64)
        e = np.ascontiguousarray(eigVec, dtype=np.complex128)
        v = np.ascontiguousarray(dVscfq, dtype=np.complex128)
        self._check(self._L.lelph_gpu_compute_elphq(self.h, _ptr(q), _ptr(e), _ptr(v), int(non_loc), int(kminusq),
                                                    _ptr(out)))
        return out

    def elph_q_rotate(self, Dl, g, Dr, time_rev):
        g = np.ascontiguousarray(g, dtype=np.complex128)
        out = np.empty_like(g)
        Dl = np.ascontiguousarray(Dl, dtype=np.complex128)
        Dr = np.ascontiguousarray(Dr, dtype=np.complex128)
        self._check(self._L.lelph_gpu_elph_q_rotate(self.h, _ptr(Dl), _ptr(g), _ptr(Dr), int(time_rev), _ptr(out)))
        return out

    def gvec_map(self, kbz, ulm=(0, 0, 0)):
        npw = len(self.sys.gvec[self.sys.kmap[kbz][0]])
        out = np.empty((npw, 3), np.int32)
        u = np.ascontiguousarray(ulm, dtype=np.int32)
        self._check(self._L.lelph_gpu_debug_gvec_map(self.h, kbz, _ptr(u, _ip), _ptr(out, _ip)))
        return out

    def set_profiling(self, on=True):
        self._check(self._L.lelph_gpu_set_profiling(self.h, int(on)))

    def set_wait_limit(self, ns=0):
        """Limit of every pipeline wait of the tensor-core sandwich (0: default)."""
        self._check(self._L.lelph_gpu_set_wait_limit(self.h, int(ns)))

    def stats(self):
        st = Stats()
        self._check(self._L.lelph_gpu_stats_get(self.h, C.byref(st)))
        out = {f: getattr(st, f) for f, _ in Stats._fields_}
        out["product_grid"] = tuple(out["product_grid"])
        return out

    def stream(self):
        return self._L.lelph_gpu_stream(self.h)


def compute_elphq(s, iq, precision="fp64", non_loc=True, kminusq=False):
    """One-shot convenience: the reference's per-q stage on the GPU."""
    with LelphGPU(s, precision) as ctx:
        return ctx.compute_elphq(s.qpts[iq], s.eigVec[iq], s.dVscf[iq], non_loc=non_loc, kminusq=kminusq)
