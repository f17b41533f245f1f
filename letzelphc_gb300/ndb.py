"""ctypes mirror of the ndb.elph writer (include/lelph_ndb.h).

Writes the variables the reference puts into ndb.elph (elph_driver.c:152-187,
write_basic_data.c:15-215) in the netCDF classic 64-bit-offset format; see the
header for the layout and what differs from the reference's NetCDF-4 storage.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .elph import load_library

EXPORTS = ["lelph_ndb_create", "lelph_ndb_put_elph", "lelph_ndb_put_phonon", "lelph_ndb_close"]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class NdbDesc(C.Structure):
    _fields_ = [
        ("nq_BZ", C.c_int), ("nq_iBZ", C.c_int), ("nkpts_BZ", C.c_int), ("nmodes", C.c_int), ("natom", C.c_int),
        ("nspin", C.c_int), ("nbnds", C.c_int), ("nph_sym", C.c_int), ("start_band", C.c_int),
        ("end_band", C.c_int), ("io_double", C.c_int),
        ("kpoints", _dp), ("qpoints", _dp), ("qpoints_iBZ", _dp), ("qmap", _ip), ("kmap", _ip),
        ("sym_Rmat", _dp), ("sym_tau", _dp), ("sym_time_rev", _ip), ("kernel", C.c_char_p), ("kminusq", C.c_int),
        ("epsilon", _dp), ("Zborn", _dp), ("Qpole", _dp),
    ]


def _lib():
    L = load_library()
    if not getattr(L, "_ndb_declared", False):
        vp = C.c_void_p
        L.lelph_ndb_create.argtypes = [C.c_char_p, C.POINTER(NdbDesc), C.POINTER(vp)]
        L.lelph_ndb_put_elph.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, C.c_int]
        L.lelph_ndb_put_phonon.argtypes = [vp, C.c_int, _dp, _dp]
        L.lelph_ndb_close.argtypes = [vp]
        for n in EXPORTS:
            getattr(L, n).restype = C.c_int
        L._ndb_declared = True
    return L


class NdbElph:
    """Writer of one ndb.elph file.  `s` carries the lattice fields
    (kbz_crys, kmap, nmodes, nspin, nbnds, atom_pos); qpts_BZ / qmap the full
    q list and its map to (iBZ q, symmetry); the phonon symmetries default to
    the system's."""

    def __init__(self, path, s, qpts_BZ, qpts_iBZ, qmap, kernel="dfpt", kminusq=False, io_double=True,
                 sym_R=None, sym_tau=None, sym_trev=None, start_band=1, end_band=None,
                 epsilon=None, Zborn=None, Qpole=None):
        self._L = _lib()
        keep = self._keep = []

        def arr(x, dt):
            a = np.ascontiguousarray(x, dtype=dt)
            keep.append(a)
            return a

        R = s.sym_R if sym_R is None else sym_R
        d = NdbDesc()
        d.nq_BZ, d.nq_iBZ, d.nkpts_BZ = len(qpts_BZ), len(qpts_iBZ), s.nk_bz
        d.nmodes, d.natom, d.nspin, d.nbnds, d.nph_sym = s.nmodes, len(s.atom_pos), s.nspin, s.nbnds, len(R)
        d.start_band = start_band
        d.end_band = start_band + s.nbnds - 1 if end_band is None else end_band
        d.io_double = int(io_double)
        d.kpoints = arr(s.kbz_crys, np.float64).ctypes.data_as(_dp)
        d.qpoints = arr(qpts_BZ, np.float64).ctypes.data_as(_dp)
        d.qpoints_iBZ = arr(qpts_iBZ, np.float64).ctypes.data_as(_dp)
        d.qmap = arr(qmap, np.int32).ctypes.data_as(_ip)
        d.kmap = arr(s.kmap, np.int32).ctypes.data_as(_ip)
        d.sym_Rmat = arr(R, np.float64).ctypes.data_as(_dp)
        d.sym_tau = arr(s.sym_tau if sym_tau is None else sym_tau, np.float64).ctypes.data_as(_dp)
        d.sym_time_rev = arr(np.asarray(s.sym_trev if sym_trev is None else sym_trev).astype(np.int32),
                             np.int32).ctypes.data_as(_ip)
        kb = kernel.encode()
        keep.append(kb)
        d.kernel = kb
        d.kminusq = int(kminusq)
        for name, v in (("epsilon", epsilon), ("Zborn", Zborn), ("Qpole", Qpole)):
            setattr(d, name, arr(v, np.float64).ctypes.data_as(_dp) if v is not None else _dp())
        h = C.c_void_p()
        rc = self._L.lelph_ndb_create(path.encode(), C.byref(d), C.byref(h))
        if rc != 0:
            raise OSError(f"lelph_ndb_create failed with status {rc}")
        self.h = h

    def put_elph(self, iq_BZ, k0, g):
        """elph_mat[iq_BZ][k0 .. k0 + len(g)) from g (nk, nmodes, nspin, nb, nb)."""
        g = np.ascontiguousarray(g)
        c64 = 1 if g.dtype == np.complex64 else 0
        if not c64:
            g = np.ascontiguousarray(g, dtype=np.complex128)
        rc = self._L.lelph_ndb_put_elph(self.h, int(iq_BZ), int(k0), len(g), g.ctypes.data_as(C.c_void_p), c64)
        if rc != 0:
            raise OSError(f"lelph_ndb_put_elph failed with status {rc}")

    def put_phonon(self, iq_BZ, eig=None, omega=None):
        e = np.ascontiguousarray(eig, dtype=np.complex128) if eig is not None else None
        w = np.ascontiguousarray(omega, dtype=np.float64) if omega is not None else None
        rc = self._L.lelph_ndb_put_phonon(self.h, int(iq_BZ), e.ctypes.data_as(_dp) if e is not None else None,
                                          w.ctypes.data_as(_dp) if w is not None else None)
        if rc != 0:
            raise OSError(f"lelph_ndb_put_phonon failed with status {rc}")

    def close(self):
        if self.h:
            rc = self._L.lelph_ndb_close(self.h)
            self.h = None
            if rc != 0:
                raise OSError(f"lelph_ndb_close failed with status {rc}")

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
