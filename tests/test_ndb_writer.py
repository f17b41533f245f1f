"""The ndb.elph writer (include/lelph_ndb.h) on CPU: the file it writes is a
netCDF classic 64-bit-offset file that an independent reader (scipy.io.netcdf)
opens, with exactly the variables, dimension names, shapes and types of the
reference's ndb.elph, and elph_mat holding the reference's own matrix
elements (the q-star fixture) bit for bit."""
import os
import subprocess
import tempfile

import ctypes
import numpy as np
import pytest

from golden_util import load_star
from letzelphc_gb300.build import build_library

netcdf = pytest.importorskip("scipy.io").netcdf_file

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# The reference's def_ncVar calls for ndb.elph: name -> (dimension names,
# element type): src/elph/elph_driver.c:152-187, src/io/write_basic_data.c:29-177
REF_LAYOUT = {
    "POLARIZATION_VECTORS": (("nq", "nmodes", "atom", "pol", "re_im"), "real"),
    "FREQ": (("nq", "nmodes"), "real"),
    "elph_mat": (("nq", "nk", "nmodes", "nspin", "initial_band", "final_band_PH_abs", "re_im"), "real"),
    "kpoints": (("nk", "pol"), "real"),
    "qpoints": (("nq", "pol"), "real"),
    "qpoints_iBZ": (("nq_iBZ", "pol"), "real"),
    "qmap": (("nq", "dim_two"), "int"),
    "kmap": (("nk", "dim_two"), "int"),
    "bands": (("two_scalars",), "int"),
    "number_of_phonon_symmetries": (("scalar",), "int"),
    "time_reversal_phonon": (("scalar",), "int"),
    "symmetry_matrices": (("nsym_ph", "pol", "pol"), "real"),
    "fractional_translation": (("nsym_ph", "pol"), "real"),
    "kernel": (("kernel_str_size",), "char"),
    "convention": (("convention_str_size",), "char"),
    "epsilon": (("pol", "pol"), "real"),
    "Born_charges": (("natoms", "pol", "pol"), "real"),
    "Quadrupole_tensor": (("natoms", "pol", "pol", "pol"), "real"),
}


def _write_star_file(path, io_double, kmq_override=None):
    from letzelphc_gb300.ndb import NdbElph
    z, s, kmq = load_star("star_c0")
    ns, qs = z["nqstar"], z["qsym"]
    qmap, qbz = [], []
    pos = 0
    for iq in range(len(s.qpts)):
        for j in range(ns[iq]):
            qmap.append((iq, int(qs[pos])))
            R = s.sym_R[qs[pos]]
            qc = np.linalg.solve(s.alat.T, s.qpts[iq])
            qbz.append(s.alat.T @ (R @ qc))
            pos += 1
    rng = np.random.default_rng(3)
    eig = rng.standard_normal((len(qmap), s.nmodes, s.nmodes)) + 1j * rng.standard_normal((len(qmap), s.nmodes, s.nmodes))
    om = rng.standard_normal((len(qmap), s.nmodes))
    with NdbElph(path, s, qbz, s.qpts, qmap, kernel="dfpt", kminusq=kmq if kmq_override is None else kmq_override,
                 io_double=io_double) as f:
        for iq in range(len(qmap)):
            f.put_elph(iq, 0, z["g"][iq])
            f.put_phonon(iq, eig[iq], om[iq])
    return z, s, np.array(qbz), np.array(qmap), eig, om


def test_layout_and_values_match_reference():
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ndb.elph")
        z, s, qbz, qmap, eig, om = _write_star_file(path, io_double=True)
        with netcdf(path, "r", mmap=False) as f:
            assert set(f.variables) == set(REF_LAYOUT)
            for name, (dims, kind) in REF_LAYOUT.items():
                v = f.variables[name]
                assert v.dimensions == dims, name
                assert {"real": "d", "int": "i", "char": "c"}[kind] == v.typecode(), name
            g = f.variables["elph_mat"].data
            ref = z["g"]
            assert g.shape == ref.shape + (2,)
            assert np.array_equal(g[..., 0] + 1j * g[..., 1], ref)
            pv = f.variables["POLARIZATION_VECTORS"].data
            assert np.array_equal(pv[..., 0] + 1j * pv[..., 1], eig.reshape(pv.shape[:-1]))
            assert np.array_equal(f.variables["FREQ"].data, om)
            assert np.array_equal(f.variables["kpoints"].data, s.kbz_crys)
            assert np.array_equal(f.variables["qpoints"].data, qbz)
            assert np.array_equal(f.variables["qpoints_iBZ"].data, s.qpts)
            assert np.array_equal(f.variables["qmap"].data, qmap)
            assert np.array_equal(f.variables["kmap"].data, s.kmap)
            assert list(f.variables["bands"].data) == [1, s.nbnds]
            assert int(f.variables["number_of_phonon_symmetries"].data[0]) == len(s.sym_R)
            assert int(f.variables["time_reversal_phonon"].data[0]) == int(s.sym_trev.any())
            assert np.array_equal(f.variables["symmetry_matrices"].data, s.sym_R)
            assert np.array_equal(f.variables["fractional_translation"].data, s.sym_tau)
            assert f.variables["kernel"].data.tobytes() == b"dfpt\0"
            assert f.variables["convention"].data.tobytes() == b"standard\0"
            assert not f.variables["epsilon"].data.any() and not f.variables["Born_charges"].data.any()


def test_float_file_and_yambo_convention():
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ndb.elph")
        z, s, *_ = _write_star_file(path, io_double=False, kmq_override=True)
        with netcdf(path, "r", mmap=False) as f:
            g = f.variables["elph_mat"]
            assert g.typecode() == "f"
            ref = z["g"].astype(np.complex64)
            assert np.array_equal(g.data[..., 0] + 1j * g.data[..., 1], ref)
            assert f.variables["convention"].data.tobytes() == b"yambo\0"


def test_unwritten_rows_read_zero_and_bad_arguments():
    from letzelphc_gb300.ndb import NdbElph
    z, s, kmq = load_star("star_c0")
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ndb.elph")
        with NdbElph(path, s, np.zeros((2, 3)), s.qpts[:1], [(0, 0), (0, 1)]) as f:
            f.put_elph(1, 3, z["g"][0, :2])
            with pytest.raises(OSError):
                f.put_elph(2, 0, z["g"][0, :1])       # q beyond nq
            with pytest.raises(OSError):
                f.put_elph(0, s.nk_bz - 1, z["g"][0, :2])  # k beyond nk
        with netcdf(path, "r", mmap=False) as f:
            g = f.variables["elph_mat"].data
            assert not g[0].any() and not g[1, :3].any() and not g[1, 5:].any()
            assert np.array_equal(g[1, 3:5, ..., 0] + 1j * g[1, 3:5, ..., 1], z["g"][0, :2])


def test_ndb_descriptor_layout_matches_c():
    from letzelphc_gb300.ndb import NdbDesc
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "lelph_ndb.h"
int main(void){
  printf("%zu %zu %zu %zu\n", sizeof(lelph_ndb_desc), offsetof(lelph_ndb_desc, kpoints),
         offsetof(lelph_ndb_desc, kernel), offsetof(lelph_ndb_desc, Qpole));
  return 0; }
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert out == [ctypes.sizeof(NdbDesc), NdbDesc.kpoints.offset, NdbDesc.kernel.offset, NdbDesc.Qpole.offset]
