"""The reference-side binding, compiled and run in the reference's own program.

letzelphc_gb300/binding/compute_elph_matq_gpu.c is what a LetzElPhC
maintainer compiles in place of src/elph/compute_elph_matq.c.  oracle/Makefile
(target gpu, run by __graft_entry__.build()) links it into the same harness as
the unmodified reference (the reference's objects, the single-rank MPI /
FFTW-API / netCDF stand-ins), so both programs read one input file and write
elph_mat through the same nc_put_vara.  These tests run both on the same
files and compare what they wrote:

* double build (-DCOMPILE_ELPH_DOUBLE): the binding hands the arrays over as
  they are and runs the library's FP64 form: <= 1e-10 relative to max|g|;
* default single-precision build: the binding widens the float inputs, runs
  the mixed form and narrows g back to float complex; against the reference's
  double build its error (the metric's definition) is of the order of that of
  the reference's own single-precision build on the same file (within 4x on
  these small systems, where a few hundred elements make the maximum a
  matter of chance; the configuration-sized tests in test_gpu_configs.py hold
  the mixed form to no more than the reference's error) and within the
  metric's 1e-5 in RMS and norm;
* q stars: with one k pool the binding expands the star on the device; with
  two it computes its pool's k-points and rotates them with the Dmats the
  harness serves through nc_get_vara, as the reference does.
"""
import os
import platform
import subprocess
import tempfile

import numpy as np
import pytest

from golden_util import errors
from letzelphc_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARCH = platform.machine()
FP64_TOL = 1e-10


def _exe(single, gpu):
    d = os.path.join(ROOT, "oracle", "_ref", ARCH + ("-f32" if single else ""))
    p = os.path.join(d, "lelph_ref_gpu" if gpu else "lelph_ref")
    if not os.access(p, os.X_OK):
        pytest.skip(f"{p} was not built (the reference sources were not available to build())")
    return p


def _run(exe, sysf, nq_rows, s, extra=(), kpools=1):
    env = dict(os.environ, LELPH_REF_KPOOLS=str(kpools), OMP_NUM_THREADS=str(os.cpu_count() or 1))
    outs = []
    for pool in range(kpools):
        gf = sysf + f".{os.path.basename(exe)}.{pool}.g"
        env["LELPH_REF_KPOOL"] = str(pool)
        subprocess.run([exe, sysf, gf, *extra], check=True, env=env, stdout=subprocess.DEVNULL)
        outs.append(np.fromfile(gf, np.complex128).reshape(nq_rows, s.nk_bz, s.nmodes, s.nspin, s.nbnds, s.nbnds))
    # every pool writes its own k rows (and their star images); the rest stay zero
    return sum(outs)


SYSTEMS = {
    "c0": ("c0", {}, False),
    "zb_tr_kmq": ("c0", {"kind": "zincblende", "timerev": True, "nbnds": 6, "kgrid": (2, 2, 2),
                         "qpts": [(0.5, 0, 0)]}, True),
    "lsda": ("c0", {"nspin": 2, "nbnds": 4, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]}, False),
    "soc": ("c0", {"kind": "zincblende", "timerev": True, "nspinor": 2, "nmag": 4, "soc": True,
                   "ls": (0, 1, 2), "nbnds": 2, "npw": 150, "fft": (20, 20, 20), "kgrid": (2, 2, 2),
                   "qpts": [(0.5, 0.5, 0)]}, False),
}


@pytest.mark.parametrize("kpools", [1, 2])
@pytest.mark.parametrize("name", list(SYSTEMS))
def test_binding_double_build_matches_reference(name, kpools):
    base, ov, kmq = SYSTEMS[name]
    s = synth.make_system(base, dict(ov))
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "s.bin")
        synth.write_system(s, f, kminusq=kmq)
        ref = _run(_exe(False, False), f, len(s.qpts), s, kpools=kpools)
        gpu = _run(_exe(False, True), f, len(s.qpts), s, kpools=kpools)
    err = np.abs(gpu - ref).max() / np.abs(ref).max()
    assert err < FP64_TOL, err


@pytest.mark.parametrize("name", ["c0", "soc"])
def test_binding_single_build_within_reference_single_precision_error(name):
    base, ov, kmq = SYSTEMS[name]
    s = synth.make_system(base, dict(ov))
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "s.bin")
        synth.write_system(s, f, kminusq=kmq)
        g64 = _run(_exe(False, False), f, len(s.qpts), s)
        g32 = _run(_exe(True, False), f, len(s.qpts), s)
        gpu = _run(_exe(True, True), f, len(s.qpts), s)
    e_ref, e_gpu = errors(g32, g64), errors(gpu, g64)
    print(f"{name}: binding (mixed form) max {e_gpu[0]:.2e} rms {e_gpu[1]:.2e} norm {e_gpu[2]:.2e}; "
          f"reference single-precision build max {e_ref[0]:.2e} rms {e_ref[1]:.2e} norm {e_ref[2]:.2e}")
    assert all(eg <= 4 * er for eg, er in zip(e_gpu, e_ref)), (e_gpu, e_ref)
    assert e_gpu[1] < 1e-5 and e_gpu[2] < 1e-5, e_gpu


@pytest.mark.parametrize("kpools", [1, 2])
def test_binding_q_star_expansion(kpools):
    import elph_oracle as O
    s = synth.make_system("c0", {"kgrid": (2, 2, 2), "nbnds": 3, "qpts": [(0.5, 0, 0), (0.5, 0.5, 0)]})
    stars = [O.q_star(s, q) for q in s.qpts]
    ns = np.array([len(m) for m, _ in stars], np.int32)
    qs = np.concatenate([sy for _, sy in stars]).astype(np.int32)
    assert ns.max() > 1
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "s.bin")
        synth.write_system(s, f)
        spec = os.path.join(d, "star.bin")
        with open(spec, "wb") as fh:
            fh.write(b"LELPHSYS")
            synth._rec(fh, "nqstar", ns)
            synth._rec(fh, "qsym", qs)
            fh.write(b"END\0" + b"\0" * 28)
        ref = _run(_exe(False, False), f, int(ns.sum()), s, extra=("star", spec), kpools=kpools)
        gpu = _run(_exe(False, True), f, int(ns.sum()), s, extra=("star", spec), kpools=kpools)
    assert (np.abs(ref).reshape(int(ns.sum()), s.nk_bz, -1).max(axis=2) > 0).all()   # every row written
    err = np.abs(gpu - ref).max() / np.abs(ref).max()
    assert err < FP64_TOL, err
