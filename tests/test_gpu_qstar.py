"""GPU q-star expansion (compute_and_write_elphq's star loop,
src/elph/compute_elph_matq.c:159-217, elph_q_rotate) through the C ABI.

* plain form: every star member at every S k against the reference's output
  (tests/golden/star_*.npz) to 1e-10 of max|g|;
* mixed form: the same with the metric's error definition (RMS and normwise
  <= 1e-5 of the FP64 reference);
* Dmats taken from the resident block of lelph_gpu_dmats give the same
  result as Dmats computed for the star on the fly;
* star_sym[0] other than the identity is refused as the reference refuses it.
"""
import numpy as np
import pytest

from golden_util import STAR_NAMES, load_star
from letzelphc_gb300.elph import LelphError, LelphGPU

pytestmark = pytest.mark.gpu


def _rows(z, iq):
    ns = z["nqstar"]
    pos = int(ns[:iq].sum())
    return pos, int(ns[iq])


@pytest.mark.parametrize("name", STAR_NAMES)
def test_qstar_fp64_matches_reference(name):
    z, s, kmq = load_star(name)
    with LelphGPU(s, "fp64") as ctx:
        for iq in range(len(s.qpts)):
            pos, n = _rows(z, iq)
            g = ctx.compute_elphq_star(s.qpts[iq], s.eigVec[iq], s.dVscf[iq], z["qsym"][pos:pos + n], kminusq=kmq)
            ref = z["g"][pos:pos + n]
            assert np.abs(g - ref).max() < 1e-10 * np.abs(ref).max(), (name, iq)


@pytest.mark.parametrize("name", ["star_c0", "star_l12", "star_soc"])
def test_qstar_mixed_error(name):
    z, s, kmq = load_star(name)
    with LelphGPU(s, "mixed") as ctx:
        for iq in range(len(s.qpts)):
            pos, n = _rows(z, iq)
            g = ctx.compute_elphq_star(s.qpts[iq], s.eigVec[iq], s.dVscf[iq], z["qsym"][pos:pos + n], kminusq=kmq)
            ref = z["g"][pos:pos + n]
            a, b = np.abs(g), np.abs(ref)
            e = np.abs(a - b) / np.maximum(b, 1e-6 * b.max())
            assert np.sqrt((e ** 2).mean()) < 1e-5, (name, iq)
            assert np.linalg.norm(g - ref) < 1e-5 * np.linalg.norm(ref), (name, iq)


def test_qstar_resident_dmats_equal_on_the_fly():
    z, s, kmq = load_star("star_c0")
    pos, n = _rows(z, 0)
    star = z["qsym"][pos:pos + n]
    with LelphGPU(s, "fp64") as ctx:
        g1 = ctx.compute_elphq_star(s.qpts[0], s.eigVec[0], s.dVscf[0], star)
        ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev, host=False)   # whole table resident
        g2 = ctx.compute_elphq_star(s.qpts[0], s.eigVec[0], s.dVscf[0], star)
    assert np.array_equal(g1, g2)


def test_qstar_rejects_non_identity_first_member():
    z, s, kmq = load_star("star_c0")
    with LelphGPU(s, "fp64") as ctx:
        with pytest.raises(LelphError) as e:
            ctx.compute_elphq_star(s.qpts[0], s.eigVec[0], s.dVscf[0], [3, 0])
        assert e.value.status == -1


def test_qstar_rows_through_the_ndb_writer(tmp_path):
    """The drop-in output path: star rows from the device written with the
    ndb.elph writer and read back by an independent netCDF reader equal the
    reference's elph_mat."""
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    from letzelphc_gb300.ndb import NdbElph
    z, s, kmq = load_star("star_c0")
    ns, qs = z["nqstar"], z["qsym"]
    qmap = [(iq, int(qs[int(ns[:iq].sum()) + j])) for iq in range(len(s.qpts)) for j in range(ns[iq])]
    path = str(tmp_path / "ndb.elph")
    with LelphGPU(s, "fp64") as ctx, NdbElph(path, s, np.zeros((len(qmap), 3)), s.qpts, qmap) as f:
        for iq in range(len(s.qpts)):
            pos, n = _rows(z, iq)
            g = ctx.compute_elphq_star(s.qpts[iq], s.eigVec[iq], s.dVscf[iq], qs[pos:pos + n], kminusq=kmq)
            for j in range(n):
                f.put_elph(pos + j, 0, g[j])
    with netcdf(path, "r", mmap=False) as f:
        g = f.variables["elph_mat"].data
        got = g[..., 0] + 1j * g[..., 1]
    assert np.abs(got - z["g"]).max() < 1e-10 * np.abs(z["g"]).max()
