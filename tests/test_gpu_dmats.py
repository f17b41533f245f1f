"""GPU parity of the Dmats (compute_and_write_dmats, src/elph/compute_dmats.c:20;
electronic_reps, src/symmetries/elec_reps.c:16-413) through the C ABI.

* plain form (FP64): every (symmetry, full-BZ k) pair of each golden system
  against the oracle to 1e-10 and against the reference's stored pairs;
* mixed form (FP32 operands and contraction, FP64 phase reduction and
  group sums): max abs error <= 2e-6 (the matrices have entries of modulus
  up to 1);
* a block (first, count) equals the same rows of the whole table, as a pool
  of distribute_to_grps computes it;
* an operation that sends k off the grid, or is not integral on the lattice,
  returns LELPH_GPU_ERR_GEOMETRY.
"""
import numpy as np
import pytest

import elph_oracle as O
from golden_util import load_dmats
from letzelphc_gb300.elph import LelphError, LelphGPU

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 2e-6


@pytest.fixture(scope="module")
def golden():
    return load_dmats()


@pytest.mark.parametrize("name", ["c0", "zb_tr", "l12", "soc_tr", "lsda", "hex_ragged"])
def test_dmats_fp64_match_oracle_and_reference(golden, name):
    z, systems = golden
    s = systems[name]
    ref = O.dmats(s).reshape(-1, s.nspin, s.nbnds, s.nbnds)
    with LelphGPU(s, "fp64") as ctx:
        D = ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev)
    assert D.shape == ref.shape
    assert np.abs(D - ref).max() < FP64_TOL, name
    assert np.abs(D[::int(z["stride"])] - z[name + "_sub"]).max() < FP64_TOL, name


@pytest.mark.parametrize("name", ["c0", "l12", "soc_tr", "lsda"])
def test_dmats_mixed_error(golden, name):
    z, systems = golden
    s = systems[name]
    ref = O.dmats(s).reshape(-1, s.nspin, s.nbnds, s.nbnds)
    with LelphGPU(s, "mixed") as ctx:
        D = ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev)
    err = np.abs(D - ref).max()
    assert err < MIXED_TOL, (name, err)


def test_dmats_block_equals_table(golden):
    z, systems = golden
    s = systems["l12"]
    with LelphGPU(s, "fp64") as ctx:
        full = ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev)
        part = ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev, first=37, count=101)
    assert np.array_equal(part, full[37:138])


def test_dmats_reject_bad_operations(golden):
    z, systems = golden
    s = systems["c0"]
    c, sn = np.cos(np.pi / 6), np.sin(np.pi / 6)
    R30 = np.array([[c, -sn, 0.0], [sn, c, 0.0], [0.0, 0.0, 1.0]])  # not a lattice symmetry
    with LelphGPU(s, "fp64") as ctx:
        with pytest.raises(LelphError) as e:
            ctx.dmats(R30[None], np.zeros((1, 3)), np.zeros(1, np.int32))
        assert e.value.status == -5
        with pytest.raises(LelphError):
            ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev, first=len(s.sym_R) * s.nk_bz - 2, count=5)


# ---- the mixed form on the tensor cores (k_dmats_tc, LELPH_DMATS_TC=1) against
# the SIMT kernel (the default): groups of jobs that share k1 (up to 4 jobs of
# 32 bands per unit), one job per unit in band tiles above 64 bands, both
# spinor counts, two spins, ragged plane-wave counts.
def _dmats_both(s, monkeypatch, **kw):
    monkeypatch.setenv("LELPH_DMATS_TC", "0")
    with LelphGPU(s, "mixed") as ctx:
        d_simt = ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev, **kw)
    monkeypatch.setenv("LELPH_DMATS_TC", "1")
    with LelphGPU(s, "mixed") as ctx:
        d_tc = ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev, **kw)
    return d_tc, d_simt


@pytest.mark.parametrize("name", ["c0", "l12", "soc_tr", "lsda", "hex_ragged"])
def test_dmats_tensor_cores_match_simt(golden, name, monkeypatch):
    z, systems = golden
    s = systems[name]
    ref = O.dmats(s).reshape(-1, s.nspin, s.nbnds, s.nbnds)
    d_tc, d_simt = _dmats_both(s, monkeypatch)
    e_tc, e_simt = np.abs(d_tc - ref).max(), np.abs(d_simt - ref).max()
    print(f"{name}: max|D - D_fp64| tensor cores {e_tc:.2e}, SIMT {e_simt:.2e}")
    assert e_tc < MIXED_TOL, (name, e_tc)
    assert np.abs(d_tc - d_simt).max() < MIXED_TOL, name


@pytest.mark.parametrize("nbnds", [80, 136])
def test_dmats_tensor_cores_band_tiles(monkeypatch, nbnds):
    from letzelphc_gb300 import synth
    s = synth.make_system("c0", {"nbnds": nbnds, "npw": 600, "kgrid": (2, 2, 2)})
    with LelphGPU(s, "fp64") as ctx:
        ref = ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev)
    d_tc, d_simt = _dmats_both(s, monkeypatch)
    e_tc, e_simt = np.abs(d_tc - ref).max(), np.abs(d_simt - ref).max()
    print(f"{nbnds} bands: max|D - D_fp64| tensor cores {e_tc:.2e}, SIMT {e_simt:.2e}")
    assert e_tc < MIXED_TOL, e_tc


def test_dmats_tensor_cores_block_equals_table(golden, monkeypatch):
    # a block groups its jobs differently from the whole table; each job's
    # matrix does not depend on its group
    z, systems = golden
    s = systems["l12"]
    monkeypatch.setenv("LELPH_DMATS_TC", "1")
    with LelphGPU(s, "mixed") as ctx:
        full = ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev)
        part = ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev, first=37, count=101)
    assert np.abs(part - full[37:138]).max() < 1e-12
