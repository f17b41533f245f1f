"""GPU parity of the CUDA path through the C ABI.

* integer symmetry maps: the device's rotated (and umklapp-shifted) Miller
  indices equal, bit for bit, the sorted integer G vectors of the reference's
  rotateGvecs + Sort_pw as restated in the oracle;
* FP64 form against the reference's own output (tests/golden/), tolerance
  1e-10 relative to max|g| (the FP64 bar);
* mixed forms against the FP64 GPU form on the same inputs, errors measured
  as e_i = ||g_mixed| - |g_fp64|| / max(|g_fp64|, 1e-6 max|g_fp64|) and as
  the complex norm ratio ||g_mixed - g_fp64|| / ||g_fp64||; tolerances are
  written next to each assertion.
"""
import numpy as np
import pytest

import elph_oracle as O
from golden_util import NAMES, load
from letzelphc_gb300 import synth
from letzelphc_gb300.elph import LelphGPU, LelphError, OUT_C64

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def run_all(s, prec, non_loc=True, kminusq=False, out=0):
    with LelphGPU(s, prec) as ctx:
        for iq in range(len(s.qpts)):
            ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
        nk = s.nk_bz
        qs = np.repeat(np.arange(len(s.qpts)), nk)
        ks = np.tile(np.arange(nk), len(s.qpts))
        g = ctx.run(qs, ks, non_loc=non_loc, kminusq=kminusq, out=out)
    return g.reshape(len(s.qpts), nk, *g.shape[1:])


def errors(g, ref):
    a, b = np.abs(g), np.abs(ref)
    floor = 1e-6 * b.max()
    e = np.abs(a - b) / np.maximum(b, floor)
    norm = np.linalg.norm((g - ref).ravel()) / np.linalg.norm(ref.ravel())
    return e.max(), np.sqrt(np.mean(e * e)), norm


@pytest.mark.parametrize("name", ["c0", "zb_tr", "soc_tr", "l12_small"])
def test_gvec_maps_bit_exact(name):
    s, _, _, _ = load(name)
    with LelphGPU(s, "fp64") as ctx:
        for kbz in range(0, s.nk_bz, max(1, s.nk_bz // 9)):
            ik, isym = s.kmap[kbz]
            ulm = (1, -1, 0) if kbz % 2 else (0, 0, 0)
            dev = ctx.gvec_map(kbz, ulm)
            G0 = np.linalg.solve(s.alat.T, np.array(ulm, float))  # cartesian vector with crystal coordinates ulm
            gf = O.rotate_gvecs(s.gvec[ik], s.sym_R[isym], s.alat, G0 if kbz % 2 else None)
            gi, _ = O.sort_pw(gf, np.zeros((1, len(gf))))
            order = np.lexsort((dev[:, 2], dev[:, 1], dev[:, 0]))
            assert np.array_equal(dev[order], gi.astype(np.int32)), (name, kbz)


@pytest.mark.parametrize("name", NAMES)
def test_fp64_matches_reference(name):
    s, g_ref, kmq, nl = load(name)
    g = run_all(s, "fp64", non_loc=nl, kminusq=kmq)
    err = np.abs(g - g_ref).max() / np.abs(g_ref).max()
    assert err < FP64_TOL, err


def test_compute_elphq_entry_matches_reference():
    s, g_ref, kmq, nl = load("c0")
    with LelphGPU(s, "fp64") as ctx:
        g = ctx.compute_elphq(s.qpts[0], s.eigVec[0], s.dVscf[0], non_loc=nl, kminusq=kmq)
    assert np.abs(g - g_ref[0]).max() / np.abs(g_ref).max() < FP64_TOL


@pytest.mark.parametrize("prec", ["mixed_f16", "mixed_bf16"])
@pytest.mark.parametrize("name", ["c0", "zb_tr", "lsda", "soc_tr", "spinor_nosoc"])
def test_mixed_against_fp64(name, prec):
    s, g_ref, kmq, nl = load(name)
    g64 = run_all(s, "fp64", non_loc=nl, kminusq=kmq)
    gm = run_all(s, prec, non_loc=nl, kminusq=kmq)
    emax, erms, enorm = errors(gm, g64)
    print(f"{name} {prec}: max {emax:.2e} rms {erms:.2e} norm {enorm:.2e}")
    # complex-norm error: split-f16 carries ~22 significand bits, split-bf16 ~16
    assert enorm < (2e-6 if prec == "mixed_f16" else 2e-5), enorm
    assert erms < (2e-5 if prec == "mixed_f16" else 2e-4), erms


@pytest.mark.parametrize("stage", ["64", "32"])
@pytest.mark.parametrize("name", ["c0", "soc_tr", "l12_small"])
def test_mixed_both_stage_sizes(name, stage, monkeypatch):
    """The tensor-core sandwich with 64- and 32-point pipeline stages (the
    latter is what wide tiles use) against the FP64 form."""
    monkeypatch.setenv("LELPH_TC_STAGE", stage)
    s, _, kmq, nl = load(name)
    g64 = run_all(s, "fp64", non_loc=nl, kminusq=kmq)
    g = run_all(s, "mixed_f16", non_loc=nl, kminusq=kmq)
    emax, erms, enorm = errors(g, g64)
    assert enorm < 2e-6, enorm
    assert erms < 2e-5, erms


def test_c64_output_matches_c128():
    s, g_ref, kmq, nl = load("c0")
    g = run_all(s, "mixed", out=OUT_C64)
    assert g.dtype == np.complex64
    assert np.linalg.norm((g - g_ref).ravel()) / np.linalg.norm(g_ref.ravel()) < 2e-6


@pytest.mark.parametrize("name", ["c0", "soc_tr", "lsda"])
def test_c64_epilogue_matches_c128_epilogue(name):
    """The mixed form's complex64 output (float error-free epilogue: TwoSum of
    the chunk partials, exact FMA products, 1/M as a float pair) against its
    complex128 output (FP64 epilogue) from the same partial sums: one value
    rounded once to float, so they differ by at most an ulp of float, plus
    2^-40 of max|g| where the local and nonlocal terms cancel."""
    s, _, kmq, nl = load(name)
    g128 = run_all(s, "mixed_f16", non_loc=nl, kminusq=kmq)
    g64 = run_all(s, "mixed_f16", non_loc=nl, kminusq=kmq, out=OUT_C64)
    assert g64.dtype == np.complex64 and g128.dtype == np.complex128
    ref = g128.astype(np.complex64).astype(np.complex128)
    d = np.maximum(np.abs(g64.real - ref.real), np.abs(g64.imag - ref.imag))
    bound = 2.0**-22 * np.maximum(np.abs(g128.real), np.abs(g128.imag)) + 2.0**-40 * np.abs(g128).max()
    assert np.all(d <= bound), (d / bound).max()


def test_l12_at_bench_grid_against_oracle():
    # the 4-atom cell on its 48^3 grid with npw ~2500, a few pairs of two q
    s = synth.make_system("c1", {"nbnds": 8, "qpts": [(0.125, 0, 0), (0.25, 0.125, 0.125)]})
    ks = [0, 77, 300, 511]
    with LelphGPU(s, "fp64") as c64, LelphGPU(s, "mixed") as cm:
        for iq in range(2):
            c64.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
            cm.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
        for iq in range(2):
            ref = O.compute_elphq(s, iq, k_list=ks)
            g = c64.run([iq] * len(ks), ks)
            assert np.abs(g - ref).max() / np.abs(ref).max() < FP64_TOL
            gm = cm.run([iq] * len(ks), ks)
            assert np.linalg.norm((gm - ref).ravel()) / np.linalg.norm(ref.ravel()) < 2e-6


def test_q_rotate_matches_reference():
    import os
    from golden_util import GOLDEN_DIR
    z = np.load(os.path.join(GOLDEN_DIR, "q_rotate.npz"))
    s = synth.make_system("c0", {"nbnds": 5})
    with LelphGPU(s, "fp64") as ctx:
        for trev, key in ((0, "out_notr"), (1, "out_tr")):
            out = ctx.elph_q_rotate(z["Dl"], z["g"], z["Dr"], trev)
            assert np.abs(out - z[key]).max() < 1e-12 * np.abs(z[key]).max()


def test_errors_are_statuses_not_aborts():
    s = synth.make_system("c0", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)], "nbnds": 2})
    with LelphGPU(s, "fp64") as ctx:
        with pytest.raises(LelphError) as e:
            ctx.run([0], [0])                      # q slot never loaded
        assert e.value.status == -6
        ctx.set_q(0, [0.25, 0, 0], s.eigVec[0], s.dVscf[0])   # q not on the 2x2x2 grid
        with pytest.raises(LelphError) as e:
            ctx.run([0], [0])
        assert e.value.status == -5
        ctx.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        g = ctx.run([0], [1])                      # context still usable
        assert np.isfinite(g).all()
