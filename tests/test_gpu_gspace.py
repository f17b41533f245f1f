"""GPU parity of the G-space route of the local sandwich (the reference's own
order of work: forward FFT of dV psi_k pruned to the k+q sphere, GEMM over
the sphere), through the C ABI.

* FP64 form against the reference's own output (tests/golden/), tolerance
  1e-10 relative to max|g|, every golden system (spinors, SOC, LSDA,
  time reversal, k-q convention);
* mixed form (FP32 FFTs and GEMM, chunk sums in FP64) against the FP64
  real-space route, errors as e_i = ||g_mixed| - |g_fp64|| /
  max(|g_fp64|, 1e-6 max|g_fp64|) and the complex norm ratio;
* the automatic route choice: the mixed form above 64 bands (beyond the
  tensor-core tile of the real-space route) runs on the G-space route;
* the 4-atom cell on its 48^3 box against the oracle.
"""
import numpy as np
import pytest

import elph_oracle as O
from golden_util import NAMES, load
from letzelphc_gb300 import synth
from letzelphc_gb300.elph import LelphGPU, ROUTE_GSPACE, ROUTE_REAL

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def run_all(s, prec, route, non_loc=True, kminusq=False):
    with LelphGPU(s, prec, route=route) as ctx:
        for iq in range(len(s.qpts)):
            ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
        nk = s.nk_bz
        qs = np.repeat(np.arange(len(s.qpts)), nk)
        ks = np.tile(np.arange(nk), len(s.qpts))
        g = ctx.run(qs, ks, non_loc=non_loc, kminusq=kminusq)
        used = ctx.stats()["route"]
    return g.reshape(len(s.qpts), nk, *g.shape[1:]), used


def errors(g, ref):
    a, b = np.abs(g), np.abs(ref)
    floor = 1e-6 * b.max()
    e = np.abs(a - b) / np.maximum(b, floor)
    norm = np.linalg.norm((g - ref).ravel()) / np.linalg.norm(ref.ravel())
    return e.max(), np.sqrt(np.mean(e * e)), norm


@pytest.mark.parametrize("name", NAMES)
def test_gspace_fp64_matches_reference(name):
    s, g_ref, kmq, nl = load(name)
    g, used = run_all(s, "fp64", "gspace", non_loc=nl, kminusq=kmq)
    assert used == ROUTE_GSPACE
    err = np.abs(g - g_ref).max() / np.abs(g_ref).max()
    assert err < FP64_TOL, err


@pytest.mark.parametrize("name", ["c0", "zb_tr", "lsda", "soc_tr", "spinor_nosoc"])
def test_gspace_mixed_against_fp64(name):
    s, _, kmq, nl = load(name)
    g64, _ = run_all(s, "fp64", "real", non_loc=nl, kminusq=kmq)
    gm, used = run_all(s, "mixed", "gspace", non_loc=nl, kminusq=kmq)
    assert used == ROUTE_GSPACE
    emax, erms, enorm = errors(gm, g64)
    print(f"{name} gspace mixed: max {emax:.2e} rms {erms:.2e} norm {enorm:.2e}")
    # FP32 FFTs and FP32 products summed over 1024-point chunks, chunks in FP64
    assert enorm < 2e-6, enorm
    assert erms < 2e-5, erms


def test_auto_route_takes_gspace_above_64_bands():
    s = synth.make_system("c0", {"nbnds": 72, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]})
    with LelphGPU(s, "mixed") as cm, LelphGPU(s, "fp64") as c64:
        assert cm.stats()["route"] == ROUTE_GSPACE
        assert c64.stats()["route"] == ROUTE_REAL
        cm.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        c64.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        ks = list(range(s.nk_bz))
        gm = cm.run([0] * len(ks), ks)
        g64 = c64.run([0] * len(ks), ks)
    emax, erms, enorm = errors(gm, g64)
    assert enorm < 2e-6, enorm


def test_gspace_l12_at_bench_grid_against_oracle():
    # the 4-atom cell on its 48^3 box with npw ~2500, a few pairs of two q
    s = synth.make_system("c1", {"nbnds": 8, "qpts": [(0.125, 0, 0), (0.25, 0.125, 0.125)]})
    ks = [0, 77, 300, 511]
    with LelphGPU(s, "fp64", route="gspace") as c64, LelphGPU(s, "mixed", route="gspace") as cm:
        for iq in range(2):
            c64.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
            cm.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
        for iq in range(2):
            ref = O.compute_elphq(s, iq, k_list=ks)
            g = c64.run([iq] * len(ks), ks)
            assert np.abs(g - ref).max() / np.abs(ref).max() < FP64_TOL
            gm = cm.run([iq] * len(ks), ks)
            assert np.linalg.norm((gm - ref).ravel()) / np.linalg.norm(ref.ravel()) < 2e-6


def test_gspace_batch_order_independent():
    """Pairs are visited grouped by k (psi(r) once per k): a shuffled pair
    list gives the same rows in the caller's order."""
    s, _, _, _ = load("zb_tr")
    with LelphGPU(s, "fp64", route="gspace") as ctx:
        for iq in range(len(s.qpts)):
            ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
        nk = s.nk_bz
        qs = np.repeat(np.arange(len(s.qpts)), nk)
        ks = np.tile(np.arange(nk), len(s.qpts))
        g = ctx.run(qs, ks)
        perm = np.random.default_rng(3).permutation(len(qs))
        gp = ctx.run(qs[perm], ks[perm])
    assert np.array_equal(gp, g[perm])


@pytest.mark.parametrize("route", ["real", "gspace"])
def test_sixteen_atoms_against_oracle(route):
    """48 displacement components: the finish runs tiled over bands (the
    per-pair form holds at most 24); both routes, both forms, vs the oracle."""
    s = synth.make_system("c4", {"nbnds": 6, "npw": 300, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)],
                                 "fft": (24, 24, 24)})
    ks = list(range(s.nk_bz))
    ref = O.compute_elphq(s, 0, k_list=ks)
    with LelphGPU(s, "fp64", route=route) as c64, LelphGPU(s, "mixed", route=route) as cm:
        c64.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        cm.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        g = c64.run([0] * len(ks), ks)
        gm = cm.run([0] * len(ks), ks)
    assert np.abs(g - ref).max() / np.abs(ref).max() < FP64_TOL
    assert np.linalg.norm((gm - ref).ravel()) / np.linalg.norm(ref.ravel()) < 2e-6
