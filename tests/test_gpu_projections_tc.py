"""KB projections of the mixed form on the tensor cores (projections_tc.cu).

The mixed form computes Pi[k][row][set] = sum_G beta_row(G) conj(c^_set(G))
with the tcgen05 TF32-split kernel by default and with the SIMT kernel
(FP32 products, FP64 chunk sums) when LELPH_PROJ_TC=0.  Both enter the same
finish; the matrix elements of the two must agree to the TF32 split's
precision, and both must stay within the FP64 bounds the parity tests use.
Shapes: one projector tile with one drain group (c0, spinors with SOC, LSDA)
and the 16-atom cell (256 projector rows: two 128-row tiles, two drain
groups).
"""
import numpy as np
import pytest

from golden_util import load
from letzelphc_gb300 import synth
from letzelphc_gb300.elph import LelphGPU

pytestmark = pytest.mark.gpu


def run(s, prec, kmq=False, npairs=None):
    with LelphGPU(s, prec) as ctx:
        for iq in range(len(s.qpts)):
            ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
        nk = s.nk_bz if npairs is None else min(s.nk_bz, npairs)
        qs = np.repeat(np.arange(len(s.qpts)), nk)
        ks = np.tile(np.arange(nk), len(s.qpts))
        return ctx.run(qs, ks, non_loc=True, kminusq=kmq)


def norm_err(g, ref):
    return np.linalg.norm((g - ref).ravel()) / np.linalg.norm(ref.ravel())


@pytest.mark.parametrize("name", ["c0", "soc_tr", "lsda", "zb_tr"])
def test_tensor_core_projections_match_simt(name, monkeypatch):
    s, _, kmq, _ = load(name)
    g64 = run(s, "fp64", kmq)
    monkeypatch.setenv("LELPH_PROJ_TC", "0")
    g_simt = run(s, "mixed_f16", kmq)
    monkeypatch.setenv("LELPH_PROJ_TC", "1")
    g_tc = run(s, "mixed_f16", kmq)
    d = np.abs(g_tc - g_simt).max() / np.abs(g64).max()
    e_tc, e_simt = norm_err(g_tc, g64), norm_err(g_simt, g64)
    print(f"{name}: max|tc - simt|/max|g| {d:.2e}; norm error vs FP64 tc {e_tc:.2e} simt {e_simt:.2e}")
    # the two differ by the TF32 split (hi + lo carries about 2^-22 of each operand)
    # and the order of the sums; the tensor-core form's error against FP64 is that
    # of the SIMT form
    assert d < 1e-6, d
    assert e_tc < 2e-6 and e_tc < 1.25 * e_simt + 5e-8, (e_tc, e_simt)


def test_tensor_core_projections_two_tiles(monkeypatch):
    # 16 atoms, l = 0, 1 projectors: 256 rows -> two 128-row tiles, two drain groups
    s = synth.make_system("c4", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)], "nbnds": 24, "fft": (48, 48, 48),
                                 "npw": 1500})
    g64 = run(s, "fp64", npairs=2)
    monkeypatch.setenv("LELPH_PROJ_TC", "0")
    g_simt = run(s, "mixed_f16", npairs=2)
    monkeypatch.setenv("LELPH_PROJ_TC", "1")
    g_tc = run(s, "mixed_f16", npairs=2)
    d = np.abs(g_tc - g_simt).max() / np.abs(g64).max()
    e_tc, e_simt = norm_err(g_tc, g64), norm_err(g_simt, g64)
    print(f"c4 cell: max|tc - simt|/max|g| {d:.2e}; norm error vs FP64 tc {e_tc:.2e} simt {e_simt:.2e}")
    assert d < 1e-6, d
    assert e_tc < 2e-6 and e_tc < 1.25 * e_simt + 5e-8, (e_tc, e_simt)
