"""GPU parity at the shapes of the benchmark configurations, and at tensor-core
tile shapes whose mode tiles leave rows of the 128-row tile unused.

Every case runs the first k-points of one q (the reference's own k-pool split):
* FP64 form against the numpy oracle (a restatement of the reference pinned to
  its compiled output) on one or two pairs: <= 1e-10 relative to max|g|;
* mixed form (split-f16 tensor cores, FP32 FFTs) against the FP64 form on the
  same pairs, with the metric's error e_i = ||g_mixed| - |g_fp64|| /
  max(|g_fp64|, 1e-6 max|g_fp64|): RMS and complex-norm error <= 1e-5, and the
  maximum no larger than that of the reference's own default single-precision
  build (src/elphC.h:21-31) against its double build on the same pairs
  (tests/golden/ref_f32.npz, made by tests/golden/make_golden.py f32).

Shapes:
* tile48: 4-atom cell, 48 bands x 12 modes (two whole modes per tile, six
  tiles, 32 rows of the last one unused), 48^3 grid;
* tile36: 8-atom cell, 36 bands x 24 modes (three modes per tile, eight tiles);
* c1s: the 4-atom cell at its 32 bands and 48^3 grid (the bench's tile: four
  modes per tile, three tiles);
* c2s: the 3-atom hexagonal slab, 36 x 36 x 216 grid, 40 bands, npw 1800-2600;
* c3s: the 8-atom spinor cell with spin-orbit projectors, 60^3 grid, nmag 4,
  64 bands;
* c4s: the 16-atom cell on its 96^3 grid (60^3 product grid) through the
  G-space route's compile-time kernels, 80 bands (the oracle checks the FP64
  G-space route at 8 bands on the same grid).
"""
import numpy as np
import pytest

import elph_oracle as O
from golden_util import errors, load_f32, load_f32_stats
from letzelphc_gb300.elph import LelphGPU

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
METRIC_TOL = 1e-5   # the metric's bound, met by the RMS and the complex-norm error

# name -> (route of both forms, k-points checked against the oracle, band count
# of the oracle check when the oracle would take minutes at the full count)
CASES = {
    "tile48": ("real", [0, 1], None),
    "tile36": ("real", [0, 1], None),
    "c1s": ("real", [0, 3], None),
    "c2s": ("auto", [0], None),
    "c3s": ("auto", [0], 16),
}


def _load(name):
    """(system, nk, (max, rms, norm) of the reference's single-precision build)."""
    if name == "c1s":
        s, g32, _, _ = load_f32(name)
        return s, g32.shape[1], None, g32
    s, st, nk = load_f32_stats(name)
    return s, nk, st, None


@pytest.mark.parametrize("name", list(CASES))
def test_config_shape(name):
    route, ks_oracle, nb_oracle = CASES[name]
    s, nk, st, g32 = _load(name)
    ks = list(range(nk))
    with LelphGPU(s, "fp64", route=route) as c64:
        c64.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        g64 = c64.run([0] * nk, ks)
    if nb_oracle is None:
        ref = O.compute_elphq(s, 0, k_list=ks_oracle)
        err = np.abs(g64[ks_oracle] - ref).max() / np.abs(ref).max()
    else:
        # the same cell, grid, plane waves and q with fewer bands
        from letzelphc_gb300 import synth
        import json
        import os
        from golden_util import GOLDEN_DIR
        spec = json.loads(str(np.load(os.path.join(GOLDEN_DIR, "ref_f32.npz"))[name + "_spec"]))
        ov = dict(spec["overrides"], nbnds=nb_oracle)
        ov["qpts"] = [tuple(q) for q in ov["qpts"]]
        sb = synth.make_system(spec["base"], ov)
        with LelphGPU(sb, "fp64", route=route) as cb:
            cb.set_q(0, sb.qpts[0], sb.eigVec[0], sb.dVscf[0])
            gb = cb.run([0] * len(ks_oracle), ks_oracle)
        ref = O.compute_elphq(sb, 0, k_list=ks_oracle)
        err = np.abs(gb - ref).max() / np.abs(ref).max()
    assert err < FP64_TOL, err
    with LelphGPU(s, "mixed", route=route) as cm:
        cm.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        gm = cm.run([0] * nk, ks)
    emax, erms, enorm = errors(gm, g64)
    if g32 is not None:
        st = errors(g32[0], g64)
    print(f"{name}: mixed max {emax:.2e} rms {erms:.2e} norm {enorm:.2e}; "
          f"reference single-precision build max {st[0]:.2e} rms {st[1]:.2e} norm {st[2]:.2e}")
    assert erms < METRIC_TOL and enorm < METRIC_TOL, (erms, enorm)
    assert emax <= st[0], (emax, st[0])
    assert erms <= st[1] and enorm <= st[2], (erms, enorm, st)


def test_c4_grid_gspace_fp64_against_oracle():
    """The 16-atom cell on its 96^3 grid (60^3 product grid), FP64 G-space
    route, one pair at 8 bands against the oracle."""
    from letzelphc_gb300 import synth
    s = synth.make_system("c4", {"nbnds": 8, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]})
    with LelphGPU(s, "fp64", route="gspace") as c:
        c.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        g = c.run([0], [0])
        assert tuple(c.stats()["product_grid"]) == (60, 60, 60)
    ref = O.compute_elphq(s, 0, k_list=[0])
    assert np.abs(g - ref).max() / np.abs(ref).max() < FP64_TOL


def test_c4_grid_gspace_mixed_against_fp64():
    """The 16-atom cell at 80 bands on the G-space route: the mixed form runs
    the compile-time plane pass (60 x 60 planes, eight modes per CTA), the
    compile-time x pass and the 256-row FP32 GEMM tile of 40 bands; against
    the FP64 G-space route on the same pair, bounded like the other shapes by
    the reference's single-precision build."""
    s, st, nk = load_f32_stats("c4s")
    ks = list(range(nk))
    out = {}
    for prec in ("fp64", "mixed"):
        with LelphGPU(s, prec, route="gspace") as c:
            c.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
            out[prec] = c.run([0] * nk, ks)
            assert tuple(c.stats()["product_grid"]) == (60, 60, 60)
    emax, erms, enorm = errors(out["mixed"], out["fp64"])
    print(f"c4s: mixed max {emax:.2e} rms {erms:.2e} norm {enorm:.2e}; reference single-precision build "
          f"max {st[0]:.2e} rms {st[1]:.2e} norm {st[2]:.2e}")
    assert erms < METRIC_TOL and enorm < METRIC_TOL, (erms, enorm)
    assert emax <= st[0] and erms <= st[1] and enorm <= st[2], (emax, erms, enorm, st)
