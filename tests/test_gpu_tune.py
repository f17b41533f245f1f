"""lelph_gpu_tune: the measured choice of route and tile options.

Every candidate the system allows runs as its own context on real inputs; the
choice is the fastest measured, a context built with it computes the same
matrix elements as the automatic one, and a second call with the same cache
file returns the stored result without measuring."""
import os
import tempfile

import numpy as np
import pytest

from letzelphc_gb300 import synth
from letzelphc_gb300.elph import LelphGPU, tune

pytestmark = pytest.mark.gpu

ROUTE_OF = {"real": "real-space", "gspace": "G-space"}


def test_tune_mixed_picks_the_fastest_candidate_and_caches_it():
    s = synth.make_system("c0", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]})
    with tempfile.TemporaryDirectory() as d:
        cache = os.path.join(d, "tune.txt")
        t = tune(s, "mixed", npairs=4, cache_path=cache)
        assert not t["cached"]
        ms = t["ms_per_pair"]
        measured = {k: v for k, v in ms.items() if v > 0}
        assert measured, ms
        fastest = min(measured, key=measured.get)
        assert fastest.startswith(ROUTE_OF[t["route"]])
        if t["route"] == "real":
            assert t["tile_points"] in (32, 64) and t["gs_gemm"] == 0
        else:
            assert t["gs_gemm"] in (1, 2) and t["tile_points"] == 0
        assert ms["G-space, SIMT GEMM"] > 0 and ms["real-space, 32-point stages"] > 0
        t2 = tune(s, "mixed", npairs=4, cache_path=cache)
        assert t2["cached"] and t2["route"] == t["route"] and t2["tile_points"] == t["tile_points"]
        assert t2["gs_gemm"] == t["gs_gemm"]
    ks = list(range(s.nk_bz))
    with LelphGPU(s, "fp64") as c64, LelphGPU(s, "mixed", route=t["route"], tile_points=t["tile_points"],
                                               gs_gemm=t["gs_gemm"]) as cm:
        for c in (c64, cm):
            c.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        g64 = c64.run([0] * len(ks), ks)
        gm = cm.run([0] * len(ks), ks)
    assert np.linalg.norm((gm - g64).ravel()) / np.linalg.norm(g64.ravel()) < 2e-6


def test_tune_fp64_has_one_kernel_per_route():
    s = synth.make_system("c0", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)], "nbnds": 4})
    t = tune(s, "fp64", npairs=2)
    ms = t["ms_per_pair"]
    assert ms["real-space, 64-point stages"] > 0 and ms["G-space, SIMT GEMM"] > 0
    assert ms["real-space, 32-point stages"] < 0 and ms["G-space, tensor-core GEMM"] < 0
