"""Preparation of the mixed real-space route, first and later calls.

The first preparation clears every box and records, per full-BZ k, which
z-columns and x planes its sphere occupies; later preparations zero only the
occupied columns before the scatter, the y pass reads unoccupied columns as
zero and the x pass unoccupied planes, so stale data left in a box by another
k-point is never read.  A context prepared again on other wavefunctions of
the same geometry must give the bits of a fresh context on those
wavefunctions, with one chunk of boxes and with several (the chunk's k-points
share the boxes of the previous chunk's).
"""
import dataclasses

import numpy as np
import pytest

from golden_util import load
from letzelphc_gb300.elph import LelphGPU

pytestmark = pytest.mark.gpu


def run(ctx, s):
    for iq in range(len(s.qpts)):
        ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
    qs = np.repeat(np.arange(len(s.qpts)), s.nk_bz)
    ks = np.tile(np.arange(s.nk_bz), len(s.qpts))
    return ctx.run(qs, ks)


@pytest.mark.parametrize("chunk_k", [None, 3])
@pytest.mark.parametrize("name", ["c0", "soc_tr"])
def test_second_preparation_matches_a_fresh_context(name, chunk_k, monkeypatch):
    if chunk_k:
        monkeypatch.setenv("LELPH_PREP_CHUNK_K", str(chunk_k))
    s, _, _, _ = load(name)
    # other wavefunctions, same geometry: the bands in reverse order, a phase
    w2 = [np.ascontiguousarray(w[:, ::-1] * np.exp(0.7j)) for w in s.wfc]
    s2 = dataclasses.replace(s, wfc=w2)
    with LelphGPU(s, "mixed_f16", route="real") as ctx:
        g_first = run(ctx, s)
        ctx.set_wavefunctions(w2)
        g_again = run(ctx, s2)
    with LelphGPU(s2, "mixed_f16", route="real") as fresh:
        g_fresh = run(fresh, s2)
    assert np.isfinite(g_again).all()
    assert np.array_equal(g_again, g_fresh)
    assert not np.array_equal(g_first, g_again)
