"""GPU dV_scf ingest (read_dvscf_qe, src/io/qe/read_dvscf.c:15-172) through the
C ABI: the mode-basis dV from QE's (pattern, nmag, Nz, Ny, Nx) layout equals
the oracle on the whole box to 1e-12 and the reference's samples; a slot
loaded this way gives the same matrix elements as one loaded with the
converted dV through lelph_gpu_set_q (and, with induced, through
lelph_gpu_set_q_induced)."""
import numpy as np
import pytest

import elph_oracle as O
from golden_util import load_dvscf_qe
from letzelphc_gb300.elph import LelphGPU

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    return load_dvscf_qe()


@pytest.mark.parametrize("name", ["c0", "lsda", "soc", "hex_odd"])
def test_dvscf_ingest_matches_oracle_and_reference(golden, name):
    z, cases = golden
    s, raw, pats = cases[name]
    ref = O.read_dvscf_qe(raw, s.eigVec[0], pats, s.nmag, s.fft_dims)
    with LelphGPU(s, "fp64") as ctx:
        dv = ctx.set_q_dvscf_qe(0, s.qpts[0], s.eigVec[0], pats, raw, want_dv=True)
    assert np.abs(dv - ref).max() < 1e-12 * np.abs(ref).max(), name
    smp = z[name + "_sample"]
    assert np.abs(dv.reshape(-1)[::int(z["sample"])] - smp).max() < 1e-12 * np.abs(smp).max(), name


def test_ingested_slot_gives_same_matrix_elements(golden):
    z, cases = golden
    s, raw, pats = cases["c0"]
    dv = O.read_dvscf_qe(raw, s.eigVec[0], pats, s.nmag, s.fft_dims)
    with LelphGPU(s, "fp64") as ctx:
        ctx.set_q_dvscf_qe(0, s.qpts[0], s.eigVec[0], pats, raw)
        ctx.set_q(1, s.qpts[0], s.eigVec[0], dv)
        ks = np.arange(s.nk_bz, dtype=np.int32)
        g0 = ctx.run(np.zeros(s.nk_bz, np.int32), ks)
        g1 = ctx.run(np.ones(s.nk_bz, np.int32), ks)
        assert np.abs(g0 - g1).max() < 1e-12 * np.abs(g1).max()
        ctx.set_local_pseudo()
        ctx.set_q_dvscf_qe(0, s.qpts[0], s.eigVec[0], pats, raw, induced=True)
        ctx.set_q_induced(1, s.qpts[0], s.eigVec[0], dv)
        g0 = ctx.run(np.zeros(s.nk_bz, np.int32), ks)
        g1 = ctx.run(np.ones(s.nk_bz, np.int32), ks)
        assert np.abs(g0 - g1).max() < 1e-12 * np.abs(g1).max()
