"""GPU parity of the local bare potential added per q before the stage.

The reference computes, per q, dVlocq (src/dvloc/dVbare_loc.c:16-231) from a
V_loc(|G|) table (create_vlocg_table, src/dvloc/vlocg_table.c:16-154) and adds
it to QE's induced dV_scf with add_dvscf_qe (src/dvloc/add_dvscf.c:12-92)
before compute_and_write_elphq (src/elph/elph_driver.c:234-306).  Here:

* lelph_gpu_dvlocq against the oracle (all points) and against the compiled
  reference's samples in tests/golden/dvloc_*.npz, FP64, 1e-10 relative;
* lelph_gpu_set_q_induced + run (FP64 form) against the reference's matrix
  elements computed from the summed dV, 1e-10 relative to max|g|;
* the mixed form on the summed dV against the FP64 form (the mixed-form
  tolerances of test_gpu_parity.py);
* the bare kernels (no induced part) against the oracle;
* call-order errors as status codes.
"""
import numpy as np
import pytest

import elph_oracle as O
from golden_util import DVLOC_NAMES, load_dvloc
from letzelphc_gb300.elph import LelphError, LelphGPU

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def _all_pairs(s):
    nk = s.nk_bz
    return np.repeat(np.arange(len(s.qpts)), nk), np.tile(np.arange(nk), len(s.qpts))


@pytest.mark.parametrize("name", DVLOC_NAMES)
def test_dvlocq_matches_oracle_and_reference(name):
    s, z = load_dvloc(name)
    step = int(z["sample"])
    tab = O.vloc_table(s, np.ceil(np.abs(s.qpts).max()) + 1)
    with LelphGPU(s, "fp64") as ctx:
        ctx.set_local_pseudo()
        for iq in range(len(s.qpts)):
            v = ctx.dvlocq(s.qpts[iq], s.eigVec[iq])
            ref = O.dvlocq(s, s.qpts[iq], s.eigVec[iq], tab)
            err = np.abs(v - ref).max() / np.abs(ref).max()
            assert err < FP64_TOL, (name, iq, err)
            flat = v.reshape(-1)
            zs = z["vloc_sample"][iq]
            assert np.abs(flat[::step] - zs).max() < FP64_TOL * np.abs(zs).max()


@pytest.mark.parametrize("name", DVLOC_NAMES)
def test_set_q_induced_fp64_matches_reference(name):
    s, z = load_dvloc(name)
    qs, ks = _all_pairs(s)
    with LelphGPU(s, "fp64") as ctx:
        ctx.set_local_pseudo()
        for iq in range(len(s.qpts)):
            ctx.set_q_induced(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
        g = ctx.run(qs, ks, non_loc=True).reshape(z["g"].shape)
    err = np.abs(g - z["g"]).max() / np.abs(z["g"]).max()
    assert err < FP64_TOL, err


@pytest.mark.parametrize("name", ["dvloc_c0", "dvloc_lsda"])
def test_set_q_induced_mixed_matches_fp64(name):
    s, z = load_dvloc(name)
    qs, ks = _all_pairs(s)
    with LelphGPU(s, "mixed_f16") as ctx:
        ctx.set_local_pseudo()
        for iq in range(len(s.qpts)):
            ctx.set_q_induced(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
        g = ctx.run(qs, ks, non_loc=True).reshape(z["g"].shape)
    ref = z["g"]
    a, b = np.abs(g), np.abs(ref)
    e = np.abs(a - b) / np.maximum(b, 1e-6 * b.max())
    norm = np.linalg.norm((g - ref).ravel()) / np.linalg.norm(ref.ravel())
    assert norm < 2e-6, norm                       # split-f16 bar of the mixed form
    assert np.sqrt(np.mean(e * e)) < 2e-5


def test_bare_kernel_matches_oracle():
    """kernel 'bare': no induced part, dV = dV_loc only (src/elph/set_kernel.c:18-51)."""
    s, _ = load_dvloc("dvloc_c0")
    tab = O.vloc_table(s, np.ceil(np.abs(s.qpts).max()) + 1)
    qs, ks = _all_pairs(s)
    with LelphGPU(s, "fp64") as ctx:
        ctx.set_local_pseudo()
        for iq in range(len(s.qpts)):
            ctx.set_q_induced(iq, s.qpts[iq], s.eigVec[iq], None)
        g = ctx.run(qs, ks, non_loc=False)
    ref = []
    for iq in range(len(s.qpts)):
        v = O.dvlocq(s, s.qpts[iq], s.eigVec[iq], tab)
        dv = O.add_dvscf_qe(np.zeros_like(s.dVscf[iq]), v, s.nmag)
        ref.append(O.compute_elphq(s, iq, dVscfq=dv, non_loc=False))
    ref = np.array(ref).reshape(g.shape)
    assert np.abs(g - ref).max() < FP64_TOL * np.abs(ref).max()


def test_local_potential_call_order_errors():
    s, _ = load_dvloc("dvloc_c0")
    with LelphGPU(s, "fp64") as ctx:
        with pytest.raises(LelphError) as e:
            ctx.dvlocq(s.qpts[0], s.eigVec[0])
        assert e.value.status == -6
        with pytest.raises(LelphError) as e:
            ctx.set_q_induced(0, s.qpts[0], s.eigVec[0], None)
        assert e.value.status == -6
