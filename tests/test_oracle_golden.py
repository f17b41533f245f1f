"""The CPU restatement (oracle/elph_oracle.py) against the reference's own
output (tests/golden/, made by the compiled reference, FP64 build)."""
import numpy as np
import pytest

import elph_oracle as O
from golden_util import DVLOC_NAMES, NAMES, load, load_dvloc


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference(name):
    s, g_ref, kmq, nl = load(name)
    g = np.array([O.compute_elphq(s, iq, non_loc=nl, kminusq=kmq) for iq in range(len(s.qpts))])
    err = np.abs(g - g_ref).max() / np.abs(g_ref).max()
    assert err < 1e-12, err


@pytest.mark.parametrize("name", DVLOC_NAMES)
def test_local_bare_potential_matches_reference(name):
    """V_loc table + dVlocq + add_dvscf_qe, then the stage on the summed dV."""
    s, z = load_dvloc(name)
    step = int(z["sample"])
    tab = O.vloc_table(s, np.ceil(np.abs(s.qpts).max()) + 1)
    g = []
    for iq in range(len(s.qpts)):
        v = O.dvlocq(s, s.qpts[iq], s.eigVec[iq], tab).reshape(-1)
        dv = O.add_dvscf_qe(s.dVscf[iq], v.reshape(s.nmodes, *s.fft_dims), s.nmag)
        assert np.abs(v[::step] - z["vloc_sample"][iq]).max() < 1e-12 * np.abs(z["vloc_sample"][iq]).max()
        assert abs(np.linalg.norm(v) - z["vloc_norm"][iq]) < 1e-12 * z["vloc_norm"][iq]
        flat = dv.reshape(-1)
        assert np.abs(flat[::step] - z["dv_sample"][iq]).max() < 1e-12 * np.abs(z["dv_sample"][iq]).max()
        assert abs(np.linalg.norm(flat) - z["dv_norm"][iq]) < 1e-12 * z["dv_norm"][iq]
        g.append(O.compute_elphq(s, iq, dVscfq=dv, non_loc=True))
    g = np.array(g)
    assert np.abs(g - z["g"]).max() < 1e-12 * np.abs(z["g"]).max()


def test_q_rotate_matches_reference():
    import os
    from golden_util import GOLDEN_DIR
    z = np.load(os.path.join(GOLDEN_DIR, "q_rotate.npz"))
    for trev, key in ((False, "out_notr"), (True, "out_tr")):
        out = O.elph_q_rotate(z["Dl"], z["g"], z["Dr"], trev)
        assert np.abs(out - z[key]).max() < 1e-12 * np.abs(z[key]).max()


def test_synthetic_generator_shapes():
    from letzelphc_gb300 import synth
    s = synth.make_system("c0")
    assert s.nk_bz == 64 and s.nk_ibz == 8 and len(s.sym_R) == 48
    assert 360 <= s.npw.min() and s.npw.max() <= 440
    # bz_expand's kmap reproduces every full-BZ point from its iBZ point
    for i, (ik, isym) in enumerate(s.kmap):
        k = s.alat.T @ (s.sym_R[isym] @ s.kibz[ik])
        assert np.allclose(k, s.kbz_crys[i])


def _rotdv_cases():
    import json
    import os
    from golden_util import GOLDEN_DIR
    z = np.load(os.path.join(GOLDEN_DIR, "rotate_dvscf.npz"))
    return z, json.loads(str(z["cases"])), json.loads(str(z["systems"]))


def rotdv_system(systems, name):
    from letzelphc_gb300 import synth
    base, ov = systems[name]
    ov = {k: (tuple(v) if isinstance(v, list) and k in ("kgrid", "fft", "ls") else v) for k, v in ov.items()}
    return synth.make_system(base, ov)


def test_rotate_dvscf_matches_reference():
    """Box permutation bit-exact, rotated dV to 1e-12 (src/symmetries/rotate_dvscf.c)."""
    z, cases, systems = _rotdv_cases()
    cache = {}
    for sysname, isym, trev_ov, comp in cases:
        s = cache.setdefault(sysname, rotdv_system(systems, sysname))
        trev = int(s.sym_trev[isym]) if trev_ov is None else trev_ov
        key = f"{sysname}_{isym}_{trev}_{comp}"
        if key + "_idx" in z.files:
            idx = O.rotate_dvscf_index(s, s.sym_R[isym], s.sym_tau[isym], trev)
            assert np.array_equal(idx, z[key + "_idx"]), key
        out = O.rotate_dvscf(s, s.qpts[0], s.dVscf[0], s.sym_R[isym], s.sym_tau[isym], trev, comp)
        smp = z[key + "_sample"]
        assert np.abs(out.reshape(-1)[::97] - smp).max() < 1e-12 * np.abs(smp).max(), key
        assert abs(np.linalg.norm(out) - float(z[key + "_norm"])) < 1e-12 * float(z[key + "_norm"])


def test_dmats_match_reference():
    """electronic_reps (src/symmetries/elec_reps.c:16-413) for every
    (symmetry, full-BZ k) pair: stored pairs to 1e-12, norms of all pairs to
    1e-12; the systems cover time reversal, fractional translations, spinors,
    two spins and k-points with different plane-wave spheres."""
    from golden_util import load_dmats
    z, systems = load_dmats()
    st = int(z["stride"])
    for name, s in systems.items():
        D = O.dmats(s).reshape(-1, s.nspin, s.nbnds, s.nbnds)
        ref = z[name + "_sub"]
        assert np.abs(D[::st] - ref).max() < 1e-12, name
        nrm = np.linalg.norm(D.reshape(len(D), -1), axis=1)
        assert np.abs(nrm - z[name + "_norm"]).max() < 1e-12, name


def test_qstar_expansion_matches_reference():
    """The stage's q-star loop (src/elph/compute_elph_matq.c:159-217, Dmats from
    electronic_reps): every star member at every S k to 1e-12 of max|g|, with
    time reversal, the k-q convention and spinors among the systems."""
    from golden_util import STAR_NAMES, load_star
    for name in STAR_NAMES:
        z, s, kmq = load_star(name)
        D = O.dmats(s).reshape(len(s.sym_R), s.nk_bz, s.nspin, s.nbnds, s.nbnds)
        ns, qs = z["nqstar"], z["qsym"]
        stars = [O.q_star(s, q) for q in s.qpts]
        assert [len(m) for m, _ in stars] == list(ns), name
        assert np.array_equal(np.concatenate([sy for _, sy in stars]), qs), name
        ref = z["g"]
        pos = 0
        for iq in range(len(s.qpts)):
            g = O.compute_elphq_star(s, iq, qs[pos:pos + ns[iq]], D, kminusq=kmq)
            r = ref[pos:pos + ns[iq]]
            assert np.abs(g - r).max() < 1e-12 * np.abs(r).max(), (name, iq)
            pos += ns[iq]


def test_dvscf_ingest_matches_reference():
    """read_dvscf_qe (src/io/qe/read_dvscf.c:15-172): transpose of QE's layout and
    pattern -> mode basis, samples and per-mode norms to 1e-12 (nmag 1, 2, 4 and
    a box whose sides are not multiples of the device tile)."""
    from golden_util import load_dvscf_qe
    z, cases = load_dvscf_qe()
    st = int(z["sample"])
    for name, (s, raw, pats) in cases.items():
        out = O.read_dvscf_qe(raw, s.eigVec[0], pats, s.nmag, s.fft_dims).reshape(-1)
        smp = z[name + "_sample"]
        assert np.abs(out[::st] - smp).max() < 1e-12 * np.abs(smp).max(), name
        nrm = np.linalg.norm(out.reshape(s.nmodes, -1), axis=1)
        assert np.abs(nrm - z[name + "_norm"]).max() < 1e-12 * nrm.max(), name


@pytest.mark.parametrize("name", NAMES)
def test_reference_single_precision_build_fixture(name):
    """ref_f32.npz holds the reference's default single-precision build
    (src/elphC.h:21-31) on the inputs of the FP64 fixtures: it must differ from
    the FP64 build like a single-precision result does (not be an FP64 copy,
    not be wrong), since the GPU tests use its error as the yardstick of the
    mixed form."""
    from golden_util import errors, load_f32
    s, g32, _, _ = load_f32(name)
    _, g64, _, _ = load(name)
    emax, erms, enorm = errors(g32, g64)
    assert g32.dtype == np.complex64 and g32.shape == g64.shape
    assert 1e-8 < enorm < 1e-5, enorm
    assert erms < 1e-4 and emax > 1e-7, (emax, erms)
