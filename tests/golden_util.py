"""Helpers to load the golden fixtures (tests/golden/*.npz) and rebuild the
synthetic system each was generated from."""
import json
import os

import numpy as np

from letzelphc_gb300 import synth

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["c0", "c0_local", "zb_tr", "zb_tr_kmq", "lsda", "soc_tr", "spinor_nosoc", "l12_small"]
# fixtures whose dVscf is the induced part; the reference added the local bare potential
DVLOC_NAMES = ["dvloc_c0", "dvloc_2d", "dvloc_lsda", "dvloc_soc"]


def load(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    spec = json.loads(str(z["spec"]))
    ov = {k: (tuple(v) if isinstance(v, list) and k in ("kgrid", "fft", "ls") else v)
          for k, v in spec["overrides"].items()}
    s = synth.make_system(spec["base"], ov)
    # the regenerated inputs must be the ones the fixture was made from
    assert np.allclose([np.abs(w).sum() for w in s.wfc], z["wfc_sum"], rtol=1e-12)
    assert np.isclose(np.abs(s.dVscf).sum(), float(z["dv_sum"]), rtol=1e-12)
    return s, z["g"], bool(spec["kminusq"]), bool(spec["non_loc"])


def load_dvloc(name):
    """(system, fixture) of a dvloc_* fixture: g from the summed dV, every
    `sample`-th element of V_loc(r) and of the summed dV per q, their norms."""
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    s, _, _, _ = load(name)
    return s, z


def load_dmats():
    """(npz, {name: System}) of tests/golden/dmats.npz: D of the reference's
    electronic_reps for every (symmetry, full-BZ k) pair of each system,
    every ``stride``-th pair stored whole and the norms of all of them."""
    import json
    from letzelphc_gb300 import synth
    z = np.load(os.path.join(GOLDEN_DIR, "dmats.npz"))
    systems = {}
    for name, (base, ov) in json.loads(str(z["systems"])).items():
        ov = {k: (tuple(v) if isinstance(v, list) and k in ("kgrid", "fft", "ls", "npw") else v)
              for k, v in ov.items()}
        systems[name] = synth.make_system(base, ov)
    return z, systems


STAR_NAMES = ["star_c0", "star_zb_tr_kmq", "star_l12", "star_soc"]


def load_star(name):
    """(npz, System, kminusq) of a q-star fixture: g of every star member
    from the reference's stage, with the stars (nqstar, qsym) it used."""
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    spec = json.loads(str(z["spec"]))
    ov = {k: (tuple(v) if isinstance(v, list) and k in ("kgrid", "fft", "ls", "npw") else v)
          for k, v in spec["overrides"].items()}
    return z, synth.make_system(spec["base"], ov), bool(spec["kminusq"])


def load_dvscf_qe():
    """(npz, {name: (System, raw, pats)}) of tests/golden/dvscf_qe.npz: the
    QE-layout dvscf inputs are regenerated from their seeds (the arithmetic of
    tests/golden/make_golden.py:dvscf_inputs)."""
    z = np.load(os.path.join(GOLDEN_DIR, "dvscf_qe.npz"))
    out = {}
    for name, (base, ov, seed) in json.loads(str(z["systems"])).items():
        ov = {k: (tuple(v) if isinstance(v, list) and k in ("kgrid", "fft", "ls", "npw") else v)
              for k, v in ov.items()}
        s = synth.make_system(base, ov)
        rng = np.random.default_rng(seed)
        Nx, Ny, Nz = s.fft_dims
        nm = s.nmodes
        raw = rng.standard_normal((nm, s.nmag, Nz, Ny, Nx)) + 1j * rng.standard_normal((nm, s.nmag, Nz, Ny, Nx))
        pats = np.linalg.qr(rng.standard_normal((nm, nm)) + 1j * rng.standard_normal((nm, nm)))[0]
        out[name] = (s, raw, pats)
    return z, out


def load_f32(name):
    """(system, g32, kminusq, non_loc) of one system of tests/golden/ref_f32.npz:
    the output of the reference's default single-precision build (complex64,
    the first nk k-points of each q when the fixture was a k-pool sample)."""
    z = np.load(os.path.join(GOLDEN_DIR, "ref_f32.npz"))
    spec = json.loads(str(z[name + "_spec"]))
    ov = {k: (tuple(v) if isinstance(v, list) and k in ("kgrid", "fft", "ls") else v)
          for k, v in spec["overrides"].items()}
    if "qpts" in ov:
        ov["qpts"] = [tuple(q) for q in ov["qpts"]]
    s = synth.make_system(spec["base"], ov)
    assert np.allclose([np.abs(w).sum() for w in s.wfc], z[name + "_wfc_sum"], rtol=1e-12)
    assert np.isclose(np.abs(s.dVscf).sum(), float(z[name + "_dv_sum"]), rtol=1e-12)
    return s, z[name + "_g32"], bool(spec["kminusq"]), bool(spec["non_loc"])


def errors(g, ref):
    """The metric's error of g against ref: e_i = ||g_i| - |ref_i|| /
    max(|ref_i|, 1e-6 max|ref|); returns (max e, RMS e, ||g - ref|| / ||ref||)."""
    a, b = np.abs(g), np.abs(ref)
    e = np.abs(a - b) / np.maximum(b, 1e-6 * b.max())
    return float(e.max()), float(np.sqrt(np.mean(e * e))), float(np.linalg.norm((g - ref).ravel()) /
                                                                np.linalg.norm(ref.ravel()))


def load_f32_stats(name):
    """(system, (max, RMS, norm), nk) of a stats-only entry of ref_f32.npz: the
    error of the reference's single-precision build against its double build
    on the first nk k-points of the system's q."""
    z = np.load(os.path.join(GOLDEN_DIR, "ref_f32.npz"))
    spec = json.loads(str(z[name + "_spec"]))
    ov = {k: (tuple(v) if isinstance(v, list) and k in ("kgrid", "fft", "ls") else v)
          for k, v in spec["overrides"].items()}
    if "qpts" in ov:
        ov["qpts"] = [tuple(q) for q in ov["qpts"]]
    s = synth.make_system(spec["base"], ov)
    assert np.allclose([np.abs(w).sum() for w in s.wfc], z[name + "_wfc_sum"], rtol=1e-12)
    assert np.isclose(np.abs(s.dVscf).sum(), float(z[name + "_dv_sum"]), rtol=1e-12)
    return s, z[name + "_stats"], int(z[name + "_nk"])
