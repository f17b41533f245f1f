"""Generate the golden fixtures of tests/golden/ from the compiled reference.

Each fixture is a small seeded synthetic system (regenerated bit-for-bit by
letzelphc_gb300.synth.make_system from the spec stored in the fixture) and
the elph matrix elements that the reference's own per-q stage
(compute_and_write_elphq, src/elph/compute_elph_matq.c:20, FP64 build)
produced for it, run through oracle/_ref/lelph_ref (oracle/Makefile).
A second fixture pins elph_q_rotate (src/symmetries/elphq_expand.c:16), and
the dvloc_* fixtures pin the local bare potential added per q before the
stage (create_vlocg_table / dVlocq / add_dvscf_qe, src/dvloc/), with the
matrix elements computed from the summed dV; rotate_dvscf.npz pins
rotate_dvscf, dmats.npz the electronic representation matrices
(electronic_reps, src/symmetries/elec_reps.c:16) and star_*.npz the stage's
q-star expansion (src/elph/compute_elph_matq.c:159-217); dvscf_qe.npz pins
the dV_scf ingest (read_dvscf_qe, src/io/qe/read_dvscf.c:15); ref_f32.npz
holds the output of the reference's default single-precision build
(oracle/_ref/f32/lelph_ref, no -DCOMPILE_ELPH_DOUBLE, src/elphC.h:21-31) on two
systems, the yardstick for the error of the mixed form.

Run from the repo root after ``make -C oracle``:
    python tests/golden/make_golden.py            (every fixture)
    python tests/golden/make_golden.py dmats      (only dmats.npz)
    python tests/golden/make_golden.py star       (only star_*.npz)
    python tests/golden/make_golden.py dvscf      (only dvscf_qe.npz)
    python tests/golden/make_golden.py f32        (only ref_f32.npz; needs
        make -C oracle OUT=_ref/f32 DEFS= as well)
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from letzelphc_gb300 import synth  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "lelph_ref")

# name -> (base config, overrides, kminusq, non_loc)
GOLDEN = {
    "c0": ("c0", {}, False, True),
    "c0_local": ("c0", {}, False, False),
    "zb_tr": ("c0", {"kind": "zincblende", "timerev": True, "nbnds": 6}, False, True),
    "zb_tr_kmq": ("c0", {"kind": "zincblende", "timerev": True, "nbnds": 6}, True, True),
    "lsda": ("c0", {"nspin": 2, "nbnds": 4, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]}, False, True),
    "soc_tr": ("c0", {"kind": "zincblende", "timerev": True, "nspinor": 2, "nmag": 4, "soc": True,
                      "ls": (0, 1, 2), "nbnds": 2, "npw": 150, "fft": (20, 20, 20), "kgrid": (4, 4, 4),
                      "qpts": [(0.25, 0.25, 0)]}, False, True),
    "spinor_nosoc": ("c0", {"nspinor": 2, "nmag": 1, "nbnds": 4, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)],
                            "ls": (0, 1, 2)}, False, True),
    "l12_small": ("c1", {"nbnds": 6, "kgrid": (2, 2, 2), "npw": 300, "fft": (24, 24, 24),
                         "qpts": [(0.5, 0, 0), (0.5, 0.5, 0.5)]}, False, True),
}


def run(name, base, ov, kmq, nl, tmp):
    s = synth.make_system(base, dict(ov))
    sysf = os.path.join(tmp, name + ".bin")
    gf = os.path.join(tmp, name + "_g.bin")
    synth.write_system(s, sysf, kminusq=kmq, non_loc=nl)
    subprocess.run([REF, sysf, gf], check=True)
    g = synth.read_g(gf, s, len(s.qpts))
    spec = json.dumps({"base": base, "overrides": ov, "kminusq": kmq, "non_loc": nl})
    np.savez(os.path.join(ROOT, "tests", "golden", name + ".npz"), g=g, spec=np.array(spec),
             wfc_sum=np.array([np.abs(w).sum() for w in s.wfc]), dv_sum=np.abs(s.dVscf).sum())
    print(name, g.shape, float(np.abs(g).max()))


# systems whose dVscf is the induced part: the reference adds the local bare
# potential (create_vlocg_table, dVlocq, add_dvscf_qe) before the stage
# name -> (base config, overrides, kminusq, non_loc)
GOLDEN_DVLOC = {
    "dvloc_c0": ("c0", {"kgrid": (2, 2, 2), "nbnds": 4, "qpts": [(0, 0, 0), (0.5, 0, 0)]}, False, True),
    "dvloc_2d": ("c2", {"kgrid": (3, 3, 1), "fft": (15, 15, 60), "nbnds": 4, "npw": 100,
                        "qpts": [(1 / 3, 0, 0)]}, False, True),
    "dvloc_lsda": ("c0", {"nspin": 2, "nbnds": 4, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]}, False, True),
    "dvloc_soc": ("c0", {"kind": "zincblende", "timerev": True, "nspinor": 2, "nmag": 4, "soc": True,
                         "ls": (0, 1, 2), "nbnds": 2, "npw": 150, "fft": (20, 20, 20), "kgrid": (2, 2, 2),
                         "qpts": [(0.5, 0.5, 0)]}, False, True),
}
SAMPLE = 4099  # every SAMPLE-th element of V_loc(r) and of the summed dV is stored


def run_dvloc(name, base, ov, kmq, nl, tmp):
    s = synth.make_system(base, dict(ov))
    sysf = os.path.join(tmp, name + ".bin")
    gf = os.path.join(tmp, name + "_g.bin")
    vf = os.path.join(tmp, name + "_v.bin")
    synth.write_system(s, sysf, kminusq=kmq, non_loc=nl)
    subprocess.run([REF, sysf, gf, "dvloc", vf], check=True)
    g = synth.read_g(gf, s, len(s.qpts))
    N = int(np.prod(s.fft_dims))
    raw = np.fromfile(vf, np.complex128).reshape(len(s.qpts), -1)
    vloc = raw[:, :s.nmodes * N]
    dv = raw[:, s.nmodes * N:]
    spec = json.dumps({"base": base, "overrides": ov, "kminusq": kmq, "non_loc": nl})
    np.savez(os.path.join(ROOT, "tests", "golden", name + ".npz"), g=g, spec=np.array(spec),
             vloc_sample=vloc[:, ::SAMPLE], dv_sample=dv[:, ::SAMPLE], sample=np.array(SAMPLE),
             vloc_norm=np.linalg.norm(vloc, axis=1), dv_norm=np.linalg.norm(dv, axis=1),
             wfc_sum=np.array([np.abs(w).sum() for w in s.wfc]), dv_sum=np.abs(s.dVscf).sum())
    print(name, g.shape, float(np.abs(g).max()), float(np.abs(vloc).max()))


# rotate_dvscf (src/symmetries/rotate_dvscf.c:22) cases:
# name -> (base config, overrides, symmetry index, time-reversal override, composite form)
ROTDV_SYS = {
    "c0": ("c0", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]}),
    "soc": ("c0", {"kind": "zincblende", "timerev": True, "nspinor": 2, "nmag": 4, "soc": True, "ls": (0, 1, 2),
                   "nbnds": 2, "npw": 150, "fft": (20, 20, 20), "kgrid": (2, 2, 2), "qpts": [(0.5, 0.5, 0)]}),
}
ROTDV_CASES = [("c0", 5, None, 0), ("c0", 24, None, 0), ("c0", 47, None, 0), ("c0", 7, 1, 0),
               ("soc", 3, None, 0), ("soc", 11, None, 1), ("soc", 47, None, 0), ("soc", 47, None, 1)]


def rotdv_fixture(tmp):
    """Outputs of the reference's rotate_dvscf and the box permutation it used,
    recovered exactly from its output (the inputs are distinct random values)."""
    rec = {}
    for sysname, isym, trev_ov, comp in ROTDV_CASES:
        base, ov = ROTDV_SYS[sysname]
        s = synth.make_system(base, dict(ov))
        sysf = os.path.join(tmp, "rot_" + sysname + ".bin")
        synth.write_system(s, sysf)
        R, tau = s.sym_R[isym], s.sym_tau[isym]
        trev = int(s.sym_trev[isym]) if trev_ov is None else trev_ov
        dv = s.dVscf[0]
        spec = os.path.join(tmp, "rotspec.bin")
        with open(spec, "wb") as f:
            f.write(b"LELPHSYS")
            synth._rec(f, "rq", np.asarray(s.qpts[0], float))
            synth._rec(f, "rR", np.asarray(R, float))
            synth._rec(f, "rtau", np.asarray(tau, float))
            synth._rec(f, "rtrev", np.array([trev], np.int32))
            synth._rec(f, "rcomp", np.array([comp], np.int32))
            synth._rec(f, "rdv", dv)
            f.write(b"END\0" + b"\0" * 28)
        out_f = os.path.join(tmp, "rotout.bin")
        subprocess.run([REF, sysf, os.path.join(tmp, "unused.bin"), "rotdv", spec, out_f], check=True)
        out = np.fromfile(out_f, np.complex128).reshape(dv.shape)
        key = f"{sysname}_{isym}_{trev}_{comp}"
        if s.nmag == 1:
            # output point i holds ph * in[idx[i]] (conjugated when time-reversed)
            a = out[0, 0].reshape(-1)
            a = np.conj(a) if trev else a
            b = dv[0, 0].reshape(-1)
            # the phase has modulus 1: match by modulus, then check one common phase
            lookup = {round(float(abs(v)), 11): j for j, v in enumerate(b)}
            assert len(lookup) == len(b)
            idx = np.array([lookup[round(float(abs(v)), 11)] for v in a], np.int32)
            ratio = a / b[idx]
            assert np.abs(ratio - ratio[0]).max() < 1e-12 and abs(abs(ratio[0]) - 1) < 1e-12
            rec[key + "_idx"] = idx
        rec[key + "_sample"] = out.reshape(-1)[::97]
        rec[key + "_norm"] = np.array(np.linalg.norm(out))
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "rotate_dvscf.npz"),
                        cases=np.array(json.dumps([list(c) for c in ROTDV_CASES])),
                        systems=np.array(json.dumps(ROTDV_SYS)), **rec)
    print("rotate_dvscf", len(ROTDV_CASES))


def rotate_fixture(tmp):
    s = synth.make_system("c0", {"nbnds": 5})
    rng = np.random.default_rng(7)
    nm, ns, nb = s.nmodes, s.nspin, s.nbnds
    g = rng.standard_normal((nm, ns, nb, nb)) + 1j * rng.standard_normal((nm, ns, nb, nb))
    Dl = rng.standard_normal((ns, nb, nb)) + 1j * rng.standard_normal((ns, nb, nb))
    Dr = rng.standard_normal((ns, nb, nb)) + 1j * rng.standard_normal((ns, nb, nb))
    out = {}
    for trev in (0, 1):
        sysf = os.path.join(tmp, "rot_sys.bin")
        synth.write_system(s, sysf)
        df = os.path.join(tmp, "rot_in.bin")
        with open(df, "wb") as f:
            f.write(b"LELPHSYS")
            synth._rec(f, "g", g)
            synth._rec(f, "Dl", Dl)
            synth._rec(f, "Dr", Dr)
            synth._rec(f, "trev", np.array([trev], np.int32))
            f.write(b"END\0" + b"\0" * 28)
        of = os.path.join(tmp, "rot_out.bin")
        subprocess.run([REF, sysf, os.path.join(tmp, "ignore.bin"), "rotate", df, of], check=True)
        out[trev] = np.fromfile(of, np.complex128).reshape(g.shape)
    np.savez(os.path.join(ROOT, "tests", "golden", "q_rotate.npz"), g=g, Dl=Dl, Dr=Dr,
             out_notr=out[0], out_tr=out[1])
    print("q_rotate", g.shape)


# Dmats (electronic_reps, src/symmetries/elec_reps.c:16, for every symmetry
# of the system and every full-BZ k): name -> (base config, overrides)
DMATS_SYS = {
    "c0": ("c0", {"kgrid": (2, 2, 2), "nbnds": 4}),
    "zb_tr": ("c0", {"kind": "zincblende", "timerev": True, "nbnds": 3, "kgrid": (2, 2, 2)}),
    "l12": ("c1", {"nbnds": 4, "kgrid": (2, 2, 2), "npw": 300, "fft": (24, 24, 24), "qpts": [(0.5, 0, 0)]}),
    "soc_tr": ("c0", {"kind": "zincblende", "timerev": True, "nspinor": 2, "nmag": 4, "soc": True,
                      "ls": (0, 1, 2), "nbnds": 2, "npw": 150, "fft": (20, 20, 20), "kgrid": (2, 2, 2),
                      "qpts": [(0.5, 0.5, 0)]}),
    "lsda": ("c0", {"nspin": 2, "nbnds": 3, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]}),
    "hex_ragged": ("c2", {"kgrid": (3, 3, 1), "fft": (15, 15, 60), "nbnds": 3, "npw": (80, 120),
                          "qpts": [(1 / 3, 0, 0)]}),
}
DMATS_STRIDE = 3  # every third (symmetry, k) pair is stored whole; the norms of all of them


def dmats_fixture(tmp):
    rec = {}
    for name, (base, ov) in DMATS_SYS.items():
        s = synth.make_system(base, dict(ov))
        sysf = os.path.join(tmp, "dm_" + name + ".bin")
        synth.write_system(s, sysf)
        out_f = os.path.join(tmp, "dm_out.bin")
        subprocess.run([REF, sysf, os.path.join(tmp, "unused.bin"), "dmats", out_f], check=True)
        D = np.fromfile(out_f, np.complex128).reshape(len(s.sym_R) * s.nk_bz, s.nspin, s.nbnds, s.nbnds)
        rec[name + "_sub"] = D[::DMATS_STRIDE]
        rec[name + "_norm"] = np.linalg.norm(D.reshape(len(D), -1), axis=1)
        print("dmats", name, D.shape, float(np.abs(D).max()))
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "dmats.npz"), systems=np.array(json.dumps(DMATS_SYS)),
                        stride=np.array(DMATS_STRIDE), **rec)


# q stars (the stage's star loop, src/elph/compute_elph_matq.c:159-217, with
# Dmats from electronic_reps): name -> (base config, overrides, kminusq)
STAR_SYS = {
    "star_c0": ("c0", {"kgrid": (2, 2, 2), "nbnds": 3, "qpts": [(0.5, 0, 0), (0.5, 0.5, 0)]}, False),
    "star_zb_tr_kmq": ("c0", {"kind": "zincblende", "timerev": True, "nbnds": 3, "kgrid": (2, 2, 2),
                              "qpts": [(0.5, 0, 0)]}, True),
    "star_l12": ("c1", {"nbnds": 3, "kgrid": (2, 2, 2), "npw": 300, "fft": (24, 24, 24),
                        "qpts": [(0.5, 0.5, 0)]}, False),
    "star_soc": ("c0", {"kind": "zincblende", "timerev": True, "nspinor": 2, "nmag": 4, "soc": True,
                        "ls": (0, 1, 2), "nbnds": 2, "npw": 150, "fft": (20, 20, 20), "kgrid": (2, 2, 2),
                        "qpts": [(0.5, 0.5, 0)]}, False),
}


def star_fixture(tmp):
    """g of every member of each q's star from the reference's own stage; the
    stars (members and the first symmetry producing each) are built here the
    way a phonon code lists them and stored with the output."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import elph_oracle as O
    for name, (base, ov, kmq) in STAR_SYS.items():
        s = synth.make_system(base, dict(ov))
        stars = [O.q_star(s, q) for q in s.qpts]
        ns = np.array([len(m) for m, _ in stars], np.int32)
        qs = np.concatenate([sy for _, sy in stars]).astype(np.int32)
        sysf = os.path.join(tmp, name + ".bin")
        synth.write_system(s, sysf, kminusq=kmq)
        spec_f = os.path.join(tmp, name + "_star.bin")
        with open(spec_f, "wb") as f:
            f.write(b"LELPHSYS")
            synth._rec(f, "nqstar", ns)
            synth._rec(f, "qsym", qs)
            f.write(b"END\0" + b"\0" * 28)
        gf = os.path.join(tmp, name + "_g.bin")
        subprocess.run([REF, sysf, gf, "star", spec_f], check=True, stdout=subprocess.DEVNULL)
        g = np.fromfile(gf, np.complex128).reshape(int(ns.sum()), s.nk_bz, s.nmodes, s.nspin, s.nbnds, s.nbnds)
        spec = json.dumps({"base": base, "overrides": ov, "kminusq": kmq, "non_loc": True})
        np.savez_compressed(os.path.join(ROOT, "tests", "golden", name + ".npz"), g=g, spec=np.array(spec),
                            nqstar=ns, qsym=qs)
        print(name, g.shape, ns.tolist(), float(np.abs(g).max()))


# read_dvscf_qe (src/io/qe/read_dvscf.c:15): seeded QE-layout dvscf files and
# patterns; name -> (base config, overrides, seed)
DVSCF_SYS = {
    "c0": ("c0", {"kgrid": (2, 2, 2), "nbnds": 2, "qpts": [(0.5, 0, 0)]}, 11),
    "lsda": ("c0", {"nspin": 2, "nbnds": 2, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]}, 12),
    "soc": ("c0", {"kind": "zincblende", "timerev": True, "nspinor": 2, "nmag": 4, "soc": True, "ls": (0, 1, 2),
                   "nbnds": 2, "npw": 150, "fft": (20, 20, 20), "kgrid": (2, 2, 2), "qpts": [(0.5, 0.5, 0)]}, 13),
    "hex_odd": ("c2", {"kgrid": (3, 3, 1), "fft": (15, 15, 60), "nbnds": 2, "npw": 100,
                       "qpts": [(1 / 3, 0, 0)]}, 14),
}
DVSCF_SAMPLE = 997


def dvscf_inputs(s, seed):
    """QE-layout dvscf (patterns, nmag, Nz, Ny, Nx) and unitary patterns, seeded."""
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz = s.fft_dims
    nm = s.nmodes
    raw = rng.standard_normal((nm, s.nmag, Nz, Ny, Nx)) + 1j * rng.standard_normal((nm, s.nmag, Nz, Ny, Nx))
    pats = np.linalg.qr(rng.standard_normal((nm, nm)) + 1j * rng.standard_normal((nm, nm)))[0]
    return raw, pats


def dvscf_fixture(tmp):
    rec = {}
    for name, (base, ov, seed) in DVSCF_SYS.items():
        s = synth.make_system(base, dict(ov))
        raw, pats = dvscf_inputs(s, seed)
        sysf = os.path.join(tmp, "dvs_" + name + ".bin")
        synth.write_system(s, sysf)
        spec = os.path.join(tmp, "dvs_spec.bin")
        with open(spec, "wb") as f:
            f.write(b"LELPHSYS")
            synth._rec(f, "eig", s.eigVec[0])
            synth._rec(f, "pats", pats)
            f.write(b"END\0" + b"\0" * 28)
        rawf = os.path.join(tmp, "dvscf_raw.bin")
        raw.astype(np.complex128).tofile(rawf)
        outf = os.path.join(tmp, "dvscf_out.bin")
        subprocess.run([REF, sysf, os.path.join(tmp, "unused.bin"), "dvscf", spec, rawf, outf], check=True)
        out = np.fromfile(outf, np.complex128)
        rec[name + "_sample"] = out[::DVSCF_SAMPLE]
        rec[name + "_norm"] = np.linalg.norm(out.reshape(s.nmodes, -1), axis=1)
        print("dvscf", name, out.shape, float(np.abs(out).max()))
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "dvscf_qe.npz"), systems=np.array(json.dumps(DVSCF_SYS)),
                        sample=np.array(DVSCF_SAMPLE), **rec)


# the reference's single-precision build on every system of GOLDEN and on the
# first k-points of one q of the 4-atom c1 system (32 bands, 48^3 grid, its own
# k-pool split LELPH_REF_KPOOLS); name -> (base, overrides, kminusq, non_loc, k pools)
F32_SYS = dict({n: (b, o, kmq, nl, 1) for n, (b, o, kmq, nl) in GOLDEN.items()},
               c1s=("c1", {"qpts": [(0.125, 0, 0)]}, False, True, 128))


# systems at the shapes of the benchmark configurations and of tensor-core
# tiles that hold whole modes (48 bands x 12 modes, 36 bands x 24 modes): both
# builds of the reference run the first nk_BZ / kpools k-points of one q and
# only the error statistics of the single-precision build against the double
# one are stored (the metric's definition: max and RMS of e_i, complex norm);
# name -> (base, overrides, k pools)
F32_STATS = {
    "tile48": ("c1", {"nbnds": 48, "kgrid": (4, 4, 4), "qpts": [(0.25, 0, 0)]}, 32),
    "tile36": ("c3", {"nbnds": 36, "nspinor": 1, "nmag": 1, "soc": False, "ls": (0, 1), "npw": 1500,
                      "fft": (40, 40, 40), "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]}, 4),
    "c2s": ("c2", {"qpts": [(1 / 12, 0, 0)]}, 36),
    "c3s": ("c3", {"qpts": [(1 / 6, 0, 0)]}, 54),
    "c4s": ("c4", {"nbnds": 80, "kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)]}, 8),
}


def f32_stats(name, base, ov, kpools, tmp):
    s = synth.make_system(base, dict(ov))
    sysf = os.path.join(tmp, "f32s_" + name + ".bin")
    synth.write_system(s, sysf)
    env = dict(os.environ, LELPH_REF_KPOOLS=str(kpools))
    nk = s.nk_bz // kpools + (1 if s.nk_bz % kpools else 0)
    g = {}
    for tag, exe in (("64", REF), ("32", os.path.join(ROOT, "oracle", "_ref", "f32", "lelph_ref"))):
        gf = os.path.join(tmp, "f32s_" + name + tag + ".bin")
        subprocess.run([exe, sysf, gf], check=True, env=env, stdout=subprocess.DEVNULL)
        g[tag] = synth.read_g(gf, s, len(s.qpts))[:, :nk]
    a, b = np.abs(g["32"]), np.abs(g["64"])
    e = np.abs(a - b) / np.maximum(b, 1e-6 * b.max())
    st = np.array([e.max(), np.sqrt(np.mean(e * e)),
                   np.linalg.norm((g["32"] - g["64"]).ravel()) / np.linalg.norm(g["64"].ravel())])
    print("f32 stats", name, nk, st.tolist(), flush=True)
    return {name + "_stats": st, name + "_nk": np.array(nk),
            name + "_spec": np.array(json.dumps({"base": base, "overrides": ov, "kminusq": False, "non_loc": True})),
            name + "_wfc_sum": np.array([np.abs(w).sum() for w in s.wfc]), name + "_dv_sum": np.abs(s.dVscf).sum()}


def f32_fixture(tmp):
    ref32 = os.path.join(ROOT, "oracle", "_ref", "f32", "lelph_ref")
    rec = {}
    for name, (base, ov, kpools) in F32_STATS.items():
        rec.update(f32_stats(name, base, ov, kpools, tmp))
    for name, (base, ov, kmq, nl, kpools) in F32_SYS.items():
        s = synth.make_system(base, dict(ov))
        sysf = os.path.join(tmp, "f32_" + name + ".bin")
        synth.write_system(s, sysf, kminusq=kmq, non_loc=nl)
        gf = os.path.join(tmp, "f32_" + name + "_g.bin")
        env = dict(os.environ, LELPH_REF_KPOOLS=str(kpools))
        subprocess.run([ref32, sysf, gf], check=True, env=env, stdout=subprocess.DEVNULL)
        nk = s.nk_bz // kpools + (1 if s.nk_bz % kpools else 0)
        g = synth.read_g(gf, s, len(s.qpts))[:, :nk]
        rec[name + "_g32"] = g.astype(np.complex64)
        rec[name + "_spec"] = np.array(json.dumps({"base": base, "overrides": ov, "kminusq": kmq,
                                                   "non_loc": nl}))
        rec[name + "_wfc_sum"] = np.array([np.abs(w).sum() for w in s.wfc])
        rec[name + "_dv_sum"] = np.abs(s.dVscf).sum()
        print("f32", name, g.shape, float(np.abs(g).max()))
    np.savez(os.path.join(ROOT, "tests", "golden", "ref_f32.npz"), **rec)


if __name__ == "__main__":
    only = sys.argv[1:]
    with tempfile.TemporaryDirectory() as tmp:
        if not only:
            for name, (base, ov, kmq, nl) in GOLDEN.items():
                run(name, base, ov, kmq, nl, tmp)
            for name, (base, ov, kmq, nl) in GOLDEN_DVLOC.items():
                run_dvloc(name, base, ov, kmq, nl, tmp)
            rotate_fixture(tmp)
            rotdv_fixture(tmp)
        if not only or "dmats" in only:
            dmats_fixture(tmp)
        if not only or "star" in only:
            star_fixture(tmp)
        if not only or "dvscf" in only:
            dvscf_fixture(tmp)
        if not only or "f32" in only:
            f32_fixture(tmp)
