"""Times the compiled reference elph stage on bounded samples of every
configuration, on this machine's cores, for the CPU-baseline table.

The binaries are oracle/_ref/<arch>-f32/lelph_ref (the reference's default
single-precision build) and oracle/_ref/<arch>/lelph_ref (-DCOMPILE_ELPH_DOUBLE),
both the reference's unmodified per-q stage (compute_and_write_elphq,
src/elph/compute_elph_matq.c:20) built by __graft_entry__.build() with the
reference recipe's flags (-O3, OpenMP).  A sample runs the way an MPI run of
the reference with one k pool per rank does: one process per core, each the
pool of one full-BZ k-point of one q (LELPH_REF_KPOOLS = nk_BZ,
LELPH_REF_KPOOL = k), one thread, OpenBLAS GEMMs when SciPy ships an OpenBLAS
(the reference's recipe links -lopenblas).  The rate is the g elements of the
sample divided by the longest of the processes' stage times.

TEST INFRASTRUCTURE ONLY.

    python -c "import __graft_entry__ as g; g.build()"
    python oracle/time_reference.py [c0 c1 ...]
"""
import json
import os
import platform
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from letzelphc_gb300 import synth  # noqa: E402

ARCH = platform.machine()
BUILDS = {"f32": os.path.join(HERE, "_ref", ARCH + "-f32", "lelph_ref"),
          "f64": os.path.join(HERE, "_ref", ARCH, "lelph_ref")}
# config -> the q of the sample (one of its iBZ q-points)
SAMPLES = {"c0": (0.25, 0, 0), "c1": (0.125, 0, 0), "c2": (1 / 12, 0, 0), "c3": (1 / 6, 0, 0),
           "c4": (0.125, 0, 0)}


def openblas():
    import glob
    try:
        import scipy
    except ImportError:
        return ""
    libs = sorted(glob.glob(os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs",
                                         "libscipy_openblas*.so")))
    return libs[0] if libs else ""


def time_config(name, cores):
    s = synth.make_system(name, {"qpts": [SAMPLES[name]]})
    g = s.nmodes * s.nspin * s.nbnds * s.nbnds
    ks = [(i * s.nk_bz) // cores for i in range(cores)]
    out = {"config": name, "pairs": len(ks), "g_elements": len(ks) * g, "cores": cores}
    with tempfile.TemporaryDirectory() as d:
        sysf = os.path.join(d, "s.bin")
        synth.write_system(s, sysf)
        for build, exe in BUILDS.items():
            procs = []
            for i, k in enumerate(ks):
                env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", LELPH_REF_BLAS=openblas(),
                           LELPH_REF_KPOOLS=str(s.nk_bz), LELPH_REF_KPOOL=str(k))
                procs.append(subprocess.Popen([exe, sysf, os.path.join(d, f"g{i}.bin")], env=env,
                                              stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True))
            worst = 0.0
            for p in procs:
                _, err = p.communicate()
                if p.returncode:
                    raise RuntimeError(err[-400:])
                worst = max(worst, float([ln for ln in err.splitlines() if "stage_seconds" in ln][0].split()[-1]))
            out[build] = {"wall_s": worst, "g_per_s": len(ks) * g / worst}
    return out


if __name__ == "__main__":
    cores = os.cpu_count() or 1
    for name in (sys.argv[1:] or list(SAMPLES)):
        print(json.dumps(time_config(name, cores)), flush=True)
