"""Times the compiled reference elph stage on bounded samples of every
configuration, on this machine's cores, for the CPU-baseline table.

The binary is oracle/_ref/o3/lelph_ref: the reference's unmodified per-q stage
(compute_and_write_elphq, src/elph/compute_elph_matq.c:20) built by
oracle/Makefile with OUT=_ref/o3 and -O3 -march=native (FP64 build,
-DCOMPILE_ELPH_DOUBLE; OpenMP on all cores).  Each sample is one q of the
configuration and the first nk_BZ/KPOOLS k-points (the reference's own k-pool
split, LELPH_REF_KPOOLS); the rate is g elements / wall time of the run.

TEST INFRASTRUCTURE ONLY: it needs the reference tree and an x86 build here.

    make -C oracle REF=<reference tree> OUT=_ref/o3 CFLAGS="-O3 -march=native -std=gnu11 -fopenmp -DELPH_OMP_PARALLEL_BUILD"
    python oracle/time_reference.py [c0 c1 ...]
"""
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from letzelphc_gb300 import synth  # noqa: E402

REF = os.path.join(HERE, "_ref", "o3", "lelph_ref")
# config -> (overrides for a one-q sample, k pools)
SAMPLES = {
    "c0": ({}, 1),
    "c1": ({"qpts": [(0.125, 0, 0)]}, 32),
    "c2": ({"qpts": [(1 / 12, 0, 0)]}, 9),
    "c3": ({"qpts": [(1 / 6, 0, 0)]}, 27),
    "c4": ({"qpts": [(0.125, 0, 0)]}, 512),
}


def time_config(name):
    ov, kpools = SAMPLES[name]
    s = synth.make_system(name, dict(ov))
    nk = s.nk_bz
    nk_pool = nk // kpools + (1 if nk % kpools else 0)
    pairs = len(s.qpts) * nk_pool
    g = s.nmodes * s.nspin * s.nbnds * s.nbnds
    env = dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count()), LELPH_REF_KPOOLS=str(kpools))
    with tempfile.TemporaryDirectory() as d:
        sysf = os.path.join(d, "s.bin")
        synth.write_system(s, sysf)
        t0 = time.perf_counter()
        subprocess.run([REF, sysf, os.path.join(d, "g.bin")], check=True, env=env, stdout=subprocess.DEVNULL)
        wall = time.perf_counter() - t0
    return {"config": name, "pairs": pairs, "g_elements": pairs * g, "wall_s": wall,
            "g_per_s": pairs * g / wall, "cores": os.cpu_count(), "k_pools": kpools}


if __name__ == "__main__":
    for name in (sys.argv[1:] or list(SAMPLES)):
        print(json.dumps(time_config(name)), flush=True)
