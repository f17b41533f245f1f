#!/usr/bin/env python
"""Throughput of the per-q electron-phonon matrix-element stage on GB300.

Metric: g elements per second (elements g_mn^nu(k,q) of ndb.elph) for the
4-atom cell workload: 48^3 grid, npw ~2500, 8x8x8 k (512 full-BZ points
unfolded from 35 irreducible), 8 q-points, 12 modes, 32 bands, KB projectors
l = 0,1, kernel dfpt (local + nonlocal).  One step = every (k, q) pair of the
batch (4096 pairs, 5.03e7 g elements), starting from the iBZ plane-wave
coefficients and dV_scf resident in HBM: unfold + FFT all full-BZ
wavefunctions, project on the KB projectors, sandwich every pair.

* value / ms_per_step: device-resident step, mixed form (FP32 FFTs,
  split-f16 tensor-core sandwich, FP64 phases and chunk reduction).
* e2e: the same step through the C ABI with host buffers: every step copies
  the coefficients and the 8 dV_scf from pinned host memory and reads g back
  (complex64, the reference's default output type).
* fp64: the plain FP64 form on a sample of pairs (its full-BZ preparation
  plus sampled pairs, scaled to the batch), and the mixed-vs-FP64 errors.
* roofline: the local-sandwich kernel (tensor bound) against the measured
  bf16 dense peak.
* cpu_baseline: the reference's own per-q stage compiled for this machine by
  __graft_entry__.build() (its default single-precision build, OpenMP on every
  host core) on a few pairs of the workload; the numpy restatement on one core
  where that build is absent.

`--impl reference` times the reference's CPU path instead: the same compiled
stage, one (k, q) pair of the workload per step, every host core (the numpy
restatement on all cores where the compiled stage is absent).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "g elements/s per GB300, mixed vs FP64 form, at |g| rel err <= 1e-5 vs FP64"
WORKLOAD = "4-atom cell, 48^3 grid, npw~2500, 8x8x8 k, 8 q, 12 modes, 32 bands, KB l=0..1"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="mixed_f16")
    p.add_argument("--fp64-pairs", type=int, default=64)
    p.add_argument("--cpu-pairs", type=int, default=16)
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--profile-case", type=int, default=0,
                   help="profiling case for ncu: this many (k, q) pairs of one q, one step, no extras")
    p.add_argument("--workload", default="elph",
                   choices=["elph", "dmats", "star", "dvscf", "configs", "gspace", "batch", "tune"],
                   help="elph: the per-q stage (default); dmats: the electronic representation matrices "
                        "of the same system (every symmetry x full-BZ k); star: the per-q stage with the "
                        "q-star expansion of each of the 8 q; dvscf: the dV_scf ingest of the 8 q from QE's "
                        "file layout; configs: mixed vs FP64 rate and error on every config's full size; "
                        "batch: the batched uneven workload in one call, per q and per (k, q) call; "
                        "tune: the measured route and tile choice on every config's shape")
    p.add_argument("--dmat-syms", type=int, default=0, help="dmats profiling case: only this many symmetries")
    p.add_argument("--configs", default="", help="configs workload: comma-separated subset (default: all)")
    p.add_argument("--small", action="store_true",
                   help="star / dvscf workloads on the same cell with a 2x2x2 k grid (profiling cases)")
    return p.parse_args()


# ------------------------------------------------------------------ ranks

def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def shard_qpoints(rank, world):
    """q-points of this rank: rank 0 takes the workload's 8 q; other ranks
    take further irreducible q of the 8x8x8 grid (no data exchanged)."""
    from letzelphc_gb300 import synth
    base = synth.CONFIGS["c1"]["qpts"]
    if rank == 0:
        return base
    A, _, _, _ = synth._structure("l12", synth.CONFIGS["c1"]["a"])
    s = synth.make_system("c0", {"kind": "l12", "a": synth.CONFIGS["c1"]["a"], "kgrid": (2, 2, 2),
                                 "qpts": [(0, 0, 0)], "nbnds": 1, "npw": 20, "fft": (24, 24, 24)})
    qirr = synth.reduce_grid((8, 8, 8), s.sym_R, A)
    idx = [(8 * rank + i) % len(qirr) for i in range(8)]
    return [tuple(qirr[i]) for i in idx]


class Dist:
    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            backend = "nccl" if os.environ.get("LELPH_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
            td.init_process_group(backend=backend)
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())


# ------------------------------------------------------------- clocks

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index
        self.out = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ helpers

def g_elems(s, npairs):
    return npairs * s.nmodes * s.nspin * s.nbnds * s.nbnds


def tensor_flops_per_pair(s, grid=None):
    """Tensor-core work of the local sandwich per (k, q) pair: three real
    GEMMs (hi*hi, hi*lo, lo*hi) of (nmodes*nbnds) x (2*nbp) x (2*nspinor*M),
    M the points of the product grid the library chose (the reference's box
    when not given)."""
    N = int(np.prod(grid if grid is not None else s.fft_dims))
    nbp = (s.nbnds + 7) // 8 * 8
    M = s.nmodes * s.nbnds
    return 3 * 2.0 * M * (2 * nbp) * (2 * s.nspinor * N) * s.nspin


def traffic_per_launch(pairs_per_launch):
    """DRAM bytes of one k_local_tc launch: the per-pair figure of the committed
    ncu capture (dram__bytes_read + dram__bytes_write of an 8-pair launch,
    divided by 8) times the pairs of the launch."""
    path = os.path.join(ROOT, "profiles", "k_local_tc_4atom_8pairs.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_pair:"):
            return float(line.split(":")[1]) * pairs_per_launch
    return None


def err_stats(g, ref):
    a, b = np.abs(g), np.abs(ref)
    e = np.abs(a - b) / np.maximum(b, 1e-6 * b.max())
    return {"max": float(e.max()), "rms": float(np.sqrt(np.mean(e * e))),
            "norm": float(np.linalg.norm((g - ref).ravel()) / np.linalg.norm(ref.ravel()))}


def cpu_port_sample(s, pairs):
    """Time the oracle on a list of (iq, k) pairs; returns (seconds, g elements)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import elph_oracle as O
    t0 = time.perf_counter()
    for iq, k in pairs:
        O.compute_elphq(s, iq, k_list=[k])
    return time.perf_counter() - t0, g_elems(s, len(pairs))


def _port_worker(args):
    iq, k = args
    s = _port_worker.s
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import elph_oracle as O
    O.compute_elphq(s, iq, k_list=[k])
    return 1


def _port_init():
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from letzelphc_gb300 import synth
    _port_worker.s = synth.make_system("c1")


# ---------------------------------------------------------- reference arm

def ref_binary(single=True):
    """The reference's per-q stage compiled for this machine by build()
    (oracle/Makefile with the reference's own recipe flags: -O3, OpenMP), in its
    default single-precision form or the double one; None if absent."""
    import platform
    d = os.path.join(ROOT, "oracle", "_ref", platform.machine() + ("-f32" if single else ""))
    exe = os.path.join(d, "lelph_ref")
    return exe if os.access(exe, os.X_OK) else None


def openblas_path():
    """An OpenBLAS shared library for the reference's GEMMs (its recipe links
    -lopenblas): the one SciPy ships, if SciPy is installed."""
    import glob
    try:
        import scipy
    except ImportError:
        return ""
    d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    libs = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    return libs[0] if libs else ""


class RefRunner:
    """Runs the compiled reference on (q, k) pairs of a system the way an MPI
    run of it with one k pool per rank does (nkpools = ranks, one rank per
    core, src/elph/compute_elph_matq.c:51-54): one process per pair, all of a
    batch at once, each the pool of its k-point (one pool per full-BZ k) with
    one thread; the time of a batch is the longest of the harness's wall
    times of the stage calls (input loading excluded)."""

    def __init__(self, s, exe):
        import tempfile
        from letzelphc_gb300 import synth
        self.s, self.exe = s, exe
        self.dir = tempfile.mkdtemp(prefix="lelph_ref_")
        self.sysf = os.path.join(self.dir, "system.bin")
        synth.write_system(s, self.sysf)
        self.blas = openblas_path()

    def pairs(self, items):
        procs = []
        for i, (iq, k) in enumerate(items):
            env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", LELPH_REF_QPT=str(iq),
                       LELPH_REF_KPOOLS=str(self.s.nk_bz), LELPH_REF_KPOOL=str(k), LELPH_REF_BLAS=self.blas)
            procs.append(subprocess.Popen([self.exe, self.sysf, os.path.join(self.dir, f"g{i}.bin")], env=env,
                                          stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True))
        worst = 0.0
        for p in procs:
            _, err = p.communicate()
            if p.returncode != 0:
                raise RuntimeError(f"the reference harness failed: {err[-400:]}")
            t = [float(line.split()[-1]) for line in err.splitlines() if "stage_seconds" in line]
            if not t:
                raise RuntimeError("the reference harness printed no stage time")
            worst = max(worst, t[0])
        return worst

    def close(self):
        import shutil
        shutil.rmtree(self.dir, ignore_errors=True)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from letzelphc_gb300 import synth
    s = synth.make_system("c1")
    cores = os.cpu_count() or 1
    exe = ref_binary(single=True)
    rng = np.random.default_rng(0)
    ts, es = [], []
    if exe:
        # the reference's compiled stage: per step one random (k, q) pair of the
        # workload on every host core, one process (k pool) per core
        rr = RefRunner(s, exe)
        try:
            rr.pairs([(0, k) for k in range(cores)])   # warm-up: page cache, library loading
            for _ in range(args.steps):
                items = [(int(rng.integers(len(s.qpts))), int(rng.integers(s.nk_bz))) for _ in range(cores)]
                ts.append(rr.pairs(items))
                es.append(g_elems(s, cores))
        finally:
            rr.close()
        warm = 1
        kind, sample = "reference", f"{cores} random (k, q) pairs per step (one per core), {args.steps} steps"
        build = ("the reference's own per-q stage (compute_and_write_elphq and its callees, unmodified sources) "
                 "in its default single-precision build, gcc -O3 -fopenmp -DELPH_OMP_PARALLEL_BUILD, one "
                 "process per core as the k pools of an MPI run, against single-rank MPI, FFTW-API (in-house "
                 "mixed-radix FFT) and CBLAS (OpenBLAS when SciPy ships one) stand-ins")
        dtype = "f32"
    else:
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        with ctx.Pool(cores, initializer=_port_init) as pool:
            def step(n):
                pairs = [(int(rng.integers(len(s.qpts))), int(rng.integers(s.nk_bz))) for _ in range(n)]
                t0 = time.perf_counter()
                pool.map(_port_worker, pairs, chunksize=1)
                return time.perf_counter() - t0, g_elems(s, n)
            for _ in range(args.warmup):
                step(cores)
            for _ in range(args.steps):
                t, e = step(cores)
                ts.append(t)
                es.append(e)
        warm = args.warmup
        kind, sample = "port", f"{cores} random (k,q) pairs per step, {args.steps} steps"
        build = "oracle port (numpy restatement): the compiled reference is absent on this host"
        dtype = "f64"
    value = sum(es) / sum(ts)
    line = {"metric": METRIC, "value": value, "unit": "g_elements/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": warm, "ms_per_step": 1e3 * sum(ts) / len(ts), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded, c1 shapes)",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": sample, "reference_build": build},
            "cpu_baseline": {"value": value, "unit": "g_elements/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "g_elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# -------------------------------------------------------------- our arm

def run_profile_case(args):
    """A small slice of the workload for ncu captures (not a bench value)."""
    import torch
    from letzelphc_gb300 import synth
    from letzelphc_gb300.build import build_library
    from letzelphc_gb300.elph import LelphGPU, OUT_C64
    build_library()
    # the workload's cell, grid, plane waves and bands on a 2x2x2 k grid: < 1 GB on the device
    s = synth.make_system("c1", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0.0, 0.0)]})
    n = min(args.profile_case, s.nk_bz)
    qs = np.zeros(n, np.int32)
    ks = np.arange(n, dtype=np.int32)
    with LelphGPU(s, args.precision) as ctx:
        ctx.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        gdev = torch.empty(n * s.nmodes * s.nbnds * s.nbnds * 2, dtype=torch.float32, device="cuda")
        for _ in range(max(1, args.warmup)):
            ctx.prepare()
            ctx.run_device(qs, ks, gdev.data_ptr(), out=OUT_C64)
        torch.cuda.synchronize()
        ctx.set_profiling(True)
        p0 = ctx.stats()
        ctx.prepare()
        ctx.run_device(qs, ks, gdev.data_ptr(), out=OUT_C64)
        p1 = ctx.stats()
    out = {"profile_case_pairs": n, "local_ms": p1["local_ms"] - p0["local_ms"],
           "prepare_ms": p1["prepare_ms"] - p0["prepare_ms"], "finish_ms": p1["finish_ms"] - p0["finish_ms"],
           "tensor_flops": tensor_flops_per_pair(s, p1["product_grid"]) * n, "product_grid": p1["product_grid"]}
    out["local_tflops"] = out["tensor_flops"] / (out["local_ms"] * 1e-3) / 1e12
    print(json.dumps(out), flush=True)
    return 0


def path_roofline(s, value, peaks, clk_mhz):
    """The path-level roofline of the survey's measurement contract, per pair:
    T_roof = max(B_min / BW_HBM, F_fft / P_simt, F_gemm_eff / P_tc, F_nl / P_tc),
    with the reference algorithm's own counts (FFTs = nspin nb nspinor + nm nspin
    nb nspinor per pair on the reference box, each 5 [sticks Nz log2 Nz +
    x_act Ny Nz log2 Ny + N log2 Nx] flops; F_gemm_eff = 3 split products of
    8 nm nspin nb^2 nspinor npw; F_nl = 16 (4 P natom) npw nspin nb nspinor +
    8 nm 3 natom nspin nb^2) and the compulsory bytes B_min (FP32 complex).
    achieved = T_roof / T_meas, T_meas = the step's time per pair; above 1
    means the implementation does less work than the reference's algorithm
    (the real-space route needs no per-mode FFT)."""
    Nx, Ny, Nz = (int(v) for v in s.fft_dims)
    N = Nx * Ny * Nz
    ff = []
    npws = []
    for m in s.miller:
        m = np.asarray(m)
        sticks = len({(int(a) % Nx, int(b) % Ny) for a, b in m[:, :2]})
        xact = len({int(a) % Nx for a in m[:, 0]})
        ff.append(5.0 * (sticks * Nz * np.log2(Nz) + xact * Ny * Nz * np.log2(Ny) + N * np.log2(Nx)))
        npws.append(len(m))
    f_one, npw = float(np.mean(ff)), float(np.mean(npws))
    nm, sig, nb, ns = s.nmodes, s.nspin, s.nbnds, s.nspinor
    lsh = np.rint(np.asarray(s.PP_table)[:, :, 0] - 1.0).astype(int)
    P = int(max(sum(2 * l + 1 for l in lsh[:, t] if l >= 0) for t in range(lsh.shape[1])))
    f_fft = (sig * nb * ns + nm * sig * nb * ns) * f_one
    f_gemm = 3 * 8.0 * nm * sig * nb * nb * ns * npw
    f_nl = 16.0 * (4 * P * s.natom) * npw * sig * nb * ns + 8.0 * nm * 3 * s.natom * sig * nb * nb
    c = 8.0
    b_min = 2 * sig * nb * ns * npw * c + 2 * P * npw * 4 + nm * s.nmag * N * c / s.nk_bz + nm * sig * nb * nb * c
    p_simt = 152 * 128 * 2 * (clk_mhz or 2070.0) * 1e6
    p_tc = (peaks.get("bf16_tflops_sustained") or 1700.0) * 1e12
    bw = (peaks.get("hbm_gbs") or 6800.0) * 1e9
    terms = {"hbm": b_min / bw, "fft_simt": f_fft / p_simt, "gemm_tensor": f_gemm / p_tc, "nonlocal_tensor": f_nl / p_tc}
    bound = max(terms, key=terms.get)
    t_roof = terms[bound]
    t_meas = nm * sig * nb * nb / value
    return {"definition": "T_roof = max(B_min/BW_HBM, F_fft/P_simt, F_gemm_eff/P_tc, F_nl/P_tc) per pair with the "
                          "reference algorithm's counts; achieved = T_roof / T_meas",
            "bound": bound, "t_roof_us": t_roof * 1e6, "t_meas_us": t_meas * 1e6, "achieved": t_roof / t_meas,
            "per_pair": {"F_fft": f_fft, "F_gemm_eff": f_gemm, "F_nl": f_nl, "B_min": b_min},
            "peaks": {"simt_fp32_tflops": p_simt / 1e12, "tensor_tflops": p_tc / 1e12, "hbm_gbs": bw / 1e9},
            "peak_source": "FP32 SIMT: nominal 152 SMs x 128 lanes x 2 x median SM clock; tensor and HBM: "
                           "MEASURED_PEAKS.json (sustained bf16, copy)"}


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = Dist(world)
    from letzelphc_gb300 import synth
    from letzelphc_gb300.build import build_library
    from letzelphc_gb300.elph import LelphGPU, OUT_C64

    build_library()
    qpts = shard_qpoints(rank, world)
    s = synth.make_system("c1", {"qpts": qpts})
    nq, nk = len(s.qpts), s.nk_bz
    npairs = nq * nk
    qs = np.repeat(np.arange(nq), nk).astype(np.int32)
    ks = np.tile(np.arange(nk), nq).astype(np.int32)
    gsz = s.nmodes * s.nspin * s.nbnds * s.nbnds
    elems = g_elems(s, npairs)

    ctx = LelphGPU(s, args.precision, device=local)
    for iq in range(nq):
        ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
    gdev = torch.empty(npairs * gsz * 2, dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream())

    def step():
        ctx.prepare()
        ctx.run_device(qs, ks, gdev.data_ptr(), out=OUT_C64)

    for _ in range(max(3, args.warmup)):
        step()
    st0 = ctx.stats()
    clocks = ClockSampler(local)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_wall0 = time.perf_counter()
    for e0, e1 in evs:
        e0.record(stream)
        step()
        e1.record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    dist.barrier()
    clk = clocks.stop()
    st1 = ctx.stats()
    ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    ms_step = dist.max(sum(ms) / len(ms))
    launches = (st1["kernel_launches"] - st0["kernel_launches"]) // args.steps

    # per-kernel device times (events around each launch on the library stream)
    ctx.set_profiling(True)
    p0 = ctx.stats()
    step()
    p1 = ctx.stats()
    ctx.set_profiling(False)
    local_ms = p1["local_ms"] - p0["local_ms"]
    local_launches = p1["local_launches"] - p0["local_launches"]
    prep_ms = p1["prepare_ms"] - p0["prepare_ms"]
    fin_ms = p1["finish_ms"] - p0["finish_ms"]
    flops = tensor_flops_per_pair(s, p1["product_grid"]) * npairs
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak = peaks.get("bf16_tflops_sustained") or 1700.0
    # the kernel's duration inside the timed steps: the library records CUDA
    # events around every launch of it on its stream (no synchronisation) and
    # reads them after each run; the profiled step above gives the other roles
    live_n = st1["local_live_launches"] - st0["local_live_launches"]
    live_ms = (st1["local_live_ms"] - st0["local_live_ms"]) / max(1, live_n)
    flops_launch = flops / max(1, local_launches)
    achieved = flops_launch / (live_ms * 1e-3) / 1e12 if live_n > 0 and live_ms > 0 else None
    roofline = {"kernel": "k_local_tc (split-f16 tcgen05 sandwich)", "bound": "tensor",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if achieved else None,
                "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)" if peaks else "fallback",
                "flops_per_launch": flops_launch, "launches": live_n,
                "product_grid": list(p1["product_grid"]), "reference_box": list(s.fft_dims),
                "avg_launch_ms": live_ms,
                "timing": "CUDA events around every k_local_tc launch on the library stream, over the timed steps "
                          f"({live_n} launches); {local_ms / max(1, local_launches):.2f} ms in the separately "
                          "profiled step",
                "traffic": traffic_per_launch(npairs / max(1, local_launches)),
                "traffic_source": "ncu DRAM bytes per pair of profiles/k_local_tc_4atom_8pairs.md x pairs per launch",
                "step_share": live_ms / ms_step if ms_step > 0 else None,
                "prepare_ms": prep_ms, "finish_ms": fin_ms}

    # HBM rooflines of the preparation's memory-bound kernels (per step, from the
    # library's per-role profiling events): algorithmic bytes / device time
    hbm = peaks.get("hbm_gbs") or 6800.0
    Mp = int(np.prod(p1["product_grid"]))
    nsets = s.nspin * s.nbnds * s.nspinor
    nbp = (s.nbnds + 7) // 8 * 8
    npw_k = np.array([len(s.gvec[int(ik)]) for ik in s.kmap[:, 0]], dtype=np.float64)
    box_bytes = s.nk_bz * nsets * Mp * 8.0            # FP32 boxes of every full-BZ k
    # after the first preparation only the occupied z-columns are zeroed
    ncols = p1.get("box_columns", 0)
    clear_bytes = ncols * nsets * p1["product_grid"][2] * 8.0 if ncols else box_bytes
    prep_roles = {
        "k_scatter (+ column clears)": (p1["prep_scatter_ms"] - p0["prep_scatter_ms"],
                                        float((npw_k * (nsets * (16 + 8 + 8) + 12)).sum()) + clear_bytes,
                                        "FP64 iBZ coefficients and Miller indices read, FP32 box entries and "
                                        "FP32 unfolded coefficients written, the occupied z-columns zeroed "
                                        f"({ncols} columns over the full-BZ k)"),
        "k_fft_x_split": (p1["prep_xsplit_ms"] - p0["prep_xsplit_ms"],
                          box_bytes + s.nk_bz * s.nspin * s.nspinor * Mp * (2 * 2 * nbp * 4 + nbp * 8.0),
                          "FP32 boxes read (an upper bound: only occupied planes are read), split k+q rows "
                          "(hi, lo) and FP32 psi_k tiles written"),
        "k_fft_contig + k_fft_strided (z, y)": (p1["prep_fft_ms"] - p0["prep_fft_ms"], 4 * box_bytes,
                                                 "FP32 boxes read and written once per pass (an upper bound: "
                                                 "the passes skip unoccupied columns and planes)"),
    }
    hbm_roofs = [{"kernel": k, "bound": "hbm", "ms": ms, "traffic_model_bytes": by,
                  "achieved": by / (ms * 1e-3) / 1e9 if ms > 0 else None, "peak": hbm, "unit": "GB/s",
                  "frac": by / (ms * 1e-3) / 1e9 / hbm if ms > 0 else None, "bytes": what}
                 for k, (ms, by, what) in prep_roles.items()]
    roofline["memory_bound_kernels"] = hbm_roofs
    # the KB projections on the tensor cores: three TF32 products of the real GEMM
    # (2 nsets coefficient rows) x (projector rows) x (2 npw), per full-BZ k
    lsh = np.rint(np.asarray(s.PP_table)[:, :, 0] - 1.0).astype(int)  # [l shell, type] -> l (< 0: none)
    nproj_max = int(max(sum(2 * l + 1 for l in lsh[:, t] if l >= 0) for t in range(lsh.shape[1])))
    proj_rows = s.natom * nproj_max * 4
    proj_ms = p1["prep_proj_ms"] - p0["prep_proj_ms"]
    if proj_rows and proj_ms > 0:
        pf = float(3 * 2 * (2 * nsets) * proj_rows * (2 * npw_k).sum())
        tf32 = (peaks.get("bf16_tflops") or 1900.0) / 2
        roofline["tensor_kernels"] = [{
            "kernel": "k_projections_tc (KB projections, split-TF32 tcgen05)", "bound": "tensor", "ms": proj_ms,
            "flops": pf, "achieved": pf / (proj_ms * 1e-3) / 1e12, "peak": tf32, "unit": "TFLOP/s",
            "frac": pf / (proj_ms * 1e-3) / 1e12 / tf32,
            "peak_source": "half of MEASURED_PEAKS.json bf16_tflops (of measured): TF32 tensor rate",
            "note": "bound by forming its operands (tables in FP64, TF32 splits), not by the tensor pipe"}]

    # ------------------------------------------------ end to end (host buffers)
    wfc_pin = [torch.empty(w.shape, dtype=torch.complex128, pin_memory=True) for w in s.wfc]
    for t, w in zip(wfc_pin, s.wfc):
        t.numpy()[...] = w
    dv_pin = torch.empty(s.dVscf.shape, dtype=torch.complex128, pin_memory=True)
    dv_pin.numpy()[...] = s.dVscf
    g_pin = torch.empty((npairs, s.nmodes, s.nspin, s.nbnds, s.nbnds), dtype=torch.complex64, pin_memory=True)
    wnp = [t.numpy() for t in wfc_pin]
    dvnp = dv_pin.numpy()
    gnp = g_pin.numpy()
    h2d = sum(w.nbytes for w in wnp) + dvnp.nbytes + s.eigVec.nbytes
    d2h = gnp.nbytes

    def e2e_step():
        ctx.set_wavefunctions(wnp)
        for iq in range(nq):
            ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], dvnp[iq])
        ctx.run(qs, ks, out=OUT_C64, g_out=gnp)

    for _ in range(2):
        e2e_step()
    dist.barrier()
    torch.cuda.synchronize()
    e2e_ms = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        e2e_step()
        torch.cuda.synchronize()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_step_ms = dist.max(sum(e2e_ms) / len(e2e_ms))
    g_mixed = gnp.copy()

    # ------------------------------------------------ FP64 form on a sample
    fp64 = None
    if not args.no_fp64 and rank == 0:
        # every q of a few evenly spaced k-points (the batch's own mix: a route that
        # builds psi_k(r) per k amortises it over the q of that k), on both routes
        nks = max(1, min(nk, args.fp64_pairs // nq))
        kk = (np.arange(nks) * (nk // nks)).astype(np.int32)
        sel = np.sort(np.concatenate([q * nk + kk for q in range(nq)]))
        routes = {}
        g64 = None
        for route in ("real", "gspace"):
            with LelphGPU(s, "fp64", device=local, route=route) as c64:
                for iq in range(nq):
                    c64.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
                c64.prepare()
                c64.run(qs[sel[:2]], ks[sel[:2]])
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                c64.prepare()
                torch.cuda.synchronize()
                t_prep = time.perf_counter() - t0
                t0 = time.perf_counter()
                g = c64.run(qs[sel], ks[sel])
                torch.cuda.synchronize()
                t_pairs = time.perf_counter() - t0
            t_batch = t_prep + t_pairs * npairs / len(sel)
            routes[route] = {"value": elems / t_batch, "ms_per_step_est": 1e3 * t_batch}
            if g64 is None:
                g64 = g
        best = max(routes, key=lambda r: routes[r]["value"])
        fp64_rate = routes[best]["value"]
        err = err_stats(g_mixed[sel].astype(np.complex128), g64)
        fp64 = {"value": fp64_rate, "unit": "g_elements/s", "ms_per_step_est": routes[best]["ms_per_step_est"],
                "route": {"real": "real-space", "gspace": "G-space"}[best], "routes": routes,
                "sample": f"full-BZ preparation + every q of {nks} k-points ({len(sel)} of {npairs} pairs), "
                          f"pair time scaled to the batch; the faster of the two FP64 routes",
                "mixed_over_fp64": (elems / (ms_step * 1e-3)) / fp64_rate,
                "mixed_error_vs_fp64": err,
                "error_definition": "e_i = ||g_mixed|-|g_fp64|| / max(|g_fp64|, 1e-6 max|g_fp64|); "
                                    "norm = ||g_mixed - g_fp64||_2 / ||g_fp64||_2 (mixed output in complex64)"}

    # ------------------------------------------------ CPU baseline (the reference's compiled stage)
    cpu = None
    if not args.no_cpu and rank == 0:
        pairs = [(i % nq, (37 * i + 5) % nk) for i in range(args.cpu_pairs)]
        exe = ref_binary(single=True)
        if exe:
            cores = os.cpu_count() or 1
            items = [(i % nq, (37 * i + 5) % nk) for i in range(cores * max(1, args.cpu_pairs // cores))]
            rr = RefRunner(s, exe)
            try:
                t = sum(rr.pairs(items[i:i + cores]) for i in range(0, len(items), cores))
            finally:
                rr.close()
            cpu = {"value": g_elems(s, len(items)) / t, "unit": "g_elements/s", "cores": cores, "kind": "reference",
                   "sample": f"{len(items)} (k,q) pairs of the workload, the reference's default single-precision "
                             f"build, one process (k pool) per core"}
        else:
            t, e = cpu_port_sample(s, pairs)
            cpu = {"value": e / t, "unit": "g_elements/s", "cores": 1, "kind": "port",
                   "sample": f"{len(pairs)} (k,q) pairs of the workload, numpy restatement, one core"}

    value = world * elems / (ms_step * 1e-3)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "g_elements/s", "n_gpus": world, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": ms_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f16x3 split on tensor cores, f32 FFT, f64 phases",
                "data": "synthetic (seeded; no public dataset)",
                "config": {"workload": WORKLOAD, "pairs_per_step": npairs, "g_elements_per_step": elems,
                           "precision": args.precision, "parallelism": f"q-sharded x{world}",
                           "route": {1: "real-space", 2: "G-space"}.get(st1["route"], st1["route"]),
                           "l2": f"inputs larger than L2 ({st1['device_bytes'] / 1e9:.1f} GB resident on the device)"},
                "e2e": {"value": world * elems / (e2e_step_ms * 1e-3), "unit": "g_elements/s",
                        "ms_per_step": e2e_step_ms, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
                "gpu_launches": int(launches), "clocks": clk, "roofline": roofline, "fp64_form": fp64,
                "cpu_baseline": cpu, "wall_s_timed": t_wall}
        line["path_roofline"] = path_roofline(s, value / world, peaks, (clk or {}).get("sm_mhz"))
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


# ------------------------------------------------------------ Dmats workload

DMAT_METRIC = "Dmats/s per GB300 (electronic_reps, every symmetry x full-BZ k)"
DMAT_JOB_BYTES = 208  # sizeof(DmatJob): the per-matrix job table copied to the device each call


def dmat_flops(s, njobs):
    """Useful contraction flops: 8 nb^2 (nspinor npw) per Dmat and spin
    (complex multiply-add = 8 real flops), npw of the k-point's own list."""
    npw = np.array([len(g) for g in s.gvec], float)
    per_k = 8.0 * s.nbnds ** 2 * s.nspinor * s.nspin * npw[s.kmap[:, 0]]
    nsym = njobs // s.nk_bz
    return float(per_k.sum() * nsym)


def run_dmats(args):
    """Dmats of the bench system: the 48 operations of the cell on the 512
    full-BZ k (24,576 matrices of 32 x 32, contraction over ~2500 plane waves)."""
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from letzelphc_gb300 import synth
    from letzelphc_gb300.build import build_library
    from letzelphc_gb300.elph import LelphGPU
    build_library()
    s = synth.make_system("c1", {"qpts": [(0.0, 0.0, 0.0)]})
    nsym = args.dmat_syms or len(s.sym_R)
    R, T, TR = s.sym_R[:nsym], s.sym_tau[:nsym], s.sym_trev[:nsym]
    njobs = nsym * s.nk_bz
    flops = dmat_flops(s, njobs)
    prec = "mixed" if args.precision.startswith("mixed") else args.precision
    ctx = LelphGPU(s, prec, device=local)
    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(max(3, args.warmup) if not args.dmat_syms else 1):
        ctx.dmats(R, T, TR, host=False)
    if args.dmat_syms:
        ctx.close()
        return 0
    st0 = ctx.stats()
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for e0, e1 in evs:
        e0.record(stream)
        ctx.dmats(R, T, TR, host=False)
        e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    st1 = ctx.stats()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in evs) / len(evs)
    launches = (st1["kernel_launches"] - st0["kernel_launches"]) // args.steps
    host_ms = (st1["dmats_host_ms"] - st0["dmats_host_ms"]) / args.steps
    # device time of the two kernels (events around the launches on the library stream)
    ctx.set_profiling(True)
    p0 = ctx.stats()
    ctx.dmats(R, T, TR, host=False)
    p1 = ctx.stats()
    ctx.set_profiling(False)
    kern_ms = p1["dmats_ms"] - p0["dmats_ms"]
    # end to end through the C ABI: host matrices out (complex128)
    e2e = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        Dm = ctx.dmats(R, T, TR)
        e2e.append(1e3 * (time.perf_counter() - t0))
    e2e_ms = sum(e2e) / len(e2e)
    ctx.close()
    # FP64 form: one pass over a block of the table, and the mixed-form error on it
    fp64 = None
    if not args.no_fp64:
        cnt = min(njobs, 4 * s.nk_bz)
        with LelphGPU(s, "fp64", device=local) as c64:
            c64.dmats(R, T, TR, count=s.nk_bz // 8, host=False)
            t0 = time.perf_counter()
            D64 = c64.dmats(R, T, TR, count=cnt)
            t64 = time.perf_counter() - t0
        err = np.abs(Dm[:cnt] - D64)
        fp64 = {"value": cnt / t64, "unit": "Dmats/s", "sample": f"first {cnt} of {njobs} matrices",
                "mixed_over_fp64": (njobs / (ms * 1e-3)) / (cnt / t64),
                "mixed_max_abs_err": float(err.max()), "mixed_rms_err": float(np.sqrt((err ** 2).mean())),
                "max_abs_D": float(np.abs(D64).max())}
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import elph_oracle as O
        pairs = [(i % nsym, (131 * i + 7) % s.nk_bz) for i in range(8)]
        t0 = time.perf_counter()
        O.dmats(s, R, T, TR, pairs=pairs)
        tc = time.perf_counter() - t0
        cpu = {"value": len(pairs) / tc, "unit": "Dmats/s", "cores": 1, "kind": "port",
               "sample": f"{len(pairs)} (symmetry, k) pairs, numpy restatement of electronic_reps, one core"}
    sm_mhz = clk.get("sm_mhz") or 1920.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    achieved = flops / (kern_ms * 1e-3) / 1e12
    line = {"metric": DMAT_METRIC, "value": njobs / (ms * 1e-3), "unit": "Dmats/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 operands and contraction, f64 phases and sums"
            if prec != "fp64" else "f64", "data": "synthetic (seeded, c1 shapes)",
            "config": {"workload": f"Dmats of the 4-atom cell: {nsym} operations x {s.nk_bz} k, 32 bands, npw~2500",
                       "matrices_per_step": njobs, "precision": prec,
                       "l2": "operands of the 35 iBZ k (18 MB) stay in L2; one launch per step"},
            "e2e": {"value": njobs / (e2e_ms * 1e-3), "unit": "Dmats/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": int(njobs * DMAT_JOB_BYTES), "d2h_bytes_per_step": int(Dm.nbytes)},
            "gpu_launches": int(launches), "clocks": clk,
            "roofline": {"kernel": "k_dmats", "bound": "fp32 (SIMT FMA)", "achieved": achieved,
                         "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                         "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 x median SM clock under load",
                         "flops_per_launch": flops, "traffic": None, "kernel_ms": kern_ms,
                         "host_job_ms": host_ms,
                         "note": "achieved = contraction flops / device time of the map + contraction kernels; "
                                 "ms_per_step also holds the host-side job construction"},
            "fp64_form": fp64, "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)
    return 0


def run_star(args):
    """The stage with its q-star expansion: for each of the bench's 8 q, g at
    every full-BZ k and its rotation onto every member of the q's star
    (compute_elphq_star), with the Dmats of the 48 operations resident."""
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from letzelphc_gb300 import synth
    from letzelphc_gb300.build import build_library
    from letzelphc_gb300.elph import LelphGPU, OUT_C64
    build_library()
    s = synth.make_system("c1", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0), (0.5, 0.5, 0)]} if args.small else None)
    # the stars as a phonon code lists them: members S q, the first S producing each
    A, qst = s.alat, []
    for q in s.qpts:
        qc = np.linalg.solve(A.T, np.asarray(q, float))
        mem, sy = [], []
        for i, R in enumerate(s.sym_R):
            sq = A.T @ (R @ qc)
            if not any(np.linalg.norm((sq - m) - np.rint(sq - m)) < 1e-5 for m in mem):
                mem.append(sq)
                sy.append(i)
        qst.append(np.array(sy, np.int32))
    nq_bz = sum(len(x) for x in qst)
    gsz = s.nmodes * s.nspin * s.nbnds * s.nbnds
    elems = nq_bz * s.nk_bz * gsz
    prec = args.precision
    ctx = LelphGPU(s, prec, device=local)
    ctx.dmats(s.sym_R, s.sym_tau, s.sym_trev, host=False)

    def step():
        for iq in range(len(s.qpts)):
            ctx.compute_elphq_star(s.qpts[iq], s.eigVec[iq], s.dVscf[iq], qst[iq], out=OUT_C64)

    for _ in range(max(3, args.warmup)):
        step()
    st0 = ctx.stats()
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    st1 = ctx.stats()
    launches = (st1["kernel_launches"] - st0["kernel_launches"]) // args.steps
    ctx.set_profiling(True)
    p0 = ctx.stats()
    step()
    p1 = ctx.stats()
    ctx.set_profiling(False)
    ctx.close()
    qs_ms = p1["qstar_ms"] - p0["qstar_ms"]
    items = (nq_bz - len(s.qpts)) * s.nk_bz
    flops = items * s.nmodes * s.nspin * 2 * 8.0 * s.nbnds ** 3
    sm_mhz = clk.get("sm_mhz") or 1920.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    line = {"metric": "g elements/s per GB300 with the q-star expansion (every star member at every S k)",
            "value": elems / wall, "unit": "g_elements/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": 1e3 * wall, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": prec, "data": "synthetic (seeded, c1 shapes)",
            "config": {"workload": f"{WORKLOAD}; stars of the 8 q: {[len(x) for x in qst]} members, "
                                   f"{nq_bz} q in all", "g_elements_per_step": elems,
                       "timing": "host wall clock around the 8 C-ABI calls (each ends with its D2H copy)"},
            "e2e": {"value": elems / wall, "unit": "g_elements/s", "h2d_bytes_per_step": int(s.dVscf.nbytes),
                    "d2h_bytes_per_step": int(elems * 8)},
            "gpu_launches": int(launches), "clocks": clk,
            "roofline": {"kernel": "k_qstar", "bound": "fp32 (SIMT FMA)" if prec != "fp64" else "fp64",
                         "achieved": flops / (qs_ms * 1e-3) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": flops / (qs_ms * 1e-3) / 1e12 / fp32_peak, "kernel_ms": qs_ms,
                         "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 x median SM clock under load",
                         "flops_per_step": flops, "traffic": None}}
    print(json.dumps(line), flush=True)
    return 0


def run_dvscf(args):
    """dV_scf ingest of the bench's 8 q: QE-layout (pattern, nmag, Nz, Ny, Nx)
    arrays in pinned host memory -> q slots in the mode basis (transpose and
    eig pats^H on the device)."""
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from letzelphc_gb300 import synth
    from letzelphc_gb300.build import build_library
    from letzelphc_gb300.elph import LelphGPU
    build_library()
    s = synth.make_system("c1", {"kgrid": (2, 2, 2)} if args.small else None)
    rng = np.random.default_rng(5)
    nm, nq = s.nmodes, len(s.qpts)
    Nx, Ny, Nz = s.fft_dims
    raws = [torch.empty((nm, s.nmag, Nz, Ny, Nx), dtype=torch.complex128, pin_memory=True) for _ in range(nq)]
    for r in raws:
        r.numpy()[...] = s.dVscf[0].transpose(0, 1, 4, 3, 2)
    pats = np.linalg.qr(rng.standard_normal((nm, nm)) + 1j * rng.standard_normal((nm, nm)))[0]
    ctx = LelphGPU(s, args.precision, device=local)

    def step():
        for iq in range(nq):
            ctx.set_q_dvscf_qe(iq, s.qpts[iq], s.eigVec[iq], pats, raws[iq].numpy())

    for _ in range(max(3, args.warmup)):
        step()
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    ctx.set_profiling(True)
    p0 = ctx.stats()
    step()
    p1 = ctx.stats()
    ctx.set_profiling(False)
    ctx.close()
    kern = (p1["dvscf_ms"] - p0["dvscf_ms"]) / nq
    N = Nx * Ny * Nz
    byts = 2 * nm * s.nmag * N * 16  # one read of the QE layout, one write of the mode basis
    flops = 8.0 * nm * nm * s.nmag * N  # eig pats^H applied at every point (complex multiply-add = 8 flops)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs") or 6800.0
    line = {"metric": "dV_scf ingests/s per GB300 (QE layout -> mode-basis q slot)", "value": nq / wall,
            "unit": "q/s", "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": 1e3 * wall, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded, c1 shapes)",
            "config": {"workload": f"8 q of the 4-atom cell: {nm} patterns x {s.nmag} x 48^3 complex128 each "
                                   f"({nm * s.nmag * N * 16 / 1e6:.1f} MB)",
                       "timing": "host wall clock around the 8 C-ABI calls (pinned host arrays, H2D included)"},
            "e2e": {"value": nq / wall, "unit": "q/s", "h2d_bytes_per_step": int(nq * nm * s.nmag * N * 16),
                    "d2h_bytes_per_step": 0},
            "gpu_launches": nq, "clocks": clk,
            "roofline": {"kernel": "k_dvscf_ingest", "bound": "fp64",
                         "achieved": flops / (kern * 1e-3) / 1e12, "peak": 1.25, "unit": "TFLOP/s",
                         "frac": flops / (kern * 1e-3) / 1e12 / 1.25, "kernel_ms": kern,
                         "peak_source": "nominal GB300 FP64 rate (no measured FP64 peak)",
                         "flops_per_launch": flops, "hbm_gbs": byts / (kern * 1e-3) / 1e9,
                         "hbm_frac": byts / (kern * 1e-3) / 1e9 / peak, "bytes_per_launch": byts, "traffic": None}}
    print(json.dumps(line), flush=True)
    return 0


def run_gspace(args):
    """The G-space route on the 16-atom, 200-band configuration (96^3 box, 60^3
    product grid, npw ~12000): the first 8 irreducible q at a block of k
    points (16 k; with --small a 2x2x2 k grid and 2 q, the profiling case),
    device-resident output, CUDA events on the library stream; per-kernel
    device times from the library's profiling counters in a separate pass."""
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from letzelphc_gb300 import synth
    from letzelphc_gb300.build import build_library
    from letzelphc_gb300.elph import LelphGPU, OUT_C64
    build_library()
    if args.small:
        s = synth.make_system("c4", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0), (0.5, 0.5, 0)]})
        kk = np.arange(s.nk_bz)
    else:
        s = synth.make_system("c4", {"qpts": [tuple(q) for q in _c4_qpts()[:8]]})
        kk = np.arange(16) * (s.nk_bz // 16)
    nq = len(s.qpts)
    qs = np.repeat(np.arange(nq), len(kk)).astype(np.int32)
    ks = np.tile(kk, nq).astype(np.int32)
    npairs = len(qs)
    gsz = s.nmodes * s.nspin * s.nbnds * s.nbnds
    ctx = LelphGPU(s, args.precision, device=local)
    for iq in range(nq):
        ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
    ctx.prepare()
    gdev = torch.empty(npairs * gsz * 2, dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(max(3, args.warmup)):
        ctx.run_device(qs, ks, gdev.data_ptr(), out=OUT_C64)
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        ctx.run_device(qs, ks, gdev.data_ptr(), out=OUT_C64)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ctx.set_profiling(True)
    p0 = ctx.stats()
    ctx.run_device(qs, ks, gdev.data_ptr(), out=OUT_C64)
    p1 = ctx.stats()
    ctx.set_profiling(False)
    st = ctx.stats()
    ctx.close()
    d = {k: (p1[k] - p0[k]) / npairs for k in ("gs_plane_ms", "gs_xpass_ms", "gs_gemm_ms", "local_ms", "finish_ms")}
    npw = int(np.mean([len(g) for g in s.gvec]))
    gemm_flops = 8.0 * s.nmodes * s.nbnds * s.nbnds * s.nspinor * npw * s.nspin  # complex MACs x 8 per pair
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12  # nominal FP32 (non-tensor) rate at the maximum SM clock
    elems = npairs * gsz
    tc = args.precision != "fp64" and os.environ.get("LELPH_GS_TC", "1") != "0"
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    if tc:
        # three TF32 products (hi hi, hi lo, lo hi) of the real GEMM; TF32 runs at
        # half the bf16 rate of the tensor cores
        tflops = 3 * gemm_flops / (d["gs_gemm_ms"] * 1e-3) / 1e12 if d["gs_gemm_ms"] else None
        tpeak = (peaks.get("bf16_tflops") or 1900.0) / 2
        roof = {"kernel": "k_gs_gemm_tc (split-TF32 tcgen05 GEMM)", "bound": "tensor", "achieved": tflops,
                "peak": tpeak, "unit": "TFLOP/s", "frac": tflops / tpeak if tflops else None,
                "peak_source": "half of MEASURED_PEAKS.json bf16_tflops (of measured): TF32 tensor rate"
                if peaks else "half of the fallback bf16 peak", "flops_per_pair": 3 * gemm_flops, "traffic": None}
    else:
        roof = {"kernel": "k_gs_gemm_f32x2", "bound": "fp32",
                "achieved": gemm_flops / (d["gs_gemm_ms"] * 1e-3) / 1e12 if d["gs_gemm_ms"] else None,
                "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": gemm_flops / (d["gs_gemm_ms"] * 1e-3) / 1e12 / fp32_peak if d["gs_gemm_ms"] else None,
                "peak_source": "nominal GB300 FP32 SIMT rate at 2070 MHz (no measured FP32 peak)",
                "flops_per_pair": gemm_flops, "traffic": None}
    line = {"metric": "g elements/s per GB300 on the G-space route (16-atom cell, 200 bands)",
            "value": elems / (ms * 1e-3), "unit": "g_elements/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.precision, "data": "synthetic (seeded, configuration-4 shapes)",
            "config": {"workload": f"{nq} q x {len(kk)} k of the 16-atom cell ({npairs} pairs, "
                                   f"product grid {list(st['product_grid'])}, npw ~{npw})",
                       "route": {1: "real-space", 2: "G-space"}.get(st["route"]),
                       "timing": "CUDA events on the library stream, device-resident inputs and output"},
            "ms_per_pair": ms / npairs, "kernel_ms_per_pair": d, "clocks": clk,
            "gpu_launches": int(p1["kernel_launches"] - p0["kernel_launches"]),
            "roofline": roof}
    print(json.dumps(line), flush=True)
    return 0


def _c4_qpts():
    """The irreducible q of the 16-atom cell's 8x8x8 grid, as synth builds them."""
    from letzelphc_gb300 import synth
    cfg = synth.CONFIGS["c4"]
    s = synth.make_system("c4", {"qpts": [(0, 0, 0)], "kgrid": cfg["kgrid"], "nbnds": 1, "npw": 50})
    return synth.reduce_grid(cfg["kgrid"], s.sym_R, s.alat)


CONFIG_NAMES = ["c0", "c1", "c2", "c3", "c4"]


def run_configs(args):
    """Every configuration at its full size: the mixed form on all (k, q) pairs
    (device-resident, CUDA events), the FP64 form on a sample of pairs (its
    full-BZ preparation plus the sampled pairs, scaled to the batch), and the
    error of the mixed form on that sample with the metric's definition.
    Pairs run in blocks of k-points (every q of each k in one call, so a
    route that builds psi(r) per k does so once per block) into an output
    buffer of at most ~8 GB that each block overwrites: the 16-atom,
    200-band configuration has 228 GB of complex64 g in all."""
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from letzelphc_gb300 import synth
    from letzelphc_gb300.build import build_library
    from letzelphc_gb300.elph import LelphGPU, OUT_C64, LelphError
    build_library()
    names = args.configs.split(",") if args.configs else CONFIG_NAMES
    out = {}
    for name in names:
        t0 = time.perf_counter()
        s = synth.make_system(name)
        gen_s = time.perf_counter() - t0
        nq, nk = len(s.qpts), s.nk_bz
        gsz = s.nmodes * s.nspin * s.nbnds * s.nbnds
        kb = int(max(1, min(nk, (8 << 30) // (8 * gsz * nq))))
        blocks = []
        for k0 in range(0, nk, kb):
            kk = np.arange(k0, min(nk, k0 + kb))
            blocks.append((np.repeat(np.arange(nq), len(kk)).astype(np.int32), np.tile(kk, nq).astype(np.int32)))
        npairs = nq * nk
        elems = g_elems(s, npairs)
        rec = {"pairs": npairs, "g_elements": elems, "input_generation_s": gen_s}
        try:
            ctx = LelphGPU(s, args.precision, device=local)
            st0 = ctx.stats()
            rec["route"] = {1: "real-space", 2: "G-space"}.get(st0["route"], st0["route"])
            rec["product_grid"] = list(st0["product_grid"])
            for iq in range(nq):
                ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
            gdev = torch.empty(len(blocks[0][0]) * gsz * 2, dtype=torch.float32, device="cuda")
            stream = torch.cuda.ExternalStream(ctx.stream())
            big = npairs * gsz > 5e9

            def step(bl):
                ctx.prepare()
                for qs, ks in bl:
                    ctx.run_device(qs, ks, gdev.data_ptr(), out=OUT_C64)

            # warm-up: the whole batch twice, or one block where the batch takes minutes
            for _ in range(1 if big else 2):
                step(blocks[:1] if big else blocks)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = 1 if big else max(1, args.steps)
            e0.record(stream)
            for _ in range(reps):
                step(blocks)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            # FP64 sample: every q of a few evenly spaced k-points (a route that
            # builds psi_k(r) per k amortises it over the q of that k, as in the batch)
            nsel = min(args.fp64_pairs if not big else 16, npairs)
            nks = max(1, min(nk, nsel // nq))
            kk = np.arange(nks) * (nk // nks)
            qs_s = np.repeat(np.arange(nq), nks).astype(np.int32)
            ks_s = np.tile(kk, nq).astype(np.int32)
            if len(qs_s) > nsel:   # more q than the sample holds: the first q's
                qs_s, ks_s = qs_s[:nsel], ks_s[:nsel]
            gm = ctx.run(qs_s, ks_s, out=OUT_C64).astype(np.complex128)
            ctx.close()
            rec.update({"mixed_value": elems / (ms * 1e-3), "mixed_ms": ms})
            routes, g64 = {}, None
            for route in ("real", "gspace"):
                try:
                    with LelphGPU(s, "fp64", device=local, route=route) as c64:
                        for iq in range(nq):
                            c64.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
                        c64.prepare()
                        c64.run(qs_s[:1], ks_s[:1])
                        torch.cuda.synchronize()
                        t0 = time.perf_counter()
                        c64.prepare()
                        torch.cuda.synchronize()
                        t_prep = time.perf_counter() - t0
                        t0 = time.perf_counter()
                        g = c64.run(qs_s, ks_s)
                        torch.cuda.synchronize()
                        t_pairs = time.perf_counter() - t0
                    routes[route] = elems / (t_prep + t_pairs * npairs / len(qs_s))
                    if g64 is None:
                        g64 = g
                except LelphError as e:
                    routes[route] = f"unsupported: {e}"
            rates = {r: v for r, v in routes.items() if not isinstance(v, str)}
            best = max(rates, key=rates.get)
            fp64_rate = rates[best]
            rec.update({"fp64_value": fp64_rate, "fp64_route": {"real": "real-space", "gspace": "G-space"}[best],
                        "fp64_routes": routes, "mixed_over_fp64": rec["mixed_value"] / fp64_rate,
                        "error_vs_fp64": err_stats(gm, g64), "sample_pairs": len(qs_s)})
        except LelphError as e:
            rec["status"] = f"unsupported: {e}"
        out[name] = rec
        print(json.dumps({name: rec}), file=sys.stderr, flush=True)
        del s
    line = {"metric": METRIC, "unit": "g_elements/s", "n_gpus": 1, "dtype": args.precision,
            "data": "synthetic (seeded, the configurations' shapes)", "configs": out,
            "error_definition": "e_i = ||g_mixed|-|g_fp64|| / max(|g_fp64|, 1e-6 max|g_fp64|); norm = "
                                "||g_mixed - g_fp64||_2 / ||g_fp64||_2 (mixed output in complex64)"}
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args):
    """The batched uneven workload (3-atom hexagonal slab, 36x36x216 grid,
    12x12x1 k, 64 q, 9 modes, 40 bands, npw 1800-2600 across k) three ways on
    the mixed form, device-resident, CUDA events on the library stream:
    * batch: every (k, q) pair of the 64 q in one call (the tensor-core
      sandwich is one persistent launch over all pairs);
    * per q: one call per q-point (144 pairs each), the reference's per-q
      stage granularity (compute_and_write_elphq, src/elph/elph_driver.c:200-307);
    * per (k, q): one call per pair, the granularity of the reference's k
      loop (src/elph/compute_elph_matq.c:116-150), on a sample of the pairs
      and scaled to the batch.
    The full-BZ preparation (unfold, FFTs, projections) is timed once and
    counted in every rate."""
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from letzelphc_gb300 import synth
    from letzelphc_gb300.build import build_library
    from letzelphc_gb300.elph import LelphGPU, OUT_C64
    build_library()
    s = synth.make_system("c2")
    nq, nk = len(s.qpts), s.nk_bz
    gsz = s.nmodes * s.nspin * s.nbnds * s.nbnds
    npairs = nq * nk
    elems = g_elems(s, npairs)
    qs = np.repeat(np.arange(nq), nk).astype(np.int32)
    ks = np.tile(np.arange(nk), nq).astype(np.int32)
    ctx = LelphGPU(s, args.precision, device=local)
    for iq in range(nq):
        ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
    gdev = torch.empty(npairs * gsz * 2, dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream())
    es = 8 * gsz  # bytes of one pair's complex64 output

    def timed(fn, reps=1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, 1e3 * (time.perf_counter() - t0) / reps

    ctx.prepare()
    ctx.run_device(qs, ks, gdev.data_ptr(), out=OUT_C64)   # warm-up (windows, kernels loaded)
    prep_ms, _ = timed(ctx.prepare, 3)
    batch_ms, batch_wall = timed(lambda: ctx.run_device(qs, ks, gdev.data_ptr(), out=OUT_C64), max(3, args.steps))

    def per_q():
        for iq in range(nq):
            sl = slice(iq * nk, (iq + 1) * nk)
            ctx.run_device(qs[sl], ks[sl], gdev.data_ptr() + iq * nk * es, out=OUT_C64)
    perq_ms, perq_wall = timed(per_q)
    nsamp = min(npairs, 4 * nk)
    rng = np.random.default_rng(2)
    sel = np.sort(rng.choice(npairs, size=nsamp, replace=False))

    def per_pair():
        for i in sel:
            ctx.run_device(qs[i:i + 1], ks[i:i + 1], gdev.data_ptr() + int(i) * es, out=OUT_C64)
    pp_ms, pp_wall = timed(per_pair)
    pp_full_ms = pp_ms * npairs / nsamp
    pp_full_wall = pp_wall * npairs / nsamp
    st = ctx.stats()
    ctx.close()
    rate = lambda ms: elems / ((prep_ms + ms) * 1e-3)  # noqa: E731
    line = {"metric": METRIC, "unit": "g_elements/s", "n_gpus": 1, "dtype": args.precision,
            "data": "synthetic (seeded, the batched uneven workload's shapes)",
            "config": {"workload": "3-atom hexagonal slab, 36x36x216 grid, 12x12x1 k, 64 q, 9 modes, 40 bands, "
                                   "npw 1800-2600", "pairs": npairs, "g_elements": elems,
                       "route": {1: "real-space", 2: "G-space"}.get(st["route"], st["route"]),
                       "product_grid": list(st["product_grid"])},
            "prepare_ms": prep_ms,
            "batch": {"value": rate(batch_ms), "pairs_ms": batch_ms, "wall_ms": batch_wall, "calls": 1},
            "per_q": {"value": rate(perq_ms), "pairs_ms": perq_ms, "wall_ms": perq_wall, "calls": nq},
            "per_pair": {"value": rate(pp_full_ms), "pairs_ms": pp_full_ms, "wall_ms": pp_full_wall,
                         "calls": npairs, "sample_pairs": int(nsamp),
                         "note": "timed on the sample, scaled to every pair of the batch"},
            "batch_over_per_pair": (prep_ms + pp_full_ms) / (prep_ms + batch_ms),
            "batch_over_per_q": (prep_ms + perq_ms) / (prep_ms + batch_ms)}
    print(json.dumps(line), flush=True)
    return 0


def run_tune(args):
    """lelph_gpu_tune on every configuration's shape (the first q with a
    nonzero vector, its first 64 full-BZ k-points as the sample, 16 for the
    16-atom cell): the measured time per pair of each candidate and the choice
    -- the route table of the library."""
    import torch
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from letzelphc_gb300 import synth
    from letzelphc_gb300.build import build_library
    from letzelphc_gb300.elph import tune
    build_library()
    names = args.configs.split(",") if args.configs else CONFIG_NAMES
    out = {}
    for name in names:
        ov = {"qpts": [tuple(q) for q in _c4_qpts()[1:2]]} if name == "c4" else {}
        s = synth.make_system(name, ov)
        iq = 1 if len(s.qpts) > 1 else 0
        rec = {}
        npt = 16 if name == "c4" else min(s.nk_bz, 64)
        for prec in (args.precision, "fp64"):
            rec[prec] = tune(s, prec, iq=iq, npairs=npt, device=local)
        rec["pairs"] = npt
        out[name] = rec
        print(json.dumps({name: rec}), file=sys.stderr, flush=True)
        del s
    print(json.dumps({"workload": "lelph_gpu_tune on every configuration's shape (first q with a nonzero "
                                  "vector, its first 64 full-BZ k-points per candidate, 16 for c4)",
                      "configs": out}), flush=True)
    return 0


def main():
    args = parse()
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "tune":
        return run_tune(args)
    if args.workload == "configs":
        return run_configs(args)
    if args.workload == "gspace":
        return run_gspace(args)
    if args.workload == "dvscf":
        return run_dvscf(args)
    if args.workload == "dmats":
        return run_dmats(args)
    if args.workload == "star":
        return run_star(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return run_profile_case(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
