"""q pools across processes (letzelphc_gb300/qpool.py), on CPU.

* the block split equals the reference's distribute_to_grps
  (src/common/parallel.c:48-76) for many (nq, pools);
* two gloo ranks on 127.0.0.1 each compute their pool's matrix elements and
  the gathered result equals the single-process one; every q is computed by
  exactly one rank.  The per-q computation in this test is the CPU oracle
  (the GPU path is exercised by the gpu-marked tests).
"""
import os
import socket

import numpy as np
import pytest

from letzelphc_gb300.qpool import merge_pools, pool_indices, q_pool


def _reference_split(n, ngrp, igrp):
    # the arithmetic of distribute_to_grps, written out for the comparison
    n_q, n_r = n // ngrp, n % ngrp
    cnt = n_q + (1 if igrp < n_r else 0)
    shift = n_q * igrp + (igrp if igrp < n_r else n_r)
    return cnt, shift


def test_split_matches_reference():
    for n in range(0, 40):
        for p in range(1, 9):
            idx = []
            for r in range(p):
                assert q_pool(n, r, p) == _reference_split(n, p, r)
                idx += pool_indices(n, r, p)
            assert idx == list(range(n))


def test_merge_rejects_overlap_and_gaps():
    with pytest.raises(ValueError):
        merge_pools([{0: 1, 1: 2}, {1: 3}], 2)
    with pytest.raises(ValueError):
        merge_pools([{0: 1}], 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _system():
    from letzelphc_gb300 import synth
    return synth.make_system("c0", {"kgrid": (2, 2, 2), "nbnds": 3,
                                    "qpts": [(0, 0, 0), (0.5, 0, 0), (0.5, 0.5, 0)]})


def _worker(rank, world, port, outdir):
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import sys
        sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
        import elph_oracle as O
        from letzelphc_gb300.qpool import run_distributed
        s = _system()
        done = []

        def compute(iq):
            done.append(iq)
            return O.compute_elphq(s, iq, non_loc=True)

        g = run_distributed(len(s.qpts), compute)
        np.save(os.path.join(outdir, f"g{rank}.npy"), np.array(g))
        np.save(os.path.join(outdir, f"done{rank}.npy"), np.array(done, dtype=np.int64))
    finally:
        td.destroy_process_group()


def test_two_gloo_ranks_match_single_process(tmp_path):
    import torch.multiprocessing as mp
    import elph_oracle as O
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    s = _system()
    ref = np.array([O.compute_elphq(s, iq, non_loc=True) for iq in range(len(s.qpts))])
    done = [set(np.load(tmp_path / f"done{r}.npy").tolist()) for r in range(2)]
    assert done[0].isdisjoint(done[1]) and done[0] | done[1] == set(range(len(s.qpts)))
    for r in range(2):
        g = np.load(tmp_path / f"g{r}.npy")
        assert np.array_equal(g, ref)
