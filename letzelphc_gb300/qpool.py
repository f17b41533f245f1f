"""q-point pools across processes, one process per GPU.

The reference splits the irreducible q-points over `nqpool` groups in
contiguous blocks (distribute_to_grps, src/common/parallel.c:48-76, called by
src/io/qe/get_data_from_qe.c:52-54); each pool then runs the per-q stage for
its own q with no data exchanged, and the results land in disjoint q rows of
ndb.elph.  The same split is used here: every rank owns a contiguous block of
q, runs it on its own GPU through the C ABI, and only the final gather of
the (disjoint) results, if the caller wants one, crosses processes.
"""
from __future__ import annotations

from typing import Callable, Dict, List, Sequence, Tuple


def q_pool(nq: int, rank: int, world: int) -> Tuple[int, int]:
    """(count, first index) of the q block of `rank` among `world` pools:
    the first nq % world pools take one extra q."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(nq, world)
    count = base + (1 if rank < extra else 0)
    first = base * rank + min(rank, extra)
    return count, first


def pool_indices(nq: int, rank: int, world: int) -> List[int]:
    count, first = q_pool(nq, rank, world)
    return list(range(first, first + count))


def run_pool(nq: int, rank: int, world: int, compute: Callable[[int], object]) -> Dict[int, object]:
    """Run `compute(iq)` for the q of this rank's pool; returns {iq: result}."""
    return {iq: compute(iq) for iq in pool_indices(nq, rank, world)}


def merge_pools(parts: Sequence[Dict[int, object]], nq: int) -> List[object]:
    """Results of every pool in q order; every q must come from exactly one pool."""
    out: Dict[int, object] = {}
    for p in parts:
        for iq, v in p.items():
            if iq in out:
                raise ValueError(f"q {iq} computed by two pools")
            out[iq] = v
    missing = [iq for iq in range(nq) if iq not in out]
    if missing:
        raise ValueError(f"q {missing} computed by no pool")
    return [out[iq] for iq in range(nq)]


def run_distributed(nq: int, compute: Callable[[int], object], gather: bool = True):
    """Inside an initialised torch.distributed job (one rank per GPU): run this
    rank's pool; with `gather`, every rank receives all results in q order
    (all_gather_object of the disjoint parts, the only exchange)."""
    import torch.distributed as td
    rank, world = td.get_rank(), td.get_world_size()
    mine = run_pool(nq, rank, world, compute)
    if not gather:
        return mine
    parts: List[Dict[int, object]] = [None] * world  # type: ignore
    td.all_gather_object(parts, mine)
    return merge_pools(parts, nq)
