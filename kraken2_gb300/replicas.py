"""Read sharding for N GPUs, each holding a full replica of the table.

Classification shards by reads with no exchange during the work: rank r
classifies a contiguous range of fragments, cut on reader-block boundaries
so each block's -K counters stay on one rank.  At the end the ranks combine
their results on the host side of rank 0: calls and hit lists are gathered in
rank order (= input order), per-taxon read counts are summed, the -K
counters' states are united (merge_counter_states; rank 0 imports the union
and finishes the report's columns), and times are the maximum over ranks.
torch.distributed is only the transport here.
"""
from __future__ import annotations

import numpy as np


def shard(n_frags: int, rank: int, world: int, block: int = 1) -> tuple[int, int]:
    """Fragments [start, stop) of `rank`: near-equal contiguous shares whose
    boundaries fall on multiples of `block` (reader blocks)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    n_blocks = -(-n_frags // block)
    b0 = n_blocks * rank // world
    b1 = n_blocks * (rank + 1) // world
    return min(n_frags, b0 * block), min(n_frags, b1 * block)


def max_over_ranks(pg, value: float, device=None) -> float:
    """The largest `value` of all ranks (a time: the job ends with its slowest rank)."""
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, counts: np.ndarray, device=None) -> np.ndarray:
    """Element-wise sum of per-taxon counts over ranks."""
    if pg is None:
        return counts
    import torch
    t = torch.from_numpy(np.ascontiguousarray(counts).view(np.int64).copy())
    if device is not None:
        t = t.to(device)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return t.cpu().numpy().view(np.uint64)


def gather_in_order(pg, rank: int, world: int, local: np.ndarray) -> np.ndarray | None:
    """Concatenation of every rank's array in rank order, on rank 0 (None elsewhere)."""
    if pg is None:
        return local
    parts = [None] * world if rank == 0 else None
    pg.gather_object(local, parts, dst=0)
    return np.concatenate(parts) if rank == 0 else None


def merge_counter_states(states: list) -> dict:
    """The union of -K counter states (k2g_counters_export of each rank):
    distinct (taxon, encoding) entries united, add_kmer counts added, dense
    flags or-ed -- the state one k2g_counters object would hold had it seen
    every rank's reader blocks (the reference merges its threads' block
    sketches into one, src/hyperloglogplus.cc:573-651)."""
    if not states:
        raise ValueError("no states")
    ent = np.unique(np.concatenate([np.asarray(s["entries"], np.uint64) for s in states]))
    tk = np.sum([np.asarray(s["taxon_kmers"], np.uint64) for s in states], axis=0, dtype=np.uint64)
    dn = np.bitwise_or.reduce([np.asarray(s["dense"], np.uint8) for s in states], axis=0)
    return {"entries": ent, "taxon_kmers": tk, "dense": dn.astype(np.uint8)}


def gather_counter_states(pg, rank: int, world: int, state: dict) -> dict | None:
    """Every rank's counter state united on rank 0 (None elsewhere)."""
    if pg is None:
        return state
    parts = [None] * world if rank == 0 else None
    pg.gather_object(state, parts, dst=0)
    return merge_counter_states(parts) if rank == 0 else None
