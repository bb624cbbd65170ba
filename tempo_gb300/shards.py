"""Column sharding across GPUs (one process per GPU).

The column step has no exchange between columns (src/module_mp_tempo_driver.F90:
400-401 loops over independent (i, j) columns), so a domain is split into contiguous
blocks of tile rows j, one block per rank, and every rank calls the step on its own
block with its own device tables.  No collective touches the data path; the only
cross-rank operation is the reduction of timings (max over ranks) and of scalar
reports.
"""
from __future__ import annotations

from typing import Sequence


def shard_rows(jts: int, jte: int, rank: int, world: int) -> tuple[int, int]:
    """Rows [jts_r, jte_r] (1-based, inclusive) of rank `rank` among `world` ranks.

    Rows are split as evenly as possible, the first ``n % world`` ranks taking one row
    more.  A rank with no rows gets an empty range (jte_r = jts_r - 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    n = max(0, jte - jts + 1)
    base, extra = divmod(n, world)
    start = jts + rank * base + min(rank, extra)
    count = base + (1 if rank < extra else 0)
    return start, start + count - 1


def shard_bounds(bounds: Sequence[int], rank: int, world: int) -> list[int]:
    """The 18 tempo_run bounds (ids..kte in the reference's argument order
    ids, ide, jds, jde, kds, kde, ims, ime, jms, jme, kms, kme, its, ite, jts, jte,
    kts, kte) with the tile rows jts:jte narrowed to this rank's block.  Memory and
    domain bounds are unchanged: every rank may hold the whole array (host-side
    decomposition) or only its block (ims:ime, jms:jme set by the caller)."""
    b = list(bounds)
    if len(b) != 18:
        raise ValueError("expected the 18 bounds ids..kte")
    b[14], b[15] = shard_rows(b[14], b[15], rank, world)
    return b


def max_over_ranks(value: float) -> float:
    """Max of a per-rank scalar over the default process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float) -> float:
    """Sum of a per-rank scalar over the default process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
