"""Host logic of multi-GPU runs: one process per GPU, no data-path collective.

A single domain is not decomposed across GPUs (a slab decomposition would need a
one-cell halo exchange per sweep), so N GPUs run independent replicas; the
batched ensemble shards naturally -- its domains are independent -- so its
domain list is split across the ranks.  Collectives are used only to time the
run (max over ranks) and to gather end-of-run statistics.
"""
from __future__ import annotations


def partition(n_items: int, rank: int, world: int) -> range:
    """Contiguous, balanced share of n_items for this rank (sizes differ by <= 1)."""
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def world() -> tuple[int, int]:
    d = _dist()
    return (d.get_rank(), d.get_world_size()) if d else (0, 1)


def max_over_ranks(x: float, device=None) -> float:
    """Slowest rank's value (the job's time)."""
    d = _dist()
    if d is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def gather(values: list) -> list:
    """Every rank's list, concatenated in rank order (on every rank)."""
    d = _dist()
    if d is None:
        return list(values)
    out = [None] * d.get_world_size()
    d.all_gather_object(out, list(values))
    return [v for part in out for v in part]


def barrier() -> None:
    d = _dist()
    if d is not None:
        d.barrier()
