"""Atmosphere sharding over ranks (one process per GPU).

Atmospheres are independent in the LTE synthesis, its adjoint and the NLTE
iteration, so a batch splits into contiguous slices of atmospheres with no
exchange on the data path; the only collectives are the ones a caller wants
afterwards (a max of step times, a gather of spectra, a sum of chi^2).
"""
from __future__ import annotations


def shard_bounds(natm: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of rank's slice: contiguous, sizes differ by at most one,
    every atmosphere in exactly one slice."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    base, extra = divmod(natm, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def rank_seed(base: int, rank: int) -> int:
    """Seed of a rank's synthetic atmospheres (weak scaling: each rank draws
    its own batch)."""
    return base + rank


def max_over_ranks(value: float, dist=None) -> float:
    """Largest value over the ranks of the default process group (step times
    are taken as the slowest rank's)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_shards(local, dist=None) -> list:
    """Every rank's local result object, in rank order (rank slices are
    contiguous, so concatenating them restores the batch order)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [local]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, local)
    return out
