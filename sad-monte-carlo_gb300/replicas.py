"""Replicas across GPUs (one process per GPU).

Walkers never exchange anything (src/mc/energy.rs runs one independent chain per
walker), so N GPUs run N independent batches: rank r owns walkers
[r * W, (r + 1) * W) of the global numbering, seeds its configurations and Philox stream
from its global walker indices, and the only collectives are a barrier around the timed
region, a max over ranks of the elapsed time, and an optional host gather of results.
"""
import torch
import torch.distributed as dist


def walker_range(rank, walkers_per_rank):
    """Global walker indices owned by `rank` (weak scaling: fixed walkers per rank)."""
    return range(rank * walkers_per_rank, (rank + 1) * walkers_per_rank)


def rank_seed(base_seed, rank):
    """Philox seed of a rank's batch; walker w of the batch draws from (seed, w), so
    distinct seeds keep every global walker's stream distinct."""
    return (int(base_seed) + 0x9E3779B97F4A7C15 * (rank + 1)) & 0xFFFFFFFFFFFFFFFF


def max_over_ranks(value, device=None):
    """Largest value over ranks (the elapsed time of the slowest replica)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device=None):
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_to_rank0(array, device=None):
    """Host gather of equally shaped per-rank arrays (e.g. ln w planes) onto rank 0."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [array]
    t = torch.as_tensor(array, device=device)
    out = [torch.empty_like(t) for _ in range(dist.get_world_size())] if dist.get_rank() == 0 else None
    dist.gather(t, gather_list=out, dst=0)
    return [o.cpu().numpy() for o in out] if out is not None else None
