"""Replica-parallel helpers (the path has no exchange step: every transform and
product is independent, so N GPUs run N replicas over disjoint shards and the
only collectives are a barrier and the max of the timings)."""
import os


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def shard(count, rank, world):
    """Contiguous [start, end) share of `count` independent units for `rank`."""
    base, extra = divmod(count, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value, device="cpu"):
    """Max of a float over all ranks (identity without an initialised process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, seconds, device="cpu"):
    """Whole-job throughput: units of all ranks over the slowest rank's time."""
    import torch.distributed as dist
    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    return world * units_per_rank / max_over_ranks(seconds, device)
