"""Host logic of multi-GPU runs.  Frames and scenes are independent, so N
GPUs run N replicas (or N shards of a scene set) with no collective on the
data path; only the timing is combined: the whole job takes as long as its
slowest rank, and its throughput is all ranks' units over that time."""
import os


def dist_env():
    """(rank, world, local_rank) from the torchrun environment."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def shard(n_items, rank, world):
    """Contiguous, balanced range [begin, end) of n_items for this rank."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank %d of %d" % (rank, world))
    base, extra = divmod(int(n_items), world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def _reduce(value, op):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value):
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.MAX)


def sum_over_ranks(value):
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.SUM)


def job_throughput(units_local, seconds_local):
    """Units of all ranks per second of the slowest rank."""
    seconds = max_over_ranks(seconds_local)
    units = sum_over_ranks(units_local)
    return units / seconds if seconds > 0 else 0.0
