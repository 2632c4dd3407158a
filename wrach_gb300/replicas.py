"""Host logic of runs over several GPUs (one process per GPU).

A single world does not shard: N GPUs run N independent replicas of the
step, with no collective on the data path.  Batched worlds shard by world:
each rank steps a contiguous range of the worlds, again with no data-path
collective.  The only collectives are the measurement's: the slowest rank's
time (max) and the units all ranks processed (sum).
"""
import torch


def shard(count, rank, world_size):
    """Contiguous range [start, stop) of `count` items for `rank`: the first
    count % world_size ranks take one item more."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("rank %d outside a world of %d" % (rank, world_size))
    base, extra = divmod(count, world_size)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def aggregate(seconds, units, device=None):
    """(max over ranks of `seconds`, sum over ranks of `units`) when
    torch.distributed is initialised, else the arguments themselves."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(seconds), float(units)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.all_reduce(u, op=torch.distributed.ReduceOp.SUM)
    return float(t.item()), float(u.item())
