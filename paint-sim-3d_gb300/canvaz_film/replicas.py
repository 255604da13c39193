"""Replica parallelism: one process per GPU, each stepping its own canvases.

The film step shards by canvas (independent simulations), so several GPUs run
replicas with no collective on the data path.  Two pieces of host logic are
shared by the benchmark and the serving loop:
  - `shard(items, rank, world)`: the items a rank serves (round robin, every
    item on exactly one rank);
  - `whole_job_rate(units, seconds, group)`: the job-wide rate, all ranks'
    units over the slowest rank's time (one all_reduce of two scalars,
    outside the timed region).
"""


def shard(items, rank, world):
    """Round-robin share of `items` for `rank` of `world`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d of world %d" % (rank, world))
    return [x for k, x in enumerate(items) if k % world == rank]


def whole_job_rate(units, seconds, group=None):
    """(sum of units over ranks) / (max of seconds over ranks); a single
    process returns units / seconds."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return units / seconds, units, seconds
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(u.item()) / float(t.item()), float(u.item()), float(t.item())
