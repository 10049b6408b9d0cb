"""One process per GPU: which systems each rank integrates, and the
whole-job timing.

The ensemble (independent disks, each with its own step size) partitions
with no exchange between ranks: rank r owns systems [r * n, (r + 1) * n) of
the seeded ensemble, so per-GPU work stays fixed as ranks are added (weak
scaling).  A single disk does not shard; every rank integrates a replica.
The only collectives are the maximum of the ranks' timed durations and the
sum of the work they did.
"""


def ensemble_range(n_per_rank, rank, world):
    """First system and count of rank `rank` (0 <= rank < world)."""
    if not 0 <= rank < world:
        raise ValueError("rank %d outside world of %d" % (rank, world))
    return rank * n_per_rank, n_per_rank


def max_over_ranks(value, device=None):
    """Maximum of a float over all ranks of the default process group (the
    value itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device=None):
    """Sum of a float over all ranks of the default process group (the value
    itself without one): the work every rank did in the timed region."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(device=None):
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        if device is not None and dist.get_backend() == "nccl":
            dist.barrier(device_ids=[device])
        else:
            dist.barrier()
