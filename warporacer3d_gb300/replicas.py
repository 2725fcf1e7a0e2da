"""Multi-GPU runs as independent replicas.

Cars never interact, so N GPUs run N copies of the rollout, each with its own
cars (its own sim seed) and no data-path collective. The only cross-rank
steps are bookkeeping: a barrier around the timed region and the maximum of
the per-rank times, so the reported throughput is what the whole job did in
the time its slowest rank took.
"""
import os


def topology():
    """(rank, world size, local rank) from the launcher's environment (1 process when unset)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base, rank):
    """Sim seed of rank `rank`: distinct spawns per replica."""
    return base + rank


def max_over_ranks(value, dist=None, device=None):
    """Largest `value` over all ranks (the value itself in a single process)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds):
    """Units processed by all ranks per second of the slowest rank's time."""
    return units_per_rank * world / seconds
