"""Independent replicas of the sampler, one process per GPU.

The MCMC over SNP inclusion does not shard: each chain touches all p SNPs
every RB step, and chains exchange nothing (src/main.cpp:92-116 runs one
Sampler per thread on shared read-only data).  N GPUs therefore run N
independent replicas with disjoint seeds; the only collective is the
max-over-ranks of the timed region, on the host side of the measurement.
"""
import os


def rank_info():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seeds(rank, chains, seed0=1):
    """Chain seeds of one replica: distinct across ranks and chains."""
    base = seed0 + 7919 * rank
    return [base + 1000 * c for c in range(chains)]


def max_over_ranks(x, device=None):
    """Max of a float over all ranks of the default process group (x itself
    when no group is initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(seconds_max, steps, chains_per_rank, world):
    """Whole-job chain-iterations per second: the units of all ranks over the
    slowest rank's time."""
    if seconds_max <= 0:
        raise ValueError("non-positive timed region")
    return steps * chains_per_rank * world / seconds_max
