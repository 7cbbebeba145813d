"""Multi-process helpers of the benchmark (one process per GPU).

The path does not shard across GPUs here: every rank runs its own replica (its own
ensemble members of the same grid), so there is no data-path collective. The only
communication is the timing protocol: a barrier on both sides of the timed region
and the maximum elapsed time over ranks.
"""
import os


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def init(backend):
    """Initialise torch.distributed when launched with WORLD_SIZE > 1."""
    import torch.distributed as dist
    rank, world, _ = env_rank()
    if world > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend, rank=rank, world_size=world)
    return rank, world


def barrier(device=None):
    import torch.distributed as dist
    if dist.is_initialized():
        if device is not None and dist.get_backend() == "nccl":
            dist.barrier(device_ids=[device])
        else:
            dist.barrier()


def max_over_ranks(value, device="cpu"):
    """Maximum of a float over all ranks (identity without torch.distributed)."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device="cpu"):
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def member_range(nmembers, rank, world):
    """Members [lo, hi) of an ensemble owned by one rank (contiguous blocks)."""
    base, extra = divmod(nmembers, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)
