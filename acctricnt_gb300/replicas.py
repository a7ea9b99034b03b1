"""Replica helpers for runs over several GPUs of one node.

The counting path has no exchange step: every graph (or every request) is an
independent unit, so N GPUs run N independent replicas (rank r counts its own
graph, seeded seed + r) and the only collectives are the timing ones: a barrier
around the timed region, the maximum of the ranks' times and the sum of their
work.  The helpers run on NCCL (CUDA tensors) or gloo (CPU tensors).
"""
import os


def setup():
    """(rank, world, local_rank) from the torchrun environment; initialises the
    process group when world > 1 (NCCL with a GPU, gloo without)."""
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, local


def _device():
    import torch
    import torch.distributed as dist
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce(x, world, op):
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op={"max": dist.ReduceOp.MAX, "sum": dist.ReduceOp.SUM}[op])
    return float(t.item())


def max_over_ranks(x, world):
    return reduce(x, world, "max")


def sum_over_ranks(x, world):
    return reduce(x, world, "sum")


def rank_seed(seed, rank):
    """Each replica counts its own graph."""
    return seed + rank
