"""Replicas across the GPUs of one node: one process per GPU, each running the same H*psi
step on its own copy of the basis (the path does not shard on one-GPU machines: a basis and its
lookup table live in one GPU's memory, and the reference's own work unit -- one operator on one
wavefunction -- has no exchange step).  Whole-job throughput is the units all ranks processed
over the slowest rank's time.

Launched by ``torch.distributed.run`` (RANK / LOCAL_RANK / WORLD_SIZE / MASTER_* in the
environment); a single process without those variables is world size 1 and needs no process
group.
"""
import os


def env():
    """(world, rank, local_rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend="nccl"):
    """Join the process group when there is more than one rank; returns (world, rank, local)."""
    world, rank, local = env()
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return world, rank, local


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of a list of floats over all ranks (times: the slowest rank)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def aggregate_rate(units_per_rank, world, seconds):
    """Whole-job rate: every rank processed units_per_rank in at most `seconds`."""
    return units_per_rank * world / seconds


def finalize():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
