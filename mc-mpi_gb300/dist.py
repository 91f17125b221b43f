"""Multi-GPU sharding of histories (one process per GPU).

Histories are independent, so N ranks take disjoint contiguous ranges of the
source's history indices (weak or strong scaling as the caller chooses) and
the only combination step is an exact sum of the int64 fixed-point tallies
at the end: the result is bit-identical to a single GPU running every
history.  No data-path collective is needed; the final reduction uses
torch.distributed (NCCL on GPUs, gloo on CPU).
"""


def shard(n_total, world_size, rank):
    """(first, count) of rank's contiguous share of n_total histories; the
    first n_total % world_size ranks take one more (as decompose_domain
    splits cells, src/layer.cpp:23-27)."""
    if world_size <= 0 or not (0 <= rank < world_size) or n_total < 0:
        raise ValueError("bad shard arguments")
    base, extra = divmod(n_total, world_size)
    count = base + (1 if rank < extra else 0)
    first = rank * base + min(rank, extra)
    return first, count


def allreduce_tally(tally_q, group=None):
    """Exact in-place sum of int64 fixed-point tallies over all ranks."""
    import torch
    import torch.distributed as dist
    assert tally_q.dtype == torch.int64
    dist.all_reduce(tally_q, op=dist.ReduceOp.SUM, group=group)
    return tally_q


def sharded_tally(run_shard, n_total, world_size, rank, device=None, group=None):
    """This rank's share of histories 0 .. n_total-1 run by
    run_shard(first, count) -> int64 tally (numpy array or torch tensor), then
    the exact sum over all ranks (allreduce_tally).  Returns the reduced int64
    torch tensor on `device` (the GPU for NCCL, None for gloo on the CPU);
    every rank holds the result, which equals one rank running every history."""
    import numpy as np
    import torch
    first, count = shard(n_total, world_size, rank)
    q = run_shard(first, count)
    t = q if isinstance(q, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(q, np.int64))
    t = t.to(device=device, dtype=torch.int64).contiguous()
    return allreduce_tally(t, group=group)
