"""Shot sharding across ranks (one process per GPU).

Shots are independent, so a batch splits by shot with no exchange in the
forward; the adjoint gradient is a sum over shots, so the ranks' partial
gradients are summed once at the end. The sum is deterministic: every rank
gathers all partials and adds them in FP64 in rank order (an all-reduce's
internal order is not fixed), and the misfit likewise.
"""
import numpy as np


def shard(items, rank, world):
    """The items of rank `rank` of `world`: every world-th one, from rank on
    (interleaved, so windows of uneven width spread evenly)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return list(items)[rank::world]


def shard_indices(n, rank, world):
    return list(range(rank, n, world))


def allreduce_gradient(grad, misfit=None, group=None):
    """Sum of every rank's (grad, misfit) in FP64, rank order; returns
    (grad_sum float64 numpy array, misfit_sum or None). Uses
    torch.distributed (any backend; gloo on CPU tensors)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    t = torch.as_tensor(np.ascontiguousarray(grad), dtype=torch.float64).cpu()
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    total = parts[0].clone()
    for p in parts[1:]:
        total += p
    msum = None
    if misfit is not None:
        m = torch.tensor([float(misfit)], dtype=torch.float64)
        ms = [torch.empty_like(m) for _ in range(world)]
        dist.all_gather(ms, m, group=group)
        msum = 0.0
        for x in ms:
            msum += float(x.item())
    return total.numpy(), msum
