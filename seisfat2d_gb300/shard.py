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
    """Sum of every rank's (grad, misfit) in FP64, in rank order.

    grad: a torch tensor on the device the process group communicates on
    (CUDA under NCCL, CPU under gloo), or a numpy array (gathered as a CPU
    tensor, for gloo). misfit: None, a number or a one-element tensor on the
    same device. Each rank's partial is gathered as it is (no host copy of
    device tensors) and the partials are added elementwise in rank order in
    FP64, so every rank gets the same bits whatever the backend's reduction
    order. Returns (sum, misfit_sum): a float64 tensor on grad's device (a
    numpy array for numpy input) and, with misfit, a one-element float64
    tensor on that device (a float for numpy input or a number)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    as_numpy = not isinstance(grad, torch.Tensor)
    t = (torch.from_numpy(np.ascontiguousarray(grad)) if as_numpy else grad).to(torch.float64).contiguous()
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    total = parts[0].clone()
    for p in parts[1:]:
        total += p
    msum = None
    if misfit is not None:
        m_is_tensor = isinstance(misfit, torch.Tensor)
        m = (misfit.reshape(1) if m_is_tensor else torch.tensor([float(misfit)], dtype=torch.float64))
        m = m.to(torch.float64).to(t.device)
        ms = [torch.empty_like(m) for _ in range(world)]
        dist.all_gather(ms, m, group=group)
        msum = ms[0].clone()
        for x in ms[1:]:
            msum += x
        if as_numpy or not m_is_tensor:
            msum = float(msum.item())
    return (total.numpy() if as_numpy else total), msum
