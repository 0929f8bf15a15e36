"""Shot sharding over two ranks (gloo on CPU, no GPU): the ranks' shards
cover every shot once, and the rank-ordered FP64 reduction of the shard
gradients (oracle FP32 batch gradients) equals the one-process gradient of
the whole batch to FP32 rounding, with identical picks per shot; the
reduction gives the same bits for numpy input and for tensors (the form the
bench's multi-GPU step passes, there as device tensors)."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case():
    rng = np.random.default_rng(11)
    S = (1.0 / rng.uniform(1500, 3000, (50, 30))).astype(np.float32)
    shots = [(float(x), 0.0) for x in range(20, 480, 60)] + [(250.0, 40.0, 5, 30)]
    rx = np.linspace(0, 490, 20).astype(np.float32)
    rz = np.full(20, 5.0, np.float32)
    tobs = rng.normal(0.15, 0.02, (len(shots), 20)).astype(np.float32)
    return S, shots, rx, rz, tobs


def _rank(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as O
        from seisfat2d_gb300.shard import allreduce_gradient, shard, shard_indices
        S, shots, rx, rz, tobs = _case()
        Sp = O.expand_boundary(S)
        idx = shard_indices(len(shots), rank, world)
        mine = shard(shots, rank, world)
        J, g, pk, _ = O.batch_misfit_gradient(Sp, 10.0, 10.0, mine, rx, rz, tobs[idx], nthreads=1)
        gsum, Jsum = allreduce_gradient(g, J)
        # the engine's calling convention: the gradient and the misfit as tensors
        # (device tensors under NCCL; CPU tensors here under gloo), no host copy
        import torch
        gt, Jt = allreduce_gradient(torch.from_numpy(g), torch.tensor([J], dtype=torch.float64))
        assert isinstance(gt, torch.Tensor) and gt.dtype == torch.float64
        assert np.array_equal(gt.numpy(), gsum) and float(Jt.item()) == Jsum
        np.save(os.path.join(outdir, f"r{rank}.npy"), pk)
        np.save(os.path.join(outdir, f"idx{rank}.npy"), np.array(idx))
        if rank == 0:
            np.save(os.path.join(outdir, "g.npy"), gsum)
            np.save(os.path.join(outdir, "J.npy"), np.array([Jsum]))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_and_gradient(oracle, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    S, shots, rx, rz, tobs = _case()
    J, g, pk, _ = oracle.batch_misfit_gradient(oracle.expand_boundary(S), 10.0, 10.0, shots, rx, rz, tobs)
    seen = []
    for r in range(world):
        idx = np.load(tmp_path / f"idx{r}.npy")
        seen += list(idx)
        assert np.array_equal(np.load(tmp_path / f"r{r}.npy"), pk[idx], equal_nan=True)
    assert sorted(seen) == list(range(len(shots)))
    gsum = np.load(tmp_path / "g.npy")
    scale = np.abs(g).max()
    assert scale > 0
    assert np.abs(gsum - g.astype(np.float64)).max() <= 1e-6 * scale
    assert float(np.load(tmp_path / "J.npy")[0]) == pytest.approx(J, rel=1e-12)
