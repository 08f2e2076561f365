"""Multi-rank host logic (gbgpu_gb300.sharding) with two gloo ranks on CPU.

The GPU path runs one process per GPU with the same calls over nccl; here the
same functions run over gloo: the binary slices partition the batch, template
groups partition the groups, the gather rebuilds the full per-binary result in
order, and max_over_ranks returns the slowest rank's times.
"""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, G):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from gbgpu_gb300 import sharding
        lo, hi = sharding.shard_slice(n)
        full = torch.arange(n, dtype=torch.float64) * 1.5
        local = full[lo:hi].clone()                    # this rank's per-binary results
        got = sharding.gather_results(local, n)
        assert torch.equal(got, full), (rank, got[:5])
        # 2-D results (e.g. gradients per binary) gather the same way
        g2 = sharding.gather_results(torch.stack([local, -local], 1), n)
        assert torch.equal(g2[:, 1], -full)
        t = sharding.max_over_ranks([1.0 + rank, 10.0 - rank])
        assert t == [float(world), 10.0], t
        gi = torch.arange(n) % G
        (g0, g1), mask = sharding.shard_groups(G, gi)
        owned = torch.zeros(G, dtype=torch.int64)
        owned[g0:g1] = 1
        allown = owned.clone()
        dist.all_reduce(allown)
        assert torch.equal(allown, torch.ones(G, dtype=torch.int64))   # each group once
        assert bool(torch.all(mask == ((gi >= g0) & (gi < g1))))
        sharding.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n,G", [(1001, 7), (2, 3)])
def test_two_gloo_ranks(n, G):
    mp.spawn(_worker, args=(2, _free_port(), n, G), nprocs=2, join=True)


def test_single_process_defaults():
    from gbgpu_gb300 import sharding
    assert sharding.shard_slice(10) == (0, 10)
    x = torch.arange(4.0)
    assert sharding.gather_results(x, 4) is x
    assert sharding.max_over_ranks([3.0]) == [3.0]
    spans = [sharding.shard_slice(10, r, 3) for r in range(3)]
    assert spans == [(0, 4), (4, 7), (7, 10)]
