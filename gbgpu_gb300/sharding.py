"""Host-side sharding of the FastGB path over ranks (one process per GPU).

Binaries are independent and each yields per-binary scalars, so a batch is
split into contiguous slices, one per rank, with no collective on the data
path; the only exchanges are a host-side gather of the per-binary results and
the max over ranks of a step time.  Global templates shard by group: each rank
owns whole templates (a split by binary would need an all-reduce of the
templates instead).  Works with any torch.distributed backend (nccl on GPUs,
gloo on CPU) or without a process group (world size 1).
"""

import torch
import torch.distributed as dist


def _world():
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def shard_slice(n, rank=None, world=None):
    """[lo, hi) of the n items owned by ``rank``: contiguous, sizes differ by <= 1."""
    if rank is None or world is None:
        rank, world = _world()
    base, extra = divmod(int(n), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_groups(num_groups, group_index, rank=None, world=None):
    """Template groups [g0, g1) owned by ``rank`` and the mask of the binaries
    (``group_index``: (B,) tensor or array) that fill them."""
    g0, g1 = shard_slice(num_groups, rank, world)
    gi = torch.as_tensor(group_index)
    return (g0, g1), (gi >= g0) & (gi < g1)


def gather_results(local, n_total, device=None):
    """Concatenate every rank's per-binary results (rank order, slices from
    ``shard_slice(n_total)``) on every rank.  ``local``: (n_local, ...) tensor."""
    rank, world = _world()
    if world == 1:
        return local
    lo, hi = shard_slice(n_total, rank, world)
    if local.shape[0] != hi - lo:
        raise ValueError(f"rank {rank} holds {local.shape[0]} rows, its slice has {hi - lo}")
    width = shard_slice(n_total, 0, world)[1]            # rank 0 has the largest slice
    buf = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype,
                      device=local.device if device is None else device)
    buf[:local.shape[0]] = local
    parts = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    out = [parts[r][:shard_slice(n_total, r, world)[1] - shard_slice(n_total, r, world)[0]]
           for r in range(world)]
    return torch.cat(out, 0)


def max_over_ranks(values, device=None):
    """Element-wise max over ranks of a list of floats (step times)."""
    rank, world = _world()
    if world == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def barrier():
    rank, world = _world()
    if world > 1:
        dist.barrier()
