"""Multi-process sharding of independent work units (states, reactors, flamelets) over ranks, one GPU per rank.

The hot path has no exchange step: every state, reactor and flamelet is independent. A batch is split into
contiguous slices, one per rank; each rank runs its slice on its own GPU and the only collective is a host-side
concatenation of the per-rank results (and a max of per-rank times for measurement). The process group may be
gloo (host tensors) or nccl (the caller passes device tensors).
"""

import os

import numpy as np


def dist_env():
    """(rank, world_size, local_rank) from the torchrun environment; (0, 1, 0) without one."""
    return int(os.environ.get('RANK', '0')), int(os.environ.get('WORLD_SIZE', '1')), \
        int(os.environ.get('LOCAL_RANK', '0'))


def shard_range(n, rank, world):
    """Contiguous slice [lo, hi) of n units for `rank` of `world`; the first n % world ranks get one more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f'bad rank {rank} of world {world}')
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _device(device):
    """The device collectives run on: the given one, else the current CUDA device under nccl, else the host."""
    import torch
    import torch.distributed as dist
    if device is not None:
        return device
    if dist.get_backend() == 'nccl':
        return torch.device('cuda', torch.cuda.current_device())
    return torch.device('cpu')


def max_over_ranks(x, device=None):
    """Max of a float over all ranks (x itself without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device(device))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, device=None):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device(device))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_rows(local, n_total, device=None):
    """Concatenate per-rank row blocks (contiguous slices of shard_range) into the full [n_total, ...] array on every
    rank. local: numpy array of this rank's rows."""
    import torch
    import torch.distributed as dist
    local = np.ascontiguousarray(local)
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local
    world = dist.get_world_size()
    tail = local.shape[1:]
    rows = max(shard_range(n_total, r, world)[1] - shard_range(n_total, r, world)[0] for r in range(world))
    device = _device(device)
    buf = torch.zeros((rows,) + tail, dtype=torch.float64, device=device)
    buf[:local.shape[0]] = torch.as_tensor(local, dtype=torch.float64, device=device)
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    out = []
    for r in range(world):
        lo, hi = shard_range(n_total, r, world)
        out.append(parts[r][:hi - lo].cpu().numpy())
    return np.concatenate(out, axis=0)
