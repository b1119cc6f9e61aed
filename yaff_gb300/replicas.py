"""Independent replicas on several GPUs.

The force evaluation of one system does not shard across GPUs (its pair,
Ewald and valence terms all read the whole system); what scales over GPUs is
the number of independent systems -- MD replicas, serving requests, MC chains
-- with one process per GPU and no collective on the data path.  These host
helpers give each rank its share of the units and reduce the few scalars a
run reports (the slowest rank's time, unit counts).  Launch with torchrun
(RANK, WORLD_SIZE, LOCAL_RANK, MASTER_ADDR / MASTER_PORT in the environment).
"""
import os

__all__ = ['dist_env', 'init', 'shard', 'owner', 'max_over_ranks', 'sum_over_ranks']


def dist_env():
    """(world size, rank, local rank) from the launcher's environment."""
    return (int(os.environ.get('WORLD_SIZE', '1')), int(os.environ.get('RANK', '0')),
            int(os.environ.get('LOCAL_RANK', '0')))


def init(backend=None):
    """Joins the process group when the world has more than one rank
    (backend: 'nccl' when CUDA is available, else 'gloo')."""
    world, rank, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            if backend is None:
                backend = 'nccl' if torch.cuda.is_available() else 'gloo'
            if backend == 'nccl':
                torch.cuda.set_device(local)
            dist.init_process_group(backend)
    return world, rank, local


def shard(n, rank, world):
    """The units [start, stop) of `rank` among n independent units: contiguous
    blocks whose sizes differ by at most one, in rank order."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError('need 0 <= rank < world and n >= 0')
    q, r = divmod(n, world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def owner(i, n, world):
    """The rank whose shard holds unit i."""
    if not 0 <= i < n:
        raise ValueError('unit index out of range')
    q, r = divmod(n, world)
    if i < r * (q + 1):
        return i // (q + 1)
    return r + (i - r * (q + 1)) // q


def _reduce(x, op):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x):
    """The largest value over all ranks (the slowest rank's time)."""
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.MAX)


def sum_over_ranks(x):
    """The sum over all ranks (units processed)."""
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.SUM)
