"""CPU, two ranks over gloo: the replica helpers that bench.py uses under
torchrun -- every unit owned by exactly one rank (shards are a partition in
rank order, `owner` agrees with `shard`), the slowest rank's time and the
summed unit counts -- with the process group on 127.0.0.1."""
import os
import socket

import pytest

from yaff_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    os.environ.update({'MASTER_ADDR': '127.0.0.1', 'MASTER_PORT': str(port), 'RANK': str(rank),
                       'WORLD_SIZE': str(world), 'LOCAL_RANK': str(rank)})
    import torch.distributed as dist
    w, r, _ = replicas.init('gloo')
    assert (w, r) == (world, rank)
    n = 4097
    a, b = replicas.shard(n, r, w)
    got = [None] * w
    dist.all_gather_object(got, (a, b))
    tmax = replicas.max_over_ranks(1.5 + r)
    units = replicas.sum_over_ranks(b - a)
    with open(os.path.join(out_dir, 'rank%d.txt' % r), 'w') as fh:
        fh.write(repr((got, tmax, units)))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_partition_single_process():
    for n in (0, 1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[k][1] == parts[k + 1][0] for k in range(world - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
            for i in range(n):
                r = replicas.owner(i, n, world)
                assert parts[r][0] <= i < parts[r][1]


def test_two_rank_gloo(tmp_path):
    torch = pytest.importorskip('torch')
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method='spawn')
    res = [eval(open(os.path.join(str(tmp_path), 'rank%d.txt' % r)).read()) for r in range(world)]
    for got, tmax, units in res:
        assert got == [(0, 2049), (2049, 4097)]
        assert tmax == 2.5
        assert units == 4097
