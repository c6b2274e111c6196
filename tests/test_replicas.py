"""Multi-rank host logic on CPU (gloo, world size 2): shards cover every
item once, and the job throughput is all ranks' units over the slowest
rank's time."""
import os
import socket

import pytest

from vkscanlinepr_gb300 import replicas


def test_shards_partition_the_items():
    for n in (0, 1, 7, 4096):
        for world in (1, 2, 3, 8):
            got = [replicas.shard(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [e - b for b, e in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b, e = replicas.shard(4096, rank, world)
    seconds = 1.0 + rank          # rank 1 is the slower one
    q.put((rank, b, e, replicas.max_over_ranks(seconds), replicas.job_throughput(e - b, seconds)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_combine_timing():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(o[1], o[2]) for o in out] == [(0, 2048), (2048, 4096)]
    for o in out:
        assert o[3] == 2.0                 # slowest rank
        assert o[4] == pytest.approx(4096 / 2.0)
