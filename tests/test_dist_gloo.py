"""The multi-GPU plumbing on CPU: two gloo ranks shard the sources disjointly,
take the max of their timings and sum their kernels (grad.py:158-165)."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from sparc_gb300 import dist as sd
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = sd.shard_sources(32, rank, world)
    t = sd.max_over_ranks(1.0 + rank)
    k = sd.sum_kernels(np.full((3, 4), float(len(mine) * (rank + 1))))
    q.put((rank, mine, t, k.tolist()))
    dist.destroy_process_group()


def test_two_rank_sharding_and_reductions():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    s0, s1 = set(res[0][1]), set(res[1][1])
    assert not (s0 & s1) and (s0 | s1) == set(range(32))
    assert res[0][2] == res[1][2] == 2.0
    assert np.allclose(res[0][3], 16 * 1 + 16 * 2)
