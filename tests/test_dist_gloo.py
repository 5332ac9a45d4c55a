"""The multi-GPU plumbing on CPU: two gloo ranks shard the sources disjointly,
take the max of their timings and sum their kernels (grad.py:158-165).  The
kernel sum is checked on real kernels: each rank computes the oracle kernels
of its own sources, reduce_kernels sums the ranks' sums, and the result equals
the one-process sum over all sources."""
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


NSRC = 5


def _kernel_worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    from oracle_kernels import global_sources, kernel_params, source_kernels
    from cases import table_for
    from sparc_gb300 import dist as sd
    from sparc_gb300 import sources
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    O.set_threads(1)
    p = kernel_params()
    tab = table_for(p)
    planes, obs = global_sources(p, NSRC)
    series = O.forward_source(p, p.maxtime + 10) * 1e3
    pix = sources.receiver_pixels(p, n=8, radius_mm=10.0)
    r, w = sd.rank_world()
    mine = sd.shard_sources(NSRC, r, w)
    t = torch.zeros((3, p.nz, p.ny, p.nx), dtype=torch.float64)
    for i in mine:
        t += torch.from_numpy(source_kernels(O, p, tab, planes[i], series, obs[i], pix))
    sd.reduce_kernels(t)
    q.put((rank, mine, t.numpy().copy()))
    dist.destroy_process_group()


def test_sharded_oracle_kernels_sum_to_the_all_source_sum():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from oracle import oracle as O
    from oracle_kernels import global_sources, kernel_params, source_kernels
    from cases import table_for
    from sparc_gb300 import sources
    O.build()
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_kernel_worker, args=(r, world, port, q)) for r in range(world)]
    for pr in procs:
        pr.start()
    res = sorted([q.get(timeout=600) for _ in procs], key=lambda x: x[0])
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    assert set(res[0][1]).isdisjoint(res[1][1]) and set(res[0][1]) | set(res[1][1]) == set(range(NSRC))
    # both ranks hold the same sum, and it is the sum over every source
    assert np.array_equal(res[0][2], res[1][2])
    p = kernel_params()
    tab = table_for(p)
    planes, obs = global_sources(p, NSRC)
    series = O.forward_source(p, p.maxtime + 10) * 1e3
    pix = sources.receiver_pixels(p, n=8, radius_mm=10.0)
    ref = sum(source_kernels(O, p, tab, planes[i], series, obs[i], pix) for i in range(NSRC))
    assert np.abs(ref).max() > 0
    np.testing.assert_allclose(res[0][2], ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
