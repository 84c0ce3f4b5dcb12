"""Replica mode across two gloo ranks on CPU: each rank fuses its own
stream with the oracle, timings reduce by max, counts gather to all ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import PKG, REPO


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, results):
    import sys
    for p in (REPO, PKG):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.oracle import Oracle
    from vhsdf import replicas, synth
    seed = replicas.stream_seed(2, rank)
    scenes = replicas.assign(5, rank, world)
    s = synth.Scene(kind=2, seed=seed, num_frames=3, width=80, height=60)
    o = Oracle(80, 60, s.fx, s.fy, s.cx, s.cy, max_depth=4.0, voxel_size=0.04, trunc=0.12)
    for f in range(3):
        o.integrate(*s.render(f))
    times = replicas.reduce_max([float(rank + 1), 10.0 - rank])
    counts = replicas.gather_counts([rank, o.num_blocks(), len(scenes)])
    results[rank] = (times, counts, seed, scenes)
    dist.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    port = free_port()
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    procs = [ctx.Process(target=worker, args=(r, world, port, results)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    r0, r1 = results[0], results[1]
    assert r0[0] == r1[0] == [2.0, 10.0]              # max over ranks
    assert r0[1] == r1[1]                            # same gathered view
    assert [c[0] for c in r0[1]] == [0, 1]
    assert r0[2] != r1[2]                            # independent streams
    assert all(c[1] > 0 for c in r0[1])
    assert sorted(r0[3] + r1[3]) == [0, 1, 2, 3, 4]  # every scene exactly once


def test_assign_validates():
    from vhsdf import replicas
    assert replicas.assign(3, 0, 1) == [0, 1, 2]
    with pytest.raises(ValueError):
        replicas.assign(3, 2, 2)
