"""Replica parallelism on CPU: the view sharding and the gathering of results over a world of two
gloo ranks (one process each, spawned), with the CPU oracle standing in for each rank's renderer."""
import hashlib
import os
import socket

import numpy as np
import pytest

from webgs import replicas


def test_shard_covers_every_view_once_and_balances():
    costs = [5.0, 1.0, 3.0, 3.0, 2.0, 8.0, 1.0]
    for world in (1, 2, 3, 7, 9):
        parts = replicas.shard(costs, world)
        assert len(parts) == world
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in replicas.shard(costs, 2)]
    assert max(loads) - min(loads) <= max(costs)
    assert replicas.shard(costs, 2) == replicas.shard(costs, 2)
    with pytest.raises(ValueError):
        replicas.shard(costs, 0)


VIEWS = [((0.0, 0.0, -4.0), 48, 40), ((0.5, 0.2, -3.5), 64, 32), ((-0.4, 0.0, -4.5), 40, 40),
         ((0.0, 0.6, -3.0), 32, 48), ((0.3, -0.3, -4.0), 56, 24)]


def _render_digest(i):
    import oracle
    import webgs

    eye, w, h = VIEWS[i]
    packed = webgs.synth_scene(0, 800, 42)
    view = webgs.camera_view(eye, (0, 0, 0), (0, 1, 0), 60.0, w, h, 0.2, 100.0)
    r = oracle.forward_f32(webgs.view_bytes(view), packed, 800, threads=1)
    return hashlib.sha256(r["rgba8"].tobytes()).hexdigest()


def _worker(rank, world, port, q):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    sys.path[:0] = [str(root), str(root / "web-gs-renderer_gb300")]
    import torch.distributed as dist

    from webgs import replicas as R

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    costs = [R.view_cost(w, h, 800) for _, w, h in VIEWS]
    got = R.render_sharded(_render_digest, costs, rank, world)
    slowest = R.max_over_ranks(float(rank + 1))
    q.put((rank, got, slowest, R.shard(costs, world)[rank]))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_render_their_shards_and_gather():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    expected = {i: _render_digest(i) for i in range(len(VIEWS))}
    shards = {}
    for rank, got, slowest, mine in results:
        assert got == expected          # every rank holds every view's result after the gather
        assert slowest == 2.0           # max over ranks
        shards[rank] = mine
    assert sorted(shards[0] + shards[1]) == list(range(len(VIEWS))) and shards[0] and shards[1]
