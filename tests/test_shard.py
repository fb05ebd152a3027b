"""CPU: the multi-GPU host logic of the batched forms (view partition, gradient all-reduce), run as two
gloo ranks on 127.0.0.1.  The GPU work of each rank is the single-GPU batched path tested elsewhere."""

import os
import socket

import pytest
import torch
import torch.multiprocessing as mp

from vkgs_gb300 import shard
from vkgs_gb300 import synthetic as syn


class _Cam:
    def __init__(self, w, h):
        self.width, self.height = w, h


def test_view_shards_cover_every_view_once_and_balance():
    cams = [_Cam(*syn.RESOLUTIONS[i % len(syn.RESOLUTIONS)]) for i in range(64)]
    for world in (1, 2, 3, 8):
        shards = shard.view_shards(cams, world)
        flat = sorted(v for s in shards for v in s)
        assert flat == list(range(64))
        loads = [sum(shard.view_work(cams[v]) for v in s) for s in shards]
        assert max(loads) - min(loads) <= max(shard.view_work(c) for c in cams)
    assert shard.view_shards([], 2) == [[], []]
    with pytest.raises(ValueError):
        shard.view_shards(cams, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # per-splat gradient buffers of the five parameter groups (N = 5 splats), rank-dependent values
        n = 5
        grads = [torch.full((n, 3), rank + 1.0), torch.full((n, 3), 10.0 * (rank + 1)), torch.full((n, 4), -1.0),
                 torch.arange(n, dtype=torch.float32) * (rank + 1), torch.ones((n, 48)) * rank]
        shard.allreduce_gradients(grads)
        cams = [_Cam(*syn.RESOLUTIONS[i % len(syn.RESOLUTIONS)]) for i in range(16)]
        mine = shard.view_shards(cams, world)[rank]
        got = [None] * world
        dist.all_gather_object(got, mine)
        out[rank] = {"grads": [g.tolist() for g in grads], "views": got}
    finally:
        dist.destroy_process_group()


def test_gradient_allreduce_and_view_partition_two_ranks():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    n = 5
    for rank in range(world):
        g = out[rank]["grads"]
        assert torch.equal(torch.tensor(g[0]), torch.full((n, 3), 3.0))
        assert torch.equal(torch.tensor(g[1]), torch.full((n, 3), 30.0))
        assert torch.equal(torch.tensor(g[2]), torch.full((n, 4), -2.0))
        assert torch.equal(torch.tensor(g[3]), torch.arange(n, dtype=torch.float32) * 3)
        assert torch.equal(torch.tensor(g[4]), torch.ones((n, 48)))
        views = out[rank]["views"]
        assert sorted(v for s in views for v in s) == list(range(16))
        assert views[0] and views[1] and not set(views[0]) & set(views[1])


def test_render_batched_sharded_renders_exactly_the_ranks_views():
    class _Renderer:
        def __init__(self):
            self.got = None

        def render_batched(self, splats, cams, colors):
            self.got = (list(cams), list(colors))

    cams = [_Cam(*syn.RESOLUTIONS[i % len(syn.RESOLUTIONS)]) for i in range(10)]
    colors = [f"target{i}" for i in range(10)]
    seen = []
    for rank in range(3):
        r = _Renderer()
        mine = shard.render_batched_sharded(r, None, cams, colors, rank, 3)
        assert r.got == ([cams[v] for v in mine], [colors[v] for v in mine])
        seen += mine
    assert sorted(seen) == list(range(10))
