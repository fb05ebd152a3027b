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


def _fake_render_batched(params, cameras, renderer):
    """A CPU autograd stand-in for train.render_batched: one image per camera, every parameter group
    entering it (the sharded step's host logic is what is under test, not the kernels)."""
    out = []
    for c in cameras:
        s = c.width / 10.0 + c.height / 7.0
        base = ((params["means"] * s).sum() + (params["log_scales"] ** 2).sum() * 0.1 + params["quats"].sin().sum()
                + torch.sigmoid(params["opacity_logits"]).sum() + (params["sh"] * s).cos().sum())
        ramp = torch.linspace(0.0, 1.0, c.height * c.width * 4).reshape(c.height, c.width, 4)
        out.append(base * ramp + ramp * s)
    return tuple(out)


def _train_inputs():
    g = torch.Generator().manual_seed(3)
    n = 7
    params = {"means": torch.randn((n, 3), generator=g), "log_scales": torch.randn((n, 3), generator=g),
              "quats": torch.randn((n, 4), generator=g), "opacity_logits": torch.randn((n,), generator=g),
              "sh": torch.randn((n, 48), generator=g)}
    cams = [_Cam(w, h) for w, h in [(8, 6), (12, 4), (5, 5), (9, 7), (6, 10)]]
    targets = [torch.rand((c.height, c.width, 4), generator=g) * 40.0 for c in cams]
    return params, cams, targets


def _train_worker(rank, world, port, out):
    import torch.distributed as dist

    from vkgs_gb300 import train

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        train.render_batched = _fake_render_batched
        params, cams, targets = _train_inputs()
        params = {k: v.clone().requires_grad_(True) for k, v in params.items()}
        loss = shard.train_step_sharded(params, cams, lambda v, img: (img - targets[v]).abs().mean(), None, rank,
                                        world)
        out[rank] = {"loss": float(loss), "grads": {k: params[k].grad.tolist() for k in train.NAMES},
                     "views": shard.view_shards(cams, world)[rank]}
    finally:
        dist.destroy_process_group()


def test_sharded_train_step_two_ranks_equals_the_sum_over_all_views():
    """shard.train_step_sharded over two gloo ranks: each rank renders only its views, and after the
    one all-reduce every rank holds the gradient of the loss summed over ALL views, and the summed
    loss -- equal to a single process that renders every view."""
    from vkgs_gb300 import train

    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_train_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    params, cams, targets = _train_inputs()
    params = {k: v.clone().requires_grad_(True) for k, v in params.items()}
    imgs = _fake_render_batched(params, cams, None)
    loss = sum((img - t).abs().mean() for img, t in zip(imgs, targets))
    loss.backward()
    assert sorted(out[0]["views"] + out[1]["views"]) == list(range(len(cams)))
    assert out[0]["views"] and out[1]["views"]
    for rank in range(world):
        assert out[rank]["loss"] == pytest.approx(float(loss), rel=1e-6)
        for k in train.NAMES:
            got = torch.tensor(out[rank]["grads"][k])
            assert torch.allclose(got, params[k].grad, rtol=1e-5, atol=1e-6), k
