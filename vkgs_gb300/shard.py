"""Multi-GPU forms of the batched paths: views partitioned across ranks, one process per GPU.

The plain frame does not shard (one sorted sequence, one image): ranks run replicas.  The batched
views shard by view with no data-path collective -- every rank holds the splats and renders its own
cameras.  The batched differentiation shards the same way and adds one exchange step per training
step: an all-reduce (sum) of the per-splat gradient buffers, so every rank applies the gradient of
the loss summed over all views.  Collectives go through torch.distributed (NCCL between GPUs, gloo for
the CPU tests of this host logic).
"""

from __future__ import annotations

import torch


def view_work(camera) -> float:
    """Relative cost of one view: its pixels plus a fixed per-view cost (cull and sort of all splats)."""
    return float(camera.width) * float(camera.height) + 250_000.0


def view_shards(cameras, world: int) -> list[list[int]]:
    """Partitions the view indices over `world` ranks: largest views first, each to the least-loaded rank
    (ties to the lower rank), so every rank gets a similar amount of work.  Deterministic, so every rank
    computes the same partition without communicating."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(cameras)), key=lambda v: (-view_work(cameras[v]), v))
    load = [0.0] * world
    shards: list[list[int]] = [[] for _ in range(world)]
    for v in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += view_work(cameras[v])
        shards[r].append(v)
    return [sorted(s) for s in shards]


def allreduce_gradients(grads, group=None) -> None:
    """Sums the per-splat gradient buffers over all ranks, in place, with one collective: the tensors are
    packed into one flat buffer (same dtype and device) and unpacked after the all-reduce."""
    import torch.distributed as dist

    grads = [g for g in grads if g is not None]
    if not grads:
        return
    flat = torch.cat([g.reshape(-1) for g in grads])
    dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
    off = 0
    for g in grads:
        n = g.numel()
        g.copy_(flat[off:off + n].view_as(g))
        off += n


def render_batched_sharded(renderer, splats, cameras, colors, rank: int, world: int):
    """This rank's share of a batched render: renders the views view_shards assigns to `rank` into their
    colour targets and returns their indices (no collective)."""
    mine = view_shards(cameras, world)[rank]
    if mine:
        renderer.render_batched(splats, [cameras[v] for v in mine], [colors[v] for v in mine])
    return mine


def train_step_sharded(params: dict, cameras, loss_of_view, renderer, rank: int, world: int, group=None):
    """One data-parallel step of the batched differentiation: this rank renders its views
    (vkgs_gb300.train.render_batched), backpropagates the sum of loss_of_view(v, image) over them, and
    the parameter gradients are all-reduced, so every rank ends with the gradient of the loss summed
    over all views.  Returns the (all-reduced) loss."""
    import torch.distributed as dist

    from . import train

    mine = view_shards(cameras, world)[rank]
    loss = None
    if mine:
        imgs = train.render_batched(params, [cameras[v] for v in mine], renderer)
        loss = sum(loss_of_view(v, img) for v, img in zip(mine, imgs))
        loss.backward()
    for k in train.NAMES:
        if params[k].grad is None:
            params[k].grad = torch.zeros_like(params[k])
    allreduce_gradients([params[k].grad for k in train.NAMES], group)
    total = (loss.detach() if loss is not None else torch.zeros((), device=params["means"].device)).reshape(1)
    dist.all_reduce(total, op=dist.ReduceOp.SUM, group=group)
    return total[0]
