"""Autotuner for the batched form: picks render lanes and the depth-slab schedule by timing them.

The batched call (``Renderer.render_batched``) has two knobs that decide how well many views of
uneven resolution fill the GPU: how many render lanes (concurrent per-view pipelines, each with its
own scratch and stream) the views are spread over, and the depth-slab schedule each view uses.  This
module times every candidate on the caller's own scene and cameras with CUDA events, keeps the
fastest, and can cache the choice in a JSON file keyed by the batch's shape (splat count, view count,
resolutions).
"""

from __future__ import annotations

import json
import os
from dataclasses import dataclass

import torch

LANES = (1, 2, 4, 8, 12, 16, 24, 32)
SLABS = ((1024,), (128, 1024), (192, 1024), (256, 1024))


@dataclass
class Choice:
    lanes: int
    slabs: tuple
    ms: float  # one batch, CUDA-event time


def batch_key(splat_count: int, cameras) -> str:
    res = sorted(f"{int(c.width)}x{int(c.height)}" for c in cameras)
    return f"n={splat_count};views={len(cameras)};res=" + ",".join(res)


def time_batch(renderer, splats, cameras, colors, reps: int = 5, warmup: int = 2) -> float:
    """Milliseconds per render_batched call (mean of reps after warmup), CUDA events on the current stream."""
    for _ in range(warmup):
        renderer.render_batched(splats, cameras, colors)
    renderer.check()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        renderer.render_batched(splats, cameras, colors)
    e1.record()
    torch.cuda.synchronize()
    renderer.check()
    return e0.elapsed_time(e1) / reps


def autotune_batched(renderer, splats, cameras, colors, lanes=LANES, slabs=SLABS, cache: str | None = None,
                     reps: int = 5) -> Choice:
    """Times every (lanes, slab schedule) pair and leaves the renderer set to the fastest one."""
    key = batch_key(splats.count, cameras)
    if cache and os.path.exists(cache):
        with open(cache) as f:
            known = json.load(f)
        if key in known:
            c = known[key]
            choice = Choice(int(c["lanes"]), tuple(c["slabs"]), float(c["ms"]))
            renderer.set_batch_lanes(choice.lanes)
            renderer.set_slabs(choice.slabs)
            return choice
    # size the pair capacity once, with the largest lane count, before timing anything
    renderer.set_batch_lanes(max(lanes))
    renderer.render_batched_checked(splats, cameras, colors)
    best = None
    for n_lanes in lanes:
        renderer.set_batch_lanes(n_lanes)
        for ends in slabs:
            renderer.set_slabs(ends)
            ms = time_batch(renderer, splats, cameras, colors, reps=reps)
            if best is None or ms < best.ms:
                best = Choice(n_lanes, tuple(ends), ms)
    renderer.set_batch_lanes(best.lanes)
    renderer.set_slabs(best.slabs)
    if cache:
        known = {}
        if os.path.exists(cache):
            with open(cache) as f:
                known = json.load(f)
        known[key] = {"lanes": best.lanes, "slabs": list(best.slabs), "ms": best.ms}
        with open(cache, "w") as f:
            json.dump(known, f, indent=1)
    return best
