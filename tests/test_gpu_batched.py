"""GPU: the batched form (gs_render_batched) against single-view renders and the oracle."""

import numpy as np
import pytest

from tests import scenes
from vkgs_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _setup(n, seed, n_views, cam_seed):
    import torch
    from vkgs_gb300 import Camera, Splats, parse_ply

    rows = syn.splat_rows(n, seed)
    dev = torch.device("cuda", 0)
    splats = parse_ply(torch.from_numpy(rows).to(dev), syn.ply_offsets())
    specs = syn.random_cameras(n_views, seed=cam_seed)
    cams = [Camera.from_spec(s) for s in specs]
    colors = [torch.empty((c.height, c.width, 4), dtype=torch.float32, device=dev) for c in cams]
    return rows, splats, specs, cams, colors


@pytest.mark.parametrize("lanes,shared", [(0, True), (1, True), (3, True), (8, True), (3, False), (8, False)])
def test_batched_equals_single_view_renders(cuda, lanes, shared):
    """Every view of a batch is bit-identical to rendering that camera alone (same arithmetic, own
    scratch), with the shared multi-view cull pass and with per-lane culls."""
    import torch
    from vkgs_gb300 import Renderer

    _, splats, specs, cams, colors = _setup(200_000, 11, 10, 501)
    r = Renderer(200_000, 1920, 1080)
    r.set_batch_lanes(lanes)
    r.set_batch_shared_cull(shared)
    r.render_batched_checked(splats, cams, colors)
    single = Renderer(200_000, 1920, 1080)
    for cam, col in zip(cams, colors):
        img, _ = single.render_checked(splats, cam)
        assert torch.equal(img, col)


def test_batched_many_views_in_groups(cuda):
    """70 views: two shared cull launches (32 views each) per group of 64, then a second group reusing the
    per-view buffers -- every view still equals its single render."""
    import torch
    from vkgs_gb300 import Camera, Renderer

    _, splats, _, _, _ = _setup(30_000, 15, 1, 505)
    specs = syn.random_cameras(70, seed=506, resolutions=[(320, 180), (256, 256), (200, 120)])
    cams = [Camera.from_spec(sp) for sp in specs]
    colors = [torch.empty((c.height, c.width, 4), dtype=torch.float32, device="cuda") for c in cams]
    r = Renderer(30_000, 320, 256)
    r.set_batch_lanes(5)
    r.render_batched_checked(splats, cams, colors)
    single = Renderer(30_000, 320, 256)
    for cam, col in zip(cams, colors):
        img, _ = single.render_checked(splats, cam)
        assert torch.equal(img, col)


def test_batched_matches_oracle(cuda, oracle):
    from vkgs_gb300 import Renderer

    rows, splats, specs, cams, colors = _setup(50_000, 12, 5, 502)
    act = scenes.activated(oracle, rows)
    r = Renderer(50_000, 1920, 1080)
    r.set_batch_lanes(4)
    r.render_batched_checked(splats, cams, colors)
    for spec, col in zip(specs, colors):
        c = scenes.camera(oracle, spec.eye, fovy_deg=spec.fovy_deg, width=spec.width, height=spec.height)
        o = oracle.render_frame(*act, scenes.oracle_camera(oracle, c))
        err = np.abs(col.cpu().numpy().astype(np.float64) - o["image"]).max()
        assert err <= 1.0 / 255.0, err


def test_batched_graph_capture_replays(cuda):
    """The whole batch captured in one CUDA graph replays to the same images (fresh look-back state per frame)."""
    import torch
    from vkgs_gb300 import Renderer

    _, splats, specs, cams, colors = _setup(100_000, 13, 6, 503)
    r = Renderer(100_000, 1920, 1080)
    r.set_batch_lanes(3)
    r.render_batched_checked(splats, cams, colors)
    want = [c.clone() for c in colors]
    for c in colors:
        c.zero_()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        r.render_batched(splats, cams, colors)  # warm-up on the capture stream
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        r.render_batched(splats, cams, colors)
    for _ in range(3):
        for c in colors:
            c.zero_()
        g.replay()
        torch.cuda.synchronize()
        for a, b in zip(colors, want):
            assert torch.equal(a, b)
    r.check()


def test_batched_first_call_under_capture_uses_per_lane_cull(cuda):
    """A batched call captured before the shared cull's buffers exist cannot allocate them: it falls back
    to one cull per lane, and the captured batch still renders the same images."""
    import torch
    from vkgs_gb300 import Renderer

    _, splats, specs, cams, colors = _setup(100_000, 16, 5, 508)
    ref = Renderer(100_000, 1920, 1080)
    want = [ref.render_checked(splats, c)[0].clone() for c in cams]
    r = Renderer(100_000, 1920, 1080)
    for c in cams:  # size the pair capacity (single-view renders allocate nothing for the batch)
        r.render_checked(splats, c)
    r.set_batch_lanes(3)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        r.render_batched(splats, cams, colors)
    for _ in range(2):
        for c in colors:
            c.zero_()
        g.replay()
        torch.cuda.synchronize()
        for a, b in zip(colors, want):
            assert torch.equal(a, b)
    r.check()


def test_batched_capacity_overflow_recovers(cuda):
    import torch
    from vkgs_gb300 import GsError, Renderer

    _, splats, specs, cams, colors = _setup(100_000, 14, 4, 504)
    r = Renderer(100_000, 1920, 1080, max_tile_pairs=2000)
    r.set_batch_lanes(2)
    r.render_batched(splats, cams, colors)
    with pytest.raises(GsError) as e:
        r.check()
    assert e.value.status == 2 and e.value.stats["tile_pairs"] > 2000
    stats = r.render_batched_checked(splats, cams, colors)
    assert stats["visible_count"] > 0
    single = Renderer(100_000, 1920, 1080)
    img, _ = single.render_checked(splats, cams[0])
    assert torch.equal(img, colors[0])


def test_batched_rejects_bad_targets(cuda):
    import torch
    from vkgs_gb300 import GsError, Renderer

    _, splats, specs, cams, colors = _setup(1000, 15, 2, 505)
    r = Renderer(1000, 640, 360)
    big = [c for c in cams if c.width > 640 or c.height > 360]
    if big:
        with pytest.raises(GsError):
            r.render_batched(splats, big[:1], [torch.empty((big[0].height, big[0].width, 4), device="cuda")])
    with pytest.raises(ValueError):
        r.render_batched(splats, cams, colors[:1])


def test_batched_workload_at_size(cuda, oracle):
    """The batched form at its own size: 1M splats (shell layout), the 64 random cameras of 640x360 ...
    1920x1080, captured in one CUDA graph and replayed as the bench does with the autotuner's choice --
    every view bit-identical to its single-view gs_render, and five views (the largest 1920x1080 ones
    first) within 1/255 of the oracle's image."""
    import torch
    from vkgs_gb300 import Camera, Renderer, parse_ply
    from vkgs_gb300.autotune import autotune_batched

    rows, off, specs = syn.workload("batched")
    splats = parse_ply(torch.from_numpy(rows).cuda(), off)
    cams = [Camera.from_spec(sp) for sp in specs]
    colors = [torch.empty((c.height, c.width, 4), dtype=torch.float32, device="cuda") for c in cams]
    r = Renderer(splats.count, 1920, 1080)
    for c in cams:  # the bench sizes the pair capacity with single renders first
        r.render_checked(splats, c)
    choice = autotune_batched(r, splats, cams, colors, reps=1)
    single = Renderer(splats.count, 1920, 1080)
    single.set_slabs(choice.slabs)  # the same depth-slab schedule as the tuned batch
    want = [single.render_checked(splats, c)[0].clone() for c in cams]
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        r.render_batched(splats, cams, colors)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        r.render_batched(splats, cams, colors)
    for _ in range(2):
        for c in colors:
            c.zero_()
        g.replay()
        torch.cuda.synchronize()
        for k, (a, b) in enumerate(zip(colors, want)):
            assert torch.equal(a, b), k
    r.check()
    act = scenes.activated(oracle, rows)
    order = sorted(range(len(specs)), key=lambda k: -specs[k].width * specs[k].height)
    picked = order[:2] + order[len(order) // 2: len(order) // 2 + 1] + order[-2:]
    assert specs[picked[0]].width == 1920
    for k in picked:
        spec = specs[k]
        c = scenes.camera(oracle, spec.eye, fovy_deg=spec.fovy_deg, width=spec.width, height=spec.height)
        o = oracle.render_frame(*act, scenes.oracle_camera(oracle, c), want_instances=False)
        err = np.abs(colors[k].cpu().numpy().astype(np.float64) - o["image"]).max()
        assert err <= 1.0 / 255.0, (k, err)


def test_captured_batch_survives_a_larger_eager_batch(cuda):
    """A batch captured with N views keeps replaying correctly after an eager batched call with 2N views
    (the arena is not replaced while a captured graph may use it; the larger call culls per lane)."""
    import torch
    from vkgs_gb300 import Camera, Renderer

    _, splats, specs, cams, colors = _setup(60_000, 18, 4, 510)
    more = [Camera.from_spec(sp) for sp in syn.random_cameras(8, seed=511)]
    more_colors = [torch.empty((c.height, c.width, 4), device="cuda") for c in more]
    single = Renderer(60_000, 1920, 1080)
    want = [single.render_checked(splats, c)[0].clone() for c in cams]
    want_more = [single.render_checked(splats, c)[0].clone() for c in more]
    r = Renderer(60_000, 1920, 1080)
    r.set_batch_lanes(4)
    r.render_batched_checked(splats, cams, colors)  # the arena for 4 views exists before the capture
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        r.render_batched(splats, cams, colors)
    r.render_batched_checked(splats, more, more_colors)  # needs 8 views' arena
    for a, b in zip(more_colors, want_more):
        assert torch.equal(a, b)
    for _ in range(2):
        for c in colors:
            c.zero_()
        g.replay()
        torch.cuda.synchronize()
        for a, b in zip(colors, want):
            assert torch.equal(a, b)
    r.check()
