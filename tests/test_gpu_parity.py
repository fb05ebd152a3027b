"""GPU parity: the CUDA path (called through the C ABI) against the CPU oracle on identical inputs.

Bars: visible count, sorted keys and sorted index bit-exact (tie rule: ascending splat id);
projection instance records bit-exact (float equality, NaN == NaN); fragment count exact; images
within 1/255 per channel of the oracle's FP32 image (IMAGE_TOL).
"""

import math

import numpy as np
import pytest

from tests import scenes
from vkgs_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

IMAGE_TOL = 1.0 / 255.0


def render_gpu(act, c, depth=None, count_fragments=True, renderer=None, bgra=False):
    import torch
    from vkgs_gb300 import Renderer, Splats

    pos, cov, opa, sh = act
    sp = Splats.from_numpy(pos, cov, opa, sh)
    n = sp.count
    r = renderer or Renderer(max(n, 1), c["width"], c["height"])
    r.count_fragments(count_fragments)
    dev = sp.position.device
    keys = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    index = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    inst = torch.zeros(max(n, 1) * 12, dtype=torch.float32, device=dev)
    vc = torch.zeros(1, dtype=torch.int32, device=dev)
    draw = torch.zeros(12, dtype=torch.int32, device=dev)
    d = None if depth is None else torch.from_numpy(depth).to(dev)
    b8 = torch.zeros((c["height"], c["width"], 4), dtype=torch.uint8, device=dev) if bgra else None
    img = r.render(sp, scenes.product_camera(c), keys=keys, index=index, instances=inst, visible_count=vc,
                   draw_indirect=draw, depth=d, bgra8=b8, color=torch.empty((c["height"], c["width"], 4),
                                                                                 dtype=torch.float32, device=dev))
    stats = r.check()
    v = int(vc.item())
    return dict(count=v, key=keys[:v].cpu().numpy().view(np.uint32), index=index[:v].cpu().numpy().view(np.uint32),
                instance=inst[: v * 12].cpu().numpy().reshape(v, 12), image=img.cpu().numpy(),
                fragments=stats["fragments"], stats=stats, draw=draw.cpu().numpy(),
                bgra=None if b8 is None else b8.cpu().numpy())


def render_cpu(oracle, act, c, depth=None):
    pos, cov, opa, sh = act
    return oracle.render_frame(pos, cov, opa, sh, scenes.oracle_camera(oracle, c), depth_in=depth)


def assert_parity(g, o, image_tol=IMAGE_TOL, fragments=True):
    assert g["count"] == o["count"]
    np.testing.assert_array_equal(g["key"], o["key"])
    np.testing.assert_array_equal(g["index"], o["index"])
    np.testing.assert_array_equal(g["instance"][:, [0, 1, 2, 4, 5, 6, 7, 8, 9, 10, 11]],
                                  o["instance"][:, [0, 1, 2, 4, 5, 6, 7, 8, 9, 10, 11]])
    if fragments:
        assert g["fragments"] == o["fragments"]
    err = np.abs(g["image"].astype(np.float64) - o["image"])
    assert err.max() <= image_tol, f"max image error {err.max()}"
    v = g["count"]
    np.testing.assert_array_equal(g["draw"], [6 * v, 1, 0, 0, 0, 0, 0, 0, v, 1, 0, 0])
    return float(err.max())


def test_small_workload_parity(cuda, oracle):
    rows = syn.splat_rows(100_000, 0)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0))
    g = render_gpu(act, c)
    o = render_cpu(oracle, act, c)
    err = assert_parity(g, o)
    assert g["count"] > 90_000
    assert err < 1e-4


@pytest.mark.parametrize("n,w,h,seed", [(1, 64, 48, 0), (2, 33, 17, 1), (1023, 257, 131, 2), (1025, 160, 90, 3),
                                        (4097, 320, 200, 4), (33_333, 500, 301, 5)])
def test_ragged_sizes(cuda, oracle, n, w, h, seed):
    rows = syn.splat_rows(n, seed)
    act = scenes.activated(oracle, rows)
    rng = np.random.default_rng(seed)
    eye = rng.normal(size=3)
    eye = eye / np.linalg.norm(eye) * rng.uniform(2.0, 8.0)
    if abs(eye[1]) > 0.99 * np.linalg.norm(eye):
        eye[0] += 1.0
    c = scenes.camera(oracle, tuple(eye), fovy_deg=float(rng.uniform(40, 75)), width=w, height=h)
    assert_parity(render_gpu(act, c), render_cpu(oracle, act, c))


@pytest.mark.parametrize("w,h", [(2560, 1440), (3840, 2160)])
def test_high_resolution_parity(cuda, oracle, w, h):
    """More tiles than the scan keeps in shared memory (14400 and 32400 > 10240): the scan's global path."""
    rows = syn.splat_rows(60_000, 17, "shell")
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (2.0, 1.0, 7.0), width=w, height=h)
    assert_parity(render_gpu(act, c), render_cpu(oracle, act, c))


def test_empty_scene(cuda, oracle):
    act = (np.zeros((0, 3), np.float32), np.zeros((0, 6), np.float32), np.zeros(0, np.float32),
           np.zeros((0, 48), np.uint16))
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=100, height=60)
    g = render_gpu(act, c)
    assert g["count"] == 0
    exp = np.zeros((60, 100, 4), np.float32)
    exp[..., 3] = 1.0
    np.testing.assert_array_equal(g["image"], exp)


def test_everything_culled(cuda, oracle):
    rows = syn.splat_rows(5000, 9)
    rows[:, 2] += 50.0  # all splats behind a camera at z=6 looking at -z
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), center=(0.0, 0.0, 0.0), width=200, height=100)
    g = render_gpu(act, c)
    o = render_cpu(oracle, act, c)
    assert g["count"] == o["count"] == 0
    np.testing.assert_array_equal(g["image"], o["image"])


def test_equal_depth_keys_keep_ascending_id(cuda, oracle):
    # 20,000 splats on one plane facing the camera: massive key ties
    rng = np.random.default_rng(3)
    rows = syn.splat_rows(20_000, 3)
    rows[:, 0:2] = rng.uniform(-2, 2, (20_000, 2))
    rows[:, 2] = 0.0
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=320, height=180)
    g = render_gpu(act, c)
    o = render_cpu(oracle, act, c)
    assert len(np.unique(g["key"])) < g["count"] // 10
    assert_parity(g, o)


def test_degenerate_and_far_plane_splats(cuda, oracle):
    rows = scenes.rows_from([
        scenes.single_splat((0, 0, 0), scale=(0.05, 0.05, 0.05)),    # D == 0 on a square target -> not drawn
        scenes.single_splat((0.3, 0.1, 0), scale=(0.08, 0.02, 0.05)),
        scenes.single_splat((0, 0, -93.9), scale=(0.5, 0.5, 0.5)),    # near the far plane
        scenes.single_splat((0, 0, -94.1), scale=(0.5, 0.5, 0.5)),    # beyond it
    ])
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=128, height=128)
    assert_parity(render_gpu(act, c), render_cpu(oracle, act, c))


def test_depth_input(cuda, oracle):
    rows = syn.splat_rows(20_000, 6)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (1.0, 0.5, 5.0), width=300, height=200)
    rng = np.random.default_rng(6)
    depth = rng.uniform(0.975, 1.0, (200, 300)).astype(np.float32)
    g = render_gpu(act, c, depth=depth)
    o = render_cpu(oracle, act, c, depth=depth)
    assert_parity(g, o)


def test_bgra8_target_is_quantised_rgba(cuda, oracle):
    rows = syn.splat_rows(10_000, 8)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=200, height=120)
    g = render_gpu(act, c, bgra=True)
    q = np.clip(np.rint(np.clip(g["image"], 0, 1) * 255), 0, 255).astype(np.int32)
    b = g["bgra"].astype(np.int32)
    np.testing.assert_array_equal(b[..., [2, 1, 0, 3]], q)


def test_model_transform(cuda, oracle):
    rows = syn.splat_rows(20_000, 12)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.5, 1.0, 6.0), width=320, height=240, model=scenes.rotation_model())
    g = render_gpu(act, c)
    o = render_cpu(oracle, act, c)
    assert g["count"] == o["count"]
    np.testing.assert_array_equal(g["key"], o["key"])
    np.testing.assert_array_equal(g["index"], o["index"])
    np.testing.assert_allclose(g["instance"], o["instance"], rtol=1e-6, atol=1e-7)
    assert np.abs(g["image"] - o["image"]).max() <= IMAGE_TOL


def test_render_is_deterministic(cuda, oracle):
    rows = syn.splat_rows(50_000, 4)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 1.0, 5.0), width=400, height=300)
    a = render_gpu(act, c)
    b = render_gpu(act, c)
    np.testing.assert_array_equal(a["image"], b["image"])
    np.testing.assert_array_equal(a["index"], b["index"])


def test_tile_pair_overflow_is_reported_and_recoverable(cuda, oracle):
    import torch
    from vkgs_gb300 import GsError, Renderer, Splats

    rows = syn.splat_rows(20_000, 1)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=320, height=180)
    r = Renderer(20_000, 320, 180, max_tile_pairs=1000)
    sp = Splats.from_numpy(*act)
    r.render(sp, scenes.product_camera(c))
    with pytest.raises(GsError) as e:
        r.check()
    assert e.value.status == 2 and e.value.stats["tile_pairs"] > 1000
    img, stats = r.render_checked(sp, scenes.product_camera(c))
    o = render_cpu(oracle, act, c)
    assert np.abs(img.cpu().numpy() - o["image"]).max() <= IMAGE_TOL


def test_capacity_checks(cuda):
    from vkgs_gb300 import GsError, Renderer, Splats

    r = Renderer(10, 64, 64)
    sp = Splats.empty(11)
    from vkgs_gb300 import Camera

    cam = Camera.look_at((0, 0, 6), width=64, height=64)
    with pytest.raises(GsError) as e:
        r.render(sp, cam)
    assert e.value.status == 2
    with pytest.raises(GsError):
        r.render(Splats.empty(5), Camera.look_at((0, 0, 6), width=65, height=64))


def test_parse_ply_on_gpu(cuda, oracle):
    import torch
    from vkgs_gb300 import parse_ply

    rows = syn.splat_rows(50_000, 13)
    off = syn.ply_offsets()
    sp = parse_ply(torch.from_numpy(rows).cuda(), off)
    pos, cov, opa, sh = oracle.parse_ply(rows, off)
    np.testing.assert_array_equal(sp.position.cpu().numpy(), pos)
    np.testing.assert_array_equal(sp.sh.cpu().numpy().view(np.uint16), sh)
    # exp() may differ by an ulp between CUDA and libm; off-diagonal terms cancel, so bound the
    # error relative to each splat's largest variance rather than to the entry itself.
    got = sp.cov3d.cpu().numpy().astype(np.float64)
    scale = np.abs(cov[:, [0, 3, 5]]).max(axis=1, keepdims=True).astype(np.float64)
    assert (np.abs(got - cov) <= 4e-6 * scale).all()
    np.testing.assert_allclose(sp.opacity.cpu().numpy(), opa, rtol=1e-6)


def test_load_ply_file_roundtrip(cuda, oracle, tmp_path):
    from vkgs_gb300 import load, write_ply

    rows = syn.splat_rows(3000, 14)
    p = tmp_path / "scene.ply"
    write_ply(p, rows, syn.PLY_PROPERTIES)
    sp = load(p)
    pos, cov, opa, sh = oracle.parse_ply(rows, syn.ply_offsets())
    np.testing.assert_array_equal(sp.position.cpu().numpy(), pos)
    np.testing.assert_array_equal(sp.sh.cpu().numpy().view(np.uint16), sh)


@pytest.mark.parametrize("n,count", [(1, 1), (4096, 4096), (4097, 3000), (300_000, 299_999), (1 << 20, 1 << 20)])
def test_sorter_matches_stable_sort(cuda, n, count):
    import torch
    from vkgs_gb300 import Sorter

    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] = keys[n // 3: 2 * (n // 3)]  # plenty of duplicates
    vals = np.arange(n, dtype=np.uint32)
    kt = torch.from_numpy(keys.view(np.int32)).cuda()
    vt = torch.from_numpy(vals.view(np.int32)).cuda()
    s = Sorter()
    s.sort_key_value(kt, vt, count=count)
    s.check()
    order = np.argsort(keys[:count], kind="stable")
    np.testing.assert_array_equal(kt.cpu().numpy().view(np.uint32)[:count], keys[:count][order])
    np.testing.assert_array_equal(vt.cpu().numpy().view(np.uint32)[:count], vals[:count][order])
    np.testing.assert_array_equal(kt.cpu().numpy().view(np.uint32)[count:], keys[count:])


def test_sorter_count_beyond_capacity_is_reported(cuda):
    import torch
    from vkgs_gb300 import GsError, Sorter

    kt = torch.arange(1000, 0, -1, dtype=torch.int32, device="cuda")
    vt = torch.arange(1000, dtype=torch.int32, device="cuda")
    s = Sorter()
    s.sort_key_value(kt, vt, count=torch.tensor([5000], dtype=torch.int32, device="cuda"))
    with pytest.raises(GsError) as e:
        s.check()
    assert e.value.status == 2
    k = kt.cpu().numpy()
    assert np.all(k[:-1] <= k[1:])  # clamped to max_count and still sorted


@pytest.fixture(scope="module")
def large_scene(oracle):
    """The bench workload: 6M splats (shell layout, seed 1) and its nine 1600x900 cameras; the oracle's
    frame of each camera is computed once and shared by the tests below."""
    rows = syn.splat_rows(6_000_000, 1, "shell")
    act = scenes.activated(oracle, rows)
    del rows
    frames = {}

    def oracle_frame(cam_index):
        if cam_index not in frames:
            spec = syn.circle_cameras()[cam_index]
            c = scenes.camera(oracle, spec.eye, width=spec.width, height=spec.height)
            frames[cam_index] = (c, render_cpu(oracle, act, c))
        return frames[cam_index]

    return act, oracle_frame


@pytest.mark.parametrize("cam_index", range(9))
def test_large_workload_parity(cuda, oracle, large_scene, cam_index):
    """6M splats (shell layout) at 1600x900, every camera of the bench cycle, at full size: visible set,
    keys, order, instance records and the fragment count bit-exact, image within 1/255."""
    act, oracle_frame = large_scene
    c, o = oracle_frame(cam_index)
    g = render_gpu(act, c)
    assert_parity(g, o)


@pytest.mark.parametrize("cam_index", range(9))
def test_large_workload_early_stop_parity(cuda, oracle, large_scene, cam_index):
    """The production path the bench times (no fragment counting): depth slabs with finished tiles
    skipped and pixels stopped at the default transmittance floor 1e-4.  Keys, order and records stay
    bit-exact; the image is within the floor (+ FP32 noise) of the oracle's full blend."""
    act, oracle_frame = large_scene
    c, o = oracle_frame(cam_index)
    g = render_gpu(act, c, count_fragments=False)
    err = assert_parity(g, o, fragments=False)
    assert err <= 1e-4 + 2e-6, err
    assert g["stats"]["pairs_emitted"] > 0


@pytest.mark.parametrize("ends", [(1024,), (64, 256, 1024), (1, 2, 3, 1024), (512, 1024), (16, 1024)])
def test_slab_schedules(cuda, oracle, ends):
    """Every slab schedule gives the oracle's image; more slabs bin fewer pairs on a dense scene."""
    from vkgs_gb300 import Renderer

    rows = syn.splat_rows(400_000, 3, "shell")
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 8.0), width=640, height=360)
    r = Renderer(400_000, 640, 360)
    r.set_slabs(ends)
    g = render_gpu(act, c, count_fragments=False, renderer=r)
    o = render_cpu(oracle, act, c)
    assert_parity(g, o, fragments=False)
    r.set_slabs((1024,))
    one = render_gpu(act, c, count_fragments=False, renderer=r)["stats"]["pairs_emitted"]
    assert g["stats"]["pairs_emitted"] <= one
    if ends in ((64, 256, 1024), (512, 1024)):  # front slabs large enough to finish the shell's tiles
        assert g["stats"]["pairs_emitted"] < one
    if len(ends) == 1:
        assert g["stats"]["pairs_emitted"] == one


@pytest.mark.parametrize("t_floor,bound", [(1e-4, 1e-4 + 2e-6), (2.0 ** -24, 2e-6), (1.0 / 255.0, 1.0 / 255.0 + 2e-6)])
def test_transmittance_floor_bounds_the_image_error(cuda, oracle, t_floor, bound):
    """Stopping a pixel at transmittance t_floor changes no channel by more than t_floor (+ FP32 noise)."""
    from vkgs_gb300 import Renderer

    rows = syn.splat_rows(300_000, 8, "shell")
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 1.0, 8.0), width=800, height=450)
    r = Renderer(300_000, 800, 450)
    r.set_transmittance_floor(t_floor)
    g = render_gpu(act, c, count_fragments=False, renderer=r)
    o = render_cpu(oracle, act, c)
    err = assert_parity(g, o, fragments=False)
    assert err <= bound, err


def test_transmittance_floor_rejects_bad_values(cuda):
    from vkgs_gb300 import GsError, Renderer

    r = Renderer(100, 64, 64)
    for bad in (0.0, -1.0, 0.01, float("nan")):
        with pytest.raises(GsError):
            r.set_transmittance_floor(bad)


def test_slab_schedule_rejects_bad_input(cuda):
    from vkgs_gb300 import GsError, Renderer

    r = Renderer(1000, 64, 64)
    for bad in [(), (512,), (0, 1024), (512, 512, 1024), (1, 2, 3, 4, 1024), (2048,)]:
        with pytest.raises((GsError, ValueError)):
            r.set_slabs(bad)


def test_many_random_cameras(cuda, oracle):
    """500k splats, 12 random cameras of mixed resolution through one renderer."""
    from vkgs_gb300 import Renderer

    rows = syn.splat_rows(500_000, 21)
    act = scenes.activated(oracle, rows)
    specs = syn.random_cameras(12, seed=77)
    r = Renderer(500_000, 1920, 1080)
    for spec in specs:
        c = scenes.camera(oracle, spec.eye, fovy_deg=spec.fovy_deg, width=spec.width, height=spec.height)
        assert_parity(render_gpu(act, c, renderer=r), render_cpu(oracle, act, c))


def test_stage_times_cover_the_frame(cuda, oracle):
    """gs_context_stage_times (the reference's per-stage timestamp panel, engine.cc:1033-1045, 1188-1301):
    one row per timed frame, every stage positive, and the six stages summing to the frame's own
    CUDA-event time (the stages follow one another on the frame's stream, so the sum can only miss the
    gaps between them)."""
    import torch
    from vkgs_gb300 import Camera, Renderer, parse_ply

    rows = syn.splat_rows(1_000_000, 41, "shell")
    splats = parse_ply(torch.from_numpy(rows).cuda(), syn.ply_offsets())
    cams = [Camera.from_spec(s) for s in syn.circle_cameras()[:5]]
    r = Renderer(splats.count, 1600, 900)
    for cam in cams:
        r.render_checked(splats, cam)
    assert r.stage_times().shape == (0, 6)  # timing off: nothing recorded
    r.enable_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    outer = []
    for cam in cams:
        torch.cuda.synchronize()
        e0.record()
        r.render(splats, cam)
        e1.record()
        torch.cuda.synchronize()
        outer.append(e0.elapsed_time(e1))
    st = r.stage_times()
    r.enable_timing(False)
    r.check()
    assert st.shape == (len(cams), 6)
    assert (st > 0).all(), st
    total = st.sum(1)
    for k in range(len(cams)):  # the gaps (launch latency before the first stage, the tail copy) are small
        assert 0.75 * outer[k] <= total[k] <= outer[k] * 1.01 + 0.01, (k, total[k], outer[k])
    assert total.sum() >= 0.85 * sum(outer), (total, outer)
    assert r.stage_times().shape == (0, 6)  # the record was cleared
    r.render(splats, cams[0])
    assert r.stage_times().shape == (0, 6)  # and nothing is recorded after timing is turned off


@pytest.mark.parametrize("cam_index", [0, 8])
def test_staged_cull_parity(cuda, oracle, large_scene, cam_index):
    """The cull + projection with its splat partitions staged in shared memory by bulk copies
    (gs_context_set_cull_staging): the same visible set, keys, order, records, fragments and image."""
    from vkgs_gb300 import Renderer

    act, oracle_frame = large_scene
    c, o = oracle_frame(cam_index)
    r = Renderer(6_000_000, 1600, 900)
    r.set_cull_staging(True)
    assert_parity(render_gpu(act, c, renderer=r), o)


@pytest.mark.parametrize("n", [1, 255, 256, 257, 4097, 100_001])
def test_staged_cull_ragged_counts(cuda, oracle, n):
    """Partial last partitions (loaded by the threads) and counts below one partition."""
    from vkgs_gb300 import Renderer

    rows = syn.splat_rows(n, 60 + n % 7)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.3, 0.2, 5.0), width=320, height=200)
    r = Renderer(n, 320, 200)
    r.set_cull_staging(True)
    assert_parity(render_gpu(act, c, renderer=r), render_cpu(oracle, act, c))


def test_staged_cull_with_unaligned_buffers_falls_back(cuda, oracle):
    """Buffers that bulk copies cannot read (not 16-byte aligned) take the per-thread cull: same frame."""
    import torch
    from vkgs_gb300 import Renderer, Splats

    n = 5000
    rows = syn.splat_rows(n, 61)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=256, height=160)
    sp = Splats.from_numpy(*act)
    pos = torch.empty(3 * n + 1, dtype=torch.float32, device="cuda")[1:].view(n, 3)  # 4 bytes off 16
    pos.copy_(sp.position)
    shifted = Splats(pos, sp.cov3d, sp.opacity, sp.sh)
    r = Renderer(n, 256, 160)
    r.set_cull_staging(True)
    img = r.render(shifted, scenes.product_camera(c))
    r.check()
    o = render_cpu(oracle, act, c)
    assert float(np.abs(img.cpu().numpy().astype(np.float64) - o["image"]).max()) <= IMAGE_TOL


@pytest.mark.parametrize("n,w,h,seed,layout", [(400_000, 1600, 900, 71, "shell"), (40_000, 333, 201, 72, "gaussian")])
def test_lean_frames_equal_default_frames(cuda, oracle, n, w, h, seed, layout):
    """gs_context_set_lean (the launch shapes of frames that run beside others: lean cull, sort and
    emission grids, the raster with two pixels per thread in 8x8 warp blocks): the same visible set,
    keys, order, records and fragment counts and bit-identical RGBA32F and BGRA8 images, with the early
    stop and without it (fragment counting), with and without a caller depth target, at an odd width
    (the last pixel pair of each row half outside the image), and within the bar of the oracle."""
    from vkgs_gb300 import Renderer

    rows = syn.splat_rows(n, seed, layout)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.4, 0.3, 6.0), width=w, height=h)
    depth = np.random.default_rng(seed).uniform(0.975, 1.0, (h, w)).astype(np.float32)
    for d in (None, depth):
        for count in (False, True):
            frames = []
            for lean in (False, True):
                r = Renderer(n, w, h)
                r.set_lean(lean)
                frames.append(render_gpu(act, c, depth=d, count_fragments=count, renderer=r, bgra=True))
            a, b = frames
            assert a["count"] == b["count"]
            for k in ("key", "index", "instance", "image", "bgra", "draw"):
                np.testing.assert_array_equal(a[k], b[k], err_msg=f"{k} depth={d is not None} count={count}")
            assert a["fragments"] == b["fragments"]
            assert a["stats"]["fragments_blended"] == b["stats"]["fragments_blended"]
            o = render_cpu(oracle, act, c, depth=d)
            assert_parity(b, o, fragments=count)
