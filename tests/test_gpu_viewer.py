"""GPU: the viewer loop (one CUDA graph per frame, camera rewritten in the graph) against gs_render."""

import pytest

from vkgs_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def test_viewer_frames_equal_direct_renders(cuda):
    import torch
    from vkgs_gb300 import Camera, Renderer, Viewer, parse_ply

    rows = syn.splat_rows(300_000, 21, "shell")
    splats = parse_ply(torch.from_numpy(rows).cuda(), syn.ply_offsets())
    specs = syn.circle_cameras(width=800, height=450)
    cams = [Camera.from_spec(s) for s in specs]
    direct = Renderer(300_000, 800, 450)
    want = [direct.render_checked(splats, c)[0].clone() for c in cams]
    r = Renderer(300_000, 800, 450)
    for c in cams:  # size the pair capacity before the graph is captured
        r.render_checked(splats, c)
    color = torch.zeros((450, 800, 4), device="cuda")
    v = Viewer(r, splats, cams[0], color)
    for _ in range(2):
        for c, w in zip(cams, want):
            img = v.frame(c)
            torch.cuda.synchronize()
            assert torch.equal(img, w)
    r.check()
    v.close()


def test_viewer_rejects_other_resolution(cuda):
    import torch
    from vkgs_gb300 import Camera, GsError, Renderer, Viewer, parse_ply

    rows = syn.splat_rows(1000, 22)
    splats = parse_ply(torch.from_numpy(rows).cuda(), syn.ply_offsets())
    cam = Camera.from_spec(syn.CameraSpec(eye=(0.0, 0.0, 6.0), width=320, height=180))
    r = Renderer(1000, 640, 360)
    v = Viewer(r, splats, cam, torch.zeros((180, 320, 4), device="cuda"))
    with pytest.raises(GsError):
        v.frame(Camera.from_spec(syn.CameraSpec(eye=(0.0, 0.0, 6.0), width=640, height=360)))
    v.close()


@pytest.mark.parametrize("inflight", [2, 3])
def test_viewer_frames_in_flight_equal_direct_renders(cuda, inflight):
    """Frames submitted without waiting (one slot per frame in flight, own scratch and stream each) are
    the direct renders; a slot's target is read back before the slot is reused."""
    import torch
    from vkgs_gb300 import Camera, Renderer, Viewer, parse_ply

    rows = syn.splat_rows(300_000, 23, "shell")
    splats = parse_ply(torch.from_numpy(rows).cuda(), syn.ply_offsets())
    cams = [Camera.from_spec(s) for s in syn.circle_cameras(width=640, height=360)]
    direct = Renderer(300_000, 640, 360)
    want = [direct.render_checked(splats, c)[0].clone() for c in cams]
    r = Renderer(300_000, 640, 360)
    for c in cams:
        r.render_checked(splats, c)
    v = Viewer(r, splats, cams[0], torch.zeros((360, 640, 4), device="cuda"), frames_in_flight=inflight)
    main = torch.cuda.current_stream()
    got = []
    for k in range(2 * len(cams)):
        assert v.next_slot == k % inflight
        slot = v.submit(cams[k % len(cams)])
        assert slot == k % inflight
        v.wait(slot)  # the copy below is ordered after this frame, and before the slot's next submit
        got.append(v.colors[slot].clone())
        if k == 0:
            assert len(set(id(c) for c in v.colors)) == inflight
    v.check()
    main.synchronize()
    for k, img in enumerate(got):
        assert torch.equal(img, want[k % len(cams)]), k
    v.close()


def test_viewer_frames_in_flight_rejects_bad_counts(cuda):
    import torch
    from vkgs_gb300 import Camera, GsError, Renderer, Viewer, parse_ply

    rows = syn.splat_rows(1000, 24)
    splats = parse_ply(torch.from_numpy(rows).cuda(), syn.ply_offsets())
    cam = Camera.from_spec(syn.CameraSpec(eye=(0.0, 0.0, 6.0), width=320, height=180))
    r = Renderer(1000, 320, 180)
    for n in (0, 9):
        with pytest.raises((GsError, ValueError)):
            Viewer(r, splats, cam, [torch.zeros((180, 320, 4), device="cuda")] * max(n, 1), frames_in_flight=n)


def test_bench_viewer_frames_in_flight_equal_direct_renders(cuda):
    """The headline configuration as the bench runs it: 6M splats (shell layout), 1600x900, the nine
    cameras cycled for two laps through gs_viewer_submit with five frames in flight (lean launch shapes),
    the pair capacity reserved from counted frames -- every frame bit-identical to a direct gs_render of
    its camera."""
    import torch
    from vkgs_gb300 import Camera, Renderer, Viewer, parse_ply

    rows = syn.splat_rows(6_000_000, 1, "shell")
    splats = parse_ply(torch.from_numpy(rows).cuda(), syn.ply_offsets())
    del rows
    cams = [Camera.from_spec(s) for s in syn.circle_cameras()]
    direct = Renderer(6_000_000, 1600, 900)
    want = [direct.render_checked(splats, c)[0].clone() for c in cams]
    direct.close()
    r = Renderer(6_000_000, 1600, 900)
    r.count_fragments(True)
    pairs = max(r.render_checked(splats, c)[1]["tile_pairs"] for c in cams)
    r.count_fragments(False)
    r.reserve(max_tile_pairs=int(pairs * 1.05) + 1024)
    slots = 5
    v = Viewer(r, splats, cams[0], torch.zeros((900, 1600, 4), device="cuda"), frames_in_flight=slots)
    # as the bench's end-to-end loop: a slot's image is copied on a side stream after its frame, and the
    # slot is drawn into again only after that copy, so up to five frames overlap on the GPU
    main = torch.cuda.current_stream()
    copier = torch.cuda.Stream()
    copied = [torch.cuda.Event() for _ in range(slots)]
    started, got = set(), []
    for k in range(2 * len(cams)):
        slot = v.next_slot
        if slot in started:
            main.wait_event(copied[slot])
        started.add(slot)
        assert v.submit(cams[k % len(cams)], stream=main) == slot
        v.wait(slot, copier)
        with torch.cuda.stream(copier):
            got.append(v.colors[slot].clone())
        copied[slot].record(copier)
    main.wait_stream(copier)
    v.check(main)
    torch.cuda.synchronize()
    for k, img in enumerate(got):
        assert torch.equal(img, want[k % len(cams)]), k
    v.close()
    r.check()
