"""GPU: the differentiable path (gs_train_forward / gs_train_backward behind a torch.autograd.Function)
against the FP64 torch restatement of the reference (autograd) and the plain forward."""

import numpy as np
import pytest

from tests import scenes
from vkgs_gb300 import synthetic as syn
from vkgs_gb300 import train_params as tp

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-3  # per parameter group: ||g_cuda - g_fp64|| / ||g_fp64||


def _gpu_params(rows, f16_sh=False):
    import torch

    p = tp.from_rows(rows)
    if f16_sh:
        p["sh"] = p["sh"].astype(np.float16).astype(np.float32)
    return {k: torch.tensor(v, device="cuda", requires_grad=True) for k, v in p.items()}


@pytest.mark.parametrize("n,w,h,eye,seed,slabs", [
    (1000, 128, 128, (0.0, 0.0, 6.0), 3, None),
    (400, 96, 80, (1.5, 0.5, 4.0), 5, None),
    (1000, 128, 128, (0.0, 0.0, 6.0), 3, (128, 1024)),       # stacked slabs: every slab's lists kept
    (3000, 112, 96, (1.0, -0.5, 5.0), 6, (64, 320, 1024)),
    (600, 97, 61, (0.5, 0.2, 5.0), 8, None),                  # odd sizes: half-outside pixel pairs
    (1200, 113, 77, (0.8, -0.3, 5.5), 9, (128, 1024)),
])
def test_gradients_match_fp64_oracle(cuda, oracle, n, w, h, eye, seed, slabs):
    import torch
    from oracle import torch_ref
    from vkgs_gb300 import train

    rows = syn.splat_rows(n, seed)
    c = scenes.camera(oracle, eye, width=w, height=h)
    act = scenes.activated(oracle, rows)
    ocam = scenes.oracle_camera(oracle, c)
    out = oracle.render_frame(*act, ocam)
    _, rec = oracle.project(*act, out["index"], ocam)
    weights = np.random.default_rng(seed).standard_normal((h, w, 4))

    params = _gpu_params(rows)
    from vkgs_gb300 import Renderer

    r = Renderer(n, w, h)
    if slabs is not None:
        r.set_slabs(slabs)
        r.set_train_slab_min(0)
    img = train.render(params, scenes.product_camera(c), r)
    (img * torch.tensor(weights, dtype=torch.float32, device="cuda")).sum().backward()

    p64 = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in tp.from_rows(rows).items()}
    img64 = torch_ref.render(p64["means"], p64["log_scales"], p64["quats"], p64["opacity_logits"], p64["sh"],
                             torch_ref.camera_dict(c), out["index"], mask_records=rec)
    (img64 * torch.tensor(weights)).sum().backward()

    assert np.abs(img.detach().cpu().numpy() - img64.detach().numpy()).max() <= 1.0 / 255.0
    for name in train.NAMES:
        g = params[name].grad.double().cpu()
        g64 = p64[name].grad
        rel = float((g - g64).norm() / g64.norm())
        assert rel <= GRAD_RTOL, (name, rel)


def test_train_forward_equals_plain_forward(cuda, oracle):
    """With binary16-representable SH the differentiable forward draws the plain forward's frame: to
    float rounding at a floor of 2^-24, and within the floor at the default 1e-4."""
    import torch
    from vkgs_gb300 import Renderer, parse_ply, train

    rows = syn.splat_rows(50_000, 7)
    rows_f16 = rows.copy()
    off = syn.ply_offsets()
    rows_f16[:, off[10:58]] = rows[:, off[10:58]].astype(np.float16).astype(np.float32)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=640, height=360)
    cam = scenes.product_camera(c)
    splats = parse_ply(torch.from_numpy(rows_f16).cuda(), off)
    for t_floor, tol in ((2.0 ** -24, 1e-6), (1e-4, 1e-4 + 1e-6)):
        r = Renderer(50_000, 640, 360)
        r.set_transmittance_floor(t_floor)
        plain, _ = r.render_checked(splats, cam)
        rt = Renderer(50_000, 640, 360)
        rt.set_transmittance_floor(t_floor)
        img = train.render(_gpu_params(rows_f16), cam, rt)
        assert float((img.detach() - plain).abs().max()) <= tol, t_floor


def test_lean_differentiable_path_equals_default(cuda, oracle):
    """A lean context (gs_context_set_lean: the training raster with two pixels per thread on every slab)
    draws the same image bit for bit and the same gradients (to float summation order) as a default one
    (two pixels per thread on the nearest slab only), at an odd width with two slabs."""
    import torch
    from vkgs_gb300 import Renderer, train

    n, w, h = 3000, 143, 87
    rows = syn.splat_rows(n, 10)
    c = scenes.camera(oracle, (0.6, -0.4, 5.0), width=w, height=h)
    cam = scenes.product_camera(c)
    weights = torch.tensor(np.random.default_rng(10).standard_normal((h, w, 4)), dtype=torch.float32,
                           device="cuda")
    out = []
    for lean in (False, True):
        r = Renderer(n, w, h)
        r.set_slabs((128, 1024))
        r.set_train_slab_min(0)
        r.set_lean(lean)
        params = _gpu_params(rows)
        img = train.render(params, cam, r)
        (img * weights).sum().backward()
        out.append((img.detach().cpu().numpy(), {k: params[k].grad.double().cpu() for k in train.NAMES}))
    (img_a, g_a), (img_b, g_b) = out
    np.testing.assert_array_equal(img_a, img_b)
    for name in train.NAMES:
        rel = float((g_a[name] - g_b[name]).norm() / max(float(g_a[name].norm()), 1e-30))
        assert rel <= 1e-5, (name, rel)


def test_train_rejects_bad_shapes(cuda):
    import torch
    from vkgs_gb300 import Camera, Renderer, train

    r = Renderer(10, 64, 64)
    p = {k: torch.zeros((10,) + train.SHAPES[k], device="cuda") for k in train.NAMES}
    p["sh"] = torch.zeros((10, 47), device="cuda")
    cam = Camera.from_spec(syn.CameraSpec(eye=(0.0, 0.0, 6.0), width=64, height=64))
    with pytest.raises(ValueError):
        train.render(p, cam, r)


@pytest.mark.parametrize("shared", [True, False])
def test_batched_gradients_equal_sum_of_views(cuda, oracle, shared):
    """The batched differentiable path draws each view exactly as the one-view path and its gradients are
    the per-view gradients summed (atomic accumulation: equal up to FP32 summation order)."""
    import torch
    from vkgs_gb300 import Renderer, train

    n = 20_000
    rows = syn.splat_rows(n, 11)
    eyes = [(0.0, 0.0, 6.0), (1.5, 0.5, 4.0), (-2.0, 1.0, 5.0), (0.5, -1.5, 4.5), (3.0, 0.0, 3.0)]
    sizes = [(160, 120), (128, 128), (200, 90), (96, 160), (144, 144)]
    cams = [scenes.product_camera(scenes.camera(oracle, e, width=w, height=h)) for e, (w, h) in zip(eyes, sizes)]
    gen = torch.Generator(device="cuda").manual_seed(4)
    weights = [torch.randn((h, w, 4), device="cuda", generator=gen) for (w, h) in sizes]

    ref = {k: torch.zeros_like(v) for k, v in _gpu_params(rows).items()}
    single = Renderer(n, 200, 160)
    imgs1 = []
    for cam, wt in zip(cams, weights):
        p = _gpu_params(rows)
        img = train.render(p, cam, single)
        (img * wt).sum().backward()
        imgs1.append(img.detach())
        for k in train.NAMES:
            ref[k] += p[k].grad

    r = Renderer(n, 200, 160)
    r.set_batch_lanes(len(cams))
    r.set_train_slab_min(0)  # stacked depth slabs on the lanes; the one-view reference uses one slab
    r.set_batch_shared_cull(shared)  # one cull pass for all views, or one per lane
    params = _gpu_params(rows)
    imgs = train.render_batched(params, cams, r)
    sum((img * wt).sum() for img, wt in zip(imgs, weights)).backward()
    r.check()
    for img, img1 in zip(imgs, imgs1):
        assert torch.equal(img.detach(), img1)
    for k in train.NAMES:
        g, g1 = params[k].grad, ref[k]
        rel = float((g - g1).norm() / g1.norm())
        assert rel <= 1e-5, (k, rel)


def test_batched_train_needs_a_lane_per_view(cuda):
    import ctypes

    import torch
    from vkgs_gb300 import Camera, Renderer, _lib as L, train

    r = Renderer(10, 64, 64)
    p = {k: torch.zeros((10,) + train.SHAPES[k], device="cuda") for k in train.NAMES}
    p["quats"][:, 3] = 1.0
    cam = Camera.from_spec(syn.CameraSpec(eye=(0.0, 0.0, 6.0), width=64, height=64))
    r.set_batch_lanes(2)
    tensors = [p[k] for k in train.NAMES]
    imgs = [torch.empty((64, 64, 4), device="cuda") for _ in range(3)]
    tp_ = train._train_params(tensors)
    cams = (L.GsCamera * 3)(*[cam.struct()] * 3)
    ptrs = (ctypes.c_void_p * 3)(*[im.data_ptr() for im in imgs])
    st = r._lib.gs_train_forward_batched(r._h, ctypes.byref(tp_), 3, cams, ptrs, None)
    assert st == L.GS_ERROR_CAPACITY
    imgs = train.forward_batched(r, tensors, [cam] * 3)  # the Python side adds lanes
    assert r.batch_lanes == 3 and len(imgs) == 3
    r.check()


def test_sharded_train_step_single_rank_matches_batched(cuda):
    """The data-parallel step (vkgs_gb300.shard.train_step_sharded) at world size 1 over NCCL: its
    all-reduced gradients equal the batched Function's."""
    import socket

    import torch
    import torch.distributed as dist
    from vkgs_gb300 import Camera, Renderer, shard, train

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        n = 5_000
        rows = syn.splat_rows(n, 31)
        cams = [Camera.from_spec(sp) for sp in syn.random_cameras(3, seed=507, resolutions=[(160, 120), (128, 96)])]
        gen = torch.Generator(device="cuda").manual_seed(8)
        targets = [torch.rand((c.height, c.width, 4), device="cuda", generator=gen) for c in cams]
        r = Renderer(n, 160, 120)
        r.set_batch_lanes(len(cams))
        p1 = _gpu_params(rows)
        loss = shard.train_step_sharded(p1, cams, lambda v, img: (img - targets[v]).abs().mean(), r, 0, 1)
        p2 = _gpu_params(rows)
        imgs = train.render_batched(p2, cams, Renderer(n, 160, 120))
        ref = sum((img - t).abs().mean() for img, t in zip(imgs, targets))
        ref.backward()
        assert abs(float(loss) - float(ref.detach())) <= 1e-5 * abs(float(ref.detach()))
        for k in train.NAMES:
            rel = float((p1[k].grad - p2[k].grad).norm() / p2[k].grad.norm())
            assert rel <= 1e-5, (k, rel)
    finally:
        dist.destroy_process_group()


def _footprint_window(rec, w, h):
    """Pixel rectangle (x0, x1, y0, y1) holding every pixel centre a raster record's quad can cover."""
    import math

    cx, cy, hx, hy = float(rec[0]), float(rec[1]), float(rec[12]), float(rec[13])
    x0 = max(0, math.floor((cx - hx + 1.0) * w / 2 - 0.5) - 1)
    x1 = min(w, math.ceil((cx + hx + 1.0) * w / 2 - 0.5) + 2)
    y0 = max(0, math.floor((cy - hy + 1.0) * h / 2 - 0.5) - 1)
    y1 = min(h, math.ceil((cy + hy + 1.0) * h / 2 - 0.5) + 2)
    return x0, x1, y0, y1


def test_gradient_check_workload_at_size(cuda, oracle):
    """The gradient-check workload at its stated size: 1,000 splats at 256x256.  CUDA gradients of every
    parameter group within 1e-3 (relative norm) of torch-FP64 autograd, and, on 4 entries per group
    (among the largest), FP64 central differences (h = 1e-6) of the loss agreeing with torch-FP64 autograd
    to 1e-5 and with the CUDA gradient to 1e-3.  A central difference perturbs one splat, which changes
    only the pixels its quad covers, so the loss is evaluated over that footprint's rectangle."""
    import torch
    from oracle import torch_ref
    from vkgs_gb300 import Camera, Renderer, train

    rows, off, specs = syn.workload("grad_check")
    spec = specs[0]
    assert rows.shape[0] == 1000 and (spec.width, spec.height) == (256, 256)
    w, h = spec.width, spec.height
    c = scenes.camera(oracle, spec.eye, fovy_deg=spec.fovy_deg, width=w, height=h)
    act = scenes.activated(oracle, rows)
    ocam = scenes.oracle_camera(oracle, c)
    out = oracle.render_frame(*act, ocam)
    _, rec = oracle.project(*act, out["index"], ocam)
    assert out["count"] > 500
    weights = np.random.default_rng(12).standard_normal((h, w, 4))

    params = _gpu_params(rows)
    img = train.render(params, scenes.product_camera(c), Renderer(1000, w, h))
    (img * torch.tensor(weights, dtype=torch.float32, device="cuda")).sum().backward()

    p64 = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in tp.from_rows(rows).items()}
    cam = torch_ref.camera_dict(c)
    args = lambda: (p64["means"], p64["log_scales"], p64["quats"], p64["opacity_logits"], p64["sh"], cam, out["index"])
    img64 = torch_ref.render(*args(), mask_records=rec)
    (img64 * torch.tensor(weights)).sum().backward()
    assert np.abs(img.detach().cpu().numpy() - img64.detach().numpy()).max() <= 1.0 / 255.0
    grads = {}
    for name in train.NAMES:
        g = params[name].grad.double().cpu()
        g64 = p64[name].grad.clone()
        grads[name] = (g, g64)
        rel = float((g - g64).norm() / g64.norm())
        assert rel <= GRAD_RTOL, (name, rel)

    record_of = {int(s): r for r, s in enumerate(out["index"])}
    rng = np.random.default_rng(5)
    for name in train.NAMES:
        g, g64 = grads[name]
        flat = g64.reshape(g64.shape[0], -1).abs()
        top = torch.argsort(flat.reshape(-1), descending=True)[:40].numpy()
        for pick in rng.choice(top, 4, replace=False):
            i, j = divmod(int(pick), flat.shape[1])
            idx = (i,) if g64.dim() == 1 else (i, j)
            win = _footprint_window(rec[record_of[i]], w, h)
            wt = torch.tensor(weights[win[2]:win[3], win[0]:win[1]])

            def loss():
                return (torch_ref.render(*args(), mask_records=rec, window=win) * wt).sum()

            fd = torch_ref.central_difference(loss, p64[name].data, idx)
            scale = max(abs(fd), 0.1 * float(flat.max()))
            assert abs(float(g64[idx]) - fd) <= 1e-5 * max(1.0, abs(fd)), (name, idx, float(g64[idx]), fd)
            assert abs(float(g[idx]) - fd) <= 1e-3 * scale, (name, idx, float(g[idx]), fd)


def test_backward_refuses_overwritten_forward_state(cuda, oracle):
    """A render between a differentiable forward and its backward overwrites the forward's tile lists:
    the backward is refused (GS_ERROR_INVALID_ARGUMENT) instead of reading another frame's lists, for
    the one-view and the batched form; with nothing in between it runs."""
    import torch
    from vkgs_gb300 import Camera, GsError, Renderer, parse_ply, train

    n = 5_000
    rows = syn.splat_rows(n, 17)
    cams = [Camera.from_spec(sp) for sp in syn.random_cameras(3, seed=509, resolutions=[(160, 120), (128, 96)])]
    splats = parse_ply(torch.from_numpy(rows).cuda(), syn.ply_offsets())
    r = Renderer(n, 160, 120)
    img = train.render(_gpu_params(rows), cams[0], r)
    r.render(splats, cams[1])
    with pytest.raises(GsError) as e:
        img.sum().backward()
    assert e.value.status == 1
    img = train.render(_gpu_params(rows), cams[0], r)
    img.sum().backward()  # nothing in between: fine

    rb = Renderer(n, 160, 120)
    rb.set_batch_lanes(len(cams))
    colors = [torch.empty((c.height, c.width, 4), device="cuda") for c in cams]
    for between in (lambda: rb.render_batched(splats, cams, colors),
                    lambda: train.forward_batched(rb, [t.detach() for t in _gpu_params(rows).values()], cams[:2])):
        imgs = train.render_batched(_gpu_params(rows), cams, rb)
        between()
        with pytest.raises(GsError) as e:
            sum(i.sum() for i in imgs).backward()
        assert e.value.status == 1
    imgs = train.render_batched(_gpu_params(rows), cams, rb)
    sum(i.sum() for i in imgs).backward()
    rb.check()
