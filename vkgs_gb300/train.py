"""The differentiable path: raw splat parameters -> RGBA image, with hand-written CUDA backward kernels
behind a torch.autograd.Function (gs_train_forward / gs_train_backward of the C ABI).

    img = vkgs_gb300.train.render(params, camera, renderer)   # params: dict of CUDA float32 tensors
    loss = (img - target).abs().mean(); loss.backward()        # grads land in params[...].grad

params: means (N, 3), log_scales (N, 3), quats (N, 4) in (x, y, z, w) order, opacity_logits (N,),
sh (N, 48) in [channel][16 coefficients] order (see vkgs_gb300.train_params.from_rows).  One renderer
keeps the state of its last forward for the backward: render, then backward, before the next render on
the same renderer.

    imgs = vkgs_gb300.train.render_batched(params, cameras, renderer)  # many views, one call each way

draws every view concurrently over the renderer's render lanes (one lane per view) and, in the
backward, adds all views' gradients into one set of parameter gradients.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib as L
from .api import Camera, GsError, Renderer, _check, _need_cuda, _ptr, _stream

NAMES = ("means", "log_scales", "quats", "opacity_logits", "sh")
SHAPES = {"means": (3,), "log_scales": (3,), "quats": (4,), "opacity_logits": (), "sh": (48,)}


def _train_params(tensors) -> L.GsTrainParams:
    n = tensors[0].shape[0]
    for name, t in zip(NAMES, tensors):
        _need_cuda(t, name, torch.float32)
        if tuple(t.shape) != (n,) + SHAPES[name] or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous ({n}{', ' if SHAPES[name] else ''}"
                             f"{', '.join(map(str, SHAPES[name]))}) float32 CUDA tensor")
    return L.GsTrainParams(*[_ptr(t) for t in tensors], n)


def forward(renderer: Renderer, tensors, camera: Camera, stream=None, check: bool | None = None) -> torch.Tensor:
    """gs_train_forward into a new (H, W, 4) image.

    The first call on a renderer (or check=True) synchronises, checks the device error word and grows the
    pair capacity once if it overflowed; later calls stay asynchronous (no host sync inside a training
    step) and report errors at the next Renderer.check()."""
    p = _train_params(tensors)
    img = torch.empty((int(camera.height), int(camera.width), 4), dtype=torch.float32, device=tensors[0].device)
    cam = camera.struct()
    lib = renderer._lib
    _check(lib.gs_train_forward(renderer._h, ctypes.byref(p), ctypes.byref(cam), _ptr(img), _stream(stream)),
           "gs_train_forward")
    if check is None:
        check = not getattr(renderer, "_train_sized", False)
    if not check:
        return img
    renderer._train_sized = True
    try:
        renderer.check(stream)
    except GsError as e:
        if e.status != L.GS_ERROR_CAPACITY or not hasattr(e, "stats"):
            raise
        renderer.reserve(max_tile_pairs=int(e.stats["tile_pairs"] * 1.25) + 1024)
        _check(lib.gs_train_forward(renderer._h, ctypes.byref(p), ctypes.byref(cam), _ptr(img), _stream(stream)),
               "gs_train_forward")
        renderer.check(stream)
    return img


def backward(renderer: Renderer, tensors, camera: Camera, grad_img: torch.Tensor, stream=None):
    """gs_train_backward: gradients of the raw parameters (new zero-initialised tensors)."""
    p = _train_params(tensors)
    grad_img = grad_img.contiguous()
    _need_cuda(grad_img, "grad_img", torch.float32)
    grads = [torch.zeros_like(t) for t in tensors]
    g = L.GsTrainGrads(*[_ptr(t) for t in grads])
    cam = camera.struct()
    _check(renderer._lib.gs_train_backward(renderer._h, ctypes.byref(p), ctypes.byref(cam), _ptr(grad_img),
                                           ctypes.byref(g), _stream(stream)), "gs_train_backward")
    return grads


def _views(renderer: Renderer, cameras, tensors, images, name):
    n = len(cameras)
    if renderer.batch_lanes < n:
        renderer.set_batch_lanes(n)
    cams = (L.GsCamera * max(n, 1))()
    ptrs = (ctypes.c_void_p * max(n, 1))()
    for v, (cam, im) in enumerate(zip(cameras, images)):
        _need_cuda(im, f"{name}[{v}]", torch.float32)
        if tuple(im.shape) != (int(cam.height), int(cam.width), 4) or not im.is_contiguous():
            raise ValueError(f"{name}[{v}] must be a contiguous ({cam.height}, {cam.width}, 4) float32 tensor")
        cams[v] = cam.struct()
        ptrs[v] = _ptr(im)
    return n, cams, ptrs


def forward_batched(renderer: Renderer, tensors, cameras, stream=None, check: bool | None = None):
    """gs_train_forward_batched into new (H_v, W_v, 4) images, one per camera (capacity as in forward)."""
    p = _train_params(tensors)
    dev = tensors[0].device
    imgs = [torch.empty((int(c.height), int(c.width), 4), dtype=torch.float32, device=dev) for c in cameras]
    n, cams, ptrs = _views(renderer, cameras, tensors, imgs, "images")
    lib = renderer._lib

    def run():
        _check(lib.gs_train_forward_batched(renderer._h, ctypes.byref(p), n, cams, ptrs, _stream(stream)),
               "gs_train_forward_batched")

    run()
    if check is None:
        check = getattr(renderer, "_train_sized_views", 0) < n
    if not check:
        return imgs
    renderer._train_sized_views = max(n, getattr(renderer, "_train_sized_views", 0))
    try:
        renderer.check(stream)
    except GsError as e:
        if e.status != L.GS_ERROR_CAPACITY or not hasattr(e, "stats"):
            raise
        renderer.reserve(max_tile_pairs=int(e.stats["tile_pairs"] * 1.25) + 1024)
        run()
        renderer.check(stream)
    return imgs


def backward_batched(renderer: Renderer, tensors, cameras, grad_imgs, stream=None):
    """gs_train_backward_batched: gradients of the raw parameters of the loss summed over the views."""
    p = _train_params(tensors)
    grad_imgs = [g.contiguous() for g in grad_imgs]
    n, cams, ptrs = _views(renderer, cameras, tensors, grad_imgs, "grad_imgs")
    grads = [torch.zeros_like(t) for t in tensors]
    g = L.GsTrainGrads(*[_ptr(t) for t in grads])
    _check(renderer._lib.gs_train_backward_batched(renderer._h, ctypes.byref(p), n, cams, ptrs, ctypes.byref(g),
                                                   _stream(stream)), "gs_train_backward_batched")
    return grads


class RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means, log_scales, quats, opacity_logits, sh, renderer, camera):
        tensors = [t.detach().contiguous() for t in (means, log_scales, quats, opacity_logits, sh)]
        img = forward(renderer, tensors, camera)
        ctx.renderer, ctx.camera = renderer, camera
        ctx.save_for_backward(*tensors)
        return img

    @staticmethod
    def backward(ctx, grad_img):
        grads = backward(ctx.renderer, list(ctx.saved_tensors), ctx.camera, grad_img)
        return (*grads, None, None)


class BatchedRenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, renderer, cameras, means, log_scales, quats, opacity_logits, sh):
        tensors = [t.detach().contiguous() for t in (means, log_scales, quats, opacity_logits, sh)]
        imgs = forward_batched(renderer, tensors, cameras)
        ctx.renderer, ctx.cameras = renderer, list(cameras)
        ctx.save_for_backward(*tensors)
        return tuple(imgs)

    @staticmethod
    def backward(ctx, *grad_imgs):
        grad_imgs = [torch.zeros((int(c.height), int(c.width), 4), dtype=torch.float32, device=ctx.saved_tensors[0].device)
                     if g is None else g for g, c in zip(grad_imgs, ctx.cameras)]
        grads = backward_batched(ctx.renderer, list(ctx.saved_tensors), ctx.cameras, grad_imgs)
        return (None, None, *grads)


def render_batched(params: dict, cameras, renderer: Renderer):
    """Differentiable render of raw parameters from every camera: a tuple of (H_v, W_v, 4) images."""
    return BatchedRenderFunction.apply(renderer, list(cameras), *(params[k] for k in NAMES))


def render(params: dict, camera: Camera, renderer: Renderer) -> torch.Tensor:
    """Differentiable render of raw parameters (dict with NAMES keys) from one camera."""
    return RenderFunction.apply(*(params[k] for k in NAMES), renderer, camera)
