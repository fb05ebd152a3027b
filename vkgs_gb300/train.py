"""The differentiable path: raw splat parameters -> RGBA image, with hand-written CUDA backward kernels
behind a torch.autograd.Function (gs_train_forward / gs_train_backward of the C ABI).

    img = vkgs_gb300.train.render(params, camera, renderer)   # params: dict of CUDA float32 tensors
    loss = (img - target).abs().mean(); loss.backward()        # grads land in params[...].grad

params: means (N, 3), log_scales (N, 3), quats (N, 4) in (x, y, z, w) order, opacity_logits (N,),
sh (N, 48) in [channel][16 coefficients] order (see vkgs_gb300.train_params.from_rows).  One renderer
keeps the state of its last forward for the backward: render, then backward, before the next render on
the same renderer.
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


def render(params: dict, camera: Camera, renderer: Renderer) -> torch.Tensor:
    """Differentiable render of raw parameters (dict with NAMES keys) from one camera."""
    return RenderFunction.apply(*(params[k] for k in NAMES), renderer, camera)
