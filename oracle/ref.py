"""ctypes front end of the executable reference (``oracle/_ref/libvkgs_ref.so``).

TEST INFRASTRUCTURE ONLY.  The library is the reference's own shaders (src/shader/parse_ply.comp,
rank.comp, inverse_index.comp, projection.comp, splat.vert, splat.frag) compiled for the host by
``oracle/glsl/make_ref.py`` against a C++ GLSL subset (``oracle/glsl/glsl.hpp``) and driven in the
engine's dispatch order by ``oracle/glsl/ref_harness.cpp``.  It exists only where the reference
checkout does (it is built from the shader sources where they lie and never committed); it pins
``oracle/cpu_ref.c``, and ``tests/golden/make_ref_fixtures.py`` records its outputs as fixtures so
that the pin is also checked where the reference is absent.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

_lib = None


def available() -> bool:
    return lib() is not None


def lib():
    global _lib
    if _lib is None:
        from oracle.glsl import make_ref

        path = make_ref.build()
        if path is None:
            return None
        L = ctypes.CDLL(str(path))
        f32p = ctypes.POINTER(ctypes.c_float)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        u16p = ctypes.POINTER(ctypes.c_uint16)
        L.ref_parse_ply.argtypes = [f32p, ctypes.c_uint32, u32p, f32p, f32p, f32p, u16p]
        L.ref_frame_compute.argtypes = [f32p, f32p, f32p, u16p, ctypes.c_uint32, f32p, f32p, f32p, f32p,
                                        ctypes.c_uint32, ctypes.c_uint32, u32p, u32p, f32p, u32p]
        L.ref_frame_compute.restype = ctypes.c_uint32
        L.ref_draw.argtypes = [f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, f32p, ctypes.c_int, f32p]
        L.ref_draw.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _p(a, ct):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ct))


def parse_ply(rows: np.ndarray, offsets: np.ndarray):
    rows = np.ascontiguousarray(rows, np.float32)
    offsets = np.ascontiguousarray(offsets, np.uint32)
    n = rows.shape[0]
    pos = np.zeros((n, 3), np.float32)
    cov = np.zeros((n, 6), np.float32)
    opa = np.zeros(n, np.float32)
    sh = np.zeros((n, 48), np.uint16)
    lib().ref_parse_ply(_p(rows, ctypes.c_float), n, _p(offsets, ctypes.c_uint32), _p(pos, ctypes.c_float),
                        _p(cov, ctypes.c_float), _p(opa, ctypes.c_float), _p(sh, ctypes.c_uint16))
    return pos, cov, opa, sh


def frame_compute(position, cov3d, opacity, sh, cam):
    """rank -> sort -> inverse index -> projection for one camera (an ``oracle.Camera``).

    Returns dict(count, key, index, instance (V x 12, sorted order), draw_indirect (12 words))."""
    position = np.ascontiguousarray(position, np.float32)
    cov3d = np.ascontiguousarray(cov3d, np.float32)
    opacity = np.ascontiguousarray(opacity, np.float32)
    sh = np.ascontiguousarray(sh, np.uint16)
    n = position.shape[0]
    key = np.zeros(max(n, 1), np.uint32)
    idx = np.zeros(max(n, 1), np.uint32)
    inst = np.zeros((max(n, 1), 12), np.float32)
    draw = np.zeros(12, np.uint32)
    proj = np.array(cam.projection[:], np.float32)
    view = np.array(cam.view[:], np.float32)
    model = np.array(cam.model[:], np.float32)
    eye = np.array(cam.eye[:], np.float32)
    v = lib().ref_frame_compute(_p(position, ctypes.c_float), _p(cov3d, ctypes.c_float),
                                _p(opacity, ctypes.c_float), _p(sh, ctypes.c_uint16), n, _p(proj, ctypes.c_float),
                                _p(view, ctypes.c_float), _p(model, ctypes.c_float), _p(eye, ctypes.c_float),
                                cam.width, cam.height, _p(key, ctypes.c_uint32), _p(idx, ctypes.c_uint32),
                                _p(inst, ctypes.c_float), _p(draw, ctypes.c_uint32))
    return {"count": int(v), "key": key[:v].copy(), "index": idx[:v].copy(), "instance": inst[:v].copy(),
            "draw_indirect": draw}


def draw(instance, width: int, height: int, depth_in=None, unorm8: bool = False):
    """splat.vert + Vulkan rasterisation + splat.frag + depth test + blend.  Returns (image, fragments)."""
    instance = np.ascontiguousarray(instance, np.float32)
    img = np.zeros((height, width, 4), np.float32)
    d = None if depth_in is None else np.ascontiguousarray(depth_in, np.float32)
    f = lib().ref_draw(_p(instance, ctypes.c_float), instance.shape[0], width, height,
                       None if d is None else _p(d, ctypes.c_float), int(bool(unorm8)), _p(img, ctypes.c_float))
    return img, int(f)


def lib_path() -> Path | None:
    from oracle.glsl import make_ref

    return make_ref.LIB if make_ref.LIB.exists() else None
