"""ctypes front end of the CPU oracle (``cpu_ref.c``).

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline arm of ``bench.py`` -- never by the product package.

Parity status: pinned.  The reference ships no tests, fixtures or CPU code and
its GLSL shaders need a Vulkan stack, so ``oracle/glsl`` compiles the shader
bodies for the host and ``tests/test_ref_pin.py`` holds this scalar restatement
(every float operation in GLSL order, no FMA contraction) to their bits; see
``cpu_ref.c`` for the per-function shader citations.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "libcpu_ref.so"
SOURCES = [HERE / "cpu_ref.c"]
CFLAGS = ["-O2", "-fPIC", "-shared", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
          "-fno-strict-aliasing"]


def build(force: bool = False) -> Path:
    """Compile the oracle with gcc (the same recipe as ``oracle/Makefile``)."""
    BUILD_DIR.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in SOURCES + [HERE / "cpu_ref.h"])
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < newest:
        tmp = LIB_PATH.with_suffix(f".so.{os.getpid()}")
        cmd = ["gcc", *CFLAGS, *map(str, SOURCES), "-o", str(tmp), "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Camera(ctypes.Structure):
    _fields_ = [
        ("projection", ctypes.c_float * 16),
        ("view", ctypes.c_float * 16),
        ("model", ctypes.c_float * 16),
        ("eye", ctypes.c_float * 3),
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        f32p = ctypes.POINTER(ctypes.c_float)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        u16p = ctypes.POINTER(ctypes.c_uint16)
        f64p = ctypes.POINTER(ctypes.c_double)
        camp = ctypes.POINTER(Camera)
        L.or_perspective_vk.argtypes = [ctypes.c_float] * 4 + [f32p]
        L.or_look_at.argtypes = [f32p, f32p, f32p, f32p]
        L.or_orbit_eye.argtypes = [f32p, ctypes.c_float, ctypes.c_float, ctypes.c_float, f32p]
        L.or_mat4_mul.argtypes = [f32p, f32p, f32p]
        L.or_f32_to_f16.argtypes = [ctypes.c_float]
        L.or_f32_to_f16.restype = ctypes.c_uint16
        L.or_f16_to_f32.argtypes = [ctypes.c_uint16]
        L.or_f16_to_f32.restype = ctypes.c_float
        L.or_parse_ply.argtypes = [f32p, ctypes.c_uint32, u32p, f32p, f32p, f32p, u16p]
        L.or_rank.argtypes = [f32p, ctypes.c_uint32, camp, u32p, u32p]
        L.or_rank.restype = ctypes.c_uint32
        L.or_sort_kv.argtypes = [u32p, u32p, ctypes.c_uint32]
        L.or_project.argtypes = [f32p, f32p, f32p, u16p, u32p, ctypes.c_uint32, camp, f32p, f32p]
        L.or_raster.argtypes = [f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, f32p, ctypes.c_int, f32p]
        L.or_raster.restype = ctypes.c_uint64
        L.or_raster_bands.argtypes = [f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, f32p, ctypes.c_int,
                                      ctypes.c_uint32, ctypes.c_uint32, f32p]
        L.or_raster_bands.restype = ctypes.c_uint64
        L.or_render_frame.argtypes = [f32p, f32p, f32p, u16p, ctypes.c_uint32, camp, f32p, ctypes.c_int, u32p, u32p,
                                      f32p, f32p, ctypes.POINTER(ctypes.c_uint64)]
        L.or_render_frame.restype = ctypes.c_uint32
        L.or_render_frame_f64.argtypes = [f32p, f32p, f32p, u16p, ctypes.c_uint32, camp, f64p]
        L.or_render_frame_f64.restype = ctypes.c_uint32
        L.or_num_threads.restype = ctypes.c_int
        L.or_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a: np.ndarray, ct):
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data_as(ctypes.POINTER(ct))


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def make_camera(projection, view, eye, width, height, model=None) -> Camera:
    cam = Camera()
    cam.projection[:] = [float(x) for x in np.asarray(projection, np.float32).reshape(-1)]
    cam.view[:] = [float(x) for x in np.asarray(view, np.float32).reshape(-1)]
    m = np.eye(4, dtype=np.float32).reshape(-1) if model is None else np.asarray(model, np.float32).reshape(-1)
    cam.model[:] = [float(x) for x in m]
    cam.eye[:] = [float(x) for x in np.asarray(eye, np.float32).reshape(-1)]
    cam.width = int(width)
    cam.height = int(height)
    return cam


def perspective_vk(fovy, aspect, znear, zfar) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().or_perspective_vk(fovy, aspect, znear, zfar, _p(out, ctypes.c_float))
    return out


def look_at(eye, center, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    out = np.zeros(16, np.float32)
    e, c, u = _f32(eye), _f32(center), _f32(up)
    lib().or_look_at(_p(e, ctypes.c_float), _p(c, ctypes.c_float), _p(u, ctypes.c_float), _p(out, ctypes.c_float))
    return out


def orbit_eye(center, r, phi, theta) -> np.ndarray:
    out = np.zeros(3, np.float32)
    c = _f32(center)
    lib().or_orbit_eye(_p(c, ctypes.c_float), r, phi, theta, _p(out, ctypes.c_float))
    return out


def mat4_mul(a, b) -> np.ndarray:
    out = np.zeros(16, np.float32)
    a, b = _f32(a).reshape(-1), _f32(b).reshape(-1)
    lib().or_mat4_mul(_p(a, ctypes.c_float), _p(b, ctypes.c_float), _p(out, ctypes.c_float))
    return out


def f32_to_f16_bits(x: np.ndarray) -> np.ndarray:
    L = lib()
    flat = _f32(x).reshape(-1)
    return np.array([L.or_f32_to_f16(float(v)) for v in flat], np.uint16).reshape(np.shape(x))


def parse_ply(rows: np.ndarray, offsets: np.ndarray):
    rows = _f32(rows)
    offsets = np.ascontiguousarray(offsets, np.uint32)
    n = rows.shape[0]
    pos = np.zeros((n, 3), np.float32)
    cov = np.zeros((n, 6), np.float32)
    opa = np.zeros(n, np.float32)
    sh = np.zeros((n, 48), np.uint16)
    lib().or_parse_ply(_p(rows, ctypes.c_float), n, _p(offsets, ctypes.c_uint32), _p(pos, ctypes.c_float),
                       _p(cov, ctypes.c_float), _p(opa, ctypes.c_float), _p(sh, ctypes.c_uint16))
    return pos, cov, opa, sh


def rank(position, cam: Camera):
    position = _f32(position)
    n = position.shape[0]
    key = np.zeros(max(n, 1), np.uint32)
    idx = np.zeros(max(n, 1), np.uint32)
    v = lib().or_rank(_p(position, ctypes.c_float), n, ctypes.byref(cam), _p(key, ctypes.c_uint32),
                      _p(idx, ctypes.c_uint32))
    return key[:v].copy(), idx[:v].copy()


def sort_kv(key, value):
    key = np.ascontiguousarray(key, np.uint32).copy()
    value = np.ascontiguousarray(value, np.uint32).copy()
    lib().or_sort_kv(_p(key, ctypes.c_uint32), _p(value, ctypes.c_uint32), key.shape[0])
    return key, value


def project(position, cov3d, opacity, sh, sorted_index, cam: Camera):
    position, cov3d, opacity = _f32(position), _f32(cov3d), _f32(opacity)
    sh = np.ascontiguousarray(sh, np.uint16)
    sorted_index = np.ascontiguousarray(sorted_index, np.uint32)
    v = sorted_index.shape[0]
    inst = np.zeros((max(v, 1), 12), np.float32)
    rec = np.zeros((max(v, 1), 16), np.float32)
    lib().or_project(_p(position, ctypes.c_float), _p(cov3d, ctypes.c_float), _p(opacity, ctypes.c_float),
                     _p(sh, ctypes.c_uint16), _p(sorted_index, ctypes.c_uint32), v, ctypes.byref(cam),
                     _p(inst, ctypes.c_float), _p(rec, ctypes.c_float))
    return inst[:v], rec[:v]


def raster(record, width, height, depth_in=None, unorm8=False):
    record = _f32(record)
    img = np.zeros((height, width, 4), np.float32)
    d = None if depth_in is None else _f32(depth_in)
    f = lib().or_raster(_p(record, ctypes.c_float), record.shape[0], width, height,
                        None if d is None else _p(d, ctypes.c_float), int(bool(unorm8)), _p(img, ctypes.c_float))
    return img, int(f)


def raster_bands(record, width, height, band_stride, band_offset=0):
    """Blend only every band_stride-th 16-row band (a bounded timing sample); returns (image, fragments)."""
    record = _f32(record)
    img = np.zeros((height, width, 4), np.float32)
    f = lib().or_raster_bands(_p(record, ctypes.c_float), record.shape[0], width, height, None, 0,
                              int(band_stride), int(band_offset), _p(img, ctypes.c_float))
    return img, int(f)


def render_frame(position, cov3d, opacity, sh, cam: Camera, depth_in=None, unorm8=False, want_instances=True):
    """FP32 transcription of the whole frame.  Returns a dict with count, key, index, instance, image, fragments."""
    position, cov3d, opacity = _f32(position), _f32(cov3d), _f32(opacity)
    sh = np.ascontiguousarray(sh, np.uint16)
    n = position.shape[0]
    key = np.zeros(max(n, 1), np.uint32)
    idx = np.zeros(max(n, 1), np.uint32)
    inst = np.zeros((max(n, 1), 12), np.float32) if want_instances else None
    img = np.zeros((cam.height, cam.width, 4), np.float32)
    frag = ctypes.c_uint64(0)
    d = None if depth_in is None else _f32(depth_in)
    v = lib().or_render_frame(_p(position, ctypes.c_float), _p(cov3d, ctypes.c_float), _p(opacity, ctypes.c_float),
                              _p(sh, ctypes.c_uint16), n, ctypes.byref(cam),
                              None if d is None else _p(d, ctypes.c_float), int(bool(unorm8)),
                              _p(key, ctypes.c_uint32), _p(idx, ctypes.c_uint32),
                              None if inst is None else _p(inst, ctypes.c_float), _p(img, ctypes.c_float),
                              ctypes.byref(frag))
    return {
        "count": int(v),
        "key": key[:v].copy(),
        "index": idx[:v].copy(),
        "instance": None if inst is None else inst[:v].copy(),
        "image": img,
        "fragments": int(frag.value),
    }


def render_frame_f64(position, cov3d, opacity, sh, cam: Camera):
    position, cov3d, opacity = _f32(position), _f32(cov3d), _f32(opacity)
    sh = np.ascontiguousarray(sh, np.uint16)
    img = np.zeros((cam.height, cam.width, 4), np.float64)
    v = lib().or_render_frame_f64(_p(position, ctypes.c_float), _p(cov3d, ctypes.c_float),
                                  _p(opacity, ctypes.c_float), _p(sh, ctypes.c_uint16), position.shape[0],
                                  ctypes.byref(cam), _p(img, ctypes.c_double))
    return int(v), img


def num_threads() -> int:
    return int(lib().or_num_threads())


def set_num_threads(n: int) -> None:
    lib().or_set_num_threads(int(n))
