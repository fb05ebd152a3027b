"""ctypes binding of the C ABI declared in include/vkgs_gb300.h.

The shared library is built in-tree by ``vkgs_gb300.build`` (``vkgs_gb300/_lib/libvkgs_gb300.so``).
There is no fallback: if the library is missing, loading raises.
"""

from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_float, c_int, c_size_t, c_uint16, c_uint32, c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libvkgs_gb300.so"

GS_SUCCESS = 0
GS_ERROR_INVALID_ARGUMENT = 1
GS_ERROR_CAPACITY = 2
GS_ERROR_CUDA = 3
GS_ERROR_DEVICE_TIMEOUT = 4
GS_ERROR_OUT_OF_MEMORY = 5
GS_ERROR_INTERNAL = 6
GS_NUM_STAGES = 6
GS_SORT_NOALLOC_MAX_COUNT = 1 << 20  # include/vkgs_gb300.h
GS_MAX_SLABS = 4
GS_MAX_LANES = 32
GS_MAX_FRAMES_IN_FLIGHT = 8
STAGES = ("cull_project", "depth_sort", "bin", "emit", "tile_sort", "raster")


class GsSplats(ctypes.Structure):
    _fields_ = [("position", c_void_p), ("cov3d", c_void_p), ("opacity", c_void_p), ("sh", c_void_p),
                ("count", c_uint32)]


class GsSplatBuffers(ctypes.Structure):
    _fields_ = [("position", c_void_p), ("cov3d", c_void_p), ("opacity", c_void_p), ("sh", c_void_p)]


class GsCamera(ctypes.Structure):
    _fields_ = [("projection", c_float * 16), ("view", c_float * 16), ("camera_position", c_float * 3),
                ("width", c_uint32), ("height", c_uint32), ("model", c_float * 16)]


class GsTarget(ctypes.Structure):
    _fields_ = [("color_rgba32f", c_void_p), ("color_bgra8", c_void_p), ("depth", c_void_p)]


class GsFrameOutputs(ctypes.Structure):
    _fields_ = [("visible_count", c_void_p), ("keys", c_void_p), ("index", c_void_p), ("instances", c_void_p),
                ("draw_indirect", c_void_p)]


class GsContextOptions(ctypes.Structure):
    _fields_ = [("max_splats", c_uint32), ("max_width", c_uint32), ("max_height", c_uint32),
                ("max_tile_pairs", c_uint32)]


class GsFrameStats(ctypes.Structure):
    _fields_ = [("visible_count", c_uint32), ("tile_pairs", c_uint32), ("fragments", c_uint64),
                ("fragments_blended", c_uint64), ("pairs_emitted", c_uint64)]


class GsTrainParams(ctypes.Structure):
    _fields_ = [("means", c_void_p), ("log_scales", c_void_p), ("quats", c_void_p), ("opacity_logits", c_void_p),
                ("sh", c_void_p), ("count", c_uint32)]


class GsTrainGrads(ctypes.Structure):
    _fields_ = [("means", c_void_p), ("log_scales", c_void_p), ("quats", c_void_p), ("opacity_logits", c_void_p),
                ("sh", c_void_p)]


# (name, restype, argtypes) for every entry point of include/vkgs_gb300.h
SIGNATURES = [
    ("gs_status_string", c_char_p, [c_int]),
    ("gs_version", c_uint32, []),
    ("gs_sorter_create", c_int, [POINTER(c_void_p)]),
    ("gs_sorter_destroy", None, [c_void_p]),
    ("gs_sorter_key_value_storage_requirements", c_int, [c_void_p, c_uint32, POINTER(c_size_t)]),
    ("gs_sorter_sort_key_value_indirect", c_int,
     [c_void_p, c_void_p, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t]),
    ("gs_sorter_check", c_int, [c_void_p, c_void_p]),
    ("gs_sort_key_value_noalloc", c_int, [c_void_p, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("gs_context_create", c_int, [POINTER(c_void_p), POINTER(GsContextOptions)]),
    ("gs_context_destroy", None, [c_void_p]),
    ("gs_context_reserve", c_int, [c_void_p, POINTER(GsContextOptions)]),
    ("gs_context_set_count_fragments", c_int, [c_void_p, c_int]),
    ("gs_context_scratch_bytes", c_int, [POINTER(GsContextOptions), POINTER(c_size_t)]),
    ("gs_context_set_slabs", c_int, [c_void_p, c_uint32, POINTER(c_uint32)]),
    ("gs_context_set_transmittance_floor", c_int, [c_void_p, c_float]),
    ("gs_context_set_batch_lanes", c_int, [c_void_p, c_uint32]),
    ("gs_viewer_create", c_int, [POINTER(c_void_p), c_void_p, POINTER(GsSplats), POINTER(GsCamera), POINTER(GsTarget)]),
    ("gs_viewer_frame", c_int, [c_void_p, POINTER(GsCamera), c_void_p]),
    ("gs_viewer_destroy", None, [c_void_p]),
    ("gs_viewer_create_frames", c_int,
     [POINTER(c_void_p), c_void_p, POINTER(GsSplats), POINTER(GsCamera), POINTER(GsTarget), c_uint32]),
    ("gs_viewer_submit", c_int, [c_void_p, POINTER(GsCamera), c_void_p, POINTER(c_uint32)]),
    ("gs_viewer_wait", c_int, [c_void_p, c_uint32, c_void_p]),
    ("gs_viewer_check", c_int, [c_void_p, c_void_p]),
    ("gs_context_set_batch_shared_cull", c_int, [c_void_p, c_int]),
    ("gs_context_set_cull_staging", c_int, [c_void_p, c_int]),
    ("gs_context_set_lean", c_int, [c_void_p, c_int]),
    ("gs_render_batched", c_int,
     [c_void_p, POINTER(GsSplats), c_uint32, POINTER(GsCamera), POINTER(GsTarget), c_void_p]),
    ("gs_render", c_int,
     [c_void_p, POINTER(GsSplats), POINTER(GsCamera), POINTER(GsTarget), POINTER(GsFrameOutputs), c_void_p]),
    ("gs_context_check", c_int, [c_void_p, c_void_p, POINTER(GsFrameStats)]),
    ("gs_selftest_bounded_wait", c_int, [c_void_p]),
    ("gs_context_set_train_slab_min", c_int, [c_void_p, c_uint32]),
    ("gs_train_forward", c_int, [c_void_p, POINTER(GsTrainParams), POINTER(GsCamera), c_void_p, c_void_p]),
    ("gs_train_backward", c_int,
     [c_void_p, POINTER(GsTrainParams), POINTER(GsCamera), c_void_p, POINTER(GsTrainGrads), c_void_p]),
    ("gs_train_forward_batched", c_int,
     [c_void_p, POINTER(GsTrainParams), c_uint32, POINTER(GsCamera), POINTER(c_void_p), c_void_p]),
    ("gs_train_backward_batched", c_int,
     [c_void_p, POINTER(GsTrainParams), c_uint32, POINTER(GsCamera), POINTER(c_void_p), POINTER(GsTrainGrads),
      c_void_p]),
    ("gs_context_enable_timing", c_int, [c_void_p, c_int]),
    ("gs_context_stage_times", c_int, [c_void_p, c_uint32, POINTER(c_float), POINTER(c_uint32)]),
    ("gs_ply_offsets_from_header", c_int,
     [c_char_p, c_size_t, POINTER(c_uint32), POINTER(c_uint64), POINTER(c_size_t)]),
    ("gs_parse_ply", c_int, [c_void_p, c_uint32, POINTER(c_uint32), POINTER(GsSplatBuffers), c_void_p]),
    ("gs_camera_perspective", None, [c_float, c_float, c_float, c_float, POINTER(c_float)]),
    ("gs_camera_look_at", None, [POINTER(c_float), POINTER(c_float), POINTER(c_float), POINTER(c_float)]),
    ("gs_camera_orbit_eye", None, [POINTER(c_float), c_float, c_float, c_float, POINTER(c_float)]),
]

_lib = None


def load(path: Path | None = None) -> ctypes.CDLL:
    """Loads (once) and returns the library; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with `python -m vkgs_gb300.build` (nvcc, sm_103a)")
    lib = ctypes.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def status_string(code: int) -> str:
    return load().gs_status_string(int(code)).decode()


def floats(values, n):
    arr = (c_float * n)()
    for i, v in enumerate(values):
        arr[i] = float(v)
    return arr


__all__ = ["load", "LIB_PATH", "SIGNATURES", "GsSplats", "GsSplatBuffers", "GsCamera", "GsTarget", "GsFrameOutputs",
           "GsContextOptions", "GsFrameStats", "GsTrainParams", "GsTrainGrads", "status_string", "floats", "c_uint16"]
