"""GB300 (sm_103a) CUDA implementation of the vkgs per-frame splat pipeline.

The compute lives in ``libvkgs_gb300.so`` (C ABI: ``include/vkgs_gb300.h``); this package binds it
for PyTorch callers.  See ``vkgs_gb300.api`` for the tensor-level calls.
"""

from .api import (Camera, GsError, Renderer, Sorter, Splats, Viewer, load, look_at, orbit_eye, parse_ply,
                  perspective, ply_header, scratch_bytes, write_ply)

__all__ = ["Camera", "GsError", "Renderer", "Sorter", "Splats", "Viewer", "load", "look_at", "orbit_eye",
           "parse_ply", "perspective", "ply_header", "scratch_bytes", "write_ply"]
