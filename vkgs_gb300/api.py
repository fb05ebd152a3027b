"""PyTorch-facing front end of the C ABI.

PyTorch supplies device memory and streams only; every computation runs in the CUDA kernels of
``libvkgs_gb300.so``.  Names follow the reference: ``load`` mirrors pygs.load
(binding/python/pygs/__init__.py:18-25), ``Renderer.render`` is one Engine::Impl::Draw frame
(src/vkgs/engine/engine.cc:742-1378) drawn into tensors instead of a swapchain image, ``Sorter``
is the vulkan_radix_sort handle (engine.cc:509-521, 1218-1219) and ``Camera`` carries the Camera
uniform + model push constant (src/vkgs/vulkan/shader/uniforms.h:10-15).
"""

from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L


class GsError(RuntimeError):
    """A non-success gs_status from the library."""

    def __init__(self, status: int, what: str):
        self.status = int(status)
        super().__init__(f"{what}: {L.status_string(status)} (gs_status {status})")


def _check(status: int, what: str) -> None:
    if status != L.GS_SUCCESS:
        raise GsError(status, what)


def _ptr(t: torch.Tensor | None):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(stream) -> ctypes.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


def _need_cuda(t: torch.Tensor, name: str, dtype, shape_tail=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if shape_tail is not None and tuple(t.shape[1:]) != tuple(shape_tail):
        raise ValueError(f"{name} must have shape (N, {', '.join(map(str, shape_tail))}), got {tuple(t.shape)}")


# ----------------------------------------------------------------------------------------- splats

@dataclass
class Splats:
    """The reference's SoA splat storage (engine.cc:1639-1651) as CUDA tensors."""

    position: torch.Tensor  # (N, 3) float32
    cov3d: torch.Tensor     # (N, 6) float32
    opacity: torch.Tensor   # (N,)   float32
    sh: torch.Tensor        # (N, 48) float16, [channel][coefficient]

    @property
    def count(self) -> int:
        return int(self.position.shape[0])

    def validate(self) -> None:
        n = self.count
        _need_cuda(self.position, "position", torch.float32, (3,))
        _need_cuda(self.cov3d, "cov3d", torch.float32, (6,))
        _need_cuda(self.opacity, "opacity", torch.float32)
        _need_cuda(self.sh, "sh", torch.float16, (48,))
        if self.cov3d.shape[0] != n or self.opacity.shape != (n,) or self.sh.shape[0] != n:
            raise ValueError("splat buffers disagree on N")

    def struct(self) -> L.GsSplats:
        self.validate()
        return L.GsSplats(self.position.data_ptr(), self.cov3d.data_ptr(), self.opacity.data_ptr(),
                          self.sh.data_ptr(), self.count)

    @staticmethod
    def empty(n: int, device="cuda") -> "Splats":
        return Splats(torch.empty((n, 3), dtype=torch.float32, device=device),
                      torch.empty((n, 6), dtype=torch.float32, device=device),
                      torch.empty((n,), dtype=torch.float32, device=device),
                      torch.empty((n, 48), dtype=torch.float16, device=device))

    @staticmethod
    def from_numpy(position, cov3d, opacity, sh_bits, device="cuda") -> "Splats":
        """sh_bits: (N, 48) uint16 binary16 bit patterns."""
        return Splats(torch.from_numpy(np.ascontiguousarray(position, np.float32)).to(device),
                      torch.from_numpy(np.ascontiguousarray(cov3d, np.float32)).to(device),
                      torch.from_numpy(np.ascontiguousarray(opacity, np.float32)).to(device),
                      torch.from_numpy(np.ascontiguousarray(sh_bits, np.uint16).view(np.float16)).to(device))


# ----------------------------------------------------------------------------------------- camera

def perspective(fovy: float, aspect: float, znear: float, zfar: float) -> np.ndarray:
    """Camera::ProjectionMatrix (camera.cc:25-35): glm::perspective then the Vulkan conversion."""
    out = (ctypes.c_float * 16)()
    L.load().gs_camera_perspective(fovy, aspect, znear, zfar, out)
    return np.frombuffer(out, np.float32).copy()


def look_at(eye, center=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Camera::ViewMatrix (camera.cc:37): glm::lookAt, right-handed."""
    out = (ctypes.c_float * 16)()
    L.load().gs_camera_look_at(L.floats(eye, 3), L.floats(center, 3), L.floats(up, 3), out)
    return np.frombuffer(out, np.float32).copy()


def orbit_eye(center, r: float, phi: float, theta: float) -> np.ndarray:
    """Camera::Eye (camera.cc:39-45)."""
    out = (ctypes.c_float * 3)()
    L.load().gs_camera_orbit_eye(L.floats(center, 3), r, phi, theta, out)
    return np.frombuffer(out, np.float32).copy()


@dataclass
class Camera:
    """The Camera uniform (projection, view, camera_position, screen_size) + the model matrix."""

    projection: np.ndarray
    view: np.ndarray
    eye: np.ndarray
    width: int
    height: int
    model: np.ndarray | None = None

    @staticmethod
    def look_at(eye, center=(0.0, 0.0, 0.0), *, fovy_deg: float = 60.0, width: int = 1600, height: int = 900,
                near: float = 0.01, far: float = 100.0, up=(0.0, 1.0, 0.0), model=None) -> "Camera":
        proj = perspective(math.radians(fovy_deg), np.float32(width) / np.float32(height), near, far)
        return Camera(proj, look_at(eye, center, up), np.asarray(eye, np.float32), int(width), int(height), model)

    @staticmethod
    def from_spec(spec) -> "Camera":
        return Camera.look_at(spec.eye, spec.center, fovy_deg=spec.fovy_deg, width=spec.width, height=spec.height,
                              near=spec.near, far=spec.far)

    def struct(self) -> L.GsCamera:
        c = L.GsCamera()
        c.projection[:] = [float(x) for x in np.asarray(self.projection, np.float32).reshape(-1)]
        c.view[:] = [float(x) for x in np.asarray(self.view, np.float32).reshape(-1)]
        c.camera_position[:] = [float(x) for x in np.asarray(self.eye, np.float32).reshape(-1)]
        c.width = int(self.width)
        c.height = int(self.height)
        m = np.eye(4, dtype=np.float32) if self.model is None else np.asarray(self.model, np.float32)
        c.model[:] = [float(x) for x in m.reshape(-1)]
        return c


# ----------------------------------------------------------------------------------------- renderer

def scratch_bytes(max_splats: int, max_width: int, max_height: int, max_tile_pairs: int = 0) -> int:
    """Device bytes a Renderer with these capacities allocates (gs_context_scratch_bytes; no device needed)."""
    opts = L.GsContextOptions(int(max_splats), int(max_width), int(max_height), int(max_tile_pairs))
    b = ctypes.c_size_t()
    _check(L.load().gs_context_scratch_bytes(ctypes.byref(opts), ctypes.byref(b)), "gs_context_scratch_bytes")
    return int(b.value)


class Renderer:
    """A render context (gs_context): reserved scratch for up to max_splats at max_width x max_height."""

    def __init__(self, max_splats: int, max_width: int, max_height: int, max_tile_pairs: int = 0):
        self._lib = L.load()
        opts = L.GsContextOptions(int(max_splats), int(max_width), int(max_height), int(max_tile_pairs))
        h = ctypes.c_void_p()
        _check(self._lib.gs_context_create(ctypes.byref(h), ctypes.byref(opts)), "gs_context_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.gs_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reserve(self, max_splats=0, max_width=0, max_height=0, max_tile_pairs=0) -> None:
        opts = L.GsContextOptions(int(max_splats), int(max_width), int(max_height), int(max_tile_pairs))
        _check(self._lib.gs_context_reserve(self._h, ctypes.byref(opts)), "gs_context_reserve")

    def set_slabs(self, ends=(1024,)) -> None:
        """Depth-slab schedule: cumulative shares of the visible splats (1/1024 units), nearest first,
        ending at 1024.  (1024,) bins and sorts every splat in one pass."""
        ends = [int(e) for e in ends]
        arr = (ctypes.c_uint32 * len(ends))(*ends)
        _check(self._lib.gs_context_set_slabs(self._h, len(ends), arr), "gs_context_set_slabs")

    def set_transmittance_floor(self, t_floor: float = 1e-4) -> None:
        """Early stop: a pixel stops blending once its transmittance is below t_floor (image error < t_floor)."""
        _check(self._lib.gs_context_set_transmittance_floor(self._h, float(t_floor)),
               "gs_context_set_transmittance_floor")

    def set_train_slab_min(self, splats: int = 1 << 20) -> None:
        """Splat count from which the differentiable forward uses the depth-slab schedule."""
        _check(self._lib.gs_context_set_train_slab_min(self._h, int(splats)), "set_train_slab_min")

    def count_fragments(self, enable: bool = True) -> None:
        _check(self._lib.gs_context_set_count_fragments(self._h, int(bool(enable))), "count_fragments")

    def render(self, splats: Splats, camera: Camera, *, color: torch.Tensor | None = None,
               bgra8: torch.Tensor | None = None, depth: torch.Tensor | None = None,
               keys: torch.Tensor | None = None, index: torch.Tensor | None = None,
               instances: torch.Tensor | None = None, draw_indirect: torch.Tensor | None = None,
               visible_count: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """Renders one frame; returns the RGBA float32 image (H, W, 4) (or bgra8 if only that was given)."""
        dev = splats.position.device
        H, W = int(camera.height), int(camera.width)
        if color is None and bgra8 is None:
            color = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
        if color is not None:
            _need_cuda(color, "color", torch.float32)
            if tuple(color.shape) != (H, W, 4):
                raise ValueError("color must be (H, W, 4)")
        if bgra8 is not None:
            _need_cuda(bgra8, "bgra8", torch.uint8)
            if tuple(bgra8.shape) != (H, W, 4):
                raise ValueError("bgra8 must be (H, W, 4)")
        if depth is not None:
            _need_cuda(depth, "depth", torch.float32)
            if tuple(depth.shape) != (H, W):
                raise ValueError("depth must be (H, W)")
        n = splats.count
        for t, name, dt, size in ((keys, "keys", torch.int32, n), (index, "index", torch.int32, n),
                                  (instances, "instances", torch.float32, n * 12),
                                  (draw_indirect, "draw_indirect", torch.int32, 12),
                                  (visible_count, "visible_count", torch.int32, 1)):
            if t is not None:
                _need_cuda(t, name, dt)
                if t.numel() < size:
                    raise ValueError(f"{name} holds {t.numel()} elements, needs {size}")
        target = L.GsTarget(_ptr(color), _ptr(bgra8), _ptr(depth))
        outs = L.GsFrameOutputs(_ptr(visible_count), _ptr(keys), _ptr(index), _ptr(instances), _ptr(draw_indirect))
        s = splats.struct()
        cam = camera.struct()
        _check(self._lib.gs_render(self._h, ctypes.byref(s), ctypes.byref(cam), ctypes.byref(target),
                                   ctypes.byref(outs), _stream(stream)), "gs_render")
        return color if color is not None else bgra8

    def set_batch_lanes(self, lanes: int) -> None:
        """Render lanes for render_batched (sub-contexts with their own scratch and stream; 0 = none)."""
        _check(self._lib.gs_context_set_batch_lanes(self._h, int(lanes)), "gs_context_set_batch_lanes")
        self._lanes = int(lanes)

    def set_cull_staging(self, enable: bool = True) -> None:
        """Plain path: stream the cull's splat partitions into shared memory with bulk copies (faster
        alone, slower with frames in flight; same results)."""
        _check(self._lib.gs_context_set_cull_staging(self._h, int(bool(enable))), "gs_context_set_cull_staging")

    def set_lean(self, enable: bool = True) -> None:
        """Launch shapes for frames that run beside other work on the GPU (fewer SM slots per kernel,
        the two-pixels-per-thread raster): slower alone, more frames per second when several contexts
        render at once; same results.  Viewer slots (frames in flight) and render lanes always are."""
        _check(self._lib.gs_context_set_lean(self._h, int(bool(enable))), "gs_context_set_lean")

    def set_batch_shared_cull(self, enable: bool = True) -> None:
        """Batched form: one cull + projection pass for all views (default) or one per lane."""
        _check(self._lib.gs_context_set_batch_shared_cull(self._h, int(bool(enable))), "set_batch_shared_cull")

    @property
    def batch_lanes(self) -> int:
        return getattr(self, "_lanes", 0)

    def render_batched(self, splats: Splats, cameras, colors, stream=None):
        """Renders every camera into its own RGBA float32 target (H_v, W_v, 4) in one call (gs_render_batched)."""
        n = len(cameras)
        if len(colors) != n:
            raise ValueError("one colour target per camera")
        cams = (L.GsCamera * max(n, 1))()
        targets = (L.GsTarget * max(n, 1))()
        for v, (cam, col) in enumerate(zip(cameras, colors)):
            _need_cuda(col, "colors[%d]" % v, torch.float32)
            if tuple(col.shape) != (int(cam.height), int(cam.width), 4):
                raise ValueError(f"colors[{v}] must be ({cam.height}, {cam.width}, 4)")
            cams[v] = cam.struct()
            targets[v] = L.GsTarget(_ptr(col), None, None)
        s = splats.struct()
        _check(self._lib.gs_render_batched(self._h, ctypes.byref(s), n, cams, targets, _stream(stream)),
               "gs_render_batched")
        return colors

    def render_batched_checked(self, splats: Splats, cameras, colors, stream=None):
        """render_batched + check; grows the tile-pair capacity and re-renders once if it overflowed."""
        self.render_batched(splats, cameras, colors, stream)
        try:
            return self.check(stream)
        except GsError as e:
            if e.status != L.GS_ERROR_CAPACITY or not hasattr(e, "stats"):
                raise
            self.reserve(max_tile_pairs=int(e.stats["tile_pairs"] * 1.25) + 1024)
            self.render_batched(splats, cameras, colors, stream)
            return self.check(stream)

    def enable_timing(self, enable: bool = True) -> None:
        """Records CUDA events around each stage of every following frame (last 256 frames kept)."""
        _check(self._lib.gs_context_enable_timing(self._h, int(bool(enable))), "gs_context_enable_timing")

    def stage_times(self, max_frames: int = 256) -> np.ndarray:
        """(frames, 6) milliseconds per stage (L.STAGES order) of the timed frames; clears the record."""
        buf = (ctypes.c_float * (max_frames * L.GS_NUM_STAGES))()
        got = ctypes.c_uint32()
        _check(self._lib.gs_context_stage_times(self._h, max_frames, buf, ctypes.byref(got)), "stage_times")
        return np.frombuffer(buf, np.float32)[: got.value * L.GS_NUM_STAGES].reshape(-1, L.GS_NUM_STAGES).copy()

    def check(self, stream=None) -> dict:
        """Synchronises and returns {visible_count, tile_pairs, fragments, fragments_blended, pairs_emitted}
        of the last frame; raises GsError on device errors."""
        st = L.GsFrameStats()
        status = self._lib.gs_context_check(self._h, _stream(stream), ctypes.byref(st))
        stats = {"visible_count": int(st.visible_count), "tile_pairs": int(st.tile_pairs),
                 "fragments": int(st.fragments), "fragments_blended": int(st.fragments_blended),
                 "pairs_emitted": int(st.pairs_emitted)}
        if status != L.GS_SUCCESS:
            err = GsError(status, "gs_context_check")
            err.stats = stats
            raise err
        return stats

    def render_checked(self, splats: Splats, camera: Camera, **kw) -> tuple[torch.Tensor, dict]:
        """render + check; grows the tile-pair capacity and re-renders once if it overflowed."""
        img = self.render(splats, camera, **kw)
        try:
            return img, self.check(kw.get("stream"))
        except GsError as e:
            if e.status != L.GS_ERROR_CAPACITY or not hasattr(e, "stats"):
                raise
            need = e.stats["tile_pairs"]
            self.reserve(max_tile_pairs=int(need * 1.25) + 1024)
            img = self.render(splats, camera, **kw)
            return img, self.check(kw.get("stream"))


# ----------------------------------------------------------------------------------------- viewer loop

class Viewer:
    """The viewer's per-frame loop as a CUDA graph (gs_viewer_*): one captured frame of `renderer` drawing
    `splats` into `color`; frame(camera) updates the camera inside the graph and launches it.  The
    renderer must not render anything else while the viewer exists.

    frames_in_flight > 1 (the reference viewer keeps two): one captured frame per slot, each with its own
    scratch, stream and target (`color` may then be a list of targets, else they are allocated);
    submit(camera) starts the next frame without waiting for the previous ones and returns its slot,
    wait(slot) orders the current stream after that slot's latest frame, check() after all of them."""

    def __init__(self, renderer: Renderer, splats: Splats, camera: Camera, color, frames_in_flight: int = 1):
        n = int(frames_in_flight)
        shape = (int(camera.height), int(camera.width), 4)
        if isinstance(color, (list, tuple)):
            colors = list(color)
        else:
            colors = [color] + [torch.empty_like(color) for _ in range(n - 1)]
        if len(colors) != n:
            raise ValueError("one colour target per frame in flight")
        for c in colors:
            _need_cuda(c, "color", torch.float32)
            if tuple(c.shape) != shape:
                raise ValueError("color must be (H, W, 4)")
        self._lib = renderer._lib
        self.renderer, self.splats, self.colors = renderer, splats, colors  # keep the buffers alive
        self.color = colors[0]
        self._s = splats.struct()
        cam = camera.struct()
        targets = (L.GsTarget * n)(*[L.GsTarget(_ptr(c), None, None) for c in colors])
        h = ctypes.c_void_p()
        _check(self._lib.gs_viewer_create_frames(ctypes.byref(h), renderer._h, ctypes.byref(self._s),
                                                 ctypes.byref(cam), targets, n), "gs_viewer_create_frames")
        self._h = h
        self._next = 0

    def frame(self, camera: Camera, stream=None) -> torch.Tensor:
        """Renders the next frame, ordered on `stream`; returns its target."""
        slot = self.submit(camera, stream)
        self.wait(slot, stream)
        return self.colors[slot]

    def submit(self, camera: Camera, stream=None) -> int:
        cam = camera.struct()
        slot = ctypes.c_uint32()
        _check(self._lib.gs_viewer_submit(self._h, ctypes.byref(cam), _stream(stream), ctypes.byref(slot)),
               "gs_viewer_submit")
        self._next = (int(slot.value) + 1) % len(self.colors)
        return int(slot.value)

    @property
    def next_slot(self) -> int:
        """The slot the next submit will use (slots are used in turn)."""
        return self._next

    def wait(self, slot: int, stream=None) -> None:
        _check(self._lib.gs_viewer_wait(self._h, int(slot), _stream(stream)), "gs_viewer_wait")

    def check(self, stream=None) -> None:
        _check(self._lib.gs_viewer_check(self._h, _stream(stream)), "gs_viewer_check")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.gs_viewer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------------------------------- sorter

class Sorter:
    """vulkan_radix_sort's key/value sorter: ascending 32-bit keys, stable, count read on the device."""

    def __init__(self):
        self._lib = L.load()
        h = ctypes.c_void_p()
        _check(self._lib.gs_sorter_create(ctypes.byref(h)), "gs_sorter_create")
        self._h = h
        self._storage = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gs_sorter_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def storage_requirements(self, max_count: int) -> int:
        b = ctypes.c_size_t()
        _check(self._lib.gs_sorter_key_value_storage_requirements(self._h, int(max_count), ctypes.byref(b)),
               "storage requirements")
        return int(b.value)

    def sort_key_value(self, keys: torch.Tensor, values: torch.Tensor, count: torch.Tensor | int | None = None,
                       storage: torch.Tensor | None = None, stream=None) -> None:
        """Sorts keys[0:count] (int32 tensors holding uint32 bit patterns) in place, values alongside."""
        _need_cuda(keys, "keys", torch.int32)
        _need_cuda(values, "values", torch.int32)
        max_count = int(keys.numel())
        if values.numel() < max_count:
            raise ValueError("values shorter than keys")
        if count is None or isinstance(count, int):
            c = torch.tensor([max_count if count is None else int(count)], dtype=torch.int32, device=keys.device)
        else:
            _need_cuda(count, "count", torch.int32)
            c = count
        need = self.storage_requirements(max_count)
        if storage is None:
            if self._storage is None or self._storage.numel() < need:
                self._storage = torch.empty(need, dtype=torch.uint8, device=keys.device)
            storage = self._storage
        _check(self._lib.gs_sorter_sort_key_value_indirect(self._h, _stream(stream), max_count, _ptr(c), _ptr(keys),
                                                           _ptr(values), _ptr(storage), storage.numel()),
               "gs_sorter_sort_key_value_indirect")

    def check(self, stream=None) -> None:
        _check(self._lib.gs_sorter_check(self._h, _stream(stream)), "gs_sorter_check")


# ----------------------------------------------------------------------------------------- loader

def ply_header(data: bytes):
    """(offsets[60] uint32, point_count, header_bytes) from the start of a binary little-endian PLY."""
    end = data.find(b"end_header")
    if end < 0:
        raise ValueError("no end_header in PLY data")
    nl = data.find(b"\n", end)
    head = data[: (nl + 1) if nl >= 0 else len(data)]
    off = (ctypes.c_uint32 * 60)()
    cnt = ctypes.c_uint64()
    hb = ctypes.c_size_t()
    _check(L.load().gs_ply_offsets_from_header(head, len(head), off, ctypes.byref(cnt), ctypes.byref(hb)),
           "gs_ply_offsets_from_header")
    return np.frombuffer(off, np.uint32).copy(), int(cnt.value), int(hb.value)


def parse_ply(rows: torch.Tensor, offsets, stream=None) -> Splats:
    """parse_ply.comp on the GPU: rows (N, stride) float32 CUDA tensor -> activated Splats."""
    _need_cuda(rows, "rows", torch.float32)
    offsets = np.ascontiguousarray(offsets, np.uint32)
    if offsets.shape != (60,) or rows.ndim != 2 or rows.shape[1] != int(offsets[59]):
        raise ValueError("rows must be (N, offsets[59]) and offsets 60 words")
    n = int(rows.shape[0])
    out = Splats.empty(n, rows.device)
    buf = L.GsSplatBuffers(out.position.data_ptr(), out.cov3d.data_ptr(), out.opacity.data_ptr(), out.sh.data_ptr())
    off = (ctypes.c_uint32 * 60)(*[int(x) for x in offsets])
    _check(L.load().gs_parse_ply(_ptr(rows), n, off, ctypes.byref(buf), _stream(stream)), "gs_parse_ply")
    return out


def write_ply(path, rows: np.ndarray, properties) -> None:
    """Writes float32 rows as a binary little-endian PLY vertex element (the 3DGS file format)."""
    rows = np.ascontiguousarray(rows, np.float32)
    if rows.shape[1] != len(properties):
        raise ValueError("one property per column")
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {rows.shape[0]}"]
    head += [f"property float {p}" for p in properties]
    head.append("end_header")
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        f.write(rows.astype("<f4").tobytes())


def load(path, device="cuda", stream=None) -> Splats:
    """pygs.load: reads a 3DGS .ply file and activates it on the GPU (SplatLoadThread + parse_ply.comp)."""
    path = os.path.abspath(path)
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    with open(path, "rb") as f:
        head = f.read(1 << 16)
        offsets, count, hb = ply_header(head)
        stride = int(offsets[59])
        f.seek(hb)
        raw = np.fromfile(f, dtype="<f4", count=count * stride)
    if raw.size != count * stride:
        raise ValueError(f"{path}: truncated vertex data")
    host = torch.from_numpy(raw.reshape(count, stride))
    rows = host.pin_memory().to(device, non_blocking=True) if torch.cuda.is_available() else host.to(device)
    return parse_ply(rows, offsets, stream=stream)
