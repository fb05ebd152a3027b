"""CPU tests of the C ABI: the library loads, exports every declared entry point, validates its
arguments before touching the GPU, and its host-side helpers (camera, PLY header) agree with the
oracle / the reference loader's offset table."""

import ctypes
import math
import re
from pathlib import Path

import numpy as np
import pytest

from vkgs_gb300 import _lib as L
from vkgs_gb300 import build as B
from vkgs_gb300 import synthetic as syn

HEADER = Path(__file__).resolve().parents[1] / "include" / "vkgs_gb300.h"


@pytest.fixture(scope="module")
def lib():
    B.build()
    return L.load()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z_][\w \*]*?\b(gs_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_bound_entry_points():
    names = declared_functions()
    assert len(names) >= 18
    assert sorted(n for n, _, _ in L.SIGNATURES) == names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_status_strings(lib):
    for code in range(7):
        assert lib.gs_status_string(code) != b"unknown status"
    assert lib.gs_version() >= 10000


def test_null_arguments_are_rejected_without_a_device(lib):
    assert lib.gs_context_create(None, None) == L.GS_ERROR_INVALID_ARGUMENT
    h = ctypes.c_void_p()
    assert lib.gs_context_create(ctypes.byref(h), None) == L.GS_ERROR_INVALID_ARGUMENT
    zero = L.GsContextOptions(10, 0, 0, 0)
    assert lib.gs_context_create(ctypes.byref(h), ctypes.byref(zero)) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_render(None, None, None, None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_check(None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_sorter_create(None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_sorter_key_value_storage_requirements(None, 10, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_sorter_sort_key_value_indirect(None, None, 0, None, None, None, None, 0) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_sorter_check(None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_parse_ply(None, 0, None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_reserve(None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_set_count_fragments(None, 1) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_set_slabs(None, 0, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_set_transmittance_floor(None, 1e-4) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_set_batch_lanes(None, 0) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_set_batch_shared_cull(None, 1) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_set_cull_staging(None, 1) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_set_lean(None, 1) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_context_set_train_slab_min(None, 0) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_render_batched(None, None, 0, None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_train_forward(None, None, None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_train_backward(None, None, None, None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_train_forward_batched(None, None, 0, None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_train_backward_batched(None, None, 0, None, None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_viewer_create(None, None, None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_viewer_create_frames(None, None, None, None, None, 2) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_viewer_frame(None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_viewer_submit(None, None, None, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_viewer_wait(None, 0, None) == L.GS_ERROR_INVALID_ARGUMENT
    assert lib.gs_viewer_check(None, None) == L.GS_ERROR_INVALID_ARGUMENT
    lib.gs_viewer_destroy(None)
    lib.gs_context_destroy(None)
    lib.gs_sorter_destroy(None)


def test_scratch_bytes_without_a_device(lib):
    def need(n, w, h, pairs=0):
        b = ctypes.c_size_t()
        assert lib.gs_context_scratch_bytes(ctypes.byref(L.GsContextOptions(n, w, h, pairs)), ctypes.byref(b)) == 0
        return b.value

    small, big = need(100_000, 1600, 900), need(6_000_000, 1600, 900)
    assert big > small > 100_000 * 64              # at least the 64-byte raster record per splat
    assert need(6_000_000, 3840, 2160) > big          # per-pixel state grows with the target
    assert need(6_000_000, 1600, 900, 1 << 20) < big  # fewer tile pairs than the default 16 per splat
    assert lib.gs_context_scratch_bytes(None, None) == L.GS_ERROR_INVALID_ARGUMENT
    b = ctypes.c_size_t()
    assert lib.gs_context_scratch_bytes(ctypes.byref(L.GsContextOptions(10, 0, 0, 0)), ctypes.byref(b)) == \
        L.GS_ERROR_INVALID_ARGUMENT


def test_python_scratch_bytes_matches_the_abi(lib):
    import vkgs_gb300

    b = ctypes.c_size_t()
    assert lib.gs_context_scratch_bytes(ctypes.byref(L.GsContextOptions(1000, 64, 64, 0)), ctypes.byref(b)) == 0
    assert vkgs_gb300.scratch_bytes(1000, 64, 64) == b.value


def test_camera_helpers_match_oracle_bits(lib, oracle):
    from vkgs_gb300 import api

    for fovy, w, h, n, f in [(60, 1600, 900, 0.1, 100.0), (45, 640, 360, 0.01, 100.0), (75, 1920, 1080, 0.5, 50.0)]:
        a = api.perspective(math.radians(fovy), np.float32(w) / np.float32(h), n, f)
        b = oracle.perspective_vk(math.radians(fovy), np.float32(w) / np.float32(h), n, f)
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    rng = np.random.default_rng(0)
    for _ in range(20):
        eye = rng.normal(size=3) * 5
        c = rng.normal(size=3)
        a = api.look_at(eye, c)
        b = oracle.look_at(eye, c)
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    e1 = api.orbit_eye((0.1, 0.2, 0.3), 2.0, math.radians(45), math.radians(45))
    e2 = oracle.orbit_eye((0.1, 0.2, 0.3), 2.0, math.radians(45), math.radians(45))
    np.testing.assert_array_equal(e1, e2)


def _header(props, fmt="binary_little_endian 1.0", count=7, types=None):
    lines = ["ply", f"format {fmt}", f"element vertex {count}"]
    for i, p in enumerate(props):
        lines.append(f"property {(types or {}).get(p, 'float')} {p}")
    lines.append("end_header")
    return ("\n".join(lines) + "\n").encode()


def test_ply_header_offsets_match_loader_table(lib):
    from vkgs_gb300 import api

    head = _header(syn.PLY_PROPERTIES)
    off, cnt, hb = api.ply_header(head + b"\x00" * 64)
    assert cnt == 7 and hb == len(head)
    np.testing.assert_array_equal(off, syn.ply_offsets())
    # a different property order gives the matching table
    props = list(reversed(syn.PLY_PROPERTIES))
    off2, _, _ = api.ply_header(_header(props))
    np.testing.assert_array_equal(off2, syn.ply_offsets(props))


@pytest.mark.parametrize("mutate", ["missing", "ascii", "double", "magic", "noend"])
def test_ply_header_rejects_malformed(lib, mutate):
    props = list(syn.PLY_PROPERTIES)
    if mutate == "missing":
        head = _header([p for p in props if p != "f_rest_44"])
    elif mutate == "ascii":
        head = _header(props, fmt="ascii 1.0")
    elif mutate == "double":
        head = _header(props, types={"opacity": "double"})
    elif mutate == "magic":
        head = b"plx\n" + _header(props)[4:]
    else:
        head = _header(props).replace(b"end_header\n", b"")
    off = (ctypes.c_uint32 * 60)()
    cnt, hb = ctypes.c_uint64(), ctypes.c_size_t()
    st = lib.gs_ply_offsets_from_header(head, len(head), off, ctypes.byref(cnt), ctypes.byref(hb))
    assert st == L.GS_ERROR_INVALID_ARGUMENT


def test_synthetic_rows_are_deterministic():
    a = syn.splat_rows(5000, 11, "shell")
    b = syn.splat_rows(5000, 11, "shell")
    np.testing.assert_array_equal(a, b)
    r = np.linalg.norm(a[:, :3], axis=1)
    assert 0.6 < np.mean(np.abs(r - 4.0) < 0.5) < 0.8  # ~70 % on the shell
