"""GPU: failure detection without a GPU fault.  A bounded device-side wait that is never satisfied gives up,
records its timeout and returns; the status reaches the host and the device keeps working."""

import time

import pytest

from tests import scenes
from vkgs_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_device_stays_usable(cuda, oracle):
    import torch
    from vkgs_gb300 import Renderer, parse_ply
    from vkgs_gb300 import _lib as L

    lib = L.load()
    t0 = time.monotonic()
    st = lib.gs_selftest_bounded_wait(None)
    elapsed = time.monotonic() - t0
    assert st == L.GS_ERROR_DEVICE_TIMEOUT
    assert elapsed < 60.0

    # the same process renders a correct frame afterwards
    rows = syn.splat_rows(20_000, 21)
    splats = parse_ply(torch.from_numpy(rows).cuda(), syn.ply_offsets())
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=160, height=120)
    r = Renderer(20_000, 160, 120)
    img, stats = r.render_checked(splats, scenes.product_camera(c))
    act = scenes.activated(oracle, rows)
    o = oracle.render_frame(*act, scenes.oracle_camera(oracle, c))
    assert stats["visible_count"] == o["count"]
    assert float((img.cpu().double() - torch.from_numpy(o["image"])).abs().max()) <= 1.0 / 255.0
