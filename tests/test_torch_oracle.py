"""The FP64 torch restatement (gradient oracle) pinned on the CPU: its forward against the scalar C
oracle's image, its autograd against FP64 central differences."""

import numpy as np
import pytest

from tests import scenes
from vkgs_gb300 import synthetic as syn
from vkgs_gb300 import train_params as tp

torch = pytest.importorskip("torch")


def _scene(oracle, n, seed, eye, w, h):
    rows = syn.splat_rows(n, seed)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, eye, width=w, height=h)
    out = oracle.render_frame(*act, scenes.oracle_camera(oracle, c))
    return rows, c, out


def _params(rows, f16_sh=False):
    p = tp.from_rows(rows)
    if f16_sh:
        p["sh"] = p["sh"].astype(np.float16).astype(np.float32)
    return {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in p.items()}


def test_forward_matches_c_oracle(oracle):
    from oracle import torch_ref

    rows, c, out = _scene(oracle, 400, 31, (0.0, 0.0, 6.0), 96, 64)
    p = _params(rows, f16_sh=True)  # the C oracle's SH are binary16
    img = torch_ref.render(p["means"], p["log_scales"], p["quats"], p["opacity_logits"], p["sh"],
                           torch_ref.camera_dict(c), out["index"])
    err = (img.detach().numpy() - out["image"]).__abs__()
    assert err.max() <= 1.0 / 255.0
    assert np.mean(err) < 1e-5


def test_autograd_matches_central_differences(oracle):
    from oracle import torch_ref

    rows, c, out = _scene(oracle, 12, 32, (0.0, 0.0, 3.0), 24, 20)
    assert out["count"] >= 5
    p = _params(rows)
    weights = torch.tensor(np.random.default_rng(0).standard_normal((20, 24, 4)))
    cam = torch_ref.camera_dict(c)

    def loss():
        img = torch_ref.render(p["means"], p["log_scales"], p["quats"], p["opacity_logits"], p["sh"], cam,
                               out["index"])
        return (img * weights).sum()

    loss().backward()
    rng = np.random.default_rng(1)
    vis = out["index"]
    checked = 0
    for name, cols in (("means", 3), ("log_scales", 3), ("quats", 4), ("opacity_logits", 0), ("sh", 48)):
        for _ in range(4):
            i = int(vis[rng.integers(len(vis))])
            idx = (i,) if cols == 0 else (i, int(rng.integers(cols)))
            g = p[name].grad[idx].item()
            fd = torch_ref.central_difference(loss, p[name].data, idx)
            assert abs(g - fd) <= 1e-5 * max(1.0, abs(fd)), (name, idx, g, fd)
            checked += 1
    assert checked == 20


def test_window_render_equals_the_crop(oracle):
    from oracle import torch_ref

    rows, c, out = _scene(oracle, 300, 33, (0.5, 0.0, 5.0), 80, 60)
    p = _params(rows)
    cam = torch_ref.camera_dict(c)
    full = torch_ref.render(p["means"], p["log_scales"], p["quats"], p["opacity_logits"], p["sh"], cam, out["index"])
    win = torch_ref.render(p["means"], p["log_scales"], p["quats"], p["opacity_logits"], p["sh"], cam, out["index"],
                           window=(13, 47, 5, 52))
    assert torch.equal(win, full[5:52, 13:47])
