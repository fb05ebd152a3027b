"""CPU tests of the oracle (the scalar restatement of the reference shaders) against known answers.

The reference ships no tests or fixtures, so the known answers here are derived independently from
the published formulas (glm perspective/lookAt, the EWA projection, IEEE binary16 conversion) in
float64 numpy, plus structural properties (sortedness, stability, blend algebra).
"""

import math

import numpy as np
import pytest

from tests import scenes
from vkgs_gb300 import synthetic as syn

W, H = 1600, 900


def test_perspective_matches_published_formula(oracle):
    fovy, aspect, n, f = math.radians(60), np.float32(W) / np.float32(H), 0.1, 100.0
    P = oracle.perspective_vk(fovy, aspect, n, f).reshape(4, 4)  # P[col][row]
    t = math.tan(fovy / 2)
    exp = np.zeros((4, 4))
    exp[0, 0] = 1 / (aspect * t)
    exp[1, 1] = -1 / t                              # y flipped by the Vulkan conversion
    exp[2, 2] = 0.5 * (-(f + n) / (f - n)) - 0.5    # z' = z/2 + w/2
    exp[2, 3] = -1
    exp[3, 2] = 0.5 * (-(2 * f * n) / (f - n))
    np.testing.assert_allclose(P, exp, rtol=2e-7, atol=1e-9)


@pytest.mark.parametrize("eye", [(0, 0, 6), (5.0, 1.0, -3.0), (-2.0, -4.0, 7.5)])
def test_look_at_is_rigid_and_maps_eye_to_origin(oracle, eye):
    V = oracle.look_at(eye, [0, 0, 0]).reshape(4, 4).T.astype(np.float64)  # row-major
    R = V[:3, :3]
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-6)
    np.testing.assert_allclose(V @ np.array([*eye, 1.0]), [0, 0, 0, 1], atol=1e-5)
    c = V @ np.array([0, 0, 0, 1.0])  # the centre lies on the -z axis
    np.testing.assert_allclose(c[:2], [0, 0], atol=1e-5)
    assert c[2] < 0


def test_f16_conversion_is_round_to_nearest_even(oracle):
    rng = np.random.default_rng(0)
    vals = np.concatenate([
        rng.standard_normal(20000).astype(np.float32) * np.float32(3.0),
        rng.standard_normal(2000).astype(np.float32) * np.float32(1e-5),  # subnormal halves
        np.array([65504, 65519.99, 65520, 1e6, -1e6, 2.0 ** -25, 2.0 ** -24, 3 * 2.0 ** -26, 0.0, -0.0,
                  1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11, np.inf, -np.inf], np.float32),
    ])
    got = oracle.f32_to_f16_bits(vals)
    with np.errstate(over="ignore"):
        exp = vals.astype(np.float16).view(np.uint16)
    np.testing.assert_array_equal(got, exp)


def test_parse_ply_matches_float64_activation(oracle):
    rows = syn.splat_rows(2000, 7)
    off = syn.ply_offsets()
    pos, cov, opa, sh = oracle.parse_ply(rows, off)
    r = rows.astype(np.float64)
    np.testing.assert_array_equal(pos, rows[:, 0:3])
    s = np.exp(r[:, 55:58])
    q = r[:, [59, 60, 61, 58]]  # (x, y, z, w) = (rot_1, rot_2, rot_3, rot_0)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    x, y, z, w = q.T
    R = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
    ], 1)  # row-major rotation
    C = R @ (s[:, :, None] ** 2 * np.transpose(R, (0, 2, 1)))
    exp = np.stack([C[:, 0, 0], C[:, 0, 1], C[:, 0, 2], C[:, 1, 1], C[:, 1, 2], C[:, 2, 2]], -1)
    np.testing.assert_allclose(cov, exp, rtol=2e-5, atol=1e-9)
    np.testing.assert_allclose(opa, 1 / (1 + np.exp(-r[:, 54])), rtol=1e-6)
    terms = np.concatenate([rows[:, [6]], rows[:, 9:24], rows[:, [7]], rows[:, 24:39], rows[:, [8]], rows[:, 39:54]], 1)
    np.testing.assert_array_equal(sh, terms.astype(np.float16).view(np.uint16))


def test_rank_single_splat_known_key(oracle):
    c = scenes.camera(oracle, (0.0, 0.0, 6.0))
    cam = scenes.oracle_camera(oracle, c)
    key, idx = oracle.rank(np.zeros((1, 3), np.float32), cam)
    assert idx.tolist() == [0]
    n, f = 0.1, 100.0
    z_clip = 0.5 * (-(f + n) / (f - n)) * (-6.0) + 0.5 * (-(2 * f * n) / (f - n)) + 0.5 * 6.0
    z_ndc = z_clip / 6.0
    k = key.view(np.float32)[0]
    assert abs(k - (1 - z_ndc)) < 2e-7


def test_rank_culls_outside_the_frustum(oracle):
    c = scenes.camera(oracle, (0.0, 0.0, 6.0))
    cam = scenes.oracle_camera(oracle, c)
    # x extent of the frustum at depth 6: tan(30deg) * aspect * 6
    xe = math.tan(math.radians(30)) * (W / H) * 6.0
    ye = math.tan(math.radians(30)) * 6.0
    pts = np.array([[0, 0, 0], [0.999 * xe, 0, 0], [1.001 * xe, 0, 0], [0, 0.999 * ye, 0], [0, -1.001 * ye, 0],
                    [0, 0, 7.0],      # behind the camera
                    [0, 0, 5.95],     # in front of the near plane (6 - 0.1)
                    [0, 0, -93.5],    # inside the far plane (distance 99.5)
                    [0, 0, -95.0]],   # beyond the far plane (distance 101)
                   np.float32)
    _, idx = oracle.rank(pts, cam)
    assert idx.tolist() == [0, 1, 3, 7]


def test_sort_is_stable_and_ascending(oracle):
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 50, 100_000).astype(np.uint32) * np.uint32(0x01010101)
    vals = np.arange(keys.size, dtype=np.uint32)
    k, v = oracle.sort_kv(keys, vals)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(k, keys[order])
    np.testing.assert_array_equal(v, vals[order])


def test_projection_isotropic_splat_known_answer(oracle):
    sigma = 0.05
    rows = scenes.single_splat((0, 0, 0), scale=(sigma,) * 3, dc=(1.0, 0.5, -0.5))
    pos, cov, opa, sh = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0))
    cam = scenes.oracle_camera(oracle, c)
    inst, rec = oracle.project(pos, cov, opa, sh, np.array([0], np.uint32), cam)
    P = c["projection"].astype(np.float64)
    a = P[0] ** 2 * sigma ** 2 / 36 + 1 / W ** 2
    b = P[5] ** 2 * sigma ** 2 / 36 + 1 / H ** 2
    s0, s1 = math.sqrt(max(a, b)), math.sqrt(min(a, b))
    # b > a: the major axis is y, theta = pi/2, rot_scale = [[0, s0], [-s1, 0]] column-major
    np.testing.assert_allclose(inst[0, 4:8], [0.0, s0, -s1, 0.0], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(inst[0, 0:2], [0.0, 0.0], atol=1e-7)
    C0 = 0.28209479177387814
    np.testing.assert_allclose(inst[0, 8:11], np.maximum(C0 * np.array([1.0, 0.5, -0.5]) + 0.5, 0), rtol=1e-6)
    np.testing.assert_allclose(inst[0, 11], 1 / (1 + math.exp(-2.0)), rtol=1e-6)
    assert rec[0, 12] > 0  # drawn


def test_degenerate_covariance_is_not_drawn(oracle):
    # square image + isotropic splat on the optical axis: a == b, c == 0 -> D == 0 -> NaN rot_scale
    rows = scenes.single_splat((0, 0, 0), scale=(0.05,) * 3)
    pos, cov, opa, sh = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=64, height=64)
    cam = scenes.oracle_camera(oracle, c)
    r = oracle.render_frame(pos, cov, opa, sh, cam)
    assert r["count"] == 1
    assert np.isnan(r["instance"][0, 4:8]).any()
    assert r["fragments"] == 0
    exp = np.zeros((64, 64, 4), np.float32)
    exp[..., 3] = 1
    np.testing.assert_array_equal(r["image"], exp)


def test_drawn_flag_rule_on_random_scene(oracle):
    rows = syn.splat_rows(5000, 3)
    pos, cov, opa, sh = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.5, 0.3, 3.0))
    cam = scenes.oracle_camera(oracle, c)
    key, idx = oracle.rank(pos, cam)
    key, idx = oracle.sort_kv(key, idx)
    inst, rec = oracle.project(pos, cov, opa, sh, idx, cam)
    m = rec[:, 2:6]
    s1 = np.hypot(inst[:, 6], inst[:, 7])
    nz = rec[:, 6]
    expect = (s1 > 0) & np.isfinite(m).all(1) & (nz >= 0) & (nz < 1)
    np.testing.assert_array_equal(rec[:, 12] >= 0, expect)


def _blend_back_to_front(a, c):
    C = np.array([0.0, 0.0, 0.0, 1.0])
    for ai, ci in zip(a, c):
        C[:3] = ai * ci + (1 - ai) * C[:3]
        C[3] = ai * ai + (1 - ai) * C[3]
    return C


def _blend_front_to_back(a, c):
    T, C = 1.0, np.zeros(4)
    for ai, ci in zip(a[::-1], c[::-1]):
        w = ai * T
        C[:3] += w * ci
        C[3] += w * ai
        T -= w
    C[3] += T
    return C


def test_front_to_back_equals_reference_blend_order():
    rng = np.random.default_rng(5)
    for _ in range(50):
        k = int(rng.integers(1, 200))
        a = rng.uniform(0, 0.99, k)
        c = rng.uniform(0, 1, (k, 3))
        np.testing.assert_allclose(_blend_front_to_back(a, c), _blend_back_to_front(a, c), atol=1e-12)


def test_fp32_transcription_close_to_fp64(oracle):
    rows = syn.splat_rows(20000, 0)
    pos, cov, opa, sh = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=400, height=225)
    cam = scenes.oracle_camera(oracle, c)
    r = oracle.render_frame(pos, cov, opa, sh, cam)
    v64, img64 = oracle.render_frame_f64(pos, cov, opa, sh, cam)
    assert v64 == r["count"]
    d = np.abs(img64 - r["image"])
    assert np.mean(d > 1 / 255) < 1e-3      # only quad-edge coverage flips exceed 1/255
    assert np.quantile(d, 0.999) < 1 / 255
    u8 = oracle.render_frame(pos, cov, opa, sh, cam, unorm8=True)["image"]
    assert np.quantile(np.abs(u8 - r["image"]), 0.99) < 8 / 255  # per-blend 8-bit rounding drift


def test_depth_input_culls_fragments_behind_it(oracle):
    rows = syn.splat_rows(3000, 2)
    pos, cov, opa, sh = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, (0.0, 0.0, 6.0), width=160, height=90)
    cam = scenes.oracle_camera(oracle, c)
    full = oracle.render_frame(pos, cov, opa, sh, cam)
    ones = np.ones((90, 160), np.float32)
    same = oracle.render_frame(pos, cov, opa, sh, cam, depth_in=ones)
    np.testing.assert_array_equal(same["image"], full["image"])
    zero = oracle.render_frame(pos, cov, opa, sh, cam, depth_in=np.zeros((90, 160), np.float32))
    assert zero["fragments"] == 0


def test_fp32_vs_fp64_report_runs(oracle, capsys, monkeypatch):
    """The per-workload FP32-vs-FP64 report (oracle/fp32_vs_fp64.py) on the small gradient-check workload."""
    import json
    import sys

    from oracle import fp32_vs_fp64

    monkeypatch.setattr(sys, "argv", ["fp32_vs_fp64", "--workloads", "grad_check", "--cameras", "1"])
    assert fp32_vs_fp64.main() == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["workload"] == "grad_check" and line["visible"] > 0
    assert line["max_abs"] < 0.05 and line["pixels_over_1_255"] < 0.01
