"""Scene and camera builders shared by the tests (host side, numpy)."""

from __future__ import annotations

import math

import numpy as np

from vkgs_gb300 import synthetic as syn


def activated(oracle, rows, offsets=None):
    """Activate PLY rows on the host with the oracle's parse_ply restatement."""
    return oracle.parse_ply(rows, syn.ply_offsets() if offsets is None else offsets)


def camera(oracle, eye, center=(0.0, 0.0, 0.0), fovy_deg=60.0, width=1600, height=900, near=0.1, far=100.0,
           model=None):
    P = oracle.perspective_vk(math.radians(fovy_deg), np.float32(width) / np.float32(height), near, far)
    V = oracle.look_at(eye, center)
    return dict(projection=P, view=V, eye=np.asarray(eye, np.float32), width=width, height=height,
                model=np.eye(4, dtype=np.float32).reshape(-1) if model is None else np.asarray(model, np.float32))


def oracle_camera(oracle, c):
    return oracle.make_camera(c["projection"], c["view"], c["eye"], c["width"], c["height"], c["model"])


def product_camera(c):
    from vkgs_gb300 import Camera

    return Camera(c["projection"], c["view"], c["eye"], c["width"], c["height"], c["model"])


def single_splat(pos, scale=(0.05, 0.05, 0.05), quat_wxyz=(1.0, 0.0, 0.0, 0.0), opacity_logit=2.0, dc=(1.0, 0.5, -0.5),
                 rest=0.0):
    """One PLY row in the synthetic property order."""
    r = np.zeros((1, syn.ROW_FLOATS), np.float32)
    r[0, 0:3] = pos
    r[0, 55:58] = np.log(np.asarray(scale, np.float32))
    r[0, 58:62] = quat_wxyz
    r[0, 54] = opacity_logit
    r[0, 6:9] = dc
    r[0, 9:54] = rest
    return r


def rows_from(list_of_rows):
    return np.concatenate(list_of_rows, axis=0).astype(np.float32)


def rotation_model(angle_deg=20.0, axis=(0.3, 1.0, 0.2), translate=(0.2, -0.1, 0.3), scale=1.1):
    """A rigid-plus-uniform-scale model matrix (column-major float[16])."""
    a = np.asarray(axis, np.float64)
    a /= np.linalg.norm(a)
    t = math.radians(angle_deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R = np.eye(3) + math.sin(t) * K + (1 - math.cos(t)) * K @ K
    M = np.eye(4)
    M[:3, :3] = R * scale
    M[:3, 3] = translate
    return M.T.astype(np.float32).reshape(-1)  # column-major
