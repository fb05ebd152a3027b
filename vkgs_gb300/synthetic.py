"""Seeded synthetic scenes and cameras standing in for the public 3DGS scenes.

The reference was benchmarked on real scenes (bicycle, garden, bonsai) that are
not available here.  These generators draw splats with the stated per-splat
distributions and emit them as rows of a standard 3DGS PLY vertex element (62
float properties: x y z nx ny nz f_dc_0..2 f_rest_0..44 opacity scale_0..2
rot_0..3), plus the 60-entry offset table that the reference's loader builds
from the PLY header (src/vkgs/engine/splat_load_thread.cc:114-135).

Workloads
---------
* ``small``   : 100,000 splats, means ~ N(0, 1.5^2 I), one 1600x900 camera at (0,0,6).
* ``large``   : 6,000,000 splats, 70 % on a shell of radius 4 (radial sigma 0.1),
                30 % uniform in [-10,10]^3; eight 1600x900 cameras on a circle of
                radius 8 plus one zoomed-out camera at radius 20.
* ``batched`` : 1,000,000 splats (small distributions), 64 random cameras.
* ``grad``    : 1,000 splats at 256x256 and 200,000 splats at 800x800.
* ``batched_grad`` : 3,000,000 splats, 16 random views.

Shared per-splat distributions: log-scale ~ U(ln 0.01, ln 0.08) per axis,
rotation = N(0, I4) (normalised by the loader's activation), opacity logit
~ N(0, 1.5), SH DC ~ N(0, 0.5), SH bands 1-3 ~ N(0, 0.05).
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

PLY_PROPERTIES = (["x", "y", "z", "nx", "ny", "nz"] + [f"f_dc_{i}" for i in range(3)] +
                  [f"f_rest_{i}" for i in range(45)] + ["opacity"] + [f"scale_{i}" for i in range(3)] +
                  [f"rot_{i}" for i in range(4)])
ROW_FLOATS = len(PLY_PROPERTIES)  # 62
CHUNK = 1 << 20  # rows drawn per generator step (fixes the random stream independent of n)

RESOLUTIONS = [(640, 360), (960, 540), (1280, 720), (1600, 900), (1920, 1080)]
GRAD_RESOLUTIONS = [(800, 800), (1264, 832), (1600, 900)]


def ply_offsets(properties=PLY_PROPERTIES) -> np.ndarray:
    """The loader's offset table (splat_load_thread.cc:114-135), in floats."""
    at = {name: i for i, name in enumerate(properties)}
    off = np.zeros(60, np.uint32)
    off[0:3] = [at["x"], at["y"], at["z"]]
    off[3:6] = [at["scale_0"], at["scale_1"], at["scale_2"]]
    off[6:10] = [at["rot_1"], at["rot_2"], at["rot_3"], at["rot_0"]]  # (qx, qy, qz, qw)
    off[10 + 0] = at["f_dc_0"]
    off[10 + 16] = at["f_dc_1"]
    off[10 + 32] = at["f_dc_2"]
    for i in range(15):
        off[10 + 1 + i] = at[f"f_rest_{i}"]
        off[10 + 17 + i] = at[f"f_rest_{15 + i}"]
        off[10 + 33 + i] = at[f"f_rest_{30 + i}"]
    off[58] = at["opacity"]
    off[59] = len(properties)
    return off


def splat_rows(n: int, seed: int, layout: str = "gaussian") -> np.ndarray:
    """n x 62 float32 PLY rows.  layout: 'gaussian' (means ~ N(0,1.5^2 I)) or 'shell'."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rows = np.zeros((n, ROW_FLOATS), np.float32)
    shell_frac = 0.7
    for b in range(0, n, CHUNK):
        e = min(n, b + CHUNK)
        m = e - b
        if layout == "gaussian":
            means = rng.standard_normal((m, 3), dtype=np.float32) * np.float32(1.5)
        elif layout == "shell":
            u = rng.random(m)
            d = rng.standard_normal((m, 3), dtype=np.float32)
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            rad = np.float32(4.0) + rng.standard_normal(m, dtype=np.float32) * np.float32(0.1)
            uni = rng.uniform(-10.0, 10.0, (m, 3)).astype(np.float32)
            means = np.where((u < shell_frac)[:, None], d * rad[:, None], uni).astype(np.float32)
        else:
            raise ValueError(f"unknown layout {layout!r}")
        rows[b:e, 0:3] = means
        rows[b:e, 55:58] = rng.uniform(math.log(0.01), math.log(0.08), (m, 3)).astype(np.float32)
        rows[b:e, 58:62] = rng.standard_normal((m, 4), dtype=np.float32)
        rows[b:e, 54] = rng.standard_normal(m, dtype=np.float32) * np.float32(1.5)
        rows[b:e, 6:9] = rng.standard_normal((m, 3), dtype=np.float32) * np.float32(0.5)
        rows[b:e, 9:54] = rng.standard_normal((m, 45), dtype=np.float32) * np.float32(0.05)
    return rows


@dataclass
class CameraSpec:
    eye: tuple
    center: tuple = (0.0, 0.0, 0.0)
    fovy_deg: float = 60.0
    width: int = 1600
    height: int = 900
    near: float = 0.1
    far: float = 100.0


def circle_cameras(radius: float = 8.0, count: int = 8, zoomed: float | None = 20.0, width=1600, height=900):
    cams = [CameraSpec(eye=(radius * math.sin(2 * math.pi * k / count), 0.0, radius * math.cos(2 * math.pi * k / count)),
                       width=width, height=height) for k in range(count)]
    if zoomed is not None:
        cams.append(CameraSpec(eye=(0.0, 0.0, zoomed), width=width, height=height))
    return cams


def random_cameras(count: int, seed: int, radius=(6.0, 12.0), fovy=(40.0, 75.0), resolutions=RESOLUTIONS):
    """Directions uniform on the sphere (redrawn while |dir.y| > 0.99 so lookAt with up=+y is defined)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cams = []
    while len(cams) < count:
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        r = rng.uniform(*radius)
        f = rng.uniform(*fovy) if fovy is not None else 60.0
        w, h = resolutions[int(rng.integers(len(resolutions)))]
        if abs(d[1]) > 0.99:
            continue
        cams.append(CameraSpec(eye=tuple(float(x) for x in d * r), fovy_deg=float(f), width=w, height=h))
    return cams


WORKLOADS = {
    "small": dict(n=100_000, seed=0, layout="gaussian"),
    "large": dict(n=6_000_000, seed=1, layout="shell"),
    "batched": dict(n=1_000_000, seed=2, layout="shell"),
    "grad_check": dict(n=1_000, seed=3, layout="gaussian"),
    "grad": dict(n=200_000, seed=3, layout="gaussian"),
    "batched_grad": dict(n=3_000_000, seed=4, layout="shell"),
}


def workload_cameras(name: str):
    if name == "small":
        return [CameraSpec(eye=(0.0, 0.0, 6.0))]
    if name == "large":
        return circle_cameras()
    if name == "batched":
        return random_cameras(64, seed=1002)
    if name == "grad_check":
        return [CameraSpec(eye=(0.0, 0.0, 6.0), width=256, height=256)]
    if name == "grad":
        return [CameraSpec(eye=(0.0, 0.0, 6.0), width=800, height=800)]
    if name == "batched_grad":
        return random_cameras(16, seed=1004, fovy=None, resolutions=GRAD_RESOLUTIONS)
    raise KeyError(name)


def workload(name: str, n: int | None = None):
    """(rows, offsets, cameras) for a named workload; n overrides the splat count."""
    spec = WORKLOADS[name]
    rows = splat_rows(spec["n"] if n is None else n, spec["seed"], spec["layout"])
    return rows, ply_offsets(), workload_cameras(name)
