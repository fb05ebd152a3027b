"""Writes tests/golden/ref_fixtures.json: outputs of the reference's own shaders, run on the host.

    python tests/golden/make_ref_fixtures.py

Needs the reference checkout (the shaders are compiled from src/shader/* where they lie, by
oracle/glsl/make_ref.py, into oracle/_ref/).  The fixtures record, per seeded workload and camera,
SHA-256 digests of what parse_ply.comp, rank.comp + the stable key sort, and projection.comp
produce, the indirect-draw words, and -- for the draw (splat.vert, Vulkan rasterisation,
splat.frag, blend) -- the fragment count and per-row channel sums of the image.
tests/test_ref_pin.py checks the CPU oracle against them, so the pin of the oracle to the
reference holds also where the reference checkout is absent.

rot_scale (instance words 4-7) is left out of the digests: projection.comp takes
cos/sin(atan(y, x) / 2) through the C library, the oracle uses the exact half-angle identities, and
the two differ by rounding (the maximum difference, relative to the column norm, is recorded).
"""

from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "ref_fixtures.json"
INSTANCE_WORDS = [0, 1, 2, 3, 8, 9, 10, 11]  # ndc.xyz, pad, rgb, opacity


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def rot_scale_error(ref_inst: np.ndarray, orc_inst: np.ndarray) -> float:
    """max |delta| over rot_scale columns, divided by the column's norm, in units of 2^-24."""
    if ref_inst.shape[0] == 0:
        return 0.0
    worst = 0.0
    for cols in ((4, 5), (6, 7)):
        a = ref_inst[:, cols].astype(np.float64)
        b = orc_inst[:, cols].astype(np.float64)
        norm = np.maximum(np.linalg.norm(b, axis=1), 1e-30)
        ok = np.isfinite(a).all(1) & np.isfinite(b).all(1)
        if ok.any():
            worst = max(worst, float((np.abs(a - b).max(1)[ok] / norm[ok]).max()) * 2.0**24)
    return worst


def cases():
    """(name, workload, n, camera specs) of the fixtures."""
    from vkgs_gb300 import synthetic as syn

    return [("small", "small", None, syn.workload_cameras("small")),
            ("large", "large", None, syn.workload_cameras("large"))]


def main() -> int:
    from oracle import oracle, ref
    from tests import scenes
    from vkgs_gb300 import synthetic as syn

    if not ref.available():
        print("the reference checkout is not present: nothing to generate", file=sys.stderr)
        return 1
    out = {"generator": "tests/golden/make_ref_fixtures.py",
           "source": "reference shaders src/shader/{parse_ply,rank,inverse_index,projection}.comp, splat.vert, "
                     "splat.frag compiled for the host (oracle/glsl/make_ref.py) and run by oracle/glsl/ref_harness.cpp",
           "instance_words": INSTANCE_WORDS, "parse_ply": [], "frames": [], "draws": []}
    for name, wl, n, specs in cases():
        rows, off, _ = syn.workload(wl, n)
        act = ref.parse_ply(rows, off)
        out["parse_ply"].append({"workload": wl, "n": int(rows.shape[0]),
                                 **{k: digest(a) for k, a in zip(("position", "cov3d", "opacity", "sh"), act)}})
        orc = oracle.parse_ply(rows, off)
        del rows
        for ci, s in enumerate(specs):
            c = scenes.camera(oracle, s.eye, fovy_deg=s.fovy_deg, width=s.width, height=s.height, near=s.near,
                              far=s.far)
            cam = scenes.oracle_camera(oracle, c)
            r = ref.frame_compute(*act, cam)
            k, i = oracle.rank(orc[0], cam)
            k, i = oracle.sort_kv(k, i)
            inst, rec = oracle.project(*orc, i, cam)
            out["frames"].append({
                "workload": wl, "camera": ci, "eye": [float(x) for x in s.eye], "width": s.width, "height": s.height,
                "count": r["count"], "key": digest(r["key"]), "index": digest(r["index"]),
                "instance": digest(r["instance"][:, INSTANCE_WORDS]),
                "draw_indirect": [int(x) for x in r["draw_indirect"]],
                "rot_scale_max_err_2m24": rot_scale_error(r["instance"], inst)})
            print(name, ci, r["count"], flush=True)
            if wl == "small":
                for unorm8 in (False, True):
                    img, frags = ref.draw(r["instance"], s.width, s.height, unorm8=unorm8)
                    out["draws"].append({"workload": wl, "camera": ci, "unorm8": unorm8, "fragments": frags,
                                         "row_sums": np.round(img.astype(np.float64).sum(axis=1), 4).tolist()})
    OUT.write_text(json.dumps(out, separators=(",", ":")) + "\n")
    print(OUT)
    return 0


if __name__ == "__main__":
    sys.exit(main())
