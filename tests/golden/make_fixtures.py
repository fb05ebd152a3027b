"""Writes tests/golden/oracle_fixtures.json: regression fixtures of the oracle on small seeded scenes.

These are NOT reference outputs (those are tests/golden/ref_fixtures.json, written by
make_ref_fixtures.py from the reference's shaders run on the host).  They pin the oracle's own results -- visible count, a digest of the sorted keys
and ids, the fragment count and image checksums -- so that an unintended change to the restatement
shows up as a failing CPU test.  Regenerate only when the restatement is changed on purpose:

    python -m tests.golden.make_fixtures
"""

from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SCENES = [  # (splats, seed, layout, eye, width, height)
    (2_000, 31, "gaussian", (0.0, 0.0, 6.0), 160, 90),
    (5_000, 32, "shell", (3.0, 1.0, 6.0), 128, 128),
    (20_000, 33, "gaussian", (-2.0, 2.0, 5.0), 200, 120),
]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def fixture(oracle, n, seed, layout, eye, w, h) -> dict:
    from tests import scenes
    from vkgs_gb300 import synthetic as syn

    rows = syn.splat_rows(n, seed, layout)
    act = scenes.activated(oracle, rows)
    c = scenes.camera(oracle, eye, width=w, height=h)
    o = oracle.render_frame(*act, scenes.oracle_camera(oracle, c))
    img = o["image"].astype(np.float64)
    return {"splats": n, "seed": seed, "layout": layout, "eye": list(eye), "width": w, "height": h,
            "visible": o["count"], "keys_sha256": digest(o["key"]), "index_sha256": digest(o["index"]),
            "fragments": o["fragments"], "image_sum": float(img.sum()),
            "image_center": [float(x) for x in img[h // 2, w // 2]]}


def main() -> None:
    from oracle import oracle

    out = [fixture(oracle, *s) for s in SCENES]
    (HERE / "oracle_fixtures.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
