"""FP32-vs-FP64 image error of the restatement per workload (TEST INFRASTRUCTURE, CPU only).

For each named workload and a few of its cameras, renders the frame with the oracle's FP32
restatement (the arithmetic the CUDA path reproduces, see cpu_ref.c) and with its FP64 twin (the
same formulas in double, literal trigonometry), and reports per camera: the largest per-channel
difference, the share of pixels differing by more than 1/255 and the 99.9th percentile of the
per-pixel maximum difference.  The differences come from quad-edge coverage flips (a pixel centre
within rounding of the 3-sigma boundary) and from rounding in the blend.

    python -m oracle.fp32_vs_fp64 [--workloads small,large,batched,grad,batched_grad] [--cameras 2]

Prints one JSON object per camera.
"""

from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from oracle import oracle
from vkgs_gb300 import synthetic as syn


def oracle_camera(spec):
    P = oracle.perspective_vk(math.radians(spec.fovy_deg), np.float32(spec.width) / np.float32(spec.height),
                              spec.near, spec.far)
    V = oracle.look_at(spec.eye, spec.center)
    return oracle.make_camera(P, V, np.asarray(spec.eye, np.float32), spec.width, spec.height,
                              np.eye(4, dtype=np.float32).reshape(-1))


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workloads", default="small,large,batched,grad,batched_grad")
    ap.add_argument("--cameras", type=int, default=2, help="cameras per workload (spread over its list)")
    args = ap.parse_args()
    for name in args.workloads.split(","):
        rows, off, specs = syn.workload(name)
        act = oracle.parse_ply(rows, off)
        del rows
        step = max(1, len(specs) // args.cameras)
        for k in list(range(0, len(specs), step))[: args.cameras]:
            cam = oracle_camera(specs[k])
            t0 = time.time()
            out = oracle.render_frame(*act, cam, want_instances=False)
            _, img64 = oracle.render_frame_f64(*act, cam)
            d = np.abs(out["image"].astype(np.float64) - img64).max(axis=-1)
            print(json.dumps({"workload": name, "camera": k, "splats": int(act[0].shape[0]),
                              "size": f"{specs[k].width}x{specs[k].height}", "visible": out["count"],
                              "max_abs": float(d.max()), "pixels_over_1_255": float((d > 1.0 / 255.0).mean()),
                              "p99_9": float(np.quantile(d, 0.999)), "seconds": round(time.time() - t0, 1)}),
                  flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
