"""Distance of the FP32 image, and of its once-quantised BGRA8 form, to the B8G8R8A8_UNORM framebuffer
of the reference (TEST INFRASTRUCTURE, CPU only).

The reference blends into an 8-bit UNORM attachment (render_pass.cc:15, engine.cc:281-291), so every
blend result is rounded to a multiple of 1/255 before the next splat blends over it.  The oracle
emulates that (``render_frame(..., unorm8=True)``, the ``unorm8`` path of cpu_ref.c).  The CUDA path
blends in FP32 (its image equals the oracle's FP32 image to ~4e-7) and, for a BGRA8 target, rounds
once at the end.  Per workload and camera this prints both distances to the per-blend UNORM8 image:
the largest per-channel difference (in 1/255 units), the share of pixels differing by more than 1/255
and by more than 4/255, and the 99th / 99.9th percentiles of the per-pixel maximum difference.

    python -m oracle.unorm8_distance [--workloads small,large,batched,grad,batched_grad] [--cameras 2]
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np

from oracle import oracle
from oracle.fp32_vs_fp64 import oracle_camera
from vkgs_gb300 import synthetic as syn


def stats(img: np.ndarray, ref8: np.ndarray) -> dict:
    d = np.abs(img.astype(np.float64) - ref8.astype(np.float64)).max(axis=-1) * 255.0
    return {"max_255": round(float(d.max()), 2), "over_1": float((d > 1.0 + 1e-6).mean()),
            "over_4": float((d > 4.0 + 1e-6).mean()), "p99_255": round(float(np.quantile(d, 0.99)), 2),
            "p99_9_255": round(float(np.quantile(d, 0.999)), 2)}


def quantise(img: np.ndarray) -> np.ndarray:
    return np.rint(np.clip(img, 0.0, 1.0) * 255.0) / 255.0


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
            f32 = oracle.render_frame(*act, cam, want_instances=False)["image"]
            u8 = oracle.render_frame(*act, cam, unorm8=True, want_instances=False)["image"]
            print(json.dumps({"workload": name, "camera": k, "splats": int(act[0].shape[0]),
                              "size": f"{specs[k].width}x{specs[k].height}",
                              "fp32_vs_unorm8": stats(f32, u8), "bgra8_once_vs_unorm8": stats(quantise(f32), u8),
                              "seconds": round(time.time() - t0, 1)}), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
