#!/usr/bin/env python3
"""Frames/s of the vkgs per-frame splat pipeline on GB300.

Workload ("large"): 6,000,000 synthetic 3D Gaussians (70 % on a radius-4 shell, 30 % uniform in
[-10,10]^3, seed 1), 1600x900, nine cameras (eight on a radius-8 circle + one zoomed out at radius
20), FP32 with binary16 SH.  A frame is cull + depth key + compaction + projection + SH, depth sort,
per-slab tile binning, per-tile sort, tile raster + blend; a step of the headline is one lap over the
nine cameras (nine frames), issued through the viewer loop with frames in flight (gs_viewer_submit:
one captured CUDA graph per slot, the camera rewritten inside it every frame, consecutive frames
overlapping; the reference's viewer keeps two frames in flight), so K steps time 9K frames and
`value` is frames/s.  One frame in flight and one gs_render call per frame (K frames each) are
reported beside it, the latter with per-stage times.  Inputs (816 MB of splat buffers) are
resident in HBM and larger than L2, so no L2 flush is interposed.  The line also carries the batched
form (64 views of a 1M-splat scene in one graph vs the per-view loop), the differentiable form
(fwd+bwd it/s, 200k splats at 800x800) and the batched differentiation (3M splats, 16 views/step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank renders its own frames (replicas: one frame does not shard) and
the line reports the whole-job frames/s.  --impl reference times the reference algorithm's CPU
restatement (the oracle) on the host cores instead; the reference's own Vulkan shaders cannot run
on this machine (no graphics stack).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "frames/s at 6M splats 1600x900"
UNIT = "frames/s"
OPS_PER_FRAGMENT = 20  # FP32 lane-ops per covered (pixel, splat) pair, the blend's algorithmic cost
WORKLOAD = "large"
DEFAULT_SLABS = 2  # the renderer's default depth-slab schedule: nearest 3/16 of the visible splats, then the rest
FRAMES_IN_FLIGHT = 5  # viewer slots whose frames overlap on the GPU (the reference viewer keeps 2, engine.cc:743)


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=27)
    p.add_argument("--warmup", type=int, default=9)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--splats", type=int, default=None, help="override the splat count (testing only)")
    p.add_argument("--cpu-band-stride", type=int, default=8, help="one-core estimate: blend every 4k-th 16-row band")
    p.add_argument("--cpu-seconds", type=float, default=120.0,
                   help="reference arm: stop timing complete CPU frames after this long (at least 3 frames)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-forms", action="store_true", help="skip the batched / differentiation forms")
    p.add_argument("--only-form", choices=["batched", "differentiation", "batched_differentiation", "cull_forms"],
                   default=None,
                   help="run just this form and print its JSON (profiling; no headline line)")
    p.add_argument("--form", choices=["plain", "batched", "batched_differentiation"], default="plain",
                   help="plain: the headline frame (replicas under torchrun); batched / batched_differentiation: "
                        "the view-sharded multi-GPU forms, one JSON line for the whole job")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running (read-only queries)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        if not self.rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in self.rows if num(r[1])]
        mx = [num(r[2]) for r in self.rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def raster_profile() -> dict:
    """The raster's figures from the committed ncu summary (DRAM bytes per launch, issue utilisation)."""
    path = os.path.join(ROOT, "profiles", "raster_large.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def make_scene(n_override=None):
    from vkgs_gb300 import synthetic as syn

    spec = syn.WORKLOADS[WORKLOAD]
    n = spec["n"] if n_override is None else n_override
    rows = syn.splat_rows(n, spec["seed"], spec["layout"])
    return rows, syn.ply_offsets(), syn.workload_cameras(WORKLOAD), n


def cpu_frames(oracle, act, cams, frames, first: int = 0):
    """Seconds per COMPLETE frame on the host (timed, nothing extrapolated): cull/key/compaction, stable
    sort, projection and the full blend of every pixel, for cameras first, first+1, ... (cycled)."""
    from tests import scenes

    out = []
    for k in range(first, first + frames):
        spec = cams[k % len(cams)]
        c = scenes.camera(oracle, spec.eye, fovy_deg=spec.fovy_deg, width=spec.width, height=spec.height,
                          near=spec.near, far=spec.far)
        cam = scenes.oracle_camera(oracle, c)
        t0 = time.perf_counter()
        key, idx = oracle.rank(act[0], cam)
        key, idx = oracle.sort_kv(key, idx)
        _, rec = oracle.project(*act, idx, cam)
        oracle.raster(rec, spec.width, spec.height)
        out.append(time.perf_counter() - t0)
    return out


def cpu_band_estimate(oracle, act, cams, band_stride: int, steps: int):
    """Seconds per frame ESTIMATED from a sample: full cull/sort/projection + the blend of every
    band_stride-th 16-row band (offset k % band_stride at step k), blend time x band_stride."""
    from tests import scenes

    out = []
    for k in range(steps):
        spec = cams[k % len(cams)]
        c = scenes.camera(oracle, spec.eye, fovy_deg=spec.fovy_deg, width=spec.width, height=spec.height,
                          near=spec.near, far=spec.far)
        cam = scenes.oracle_camera(oracle, c)
        t0 = time.perf_counter()
        key, idx = oracle.rank(act[0], cam)
        key, idx = oracle.sort_kv(key, idx)
        _, rec = oracle.project(*act, idx, cam)
        t1 = time.perf_counter()
        oracle.raster_bands(rec, spec.width, spec.height, band_stride, k % band_stride)
        t2 = time.perf_counter()
        out.append((t1 - t0) + band_stride * (t2 - t1))
    return out


def batched_form(dev, quick: bool = False):
    """Batched views (1M splats, 64 random cameras of mixed resolution): one gs_render_batched call captured
    in a CUDA graph and replayed, against the plain per-view loop of gs_render calls on the same GPU."""
    import torch
    from vkgs_gb300 import Camera, Renderer, parse_ply, synthetic as syn
    from vkgs_gb300.autotune import autotune_batched

    rows, off, specs = syn.workload("batched")
    splats = parse_ply(torch.from_numpy(rows).to(dev), off)
    del rows
    cams = [Camera.from_spec(sp) for sp in specs]
    colors = [torch.empty((c.height, c.width, 4), dtype=torch.float32, device=dev) for c in cams]
    r = Renderer(splats.count, 1920, 1080)
    for cam, col in zip(cams, colors):
        r.render_checked(splats, cam, color=col)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 2 if quick else 5

    def loop():
        for cam, col in zip(cams, colors):
            r.render(splats, cam, color=col)

    loop()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        loop()
    e1.record()
    torch.cuda.synchronize()
    loop_ms = e0.elapsed_time(e1) / reps
    r.check()
    choice = autotune_batched(r, splats, cams, colors, reps=2 if quick else 4)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        r.render_batched(splats, cams, colors)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        r.render_batched(splats, cams, colors)
    for _ in range(2):
        graph.replay()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps * 2):
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1) / (reps * 2)
    r.check()
    n = len(cams)
    return {"workload": f"batched: {splats.count} splats (shell layout), {n} random cameras at radius 6-12, "
                        "fovy 40-75 deg, resolutions from 640x360 to 1920x1080",
            "views_per_s": n / (batch_ms / 1e3), "plain_loop_views_per_s": n / (loop_ms / 1e3),
            "speedup_vs_plain_loop": loop_ms / batch_ms, "ms_per_batch": batch_ms, "ms_plain_loop": loop_ms,
            "lanes": choice.lanes, "slabs": list(choice.slabs), "graph": "one CUDA graph per batch (replayed)",
            "form": "per-view pipelines spread over render lanes (sub-contexts + streams), forked/joined in one graph"}


def _perturbed(raw: dict, seed: int = 4) -> dict:
    """The target's parameters: means + N(0, 0.01), SH DC + N(0, 0.05)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    pert = dict(raw)
    pert["means"] = raw["means"] + rng.normal(0.0, 0.01, raw["means"].shape).astype(np.float32)
    sh = raw["sh"].reshape(-1, 3, 16).copy()
    sh[:, :, 0] += rng.normal(0.0, 0.05, sh[:, :, 0].shape).astype(np.float32)
    pert["sh"] = sh.reshape(-1, 48)
    return pert


def batched_differentiation_form(dev, quick: bool = False):
    """fwd+bwd of 16 views per step (3M splats, resolutions from {800x800, 1264x832, 1600x900}, L1 loss to
    targets rendered from perturbed parameters): the batched autograd Function, gradients of all views
    accumulated into one per-splat buffer, against a per-view loop of the one-view Function."""
    import torch
    from vkgs_gb300 import Camera, Renderer, synthetic as syn, train, train_params as tp

    import gc

    rows, _, specs = syn.workload("batched_grad")
    raw = tp.from_rows(rows)
    n = rows.shape[0]
    del rows
    cams = [Camera.from_spec(sp) for sp in specs]
    gc.collect()  # renderers of earlier forms
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free0, total = torch.cuda.mem_get_info()
    params = {k: torch.tensor(v, device=dev, requires_grad=True) for k, v in raw.items()}
    mw, mh = max(c.width for c in cams), max(c.height for c in cams)
    r = Renderer(n, mw, mh)
    r.set_batch_lanes(len(cams))
    with torch.no_grad():
        pert = {k: torch.tensor(v, device=dev) for k, v in _perturbed(raw).items()}
        targets = [t.clone() for t in train.render_batched(pert, cams, r)]
        del pert
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3 if quick else 10

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def step():
        for t in params.values():
            t.grad = None
        imgs = train.render_batched(params, cams, r)
        loss = sum((img - tgt).abs().mean() for img, tgt in zip(imgs, targets)) / len(cams)
        loss.backward()

    torch.cuda.reset_peak_memory_stats()
    step_ms = timed(step)
    r.check()
    free1, _ = torch.cuda.mem_get_info()
    # device memory outside torch's caching allocator (the renderer's arenas, CUDA context) + torch's peak,
    # less what was in use before the form started
    outside = (total - free1) - torch.cuda.memory_reserved()
    peak_gb = (outside + torch.cuda.max_memory_reserved() - (total - free0)) / 1e9
    single = Renderer(n, mw, mh)

    def loop():
        for t in params.values():
            t.grad = None
        for cam, tgt in zip(cams, targets):
            ((train.render(params, cam, single) - tgt).abs().mean() / len(cams)).backward()

    loop_ms = timed(loop)
    single.check()
    res = sorted({f"{c.width}x{c.height}" for c in cams})
    return {"workload": f"batched fwd+bwd: {n} splats (shell layout), {len(cams)} views per step at "
                        f"{', '.join(res)}, L1 loss to perturbed-parameter targets, gradients of all views "
                        "accumulated into one per-splat buffer",
            "fwd_bwd_it_per_s": 1e3 / step_ms, "ms_fwd_bwd": step_ms, "views_per_s": len(cams) * 1e3 / step_ms,
            "per_view_loop_ms": loop_ms, "speedup_vs_per_view_loop": loop_ms / step_ms,
            "peak_hbm_gb": peak_gb, "device_in_use_before_gb": (total - free0) / 1e9,
            "form": "torch.autograd.Function over gs_train_forward_batched / gs_train_backward_batched "
                    "(one render lane per view; per-tile recomputation in the blend backward, per-pixel state "
                    "= final transmittance + blended count)"}


def cull_forms(dev, quick: bool = False, n_override=None):
    """Camera 0 of the bench workload with each cull + projection form (per-thread loads, then partitions
    staged in shared memory by bulk copies) and then with the lean launch shapes of the viewer's slots
    (gs_context_set_lean: the raster is k_raster_pairs): two untimed frames each (the launches an ncu
    capture of this mode sees), then the per-stage times over `reps` frames each, CUDA events."""
    import torch
    from vkgs_gb300 import Camera, Renderer, parse_ply

    rows, off, specs, n = make_scene(n_override)
    splats = parse_ply(torch.from_numpy(rows).to(dev), off)
    del rows
    cam = Camera.from_spec(specs[0])
    r = Renderer(n, cam.width, cam.height)
    r.render_checked(splats, cam)
    out = {"workload": f"{WORKLOAD}: {n} splats, camera 0, {cam.width}x{cam.height}"}
    forms = (("per_thread", False, False), ("staged", True, False), ("lean", False, True))
    for _, staged, lean in forms:
        r.set_cull_staging(staged)
        r.set_lean(lean)
        for _ in range(2):
            r.render(splats, cam)
        r.check()
    reps = 3 if quick else 20
    for name, staged, lean in forms:
        r.set_cull_staging(staged)
        r.set_lean(lean)
        r.enable_timing(True)
        for _ in range(reps):
            r.render(splats, cam)
        st = r.stage_times(reps)
        r.enable_timing(False)
        out[name] = {"cull_project_ms": float(st[:, 0].mean()), "raster_ms": float(st[:, 5].mean()),
                     "frame_ms": float(st.sum(1).mean())}
    r.check()
    return out


def differentiation_form(dev, quick: bool = False):
    """fwd+bwd through the autograd Function (200k splats, 800x800, L1 loss to a target rendered from
    perturbed parameters: means + N(0, 0.01), SH DC + N(0, 0.05)) against the plain forward of the same frame."""
    import numpy as np
    import torch
    from vkgs_gb300 import Camera, Renderer, parse_ply, synthetic as syn, train, train_params as tp

    rows, off, specs = syn.workload("grad")
    cam = Camera.from_spec(specs[0])
    raw = tp.from_rows(rows)
    params = {k: torch.tensor(v, device=dev, requires_grad=True) for k, v in raw.items()}
    pert = _perturbed(raw)
    r = Renderer(rows.shape[0], cam.width, cam.height)
    with torch.no_grad():
        target = train.render({k: torch.tensor(v, device=dev) for k, v in pert.items()}, cam, r).clone()
    splats = parse_ply(torch.from_numpy(rows).to(dev), off)
    plain = Renderer(rows.shape[0], cam.width, cam.height)
    plain.render_checked(splats, cam)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5 if quick else 30

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    fwd_ms = timed(lambda: plain.render(splats, cam))

    def step():
        for t in params.values():
            t.grad = None
        loss = (train.render(params, cam, r) - target).abs().mean()
        loss.backward()

    step_ms = timed(step)
    r.check()
    plain.check()
    return {"workload": f"fwd+bwd: {rows.shape[0]} splats (gaussian layout), 800x800, L1 loss to a perturbed-parameter "
                        "target, gradients for means, log-scales, quaternions, opacity logits and FP32 SH",
            "fwd_bwd_it_per_s": 1e3 / step_ms, "ms_fwd_bwd": step_ms, "ms_forward": fwd_ms,
            "fwd_bwd_over_forward": step_ms / fwd_ms,
            "form": "torch.autograd.Function over gs_train_forward / gs_train_backward (loss and autograd included)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle

    oracle.build()
    rows, off, cams, n = make_scene(args.splats)
    act = oracle.parse_ply(rows, off)
    del rows
    threads = oracle.num_threads()
    # Complete frames, each timed: one untimed frame pages the scene in, then K frames (camera k mod 9),
    # capped so that the run stays within a few minutes; `steps` reports the frames actually timed.
    cpu_frames(oracle, act, cams, 1 if args.warmup > 0 else 0)
    t_start = time.perf_counter()
    times = []
    while len(times) < args.steps and (len(times) < 3 or time.perf_counter() - t_start < args.cpu_seconds):
        times += cpu_frames(oracle, act, cams, 1, first=len(times))
    value = len(times) / sum(times)
    # The same restatement on one core, estimated from a band sample (a complete one-core frame takes
    # minutes): 4 steps, cameras 0-3, every 32nd 16-row band at offsets 0-3, blend time x32.
    oracle.set_num_threads(1)
    try:
        stride = 4 * args.cpu_band_stride
        one = cpu_band_estimate(oracle, act, cams, stride, 4)
    finally:
        oracle.set_num_threads(threads)
    sample = (f"{len(times)} complete frames (cameras 0..{len(times) - 1} mod 9) of all {n} splats: cull/key/"
              "compaction, stable sort, projection and the full blend of every pixel, each timed")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": len(times), "steps_requested": args.steps, "warmup": min(args.warmup, 1),
        "ms_per_step": 1000 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{WORKLOAD}: {n} splats (70% shell r=4, 30% uniform), 1600x900, 9 cameras "
                               "(8 on an r=8 circle + 1 at r=20), SH degree 3 in binary16",
                   "parallelism": f"host threads x{threads}", "l2": "inputs (816 MB) exceed L2; no flush"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "frame_s": [round(t, 3) for t in times],
                         "one_core_estimate": {"value": 4.0 / sum(one), "unit": UNIT, "cores": 1, "steps": 4,
                                               "sample": f"ESTIMATE: cameras 0-3, full cull/key/sort/projection "
                                                         f"+ blend of every {stride}th 16-row band (offset k mod "
                                                         f"{stride} at step k), blend time x{stride}"}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's Vulkan shaders cannot run here (no graphics stack); this arm is the scalar "
                "C restatement of those shaders (oracle/cpu_ref.c, pinned to the shaders' own bits on the "
                "host) on all host cores",
    }
    print(json.dumps(line), flush=True)
    return 0


def run_sharded_form(args):
    """The view-sharded forms on N GPUs (one process per GPU under torchrun): every rank holds the whole
    scene and takes its share of the views (vkgs_gb300.shard.view_shards: largest first, least-loaded
    rank).  batched: a step renders the 64-view batch (1M splats) -- each rank its views in one captured
    graph, no collective.  batched_differentiation: a step is one fwd+bwd of the 16-view batch (3M
    splats) with the gradients all-reduced over NCCL (shard.train_step_sharded).  The batch is fixed as
    N grows (strong scaling); value = whole-job views/s or it/s over the max-over-ranks time."""
    import torch
    import torch.distributed as dist

    from vkgs_gb300 import Camera, Renderer, parse_ply, shard, synthetic as syn, train, train_params as tp

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl")
    else:
        import socket

        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    K, W = args.steps, max(args.warmup, 3)
    if args.form == "batched":
        rows, off, specs = syn.workload("batched")
        splats = parse_ply(torch.from_numpy(rows).to(dev), off)
        del rows
        cams = [Camera.from_spec(sp) for sp in specs]
        mine = shard.view_shards(cams, world)[rank]
        colors = [torch.empty((c.height, c.width, 4), device=dev) for c in cams]
        r = Renderer(splats.count, 1920, 1080)
        r.set_batch_lanes(16)
        for v in mine:
            r.render_checked(splats, cams[v], color=colors[v])
        shard.render_batched_sharded(r, splats, cams, colors, rank, world)
        r.check()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            shard.render_batched_sharded(r, splats, cams, colors, rank, world)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            shard.render_batched_sharded(r, splats, cams, colors, rank, world)
        step = g.replay
        units, unit, metric = len(cams), "views/s", "batched views/s (1M splats, 64 views of 640x360..1920x1080)"
        workload = f"batched: {splats.count} splats, 64 random cameras, sharded by view over {world} rank(s)"
    else:
        rows, _, specs = syn.workload("batched_grad")
        raw = tp.from_rows(rows)
        n = rows.shape[0]
        del rows
        cams = [Camera.from_spec(sp) for sp in specs]
        params = {k: torch.tensor(v, device=dev, requires_grad=True) for k, v in raw.items()}
        mine = shard.view_shards(cams, world)[rank]
        r = Renderer(n, max(c.width for c in cams), max(c.height for c in cams))
        r.set_batch_lanes(max(len(mine), 1))
        with torch.no_grad():
            pert = {k: torch.tensor(v, device=dev) for k, v in _perturbed(raw).items()}
            targets = [t.clone() for t in train.render_batched(pert, cams, r)]
            del pert

        def step():
            for t in params.values():
                t.grad = None
            shard.train_step_sharded(params, cams, lambda v, img: (img - targets[v]).abs().mean() / len(cams), r,
                                     rank, world)

        units, unit, metric = 1, "it/s", "batched fwd+bwd it/s (3M splats, 16 views per step)"
        workload = f"batched_grad: {n} splats, 16 views per step, sharded by view over {world} rank(s), " \
                   "gradients all-reduced (NCCL)"
    for _ in range(W):
        step()
    r.check()
    dist.barrier()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(K):
        step()
    e1.record()
    torch.cuda.synchronize()
    dist.barrier()
    r.check()
    t = torch.tensor([e0.elapsed_time(e1)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    if rank == 0:
        print(json.dumps({
            "metric": metric, "value": units * K / (ms / 1e3), "unit": unit, "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload, "parallelism": f"views sharded x{world}", "form": args.form,
                       "views_on_rank0": len(mine)},
            "gpu_launches": None}), flush=True)
    dist.destroy_process_group()
    return 0


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from vkgs_gb300 import build as vbuild

    vbuild.build()
    from vkgs_gb300 import Camera, Renderer, parse_ply
    from vkgs_gb300 import _lib as L

    if args.only_form:
        if args.only_form == "cull_forms":
            print(json.dumps({"cull_forms": cull_forms(dev, quick=args.steps < 9, n_override=args.splats)}), flush=True)
            return 0
        form = {"batched": batched_form, "differentiation": differentiation_form,
                "batched_differentiation": batched_differentiation_form}[args.only_form]
        print(json.dumps({args.only_form: form(dev, quick=args.steps < 9)}), flush=True)
        return 0
    rows, off, specs, n = make_scene(args.splats)
    rows_t = torch.from_numpy(rows).to(dev)
    host_rows = rows if (rank == 0 and not args.no_cpu_baseline) else None
    del rows
    splats = parse_ply(rows_t, off)
    del rows_t
    cams = [Camera.from_spec(s) for s in specs]
    W, H = specs[0].width, specs[0].height
    r = Renderer(n, W, H)
    color = torch.empty((H, W, 4), dtype=torch.float32, device=dev)

    # Untimed: size the tile-pair capacity and count each camera's fragments F.
    r.count_fragments(True)
    stats = []
    for cam in cams:
        _, st = r.render_checked(splats, cam, color=color)
        stats.append(st)
    r.count_fragments(False)
    r.reserve(max_tile_pairs=int(max(s["tile_pairs"] for s in stats) * 1.05) + 1024)
    for k in range(max(args.warmup, 3)):
        r.render(splats, cams[k % len(cams)], color=color)
    r.check()

    def barrier():
        if dist is not None:
            dist.barrier()

    K = args.steps
    # Per-stage times of the same frames issued call by call (CUDA events between the stages).
    r.enable_timing(True)
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(K):
        r.render(splats, cams[k % len(cams)], color=color)
    e1.record()
    torch.cuda.synchronize()
    barrier()
    r.check()
    direct_ms = e0.elapsed_time(e1) / K
    stage = r.stage_times(K)
    r.enable_timing(False)

    # The same frames with the cull's partitions staged in shared memory by bulk copies (faster alone,
    # slower with frames in flight; reported beside the default)
    r.set_cull_staging(True)
    r.enable_timing(True)
    torch.cuda.synchronize()
    e0.record()
    for k in range(K):
        r.render(splats, cams[k % len(cams)], color=color)
    e1.record()
    torch.cuda.synchronize()
    r.check()
    staged_ms = e0.elapsed_time(e1) / K
    staged_stage = r.stage_times(K)
    r.enable_timing(False)
    r.set_cull_staging(False)

    # The same frames with the launch shapes of the viewer's slots (gs_context_set_lean): what each of
    # the headline's kernels costs alone (the raster is k_raster_pairs, two pixels per thread)
    r.set_lean(True)
    r.enable_timing(True)
    torch.cuda.synchronize()
    e0.record()
    for k in range(K):
        r.render(splats, cams[k % len(cams)], color=color)
    e1.record()
    torch.cuda.synchronize()
    r.check()
    lean_ms = e0.elapsed_time(e1) / K
    lean_stage = r.stage_times(K)
    r.enable_timing(False)
    r.set_lean(False)

    # (splat, tile) pairs binned per camera on the timed path (depth slabs, finished tiles skipped)
    emitted = []
    for cam in cams:
        r.render(splats, cam, color=color)
        emitted.append(r.check()["pairs_emitted"])

    # The headline: the viewer loop (gs_viewer_frame), one captured frame replayed as a CUDA graph with
    # the camera rewritten inside it every frame, cycling the nine cameras.
    from vkgs_gb300 import Viewer

    main = torch.cuda.current_stream()

    def viewer_rate(viewer, present, steps, warmup=None):
        """ms for `steps` frames through present(k); every slot waited for inside the timed region."""
        for k in range(max(args.warmup, 3) if warmup is None else warmup):
            present(k)
        viewer.check(main)
        barrier()
        torch.cuda.synchronize()
        e0.record(main)
        for k in range(steps):
            present(k)
        for slot in range(len(viewer.colors)):
            viewer.wait(slot, main)
        e1.record(main)
        torch.cuda.synchronize()
        barrier()
        viewer.check(main)
        return e0.elapsed_time(e1)

    # One frame in flight, for comparison: each frame waits for the previous one.  An event after every
    # frame gives the per-frame latency distribution (median, p10, p90).
    viewer = Viewer(r, splats, cams[0], color)
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(K)]

    def one_frame(k):  # (warm-up frames record too; the timed frames record again afterwards)
        viewer.frame(cams[k % len(cams)], stream=main)
        if k < K:
            marks[k].record(main)

    single_ms = viewer_rate(viewer, one_frame, K)
    frame_ms = [e0.elapsed_time(marks[0])] + [marks[k - 1].elapsed_time(marks[k]) for k in range(1, K)]
    viewer.close()

    # The headline: FRAMES_IN_FLIGHT frames in flight (the reference's viewer keeps two in flight).
    viewer = Viewer(r, splats, cams[0], color, frames_in_flight=FRAMES_IN_FLIGHT)
    clocks = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if clocks:
        clocks.start()
        time.sleep(0.3)
    # a step is one lap over the nine cameras: K steps time 9K frames (W warm-up laps first)
    lap = len(cams)
    ms = viewer_rate(viewer, lambda k: viewer.submit(cams[k % lap], stream=main), K * lap,
                     warmup=max(args.warmup, 3) * lap)
    clk = clocks.stop() if clocks else None
    r.check()
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * K * lap / (ms_max / 1000.0)

    # End to end through the public API, as a viewer presents its frames: per step the camera crosses
    # into the graph (h2d, the cull node's parameters) and the finished RGBA image is copied into pinned
    # host memory (d2h).  The copy of a slot's frame (on a copy stream) overlaps the next frames; a slot
    # is drawn into again only after its previous copy has finished.
    hosts = [torch.empty((H, W, 4), dtype=torch.float32).pin_memory() for _ in range(FRAMES_IN_FLIGHT)]
    copier = torch.cuda.Stream()
    copied = [torch.cuda.Event() for _ in range(FRAMES_IN_FLIGHT)]
    started = set()

    def present(k):
        slot = viewer.next_slot
        if slot in started:
            main.wait_event(copied[slot])
        started.add(slot)
        got = viewer.submit(cams[k % len(cams)], stream=main)
        viewer.wait(got, copier)
        with torch.cuda.stream(copier):
            hosts[got].copy_(viewer.colors[got], non_blocking=True)
        copied[got].record(copier)

    # the same K laps of nine frames
    e2e_steps = K * lap
    for k in range(max(args.warmup, 3)):
        present(k)
    torch.cuda.synchronize()
    barrier()
    e0.record(main)
    for k in range(e2e_steps):
        present(k)
    main.wait_stream(copier)
    e1.record(main)
    torch.cuda.synchronize()
    barrier()
    viewer.check(main)
    viewer.close()
    r.check()
    te = torch.tensor([e0.elapsed_time(e1)], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_value = world * e2e_steps / (float(te.item()) / 1000.0)  # frames/s

    # What the early stop buys: the same viewer loop with the transmittance floor at 2^-24 (every
    # contribution above FP32 resolution blended); the pair capacity reserved above already holds a
    # frame without early stop.
    r.set_transmittance_floor(2.0 ** -24)
    viewer = Viewer(r, splats, cams[0], color, frames_in_flight=FRAMES_IN_FLIGHT)
    exact_ms = viewer_rate(viewer, lambda k: viewer.submit(cams[k % lap], stream=main), K * lap, warmup=lap)
    viewer.close()
    r.set_transmittance_floor(1e-4)
    r.check()

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # Roofline of the dominant kernel (the raster/blend: FP32 issue-bound) + the HBM-bound stages.
    peaks = measured_peaks()
    props = torch.cuda.get_device_properties(dev)
    sms = props.multi_processor_count
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = sms * 128 * sm_max * 1e6 / 1e12  # T lane-ops/s
    cam_of = [k % len(cams) for k in range(K)]
    frags = np.array([stats[c]["fragments_blended"] for c in cam_of], np.float64)
    vis = np.array([stats[c]["visible_count"] for c in cam_of], np.float64)
    raster_ms = stage[:, 5].astype(np.float64)
    achieved = float((frags * OPS_PER_FRAGMENT).sum() / (raster_ms.sum() / 1e3) / 1e12)
    achieved_lean = float((frags * OPS_PER_FRAGMENT).sum() / (lean_stage[:, 5].astype(np.float64).sum() / 1e3) / 1e12)
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    cull_bytes = 12.0 * n + (8.0 + 188.0) * vis
    sort_bytes = 64.0 * vis
    stage_mean = {name: float(stage[:, i].mean()) for i, name in enumerate(L.STAGES)}
    hbm_stages = {
        "cull_project": {"ms": stage_mean["cull_project"],
                         "gbs": float(cull_bytes.sum() / (stage[:, 0].sum() / 1e3) / 1e9)},
        "depth_sort": {"ms": stage_mean["depth_sort"], "gbs": float(sort_bytes.sum() / (stage[:, 1].sum() / 1e3) / 1e9)},
    }
    for v in hbm_stages.values():
        v["frac"] = v["gbs"] / hbm
    dominant = max(stage_mean, key=stage_mean.get)

    cpu = None
    if host_rows is not None:
        try:
            from oracle import oracle

            oracle.build()
            act = oracle.parse_ply(host_rows, off)
            del host_rows
            threads = oracle.num_threads()
            times = cpu_frames(oracle, act, specs, 3)
            cpu = {"value": len(times) / sum(times), "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": "3 complete frames (cameras 0, 1, 2), each timed: cull/key/compaction, stable sort, "
                             "projection and the full blend of every pixel",
                   "frame_s": [round(t, 3) for t in times]}
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port", "sample": f"failed: {exc}"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": ms_max / K, "frames_per_step": lap, "frames_timed": K * lap,
        "ms_per_frame": ms_max / (K * lap), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{WORKLOAD}: {n} splats (70% shell r=4, 30% uniform), 1600x900, 9 cameras "
                               "(8 on an r=8 circle + 1 at r=20), SH degree 3 in binary16",
                   "parallelism": f"replicas x{world}", "l2": "inputs (816 MB) exceed L2; no flush",
                   "depth_slabs": "nearest 192/1024 of the visible splats, then the rest",
                   "frames_in_flight": FRAMES_IN_FLIGHT},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 292 * lap,
                "d2h_bytes_per_step": H * W * 16 * lap, "frames_timed": e2e_steps,
                "form": f"gs_viewer_submit per step ({FRAMES_IN_FLIGHT} frames in flight) + the RGBA image of "
                        "each frame copied to pinned host memory; a copy overlaps the following frames"},
        "gpu_launches": None,
        "roofline": {"bound": "fp32", "kernel": "k_raster_pairs (nearest slab) + k_raster (farther slab)",
                     "achieved": achieved, "peak": fp32_peak,
                     "unit": "T lane-ops/s", "frac": achieved / fp32_peak,
                     "traffic": raster_profile().get("dram_bytes_per_launch"),
                     "issue_active_ncu": raster_profile().get("issue_active"),
                     "peak_source": f"nominal {sms} SMs x 128 FP32 lanes x {sm_max:.0f} MHz (max SM clock)",
                     "work": f"{OPS_PER_FRAGMENT} FP32 lane-ops per covered (pixel, splat) pair met front to "
                             "back while the pixel's transmittance is >= the transmittance floor (1e-4)",
                     "lean_form": {"kernel": "k_raster_pairs (every slab)", "ms": float(lean_stage[:, 5].mean()),
                                   "achieved": achieved_lean, "frac": achieved_lean / fp32_peak,
                                   "form": "the raster of the headline's viewer slots (two pixels per thread, "
                                           "packed FP32 blend), timed alone on the direct path"}},
        "roofline_hbm": {**hbm_stages, "peak_gbs": hbm, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "stages_ms": stage_mean,
        "dominant_stage": dominant,
        "frame_stats": {"visible": [s["visible_count"] for s in stats], "tile_pairs": [s["tile_pairs"] for s in stats],
                        "fragments": [s["fragments"] for s in stats],
                        "fragments_blended": [s["fragments_blended"] for s in stats],
                        "pairs_emitted": emitted},
        "cpu_baseline": cpu,
        "clocks": clk,
        "form": f"gs_viewer_submit with {FRAMES_IN_FLIGHT} frames in flight: "
                "one captured CUDA graph per slot, the camera constants rewritten in its cull node every step, "
                "each slot with its own scratch, stream and target, consecutive frames overlapping",
        "one_frame_in_flight": {"frames_per_s": world * K / (single_ms / 1e3), "ms_per_frame": single_ms / K,
                                "frame_ms_p10_median_p90": [float(np.percentile(frame_ms, q)) for q in (10, 50, 90)],
                                "form": "gs_viewer_frame: each frame waits for the previous one"},
        "direct_render": {"frames_per_s": world / (direct_ms / 1e3), "ms_per_frame": direct_ms,
                          "form": "one gs_render call per step (stages_ms are measured on this path)"},
        "floor_2m24": {"frames_per_s": world * K * lap / (exact_ms / 1e3), "frames_timed": K * lap,
                       "form": f"the headline viewer loop ({FRAMES_IN_FLIGHT} frames in flight) with the "
                               "transmittance floor at 2^-24 instead of 1e-4"},
        "direct_render_staged_cull": {
            "frames_per_s": world / (staged_ms / 1e3), "ms_per_frame": staged_ms,
            "cull_project_ms": float(staged_stage[:, 0].mean()),
            "cull_project_gbs": float(cull_bytes.sum() / (staged_stage[:, 0].sum() / 1e3) / 1e9),
            "form": "gs_render with gs_context_set_cull_staging(1): cull partitions staged in shared memory "
                    "by bulk copies"},
        "direct_render_lean": {
            "frames_per_s": world / (lean_ms / 1e3), "ms_per_frame": lean_ms,
            "stages_ms": {name: float(lean_stage[:, i].mean()) for i, name in enumerate(L.STAGES)},
            "form": "gs_render with gs_context_set_lean(1): the launch shapes of the headline's viewer slots, "
                    "each kernel alone"},
    }
    if not args.no_forms:
        line["batched"] = batched_form(dev, quick=args.steps < 9)
        line["differentiation"] = differentiation_form(dev, quick=args.steps < 9)
        line["batched_differentiation"] = batched_differentiation_form(dev, quick=args.steps < 9)
    # cull_project, depth sort (histogram + 4 passes), then per depth slab: count, giant count, scan,
    # emit, giant emit, per-tile sort, raster
    launches_per_frame = 1 + 5 + 7 * DEFAULT_SLABS
    line["gpu_launches"] = launches_per_frame * K * lap
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.form != "plain":
        return run_sharded_form(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
