"""Builds libvkgs_gb300.so (sm_103a) in-tree with nvcc, one translation unit per process.

    python -m vkgs_gb300.build          # incremental
    python -m vkgs_gb300.build --force  # rebuild everything
"""

from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libvkgs_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
          f"-I{INCLUDE}", f"-I{CSRC}"]
# Per-translation-unit numeric flags: the units that must reproduce the restated shader arithmetic
# bit for bit never contract a*b+c into an FMA.
UNITS = {
    "gs_api.cu": ["--fmad=false"],
    "gs_cull.cu": ["--fmad=false"],
    "gs_ply.cu": ["--fmad=false"],
    "gs_sort.cu": [],
    # the count and emit kernels evaluate the same tile-footprint arithmetic and must agree exactly
    "gs_bin.cu": ["--fmad=false"],
    "gs_raster.cu": ["-ftz=true"],
    "gs_noalloc.cu": [],
    # the projection backward: gradients, no bit-exactness requirement (FMA contraction on)
    "gs_train.cu": [],
}
HEADERS = ["gs_common.cuh", "gs_internal.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (cand == "nvcc" or Path(cand).exists()):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    headers = [CSRC / h for h in HEADERS] + [INCLUDE / "vkgs_gb300.h", Path(__file__)]
    jobs = []
    objs = []
    for unit, flags in UNITS.items():
        src = CSRC / unit
        obj = BUILD / (unit + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append([nvcc(), *ARCH, *COMMON, *flags, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({cmd[-3]}):\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(f".so.{os.getpid()}")
        run([nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fPIC"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
