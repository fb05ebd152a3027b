"""Builds oracle/_ref/libvkgs_ref.so: the reference's own splat shaders, executed on the host.

TEST INFRASTRUCTURE ONLY (the executable reference that pins oracle/cpu_ref.c).

The shader sources are read where they lie in the reference checkout -- src/shader/parse_ply.comp,
rank.comp, inverse_index.comp, projection.comp, splat.vert and splat.frag -- and nothing of them is
committed here.  Each file is rewritten mechanically into a C++ include under oracle/_ref/gen/:

  * `#version` / `#extension` lines and the `layout(local_size_...) in;` declaration are dropped;
  * every interface block `layout(...) uniform|buffer Name { members };` becomes its members as
    namespace-scope variables (an unsized array `T a[];` becomes a pointer `T* a`), which the
    harness binds to its buffers -- the descriptor sets and push constants of the Vulkan engine;
  * `layout(location = k) in|out T name;` becomes `T name;` (the vertex outputs / fragment inputs the
    harness interpolates), `shared` storage becomes namespace-scope storage;
  * `void main()` is renamed `shader_main()`.

Function bodies are not touched: they compile as written against oracle/glsl/glsl.hpp (the GLSL
subset in C++), and oracle/glsl/ref_harness.cpp dispatches them in the engine's order
(engine.cc:1164-1290) and rasterises the quads with Vulkan's rules.

    python oracle/glsl/make_ref.py [--reference DIR] [--force]
"""

from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
GEN = OUT / "gen"
LIB = OUT / "libvkgs_ref.so"
DEFAULT_REFERENCE = Path(os.environ.get("VKGS_REFERENCE", "/root/reference"))
SHADERS = ["parse_ply.comp", "rank.comp", "inverse_index.comp", "projection.comp", "splat.vert", "splat.frag"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-Wno-unknown-pragmas"]

_BLOCK = re.compile(
    r"layout\s*\([^)]*\)\s*(?:(?:readonly|writeonly|coherent|restrict|volatile)\s+)*(?:uniform|buffer)\s+\w+\s*"
    r"\{(?P<body>.*?)\}\s*;", re.S)
_LOCAL_SIZE = re.compile(r"layout\s*\([^)]*local_size[^)]*\)\s*in\s*;")
_IO = re.compile(r"layout\s*\([^)]*\)\s*(?:in|out)\s+(\w+)\s+(\w+)\s*;")
_MEMBER = re.compile(r"^\s*(?P<type>\w+)\s+(?P<name>\w+)\s*(?:\[(?P<dim>\w*)\])?\s*$")


def _members(body: str) -> str:
    body = re.sub(r"//[^\n]*", "", body)
    out = []
    for decl in body.split(";"):
        if not decl.strip():
            continue
        m = _MEMBER.match(decl.strip())
        if m is None:
            raise ValueError(f"unsupported interface member: {decl.strip()!r}")
        t, name, dim = m.group("type"), m.group("name"), m.group("dim")
        if dim is None:
            out.append(f"{t} {name}{{}};")
        elif dim == "":
            out.append(f"{t}* {name} = nullptr;")
        else:
            out.append(f"{t} {name}[{dim}] = {{}};")
    return " ".join(out)


def translate(src: str) -> str:
    """GLSL shader source -> C++ declarations + shader_main() (bodies verbatim)."""
    src = re.sub(r"^\s*#\s*(version|extension)\b[^\n]*$", "", src, flags=re.M)
    src = _LOCAL_SIZE.sub("", src)
    src = _BLOCK.sub(lambda m: _members(m.group("body")), src)
    src = _IO.sub(r"\1 \2;", src)
    src = re.sub(r"^(\s*)shared\s+", r"\1", src, flags=re.M)
    src, n = re.subn(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", src)
    if n != 1:
        raise ValueError("expected exactly one main()")
    return src


def build(reference: Path = DEFAULT_REFERENCE, force: bool = False) -> Path | None:
    """Generate and compile; returns the library path, or None when the reference is not present."""
    shader_dir = reference / "src" / "shader"
    if not all((shader_dir / s).is_file() for s in SHADERS):
        return None
    GEN.mkdir(parents=True, exist_ok=True)
    deps = [HERE / "glsl.hpp", HERE / "ref_harness.cpp", Path(__file__)]
    for s in SHADERS:
        src = shader_dir / s
        dst = GEN / (s.replace(".", "_") + ".inc")
        text = f"// generated by oracle/glsl/make_ref.py from src/shader/{s}\n" + translate(src.read_text())
        if force or not dst.exists() or dst.read_text() != text:
            dst.write_text(text)
        deps.append(dst)
    newest = max(p.stat().st_mtime for p in deps)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(f".so.{os.getpid()}")
        cmd = ["g++", *CXXFLAGS, f"-I{HERE}", f"-I{GEN}", str(HERE / "ref_harness.cpp"), "-o", str(tmp)]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


def main() -> int:
    p = argparse.ArgumentParser()
    p.add_argument("--reference", type=Path, default=DEFAULT_REFERENCE)
    p.add_argument("--force", action="store_true")
    a = p.parse_args()
    lib = build(a.reference, a.force)
    if lib is None:
        print(f"reference shaders not found under {a.reference}/src/shader", file=sys.stderr)
        return 1
    print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
