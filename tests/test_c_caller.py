"""CPU: a plain C11 program includes include/vkgs_gb300.h and links libvkgs_gb300.so -- the boundary a
C or C++ engine (or a cgo / JNI / ctypes stub) binds -- and calls the entry points that need no device."""

import shutil
import subprocess
from pathlib import Path

import pytest

from vkgs_gb300 import _lib as L

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "vkgs_gb300.h"

int main(void) {
  gs_context_options o = {6000000u, 1600u, 900u, 0u};
  size_t bytes = 0;
  if (gs_context_scratch_bytes(&o, &bytes) != GS_SUCCESS || bytes == 0) return 1;
  if (gs_context_scratch_bytes(NULL, &bytes) != GS_ERROR_INVALID_ARGUMENT) return 2;
  if (gs_render(NULL, NULL, NULL, NULL, NULL, NULL) != GS_ERROR_INVALID_ARGUMENT) return 3;
  if (gs_viewer_submit(NULL, NULL, NULL, NULL) != GS_ERROR_INVALID_ARGUMENT) return 4;
  if (strcmp(gs_status_string(GS_SUCCESS), "unknown status") == 0) return 5;
  float p[16];
  gs_camera_perspective(1.0471976f, 16.0f / 9.0f, 0.1f, 100.0f, p);
  if (!(p[0] > 0.0f)) return 6;
  printf("%u %zu\n", gs_version(), bytes);
  return 0;
}
"""


def test_c_program_links_and_calls_the_abi(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = L.LIB_PATH
    if not lib.exists():
        pytest.skip("library not built")
    src = tmp_path / "caller.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "caller"
    subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(lib.parent), "-l:" + lib.name, f"-Wl,-rpath,{lib.parent}"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) >= 10000 and int(out[1]) > 6_000_000 * 64
