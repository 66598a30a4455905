"""The C ABI from plain C: include/bpl_gb300.h compiles as strict C99 with
-pedantic and no warnings, and a C program links libbpl_gb300.so and calls it
(version, status text, an argument check that fails on the host before any
device work).  This is the boundary a cgo / JNI / N-API binding would
compile against; no GPU is needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C_SOURCE = r"""
#include "bpl_gb300.h"
#include <stdio.h>
#include <string.h>
int main(void) {
  if (bpl_version() < 100) return 2;
  if (strcmp(bpl_status_string(0), "ok") != 0) return 3;
  /* L out of range: rejected on the host, null pointers never touched */
  int st = bpl_lbp_forward(0, NULL, NULL, NULL, NULL, NULL, 0, NULL, 1, 4, 4, 2000, 6, 1, 1, 3, NULL);
  printf("%d %s\n", st, bpl_last_error());
  return st == 1 ? 0 : 1;
}
"""


def _cudart_dir():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    for d in ("lib64", "lib"):
        p = os.path.join(home, d)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return None


def test_header_compiles_as_c_and_links(bpl_lib, tmp_path):
    gcc = shutil.which("gcc")
    cudart = _cudart_dir()
    if gcc is None or cudart is None:
        pytest.skip("gcc or libcudart not found")
    from bpl_gb300 import _build
    libdir = os.path.dirname(_build.LIB_PATH)
    src = tmp_path / "capi.c"
    src.write_text(C_SOURCE)
    exe = tmp_path / "capi"
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
           str(src), "-o", str(exe), "-L", libdir, "-lbpl_gb300", "-Wl,-rpath," + libdir,
           "-L", cudart, "-lcudart", "-Wl,-rpath," + cudart]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "L=2000" in r.stdout
