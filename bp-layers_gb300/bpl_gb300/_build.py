"""Builds libbpl_gb300.so (the C-ABI library with all CUDA kernels) in-tree.

nvcc compiles each translation unit of csrc/ for sm_103a in parallel, then
links them (with device linking for the units that share device symbols) into
bp-layers_gb300/_build/libbpl_gb300.so.  No torch headers are involved, so
the build is a few nvcc calls.
"""
from __future__ import annotations

import glob
import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # bp-layers_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libbpl_gb300.so")

ARCH = "103a"
NVCC_FLAGS = [
    "-std=c++17", "-O3", "-lineinfo", f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}",
    "-rdc=true", "-Xcompiler", "-fPIC", "--fmad=false", "-Xptxas", "-warn-spills",
]
# Units that reference no device symbol of another unit (the device error
# word and the wait limit are declared for relocatable units only, so such a
# reference does not compile) are compiled as whole programs: relocatable code
# gave the adjoint kernels a stack frame (local loads on every step) that
# whole-program code does not have.  They link beside the relocatable units;
# only the latter take part in device linking.
WHOLE_PROGRAM_PREFIXES = ("lbp_backward", "sad.cu", "beliefs.cu", "epilogue.cu", "pyramid.cu")


def _flags(src: str):
    if os.path.basename(src).startswith(WHOLE_PROGRAM_PREFIXES):
        return [f if f != "-rdc=true" else "-rdc=false" for f in NVCC_FLAGS]
    return NVCC_FLAGS


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps_digest() -> str:
    h = hashlib.sha256()
    for f in sorted(glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(INCLUDE, "*.h"))):
        with open(f, "rb") as fh:
            h.update(os.path.basename(f).encode())
            h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS + list(WHOLE_PROGRAM_PREFIXES)).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if sources changed) and return the library path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    stamp = os.path.join(BUILD_DIR, "stamp.txt")
    digest = _deps_digest()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return LIB_PATH
    nvcc = _nvcc()
    objs = []
    cmds = []
    for src in _sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        cmds.append([nvcc, "-c", src, "-o", obj, "-I", INCLUDE] + _flags(src))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout[-20000:], r.stderr[-20000:])
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for " + cmd[2])
        return r.stderr

    with ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 4)) as ex:
        list(ex.map(run, cmds))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    run([nvcc, "-shared", "-o", tmp] + objs + [f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}", "-rdc=true",
                                            "-Xcompiler", "-fPIC", "-lcudart", "-ldl"])
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB_PATH
