"""In-tree build of the C-ABI library ``simplefluid_gb300/_lib/libsimplefluid_gb300.so``.

``build(checked=True)`` builds the checked library
``_lib/libsimplefluid_gb300_checked.so`` instead: the same sources compiled with
SF_DEVICE_CHECKS=1, whose kernels check every cell-table range end and
neighbour-list entry before use and count bad ones (``sf_index_checks``).

Every translation unit is compiled by nvcc for sm_103a only, in parallel, then
linked into one shared library.  Host code is built with -ffp-contract=off so
that x86-64 and aarch64 hosts produce identical scene coordinates; the kernel
TU is built with -fmad=false so that only explicit fmaf() calls fuse.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libsimplefluid_gb300.so")
CHECKED_LIB = os.path.join(OUT_DIR, "libsimplefluid_gb300_checked.so")
CHECKED_OBJ_DIR = os.path.join(OUT_DIR, "obj_checked")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
          "-I", os.path.join(ROOT, "include")]

# (source, extra flags)
SOURCES = [
    ("sf_grid.cu", ["-fmad=false"]),
    ("sf_density.cu", ["-fmad=false"]),
    ("sf_force.cu", ["-fmad=false"]),
    ("sf_adjoint.cu", ["-fmad=false"]),
    ("sf_render.cu", ["-fmad=false"]),
    ("sf_frame.cu", ["-fmad=false"]),
    ("sf_capi.cpp", []),
    ("sf_capi_inspect.cpp", []),
    ("sf_capi_batch.cpp", []),
    ("sf_capi_adjoint.cpp", []),
    ("sf_scenes.cpp", []),
    ("sf_noalloc.cu", ["-fmad=false"]),
    ("sf_batch.cu", ["-fmad=false"]),
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src: str, extra: list[str], verbose: bool, obj_dir: str | None = None) -> str:
    obj = os.path.join(obj_dir or OBJ_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, checked: bool = False) -> str:
    obj_dir, lib = (CHECKED_OBJ_DIR, CHECKED_LIB) if checked else (OBJ_DIR, LIB)
    flags = ["-DSF_DEVICE_CHECKS=1"] if checked else []
    os.makedirs(obj_dir, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s[0], s[1] + flags, verbose, obj_dir), SOURCES))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, checked="--checked" in sys.argv))
