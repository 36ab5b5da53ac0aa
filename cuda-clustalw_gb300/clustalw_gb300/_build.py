"""Compiles the CUDA library (csrc/*.cu) for sm_103a into lib/libcwgpu.so.

The library is built in-tree so that the process that loads it can be seen to
load this file and not an installed copy.
"""
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # cuda-clustalw_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO_ROOT, "include")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libcwgpu.so")

SOURCES = ["cwgpu.cu", "cwgpu_noalloc.cu", "cwgpu_serve.cu", "cwgpu_nj.cu", "cwgpu_fast.cu"]
HEADERS = ["cwgpu_device.cuh", "cwgpu_context.h", "cwgpu_ranges.h", "cwgpu_layout.h", "cwgpu_order.h"]
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, s) for s in SOURCES + HEADERS] + [os.path.join(INCLUDE, h) for h in ("cwgpu.h", "cwgpu_nj.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Build lib/libcwgpu.so if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    cmd = [
        nvcc_path(),
        *ARCH_FLAGS,
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler",
        "-fPIC",
        "-shared",
        "-I" + INCLUDE,
        *[os.path.join(CSRC, s) for s in SOURCES],
        "-o",
        tmp,
    ]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    # Translation units compile in parallel (-t), one -gencode.
    cmd.insert(1, "-t0")
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH
