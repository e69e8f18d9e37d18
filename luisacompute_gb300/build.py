"""Compile the sm_103a kernels and the C ABI into ``luisacompute_gb300/_lib/liblcx_accel.so``.

Plain ``nvcc`` invocations (one per translation unit, run in parallel, one
``-gencode``), then one shared-library link.  No CMake.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "liblcx_accel.so"
SOURCES = ["build.cu", "sah.cu", "traverse.cu", "capi.cu", "sort.cu", "noalloc.cu", "pathtrace.cu", "reorder.cu", "cpu_table.cu"]
HEADERS = ["lcx_internal.h", "build_util.cuh", "pt_math.cuh"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblcx_accel.so")


PUBLIC_HEADERS = ["lcx_accel.h", "lcx/bvh_device.cuh", "lcx/node_test.cuh", "lcx/accel_instances.cuh", "lcx/trace.cuh",
                  "lcx/ray_query.cuh"]


def _stamp() -> str:
    h = hashlib.sha256()
    for f in SOURCES + HEADERS:
        h.update((CSRC / f).read_bytes())
    for f in PUBLIC_HEADERS:
        h.update((ROOT / "include" / f).read_bytes())
    h.update(" ".join(NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    """Build the library if its sources changed; returns its path."""
    LIBDIR.mkdir(exist_ok=True)
    stamp_file = LIBDIR / "stamp.txt"
    stamp = _stamp()
    if not force and LIB.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return LIB
    nvcc = nvcc_path()
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)

    def compile_one(src: str):
        out = objdir / (Path(src).stem + ".o")
        cmd = [nvcc, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(out)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr, file=sys.stderr)
        return out

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    cmd = [nvcc, ARCH, "-shared", "-cudart", "shared", "-o", str(LIB), *map(str, objs),
           "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    stamp_file.write_text(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
