"""In-tree build of the CUDA library ``libaxs_gb300.so`` for sm_103a.

Every ``csrc/*.cu`` is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`` and linked into
one shared library next to this file. No torch extension machinery is used:
the library exports a plain C ABI (include/axs.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG_DIR), "include")
LIB_NAME = "libaxs_gb300.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)
BUILD_DIR = os.path.join(PKG_DIR, "_build")
HOST_DIR = os.path.join(PKG_DIR, "host")
DEMO_PATH = os.path.join(PKG_DIR, "axs_level_demo")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libaxs_gb300.so")
    return cand


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _fingerprint() -> str:
    h = hashlib.sha256()
    extra = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + sorted(glob.glob(os.path.join(HOST_DIR, "*.*")))
    for p in _sources() + extra + [os.path.join(INCLUDE, "axs.h")]:
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    h.update(" ".join(ARCH_FLAGS + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and return the path of libaxs_gb300.so."""
    stamp = LIB_PATH + ".stamp"
    fp = _fingerprint()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(DEMO_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == fp:
                return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD_DIR, os.path.basename(src).replace(".cu", ".o"))
        cmd = [cc, *ARCH_FLAGS, *NVCC_FLAGS, "-I", INCLUDE, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    build_host_demo(cc)
    with open(stamp, "w") as f:
        f.write(fp)
    return LIB_PATH


def build_host_demo(cc: str | None = None) -> str:
    """The C++ host driver (host/level_demo.cpp over host/axs_level.hpp),
    linked against libaxs_gb300.so next to it."""
    cc = cc or nvcc()
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(cc)))
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I", INCLUDE, "-I", os.path.join(cuda, "include"), "-I", HOST_DIR,
           os.path.join(HOST_DIR, "level_demo.cpp"), "-o", DEMO_PATH, "-L", PKG_DIR, "-laxs_gb300",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN",
           "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host demo build failed:\n{r.stdout}\n{r.stderr}")
    return DEMO_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
