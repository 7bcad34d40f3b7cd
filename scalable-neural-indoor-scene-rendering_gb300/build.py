"""Build recipe of libsnisr.so (CUDA kernels for sm_103a + C++ host code).

Compiles every translation unit of csrc/ in parallel with nvcc/g++ into
_build/, then links snisr/libsnisr.so.  No cmake, no torch extension
machinery: the library exposes a plain C ABI (include/snisr.h).

    python scalable-neural-indoor-scene-rendering_gb300/build.py [--force]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
OUT = os.path.join(PKG, "snisr", "libsnisr.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _sources():
    srcs = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cpp")):
            srcs.append(os.path.join(CSRC, f))
    return srcs


def _deps_mtime() -> float:
    m = os.path.getmtime(os.path.join(INCLUDE, "snisr.h"))
    for f in os.listdir(CSRC):
        m = max(m, os.path.getmtime(os.path.join(CSRC, f)))
    return m


def _compile(src: str, cuda: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    inc = ["-I", INCLUDE, "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-O3", "-lineinfo", "-std=c++17",
               "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC", *inc, "-c", src, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
               "-I", os.path.join(cuda, "include"), *inc, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= _deps_mtime():
        return OUT
    cuda = cuda_home()
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), max(2, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(lambda s: _compile(s, cuda), srcs))
    tmp = OUT + ".tmp"
    cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread",
           "-Xlinker", "--no-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    if verbose:
        print(f"built {OUT}")
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    try:
        build(force=a.force, verbose=True)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
