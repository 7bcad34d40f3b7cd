"""Recipe: compile the reference's header-only helpers for the host.

Reads the reference tree in place (/root/reference, read-only) and writes only
oracle/_ref/libref.so (git-ignored).  Test infrastructure; the reference's
own build system is not used.  Skipped (returns None) where the reference
tree is absent, e.g. on the GPU machine.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SNISR_REFERENCE_TREE", "/root/reference")
OUT = os.path.join(HERE, "_ref", "libref.so")


def build(force: bool = False):
    inc = os.path.join(REF, "rendering", "src", "include")
    if not os.path.isdir(inc):
        return None
    src = os.path.join(HERE, "ref_harness.cpp")
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(src):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cuda_inc = "/usr/local/cuda/include"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           "-I", inc, "-I", cuda_inc, src, "-o", OUT + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
