"""Recipe: compile the reference's own code for the parity checks.

1. The reference's header-only helpers for the host: oracle/_ref/libref.so.
2. The reference's CUDA kernel sources for sm_103a, device code only, one
   cubin per source file (oracle/_ref/<name>.cubin), with the nvcc flags its
   torch CUDAExtension builds pass (torch's COMMON_NVCC_FLAGS; no fast math).
   The cubins carry no host code, so they travel to the GPU host as they are;
   tests/refgpu.py loads them through the CUDA driver API.

Reads the reference tree in place (/root/reference, read-only) and writes
only under oracle/_ref/ (git-ignored).  Test infrastructure; the reference's
own build system is not used.  Skipped (returns None) where the reference
tree is absent, e.g. on the GPU host.
"""
from __future__ import annotations

import concurrent.futures
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SNISR_REFERENCE_TREE", "/root/reference")
OUT = os.path.join(HERE, "_ref", "libref.so")


# cubin name -> reference source file (path within the reference tree)
CUBINS = {
    "compute_rays": "rendering/src/compute_rays.cu",
    "raytile_tracing": "rendering/src/raytile_tracing.cu",
    "raydiffuse_render_octree_fp16": "rendering/src/raydiffuse_render_octree_fp16.cu",
    "rayreflection_render": "rendering/src/rayreflection_render.cu",
    "sampling": "rendering/src/sampling.cu",
    "volume_rendering": "rendering/src/volume_rendering.cu",
    "reorder": "rendering/src/reorder.cu",
    "Sample_kernel": "training/src/Sample_kernel.cu",
    "Helper_kernel": "training/src/Helper_kernel.cu",
    "cuda_func": "training/src/cuda_func.cu",
}
# rayreflection_render.cu:5-6 include two ATen quantized CPU headers that it
# does not use and that this torch no longer ships; empty stand-ins are found
# first on the include path.
_STUBS = ("ATen/native/quantized/cpu/embedding_packed_params.h", "ATen/native/quantized/cpu/fbgemm_utils.h")
# training/src/cuda_func.cu's host code (image and .npy file loading, a
# progress bar) uses OpenCV, cnpy and tqdm, which are not installed.  Only its
# device code goes into the cubin, but nvcc still parses the host code, so
# these stand-ins declare the few names it uses (nothing is defined: no host
# code is compiled or linked).
_DECL_STUBS = {
    "opencv2/opencv.hpp": """#pragma once
#include <string>
#define CV_8UC3 16
#define CV_32FC3 21
namespace cv {
enum { COLOR_BGR2RGB = 4, COLOR_RGB2BGR = 4 };
struct Mat {
  unsigned char* data;
  bool isContinuous() const;
  void convertTo(Mat& dst, int type, double alpha = 1.0, double beta = 0.0) const;
  static Mat zeros(int rows, int cols, int type);
};
Mat imread(const std::string& path, int flags = 1);
bool imwrite(const std::string& path, const Mat& img);
void cvtColor(const Mat& src, Mat& dst, int code);
}  // namespace cv
""",
    "cnpy.h": """#pragma once
#include <string>
namespace cnpy {
struct NpyArray {
  template <class T> T* data();
};
NpyArray npy_load(std::string path);
}  // namespace cnpy
""",
    "tqdm.h": """#pragma once
class tqdm {
 public:
  void progress(int i, int n);
  void finish();
};
""",
}


def cubin_path(name: str) -> str:
    return os.path.join(HERE, "_ref", name + ".cubin")


def _nvcc_cubin(name: str, src: str, incs: list, flags: list) -> str:
    out = cubin_path(name)
    cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-w"] + flags
    for d in incs:
        cmd += ["-I", d]
    cmd += [src, "-o", out + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def build_cubins(force: bool = False):
    """The reference's kernels as sm_103a cubins; None without the reference tree."""
    if not os.path.isdir(os.path.join(REF, "rendering", "src")):
        return None
    from torch.utils.cpp_extension import COMMON_NVCC_FLAGS, include_paths
    import sysconfig
    stub = os.path.join(HERE, "_ref", "stub")
    for h in _STUBS:
        p = os.path.join(stub, h)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        if not os.path.exists(p):
            open(p, "w").close()
    for h, text in _DECL_STUBS.items():
        p = os.path.join(stub, h)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        if not os.path.exists(p) or open(p).read() != text:
            with open(p, "w") as f:
                f.write(text)
    jobs = []
    for name, rel in CUBINS.items():
        src = os.path.join(REF, rel)
        out = cubin_path(name)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        incs = [stub, os.path.join(os.path.dirname(src), "include")] + list(include_paths()) + \
            [sysconfig.get_paths()["include"]]
        jobs.append((name, src, incs))
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for f in [ex.submit(_nvcc_cubin, n, s, i, list(COMMON_NVCC_FLAGS)) for n, s, i in jobs]:
            f.result()
    return {n: cubin_path(n) for n in CUBINS}


def build(force: bool = False):
    inc = os.path.join(REF, "rendering", "src", "include")
    if not os.path.isdir(inc):
        return None
    build_cubins(force)
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
