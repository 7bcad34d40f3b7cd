"""The camera-frame ray order (csrc/kernels.h: RayOrder, ray_pixel), checked
on the host: a permutation of the pixels for tiled and untiled image sizes,
each warp's 32 rays one 4 x 8 pixel tile, each group of 4 warps one 8 x 16
block where the image divides into them, the caller's rays in their own
order.  Frames rendered in this order are compared pixel by pixel with the
oracle by the GPU render tests."""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "scalable-neural-indoor-scene-rendering_gb300", "csrc")
EXE = os.path.join(HERE, "cpp", "_build", "ray_order")


def test_ray_order_is_a_tiled_permutation():
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda = os.environ.get("CUDA_HOME") or os.path.dirname(os.path.dirname(nvcc))
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(cuda, "include"), "-I",
           os.path.join(ROOT, "include"), "-I", CSRC, os.path.join(HERE, "cpp", "ray_order.cpp"), "-o", EXE]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([EXE], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
