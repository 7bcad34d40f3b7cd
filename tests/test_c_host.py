"""The C ABI from a C++ host (tests/cpp/render_host.cpp): it compiles
against include/snisr.h and links libsnisr.so with no Python or PyTorch
(CPU test), and on the GPU its frame equals the Python binding's render of
the same seeded scene and camera (colour max-abs <= 1e-6: the MLP's colour
atomics add in any order; depth and opacity bit-exact)."""
import os
import subprocess

import numpy as np
import pytest

import snisr
from snisr import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cpp", "render_host.cpp")
EXE = os.path.join(HERE, "cpp", "_build", "render_host")


def _build():
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", libdir, "-lsnisr", f"-Wl,-rpath,{libdir}", "-o", EXE]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return EXE


def test_c_host_compiles_and_links():
    exe = _build()
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 2 and "usage" in out.stderr


@pytest.mark.gpu
def test_c_host_frame_matches_python(cuda, tmp_path):
    exe = _build()
    cfg = snisr.CFG1
    s = snisr.SynthScene(cfg)
    cam = s.camera(2)
    (tmp_path / "p.bin").write_bytes(bytes(cfg.synth_params()))
    (tmp_path / "c.bin").write_bytes(bytes(cam))
    out = subprocess.run([exe, str(tmp_path / "p.bin"), str(tmp_path / "c.bin"), str(tmp_path / "o.bin")],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    n = cam.width * cam.height
    raw = np.fromfile(tmp_path / "o.bin", np.float32)
    assert raw.size == 5 * n
    rgb, depth, opac = raw[:3 * n].reshape(n, 3), raw[3 * n:4 * n], raw[4 * n:]
    sc = snisr.Scene(s.desc)
    try:
        ref = [t.cpu().numpy() for t in sc.render(cam, snisr.FORM_TC)]
        sc.check()
    finally:
        sc.close()
    assert np.abs(rgb - ref[0].reshape(n, 3)).max() <= 1e-6
    assert np.array_equal(depth, ref[1].reshape(n)) and np.array_equal(opac, ref[2].reshape(n))
    assert opac.max() > 0.5
