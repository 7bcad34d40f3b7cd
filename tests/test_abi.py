"""CPU checks of the C ABI (no GPU calls): the library loads, exports every
entry point declared in include/snisr.h, validates arguments before touching
CUDA, and the seeded scene generator is deterministic."""
import ctypes as C
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

import snisr
from snisr import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "snisr.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(snisr_[a-z0-9_]+)\s*\(", src)))


def test_header_functions_are_exported():
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (snisr_[a-z0-9_]+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing


def test_ctypes_table_covers_header():
    assert set(declared_functions()) <= set(_lib.exported_symbols())


def test_abi_version_and_strings():
    L = snisr.lib()
    assert L.snisr_abi_version() == 1
    assert b"sm_103a" in L.snisr_version()


def test_mlp_param_count():
    L = snisr.lib()
    assert L.snisr_mlp_param_count(32, 4, 64, 3) == (59 * 64 + 64) + 2 * (64 * 64 + 64) + (64 * 3 + 3)
    assert L.snisr_mlp_param_count(16, 4, 32, 2) == (43 * 32 + 32) + (32 * 32 + 32) + (32 * 3 + 3)


def test_invalid_arguments_are_reported_without_cuda():
    L = snisr.lib()
    h = C.c_void_p()
    assert L.snisr_scene_create(None, 0, C.byref(h)) == _lib.INVALID_ARG
    assert b"desc" in L.snisr_last_error_string()
    d = _lib.SceneDesc()
    assert L.snisr_scene_create(C.byref(d), 0, C.byref(h)) == _lib.INVALID_ARG  # zero grid
    s = snisr.SynthScene(snisr.CFG1)
    bad = _lib.SceneDesc.from_buffer_copy(s.desc)
    bad.res = 30
    assert L.snisr_scene_create(C.byref(bad), 0, C.byref(h)) == _lib.INVALID_ARG
    bad = _lib.SceneDesc.from_buffer_copy(s.desc)
    bad.mlp_hidden = 48
    assert L.snisr_scene_create(C.byref(bad), 0, C.byref(h)) == _lib.UNSUPPORTED
    bad = _lib.SceneDesc.from_buffer_copy(s.desc)
    bad.dir_freqs = 6
    assert L.snisr_scene_create(C.byref(bad), 0, C.byref(h)) == _lib.UNSUPPORTED
    # entry points reject null scenes and bad sizes before any CUDA call
    assert L.snisr_render(None, None, 0, None, None, None, None) == _lib.INVALID_ARG
    assert L.snisr_scene_check(None, None) == _lib.INVALID_ARG
    assert L.snisr_op_sample_sparse(None, None, 4, None, 0, 0, 0, 1.0, 8, 4, None, None, None) == _lib.INVALID_ARG
    assert L.snisr_op_tracing_tiles(None, 4, None, None, None, None, None, 1.0, 0, None, None) == _lib.INVALID_ARG
    assert L.snisr_diag_mma(None, None, None, 48, 0, 0, None) == _lib.INVALID_ARG
    t = _lib.Tuning(128, 16, 0, 128, 2)
    assert L.snisr_scene_set_tuning(None, C.byref(t)) == _lib.INVALID_ARG
    assert L.snisr_scene_get_tuning(None, C.byref(t)) == _lib.INVALID_ARG


def test_python_raises_on_error_status():
    with pytest.raises(snisr.SnisrError):
        _lib.check(_lib.INVALID_ARG)


def _digest(s):
    a = s.arrays()
    h = hashlib.sha256()
    for k in sorted(a):
        h.update(k.encode())
        h.update(np.ascontiguousarray(a[k]).tobytes())
    return h.hexdigest()


def test_synthetic_scene_is_deterministic():
    a, b = snisr.SynthScene(snisr.CFG1), snisr.SynthScene(snisr.CFG1)
    assert _digest(a) == _digest(b)
    ca, cb = a.camera(3), b.camera(3)
    assert bytes(ca) == bytes(cb)


def test_synthetic_scene_shapes_cfg1():
    s = snisr.SynthScene(snisr.CFG1)
    d = s.desc
    assert (d.grid[0], d.grid[1], d.grid[2], d.res, d.feat_dim, d.num_tiles) == (1, 1, 1, 64, 16, 1)
    a = s.arrays()
    occ_bits = int(sum(bin(int(w)).count("1") for w in a["occupancy"]))
    assert occ_bits == d.num_voxels
    assert a["voxel_corners"].shape == (d.num_voxels, 8)
    assert a["voxel_corners"].min() >= 0 and a["voxel_corners"].max() < d.num_vertices
    assert 0.01 < s.occupancy_fraction() < 0.12
    # features ~N(0, 0.1), density logits ~N(2, 1)
    assert abs(float(a["vertex_feat"].std()) - 0.1) < 0.01
    assert abs(float(a["vertex_density"].mean()) - 2.0) < 0.05
    assert d.num_triangles == 0


def test_synthetic_mesh_cfg2_sizes():
    s = snisr.SynthScene(snisr.CFG2.replace(res=32))
    d = s.desc
    assert 150_000 < d.num_triangles < 260_000
    a = s.arrays()
    assert a["mesh_faces"].max() < d.num_mesh_vertices
