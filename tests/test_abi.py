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
    # a march step too small to advance the tile-local position is rejected
    # (the march would otherwise repeat one sample forever)
    for step in (1e-9, 1.0 / 2048, float("nan"), 100.0):
        bad = _lib.SceneDesc.from_buffer_copy(s.desc)
        bad.step_vox = step
        assert L.snisr_scene_create(C.byref(bad), 0, C.byref(h)) == _lib.INVALID_ARG
        assert b"step_vox" in L.snisr_last_error_string()
    # entry points reject null scenes and bad sizes before any CUDA call
    assert L.snisr_render(None, None, 0, None, None, None, None) == _lib.INVALID_ARG
    assert L.snisr_scene_check(None, None) == _lib.INVALID_ARG
    assert L.snisr_op_sample_sparse(None, None, 4, None, 0, 0, 0, 1.0, 8, 4, None, None, None) == _lib.INVALID_ARG
    assert L.snisr_op_tracing_tiles(None, 4, None, None, None, None, None, 1.0, 0, None, None) == _lib.INVALID_ARG
    assert L.snisr_diag_mma(None, None, None, 48, 0, 0, None) == _lib.INVALID_ARG
    waited = C.c_int64()
    assert L.snisr_diag_wait_timeout(0, C.byref(waited), None) == _lib.INVALID_ARG
    assert L.snisr_diag_wait_timeout(11_000_000_000, C.byref(waited), None) == _lib.INVALID_ARG
    assert L.snisr_diag_wait_timeout(1000, None, None) == _lib.INVALID_ARG
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


def test_op_argument_validation_without_cuda():
    """The drop-in ops reject bad sizes and null buffers (and return at once
    for empty inputs) before any CUDA call."""
    L = snisr.lib()
    OK, BAD = _lib.OK, _lib.INVALID_ARG
    P = C.c_void_p
    fake = P(16)  # never dereferenced: every call below returns before a launch
    cnt = C.c_int64(-1)
    # sort_by_key / assign_pixels / inference_mlp (specular pass)
    assert L.snisr_op_sort_by_key(None, None, None, 0, C.byref(cnt), None) == OK and cnt.value == 0
    assert L.snisr_op_sort_by_key(None, None, None, 5, C.byref(cnt), None) == BAD
    assert L.snisr_op_sort_by_key(fake, fake, fake, -1, C.byref(cnt), None) == BAD
    assert L.snisr_op_assign_pixels(None, None, None, 0, None, None, None) == OK
    assert L.snisr_op_assign_pixels(None, None, None, 3, None, None, None) == BAD
    bufs = [None] * 9  # transparency, qpix, pixel_starts, centers, samples, rays_d, params, results, err
    assert len(_lib._SIGNATURES["snisr_op_inference_mlp"][1]) == 16
    assert L.snisr_op_inference_mlp(16, 0, 0.1, 0.01, None, 16, *bufs, None) == OK
    assert L.snisr_op_inference_mlp(0, 4, 0.1, 0.01, None, 16, *bufs, None) == BAD
    assert L.snisr_op_inference_mlp(16, 4, 0.1, 0.01, None, 16, *bufs, None) == BAD
    # FP16 octree diffuse renderer
    oct_args = lambda npix, K, tile: (None, None, npix, K) + (None,) * 8 + (1, tile, 0.1, 0.02, 18, 0.8, 0.01, 0,
                                                                           None, None, None, 0, None)
    assert L.snisr_op_rendering_diffuse_octree(*oct_args(0, 30, 6.4)) == OK
    assert L.snisr_op_rendering_diffuse_octree(*oct_args(10, 30, 6.4)) == BAD  # null buffers
    assert L.snisr_op_rendering_diffuse_octree(*oct_args(10, 0, 6.4)) == BAD
    assert L.snisr_op_rendering_diffuse_octree(*oct_args(10, 30, 0.0)) == BAD
    tiny = lambda step: (fake, fake, 10, 30) + (fake,) * 8 + (1, 6.4, 0.1, step, 18, 0.8, 0.01, 0, fake, fake, fake,
                                                              0, None)
    assert L.snisr_op_rendering_diffuse_octree(*tiny(1e-9)) == BAD  # step < voxel / 1024 would never advance z
    assert b"sample_step" in L.snisr_last_error_string()
    neg_width = list(tiny(0.02))
    neg_width[-2] = -1
    assert L.snisr_op_rendering_diffuse_octree(*neg_width) == BAD
    # pruning
    assert L.snisr_op_transparency_statistic(None, None, 0, 18, None, 1.0, 0.0625, 0.006, None, None, None,
                                             None) == OK
    assert L.snisr_op_transparency_statistic(None, None, 5, 18, None, 1.0, 0.0625, 0.006, None, None, None,
                                             None) == BAD
    assert L.snisr_op_transparency_statistic(fake, fake, 5, 2000, fake, 1.0, 0.0625, 0.006, fake, fake, fake,
                                             None) == BAD
    assert L.snisr_op_transparency_statistic(fake, fake, 5, 18, fake, 1.0, 0.0625, 1e-9, fake, fake, fake,
                                             None) == BAD
    assert b"sample_step" in L.snisr_last_error_string()
    assert L.snisr_op_dilate_boundary(None, 18, None) == BAD
    assert L.snisr_op_dilate_boundary(fake, 0, None) == BAD
    assert L.snisr_op_prune_flags(fake, fake, None, 18, 4, 0.5, 0.0, fake, None) == BAD  # 18 % 4 != 0
    assert L.snisr_op_prune_flags(None, fake, None, 16, 4, 0.5, 0.0, fake, None) == BAD
    assert L.snisr_op_pack_occupancy(fake, 16, None, fake, None) == BAD
    # training-ray preparation
    assert L.snisr_op_train_rays(fake, fake, 0, 640, fake, fake, None) == BAD
    assert L.snisr_op_train_rays(None, fake, 480, 640, fake, fake, None) == BAD
    shape = (C.c_int32 * 3)(4, 4, 1)
    smin = (C.c_float * 3)(0, 0, 0)
    assert L.snisr_op_train_tracing_tiles(None, None, 0, None, shape, smin, 3.0, 30, None, None) == OK
    assert L.snisr_op_train_tracing_tiles(fake, fake, 8, fake, shape, smin, 3.0, 0, fake, None) == BAD
    assert L.snisr_op_train_tracing_tiles(fake, fake, 8, fake, (C.c_int32 * 3)(0, 4, 1), smin, 3.0, 30, fake,
                                          None) == BAD
    assert L.snisr_op_train_bgdepth(0, None, None, 0, 30, None, None, None) == OK
    assert L.snisr_op_train_bgdepth(0, None, None, 8, 30, None, None, None) == BAD
    assert L.snisr_op_gen_diffuse(None, 0, fake, fake, fake, fake, None, None, None, 30, 4, 1, 640, fake, fake,
                                  None) == BAD
    assert L.snisr_op_gen_diffuse(None, 0, fake, fake, fake, fake, None, None, None, 30, 4, 480, 640, fake, fake,
                                  None) == BAD  # images missing for 4 views
    assert L.snisr_op_sample_bg(None, None, None, 0, 16, 0.5, None, 3.0, None, None) == OK
    assert L.snisr_op_sample_bg(fake, fake, fake, 8, 1, 0.5, fake, 3.0, fake, None) == BAD
    assert L.snisr_op_patch_capacity(720, 1280, 7) == ((720 - 7 - 3 + 6) // 7) * ((1280 - 7 - 3 + 6) // 7)
    assert L.snisr_op_patch_capacity(720, 1280, 6) == -1 and L.snisr_op_patch_capacity(5, 5, 7) == 0
    assert L.snisr_op_patch_rows(fake, 720, 1280, 8, fake, fake, fake, fake, fake, fake, fake, fake, None) == BAD
    assert L.snisr_scene_double_hits(None, fake, fake, fake, 8, 30, fake, None) == BAD
