"""ctypes binding of libsnisr.so (the C ABI declared in include/snisr.h).

The library is the product: every GPU computation goes through it.  If the
shared object is missing this module raises instead of falling back to
anything else.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsnisr.so")

OK, INVALID_ARG, OOM, CUDA_ERROR, DEVICE_TIMEOUT, CORRUPT_SCENE, OVERFLOW, UNSUPPORTED = range(8)
F32, F16 = 0, 1
FORM_PLAIN_FP32, FORM_TC = 0, 1

STATUS_NAMES = {
    OK: "OK", INVALID_ARG: "INVALID_ARG", OOM: "OOM", CUDA_ERROR: "CUDA_ERROR",
    DEVICE_TIMEOUT: "DEVICE_TIMEOUT", CORRUPT_SCENE: "CORRUPT_SCENE", OVERFLOW: "OVERFLOW",
    UNSUPPORTED: "UNSUPPORTED",
}


class SceneDesc(C.Structure):
    _fields_ = [
        ("grid", C.c_int32 * 3),
        ("scene_min", C.c_float * 3),
        ("tile_size", C.c_float),
        ("res", C.c_int32),
        ("num_tiles", C.c_int32),
        ("tile_index", C.POINTER(C.c_int32)),
        ("occupancy", C.POINTER(C.c_uint64)),
        ("num_voxels", C.c_int64),
        ("voxel_corners", C.POINTER(C.c_int32)),
        ("num_vertices", C.c_int64),
        ("feat_dim", C.c_int32),
        ("feat_type", C.c_int32),
        ("vertex_feat", C.c_void_p),
        ("vertex_density", C.c_void_p),
        ("dir_freqs", C.c_int32),
        ("mlp_hidden", C.c_int32),
        ("mlp_layers", C.c_int32),
        ("mlp_params", C.POINTER(C.c_float)),
        ("num_mesh_vertices", C.c_int64),
        ("mesh_vertices", C.POINTER(C.c_float)),
        ("num_triangles", C.c_int64),
        ("mesh_faces", C.POINTER(C.c_int32)),
        ("step_vox", C.c_float),
        ("early_stop", C.c_float),
        ("start_offset_vox", C.c_float),
        ("max_samples_per_ray", C.c_int32),
        ("max_pixels", C.c_int32),
    ]


class SceneInfo(C.Structure):
    _fields_ = [
        ("num_voxels", C.c_int64), ("num_vertices", C.c_int64), ("num_triangles", C.c_int64),
        ("bvh_nodes", C.c_int64),
        ("num_tiles", C.c_int32), ("res", C.c_int32), ("feat_dim", C.c_int32), ("mlp_in", C.c_int32),
        ("mlp_hidden", C.c_int32), ("mlp_layers", C.c_int32), ("params_per_tile", C.c_int32),
        ("device_bytes", C.c_int64), ("sample_capacity", C.c_int64),
    ]


class Camera(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32),
        ("cx", C.c_float), ("cy", C.c_float), ("inv_focal", C.c_float),
        ("c2w", C.c_float * 12),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("traverse_threads", C.c_int32), ("scatter_blocks_per_sm", C.c_int32), ("mlp_ctas_per_sm", C.c_int32),
        ("train_march_threads", C.c_int32), ("train_fwd_warps", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


class SynthParams(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("grid", C.c_int32 * 3),
        ("tile_size", C.c_float),
        ("res", C.c_int32),
        ("feat_dim", C.c_int32),
        ("feat_type", C.c_int32),
        ("mlp_hidden", C.c_int32), ("mlp_layers", C.c_int32), ("dir_freqs", C.c_int32),
        ("num_boxes", C.c_int32),
        ("box_min", C.c_float), ("box_max", C.c_float),
        ("with_mesh", C.c_int32),
        ("mesh_cell", C.c_float),
        ("density_mean", C.c_float), ("density_std", C.c_float), ("feat_std", C.c_float),
        ("seed", C.c_uint64),
        ("round_weights_f16", C.c_int32),
    ]


P = C.c_void_p
FP = C.POINTER(C.c_float)
IP = C.POINTER(C.c_int32)

# name -> (restype, argtypes); pointers are passed as plain integers/void*.
_SIGNATURES = {
    "snisr_mlp_param_count": (C.c_int64, [C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "snisr_scene_create": (C.c_int, [C.POINTER(SceneDesc), C.c_int32, C.POINTER(P)]),
    "snisr_scene_destroy": (C.c_int, [P]),
    "snisr_scene_get_info": (C.c_int, [P, C.POINTER(SceneInfo)]),
    "snisr_scene_check": (C.c_int, [P, P]),
    "snisr_scene_set_mlp": (C.c_int, [P, P, P]),
    "snisr_render": (C.c_int, [P, C.POINTER(Camera), C.c_int32, P, P, P, P]),
    "snisr_render_host": (C.c_int, [P, C.POINTER(Camera), C.c_int32, P, P, P, P]),
    "snisr_camera_rays": (C.c_int, [C.POINTER(Camera), P, P]),
    "snisr_proxy_hit": (C.c_int, [P, P, P, C.c_int64, P, P, P]),
    "snisr_trace_voxels": (C.c_int, [P, P, P, C.c_int64, C.c_int32, P, P, P]),
    "snisr_render_rays": (C.c_int, [P, P, P, C.c_int64, C.c_int32, P, P, P, P]),
    "snisr_render_rays_noalloc": (C.c_int, [P, P, P, C.c_int64, P, P, P, P]),
    "snisr_train_forward": (C.c_int, [P, P, P, P, P, P, P, C.c_int64, C.c_int32, P, P, P]),
    "snisr_train_backward": (C.c_int, [P, P, P, P, P, P, P, C.c_int64, C.c_int32, C.c_uint64, P, P, P, P, P, P]),
    "snisr_op_compute_rays": (C.c_int, [P, P, C.c_int32, C.c_int32, P, P]),
    "snisr_op_tracing_tiles": (C.c_int, [P, C.c_int64, P, P, P, P, P, C.c_float, C.c_int32, P, P]),
    "snisr_op_sample_sparse": (C.c_int, [P, P, C.c_int64, P, C.c_float, C.c_float, C.c_float, C.c_float,
                                         C.c_int32, C.c_int32, P, P, P]),
    "snisr_op_inverse_z_sampling": (C.c_int, [P, P, P, P, C.c_int64, C.c_int32, C.c_int32, P, P, P]),
    "snisr_op_integrate_points": (C.c_int, [P, P, C.c_int64, C.c_float, P, P, P]),
    "snisr_op_sort_by_key": (C.c_int, [P, P, P, C.c_int64, C.POINTER(C.c_int64), P]),
    "snisr_op_assign_pixels": (C.c_int, [P, P, P, C.c_int64, P, P, P]),
    "snisr_op_inference_mlp_param_count": (C.c_int32, []),
    "snisr_op_rendering_diffuse_octree": (C.c_int, [P, P, C.c_int64, C.c_int32, P, P, P, P, P, P, P, P, C.c_int32,
                                                    C.c_float, C.c_float, C.c_float, C.c_int32, C.c_float, C.c_float,
                                                    C.c_int32, P, P, P, C.c_int32, P]),
    "snisr_render_host_async": (C.c_int, [P, C.POINTER(Camera), C.c_int32, P, P, P, P]),
    "snisr_render_host_wait": (C.c_int, [P]),
    "snisr_op_train_rays": (C.c_int, [P, P, C.c_int32, C.c_int32, P, P, P]),
    "snisr_op_train_tracing_tiles": (C.c_int, [P, P, C.c_int64, P, C.POINTER(C.c_int32), C.POINTER(C.c_float),
                                               C.c_float, C.c_int32, P, P]),
    "snisr_scene_double_hits": (C.c_int, [P, P, P, P, C.c_int64, C.c_int32, P, P]),
    "snisr_op_train_bgdepth": (C.c_int, [C.c_int32, P, P, C.c_int64, C.c_int32, P, P, P]),
    "snisr_op_gen_diffuse": (C.c_int, [P, C.c_int32, P, P, P, P, P, P, P, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_int32, P, P, P]),
    "snisr_op_sample_bg": (C.c_int, [P, P, P, C.c_int64, C.c_int32, C.c_float, P, C.c_float, P, P]),
    "snisr_op_patch_capacity": (C.c_int64, [C.c_int32, C.c_int32, C.c_int32]),
    "snisr_op_patch_rows": (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32, P, P, P, P, P, P, P, P, P]),
    "snisr_op_transparency_statistic": (C.c_int, [P, P, C.c_int64, C.c_int32, P, C.c_float, C.c_float, C.c_float, P,
                                                  P, P, P]),
    "snisr_op_dilate_boundary": (C.c_int, [P, C.c_int32, P]),
    "snisr_op_prune_flags": (C.c_int, [P, P, P, C.c_int32, C.c_int32, C.c_float, C.c_float, P, P]),
    "snisr_op_pack_occupancy": (C.c_int, [P, C.c_int32, P, P, P]),
    "snisr_op_inference_mlp": (C.c_int, [C.c_int32, C.c_int32, C.c_float, C.c_float, P, C.c_int32, P, P, P, P, P, P, P,
                                         P, P, P]),
    "snisr_synth_create": (C.c_int, [C.POINTER(SynthParams), C.POINTER(P), C.POINTER(SceneDesc)]),
    "snisr_synth_destroy": (C.c_int, [P]),
    "snisr_synth_camera": (C.c_int, [P, C.c_uint64, C.c_int32, C.c_int32, C.c_float, C.POINTER(Camera)]),
    "snisr_diag_mma": (C.c_int, [P, P, P, C.c_int32, C.c_int32, C.c_int32, P]),
    "snisr_diag_wait_timeout": (C.c_int, [C.c_int64, C.POINTER(C.c_int64), P]),
    "snisr_diag_march_math": (C.c_int, [C.c_int32, P, C.c_int64, P, P]),
    "snisr_diag_block_distance": (C.c_int, [P, C.c_int32, P]),
    "snisr_scene_set_profiling": (C.c_int, [P, C.c_int32]),
    "snisr_scene_stage_times": (C.c_int, [P, P, C.c_int32, P]),
    "snisr_scene_frame_stats": (C.c_int, [P, P, P]),
    "snisr_scene_frame_footprint": (C.c_int, [P, P, P]),
    "snisr_scene_get_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "snisr_scene_set_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "snisr_scene_autotune_render": (C.c_int, [P, C.POINTER(Camera), C.c_int32, P, C.POINTER(Tuning), FP]),
    "snisr_scene_autotune_train": (C.c_int, [P, P, P, P, P, P, P, C.c_int64, C.c_int32, P, C.POINTER(Tuning), FP]),
    "snisr_last_error_string": (C.c_char_p, []),
    "snisr_version": (C.c_char_p, []),
    "snisr_abi_version": (C.c_int32, []),
}

_lib = None


class SnisrError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def lib() -> C.CDLL:
    """Loads libsnisr.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "`python scalable-neural-indoor-scene-rendering_gb300/build.py` (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.snisr_abi_version() != 1:
            raise RuntimeError("libsnisr ABI version mismatch")
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != OK:
        raise SnisrError(status, lib().snisr_last_error_string().decode())


def exported_symbols():
    return sorted(_SIGNATURES)
