"""snisr — GB300-native sparse-voxel tile renderer (host-side Python mirror).

The compute path is libsnisr.so (hand-written sm_103a kernels behind a C ABI,
include/snisr.h).  This package only marshals arguments: it has no compute
fallback of its own.
"""
from . import _lib
from ._lib import FORM_PLAIN_FP32, FORM_TC, F16, F32, Camera, SceneDesc, SnisrError, lib
from .configs import ALL as CONFIGS, CFG1, CFG2, CFG3, CFG4, CFG5, Config
from .scene import Scene, SynthScene, camera_rays
from . import ops

__all__ = [
    "FORM_PLAIN_FP32", "FORM_TC", "F16", "F32", "Camera", "SceneDesc", "SnisrError", "lib", "CONFIGS", "CFG1", "CFG2", "CFG3",
    "CFG4", "CFG5", "Config", "Scene", "SynthScene", "camera_rays", "build",
]


def build(force: bool = False) -> str:
    """Compiles libsnisr.so in-tree for sm_103a (see ../build.py)."""
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "build.py")
    spec = importlib.util.spec_from_file_location("snisr_build", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)
