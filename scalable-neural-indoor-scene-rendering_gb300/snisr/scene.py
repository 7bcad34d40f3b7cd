"""Host-side scene objects.

SynthScene  seeded synthetic scene generated by the library (host arrays).
Scene       device-resident scene (snisr_scene_create) with render entry
            points taking torch CUDA tensors; the role FRender plays for the
            reference renderer (rendering/src/__init__.py:98-341).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .configs import Config


def _np(ptr, count, dtype):
    if count == 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    buf = C.cast(ptr, C.POINTER(C.c_uint8 * (count * np.dtype(dtype).itemsize))).contents
    return np.frombuffer(buf, dtype=dtype, count=count)


class SynthScene:
    """Synthetic scene for a benchmark configuration (host memory)."""

    def __init__(self, cfg: Config, max_pixels: int | None = None, max_samples_per_ray: int = 48):
        L = _lib.lib()
        self.cfg = cfg
        self._handle = C.c_void_p()
        self.desc = _lib.SceneDesc()
        p = cfg.synth_params()
        _lib.check(L.snisr_synth_create(C.byref(p), C.byref(self._handle), C.byref(self.desc)))
        self.desc.max_pixels = max_pixels if max_pixels is not None else cfg.width * cfg.height
        self.desc.max_samples_per_ray = max_samples_per_ray

    def close(self):
        if self._handle:
            _lib.lib().snisr_synth_destroy(self._handle)
            self._handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def camera(self, pose: int, width: int | None = None, height: int | None = None) -> _lib.Camera:
        cam = _lib.Camera()
        _lib.check(_lib.lib().snisr_synth_camera(self._handle, self.cfg.pose_seed(pose), width or self.cfg.width,
                                                  height or self.cfg.height, self.cfg.fov, C.byref(cam)))
        return cam

    # numpy views of the description (valid while the scene lives)
    def arrays(self) -> dict:
        d = self.desc
        F = d.feat_dim
        ft = np.float16 if d.feat_type == _lib.F16 else np.float32
        ndense = d.grid[0] * d.grid[1] * d.grid[2]
        words = d.res ** 3 // 64
        P = int(_lib.lib().snisr_mlp_param_count(F, d.dir_freqs, d.mlp_hidden, d.mlp_layers))
        return {
            "tile_index": _np(d.tile_index, ndense, np.int32),
            "occupancy": _np(d.occupancy, d.num_tiles * words, np.uint64),
            "voxel_corners": _np(d.voxel_corners, d.num_voxels * 8, np.int32).reshape(-1, 8),
            "vertex_feat": _np(d.vertex_feat, d.num_vertices * F, ft).reshape(-1, F),
            "vertex_density": _np(d.vertex_density, d.num_vertices, ft),
            "mlp_params": _np(d.mlp_params, d.num_tiles * P, np.float32).reshape(d.num_tiles, P),
            "mesh_vertices": _np(d.mesh_vertices, d.num_mesh_vertices * 3, np.float32).reshape(-1, 3),
            "mesh_faces": _np(d.mesh_faces, d.num_triangles * 3, np.int32).reshape(-1, 3),
        }

    def occupancy_fraction(self) -> float:
        d = self.desc
        return d.num_voxels / float(d.num_tiles * d.res ** 3) if d.num_tiles else 0.0


def _ptr(t) -> int:
    return 0 if t is None else t.data_ptr()


def _stream(stream) -> int:
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return stream.cuda_stream


class Scene:
    """Device-resident scene; renders through the C ABI."""

    def __init__(self, desc: _lib.SceneDesc, device: int = 0):
        self._h = C.c_void_p()
        _lib.check(_lib.lib().snisr_scene_create(C.byref(desc), device, C.byref(self._h)))
        self.device = device
        self.info = _lib.SceneInfo()
        _lib.check(_lib.lib().snisr_scene_get_info(self._h, C.byref(self.info)))

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            _lib.lib().snisr_scene_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, stream=None):
        _lib.check(_lib.lib().snisr_scene_check(self._h, _stream(stream)))

    def set_profiling(self, enable: bool):
        _lib.check(_lib.lib().snisr_scene_set_profiling(self._h, 1 if enable else 0))

    def stage_times(self):
        """Per-stage ms of the last frame (see snisr_scene_stage_times)."""
        buf = (C.c_float * 8)()
        n = C.c_int32()
        _lib.check(_lib.lib().snisr_scene_stage_times(self._h, buf, 8, C.byref(n)))
        return [buf[i] for i in range(n.value)]

    def frame_stats(self, stream=None):
        out = (C.c_int64 * 4)()
        _lib.check(_lib.lib().snisr_scene_frame_stats(self._h, out, _stream(stream)))
        return {"samples": out[0], "voxel_steps": out[1], "reserved": out[2], "chunks": out[3]}

    def tuning(self) -> dict:
        """Launch shapes in use (snisr_tuning fields)."""
        t = _lib.Tuning()
        _lib.check(_lib.lib().snisr_scene_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw):
        """Sets launch-shape knobs by name; the others keep their values."""
        t = _lib.Tuning()
        _lib.check(_lib.lib().snisr_scene_get_tuning(self._h, C.byref(t)))
        for k, v in kw.items():
            if not hasattr(t, k):
                raise KeyError(k)
            setattr(t, k, int(v))
        _lib.check(_lib.lib().snisr_scene_set_tuning(self._h, C.byref(t)))

    def autotune_render(self, cam: _lib.Camera, reps: int = 3, stream=None):
        """Times launch shapes of the TC render of `cam`, keeps the fastest.
        Returns (tuning dict, ms per frame)."""
        t = _lib.Tuning()
        ms = C.c_float()
        _lib.check(_lib.lib().snisr_scene_autotune_render(self._h, C.byref(cam), int(reps), _stream(stream),
                                                          C.byref(t), C.byref(ms)))
        return t.as_dict(), float(ms.value)

    def autotune_train(self, vfeat, vdens, mlp, origins, dirs, ray_tile, reps: int = 3, stream=None):
        """Times launch shapes of the TC training step on this batch, keeps the
        fastest.  Returns (tuning dict, ms per step)."""
        t = _lib.Tuning()
        ms = C.c_float()
        _lib.check(_lib.lib().snisr_scene_autotune_train(
            self._h, _ptr(vfeat), _ptr(vdens), _ptr(mlp), _ptr(origins), _ptr(dirs), _ptr(ray_tile),
            int(origins.shape[0]), int(reps), _stream(stream), C.byref(t), C.byref(ms)))
        return t.as_dict(), float(ms.value)

    def set_mlp(self, params, stream=None):
        """Replaces the per-tile MLP parameters ([NT, P] FP32 CUDA tensor)."""
        if not params.is_cuda or not params.is_contiguous():
            raise RuntimeError("params must be a contiguous CUDA tensor")
        _lib.check(_lib.lib().snisr_scene_set_mlp(self._h, _ptr(params), _stream(stream)))

    def frame_footprint(self, stream=None):
        """Distinct voxels / vertices read by the last tensor-core frame."""
        out = (C.c_int64 * 2)()
        _lib.check(_lib.lib().snisr_scene_frame_footprint(self._h, out, _stream(stream)))
        return {"voxels": out[0], "vertices": out[1]}

    def render(self, cam: _lib.Camera, form: int = _lib.FORM_TC, out=None, stream=None):
        import torch
        n = cam.width * cam.height
        dev = torch.device("cuda", self.device)
        if out is None:
            out = (torch.empty(n, 3, device=dev), torch.empty(n, device=dev), torch.empty(n, device=dev))
        rgb, depth, opac = out
        _lib.check(_lib.lib().snisr_render(self._h, C.byref(cam), form, _ptr(rgb), _ptr(depth), _ptr(opac),
                                           _stream(stream)))
        return rgb, depth, opac

    def render_host(self, cam: _lib.Camera, form: int, rgb_h, depth_h, opac_h, stream=None):
        """Renders into host (ideally pinned) tensors; synchronises."""
        _lib.check(_lib.lib().snisr_render_host(self._h, C.byref(cam), form, _ptr(rgb_h), _ptr(depth_h),
                                                _ptr(opac_h), _stream(stream)))

    def render_host_async(self, cam: _lib.Camera, form: int, rgb_h, depth_h, opac_h, stream=None):
        """Pipelined host-output render (see snisr_render_host_async): the host
        tensors of a call are complete after the second following call or
        after render_host_wait()."""
        _lib.check(_lib.lib().snisr_render_host_async(self._h, C.byref(cam), form, _ptr(rgb_h), _ptr(depth_h),
                                                      _ptr(opac_h), _stream(stream)))

    def render_host_wait(self):
        _lib.check(_lib.lib().snisr_render_host_wait(self._h))

    def render_rays(self, origins, dirs, form: int = _lib.FORM_TC, stream=None):
        import torch
        n = origins.shape[0]
        rgb = torch.empty(n, 3, device=origins.device)
        depth = torch.empty(n, device=origins.device)
        opac = torch.empty(n, device=origins.device)
        _lib.check(_lib.lib().snisr_render_rays(self._h, _ptr(origins), _ptr(dirs), n, form, _ptr(rgb),
                                                _ptr(depth), _ptr(opac), _stream(stream)))
        return rgb, depth, opac

    def trace_voxels(self, origins, dirs, K: int, stream=None):
        import torch
        n = origins.shape[0]
        visited = torch.empty(n, K, dtype=torch.int32, device=origins.device)
        count = torch.empty(n, dtype=torch.int32, device=origins.device)
        _lib.check(_lib.lib().snisr_trace_voxels(self._h, _ptr(origins), _ptr(dirs), n, K, _ptr(visited),
                                                 _ptr(count), _stream(stream)))
        return visited, count

    def proxy_hit(self, origins, dirs, stream=None):
        import torch
        n = origins.shape[0]
        t = torch.empty(n, device=origins.device)
        tri = torch.empty(n, dtype=torch.int32, device=origins.device)
        _lib.check(_lib.lib().snisr_proxy_hit(self._h, _ptr(origins), _ptr(dirs), n, _ptr(t), _ptr(tri),
                                              _stream(stream)))
        return t, tri


def camera_rays(cam: _lib.Camera, device: int = 0, stream=None):
    import torch
    dirs = torch.empty(cam.height * cam.width, 3, device=torch.device("cuda", device))
    _lib.check(_lib.lib().snisr_camera_rays(C.byref(cam), _ptr(dirs), _stream(stream)))
    return dirs
