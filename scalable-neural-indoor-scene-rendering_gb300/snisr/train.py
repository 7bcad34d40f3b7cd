"""torch.autograd.Function over the training forward / hand-written adjoint.

Replaces, for training scripts, the graph the reference builds per batch in
Tile.train_batch (training/scripts/tile/tile.py:667-704): sparse sampling,
the MLP baked into a voxel grid, grid_sample lookup and cumprod compositing
(training/scripts/utils.py:823-837).  Here the MLP is evaluated per sample
on trilinear per-corner features and the backward is libsnisr's adjoint.
"""
from __future__ import annotations

import ctypes

from . import _lib


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def _check(t, name):
    import torch
    if not t.is_cuda or not t.is_contiguous():
        raise RuntimeError(f"{name} must be a contiguous CUDA tensor")
    if t.dtype not in (torch.float32, torch.int32):
        raise RuntimeError(f"{name} has unsupported dtype {t.dtype}")


class TileFieldFunction:
    """rgb = TileFieldFunction.apply(vfeat, vdens, mlp, scene, origins, dirs, ray_tile, form)

    vfeat [NV, F], vdens [NV], mlp [NT, P] (FP32, requires_grad as needed);
    origins/dirs [n, 3] (normalised dirs); ray_tile [n] int32, grouped by tile.
    The forward's sample records live in the scene's training workspace until
    the next forward on the same scene replaces them; each forward's id
    (generation) is kept in the autograd context, and a backward whose
    forward was replaced raises SnisrError instead of back-propagating
    through another forward's samples."""

    _fn = None

    @classmethod
    def apply(cls, *args):
        if cls._fn is None:
            cls._fn = _make_function()
        return cls._fn.apply(*args)


def _make_function():
    import torch

    class _Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, vfeat, vdens, mlp, scene, origins, dirs, ray_tile, form):
            for t, nm in ((vfeat, "vfeat"), (vdens, "vdens"), (mlp, "mlp"), (origins, "origins"), (dirs, "dirs"),
                          (ray_tile, "ray_tile")):
                _check(t, nm)
            n = origins.shape[0]
            rgb = torch.empty(n, 3, device=origins.device)
            gen = ctypes.c_uint64(0)
            _lib.check(_lib.lib().snisr_train_forward(scene.handle, vfeat.data_ptr(), vdens.data_ptr(), mlp.data_ptr(),
                                                      origins.data_ptr(), dirs.data_ptr(), ray_tile.data_ptr(), n,
                                                      int(form), rgb.data_ptr(), ctypes.byref(gen), _stream()))
            ctx.save_for_backward(vfeat, vdens, mlp, origins, dirs, ray_tile)
            ctx.scene = scene
            ctx.form = int(form)
            ctx.generation = gen.value
            return rgb

        @staticmethod
        def backward(ctx, grad_rgb):
            vfeat, vdens, mlp, origins, dirs, ray_tile = ctx.saved_tensors
            g = grad_rgb.contiguous().float()
            gF = torch.zeros_like(vfeat)
            gG = torch.zeros_like(vdens)
            gW = torch.zeros_like(mlp)
            n = origins.shape[0]
            _lib.check(_lib.lib().snisr_train_backward(ctx.scene.handle, vfeat.data_ptr(), vdens.data_ptr(),
                                                       mlp.data_ptr(), origins.data_ptr(), dirs.data_ptr(),
                                                       ray_tile.data_ptr(), n, ctx.form, ctx.generation, 0,
                                                       g.data_ptr(),
                                                       gF.data_ptr(), gG.data_ptr(), gW.data_ptr(), _stream()))
            return gF, gG, gW, None, None, None, None, None

    return _Fn


def tile_field(vfeat, vdens, mlp, scene, origins, dirs, ray_tile, form=_lib.FORM_TC):
    return TileFieldFunction.apply(vfeat, vdens, mlp, scene, origins, dirs, ray_tile, form)
