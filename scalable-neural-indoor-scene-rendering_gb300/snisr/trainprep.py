"""Training-data preparation of one tile (get_trainData_v3,
training/src/cuda_func.cu:1341-1686) on the device.

Per selected view: camera rays (get_rays), tile DDA, the two nearest
proxy-mesh hits inside every visited tile (from the scene's BVH), the
background depth and validity of the rays for the training tile, the diffuse
estimate of the hit point from all selected views (projection, depth test,
(1 - cos)^2 weights) with the background visibility test, and the patches
that hold a valid pixel as rows of 14 floats:
    rays_o (3), rays_d (3), bgdepth, gt rgb (3), diffuse (3), valid.

Images and depth maps are passed in (float RGB in [0, 1], depth along the
camera z axis); the reference reads them from PNG / .npy files.  The
projection matrices are compute_project_matrix
(training/src/include/cuda_utils.h:37-58).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .ops import _stream


def project_matrix(K, c2w) -> np.ndarray:
    """compute_project_matrix in float32, operation by operation."""
    K = np.asarray(K, np.float32).reshape(9)
    c = np.asarray(c2w, np.float32).reshape(12)
    f32 = np.float32
    fx, fy, cx, cy = K[0], K[4], K[2], K[5]
    t1 = f32(-1.0) * ((c[0] * c[3] + c[4] * c[7]) + c[8] * c[11])
    t2 = f32(-1.0) * ((c[1] * c[3] + c[5] * c[7]) + c[9] * c[11])
    t3 = f32(-1.0) * ((c[2] * c[3] + c[6] * c[7]) + c[10] * c[11])
    m = [fx * c[0] + cx * c[2], fx * c[4] + cx * c[6], fx * c[8] + cx * c[10], fx * t1 + cx * t3,
         fy * c[1] + cy * c[2], fy * c[5] + cy * c[6], fy * c[9] + cy * c[10], fy * t2 + cy * t3,
         c[2], c[6], c[10], t3]
    return np.array(m, np.float32)


class TrainPrep:
    """Device buffers for one view size; `view()` runs the per-view chain."""

    def __init__(self, scene, height: int, width: int, index_map, tile_shape, scene_min_corner, tile_size: float,
                 max_tracing_tile: int = 30, patch_size: int = 7, device=None):
        import torch
        self.scene = scene
        self.H, self.W, self.K, self.P = int(height), int(width), int(max_tracing_tile), int(patch_size)
        dev = torch.device("cuda", scene.device if device is None else device)
        self.dev = dev
        n = self.H * self.W
        self.imap = torch.as_tensor(np.ascontiguousarray(index_map, np.int32).reshape(-1), device=dev)
        self.shape = (C.c_int32 * 3)(*[int(x) for x in tile_shape])
        self.smin = (C.c_float * 3)(*[float(x) for x in scene_min_corner])
        self.tile = float(tile_size)
        self.ro = torch.empty(n, 3, device=dev)
        self.rd = torch.empty(n, 3, device=dev)
        self.visited = torch.empty(n, self.K, dtype=torch.int32, device=dev)
        self.hits = torch.empty(n, self.K, 2, device=dev)
        self.bg = torch.empty(n, device=dev)
        self.valid = torch.empty(n, dtype=torch.int32, device=dev)
        self.diffuse = torch.empty(n, 3, device=dev)
        cap = _lib.lib().snisr_op_patch_capacity(self.H, self.W, self.P)
        if cap < 0:
            raise ValueError("patch_size must be odd and positive")
        self.cap = int(cap)
        self.scratch = torch.empty(max(2 * self.cap, 1), dtype=torch.int32, device=dev)
        self.rows = torch.empty(max(self.cap, 1) * self.P * self.P, 14, device=dev)
        self.count = torch.zeros((), dtype=torch.int64, device=dev)

    def view(self, train_tile: int, K, c2w, gt_rgb, origins, images, depths, proj):
        """One view: returns (rows tensor view [count*P*P, 14], count tensor).
        K [9], c2w [12] device float32; gt_rgb [H*W,3]; origins [M,3], images
        [M,H*W,3], depths [M,H*W], proj [M,12] of the M selected views."""
        L = _lib.lib()
        s = _stream()
        n = self.H * self.W
        _lib.check(L.snisr_op_train_rays(K.data_ptr(), c2w.data_ptr(), self.H, self.W, self.ro.data_ptr(),
                                         self.rd.data_ptr(), s))
        _lib.check(L.snisr_op_train_tracing_tiles(self.ro.data_ptr(), self.rd.data_ptr(), n, self.imap.data_ptr(),
                                                  self.shape, self.smin, self.tile, self.K, self.visited.data_ptr(),
                                                  s))
        _lib.check(L.snisr_scene_double_hits(self.scene.handle, self.ro.data_ptr(), self.rd.data_ptr(),
                                             self.visited.data_ptr(), n, self.K, self.hits.data_ptr(), s))
        _lib.check(L.snisr_op_train_bgdepth(int(train_tile), self.visited.data_ptr(), self.hits.data_ptr(), n, self.K,
                                            self.bg.data_ptr(), self.valid.data_ptr(), s))
        M = int(proj.shape[0])
        _lib.check(L.snisr_op_gen_diffuse(origins.data_ptr(), int(train_tile), self.ro.data_ptr(), self.rd.data_ptr(),
                                          self.hits.data_ptr(), self.visited.data_ptr(), images.data_ptr(),
                                          depths.data_ptr(), proj.data_ptr(), self.K, M, self.H, self.W,
                                          self.diffuse.data_ptr(), self.bg.data_ptr(), s))
        _lib.check(L.snisr_op_patch_rows(self.valid.data_ptr(), self.H, self.W, self.P, self.ro.data_ptr(),
                                         self.rd.data_ptr(), self.bg.data_ptr(), gt_rgb.data_ptr(),
                                         self.diffuse.data_ptr(), self.scratch.data_ptr(), self.rows.data_ptr(),
                                         self.count.data_ptr(), s))
        return self.rows, self.count


def get_train_data(scene, train_tile: int, Ks, C2Ws, img_ids, images, depths, index_map, tile_shape,
                   scene_min_corner, tile_size: float, max_tracing_tile: int = 30, patch_size: int = 7):
    """All views' patches for one tile: float32 tensor [npatch, P*P, 14].
    Ks [nc,9], C2Ws [nc,12] (numpy), img_ids the selected views, images
    [len(img_ids),H,W,3] and depths [len(img_ids),H,W] (device float32)."""
    import torch
    M, H, W = int(images.shape[0]), int(images.shape[1]), int(images.shape[2])
    dev = images.device
    prep = TrainPrep(scene, H, W, index_map, tile_shape, scene_min_corner, tile_size, max_tracing_tile, patch_size,
                     device=dev.index)
    Ks = np.asarray(Ks, np.float32).reshape(-1, 9)
    C2Ws = np.asarray(C2Ws, np.float32).reshape(-1, 12)
    proj = torch.from_numpy(np.stack([project_matrix(Ks[i], C2Ws[i]) for i in img_ids])).to(dev)
    origins = torch.from_numpy(np.stack([C2Ws[i][[3, 7, 11]] for i in img_ids]).astype(np.float32)).to(dev)
    imgs = images.reshape(M, H * W, 3).contiguous()
    deps = depths.reshape(M, H * W).contiguous()
    out = []
    P2 = patch_size * patch_size
    for j, i in enumerate(img_ids):
        K = torch.from_numpy(Ks[i].copy()).to(dev)
        c2w = torch.from_numpy(C2Ws[i].copy()).to(dev)
        rows, count = prep.view(train_tile, K, c2w, imgs[j], origins, imgs, deps, proj)
        n = int(count)
        out.append(rows[:n * P2].clone().reshape(n, P2, 14))
    return torch.cat(out) if out else torch.empty(0, P2, 14, device=dev)
