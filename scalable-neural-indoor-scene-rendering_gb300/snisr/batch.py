"""Ray segments for batched multi-tile training.

Per-tile training uses each camera ray inside every tile it crosses (the
reference prepares per-tile training rays the same way: tile DDA over the
tile grid, training/src/cuda_func.cu:1341-1686).  Here the visited tiles of
every pixel come from the tracing_tiles op (tile DDA,
rendering/src/raytile_tracing.cu:9-60); a (pixel, tile) pair is one ray
segment, marched by the training path inside that tile only.  Every tile
then takes a seeded log-uniform number of its segments, and the batch is
returned grouped by tile, as snisr_train_forward expects.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib, ops
from .scene import camera_rays


def tile_segments(synth, views: int, device: int = 0, K: int = 30):
    """All (origin, direction, tile) segments of `views` seeded camera poses.
    Returns CUDA tensors o [m,3], d [m,3] (normalised) and tile [m] int32."""
    import torch
    dev = torch.device("cuda", device)
    desc = synth.desc
    gx, gy, gz = desc.grid[0], desc.grid[1], desc.grid[2]
    index_map = torch.from_numpy(np.ascontiguousarray(synth.arrays()["tile_index"].reshape(gx, gy, gz))).to(dev)
    shape = torch.tensor([gx, gy, gz], dtype=torch.int32, device=dev)
    smin = torch.tensor(list(desc.scene_min), dtype=torch.float32, device=dev)
    size = torch.tensor([gx * desc.tile_size, gy * desc.tile_size, gz * desc.tile_size], dtype=torch.float32,
                        device=dev)
    os_, ds_, ts_ = [], [], []
    for v in range(views):
        cam = synth.camera(v)
        d = camera_rays(cam, device)
        origin = torch.tensor([cam.c2w[3], cam.c2w[7], cam.c2w[11]], dtype=torch.float32, device=dev)
        visited = torch.empty(cam.height, cam.width, K, dtype=torch.int32, device=dev)
        ops.tracing_tiles(d, index_map, origin, shape, smin, size, float(desc.tile_size), 0, visited)
        pix, slot = torch.nonzero(visited.view(-1, K) >= 0, as_tuple=True)
        ts_.append(visited.view(-1, K)[pix, slot])
        ds_.append(d[pix])
        os_.append(origin.expand(pix.numel(), 3))
    return torch.cat(os_).contiguous(), torch.cat(ds_).contiguous(), torch.cat(ts_).contiguous()


def tile_batch(synth, views: int = 8, lo: int = 1024, hi: int = 65536, seed: int = 0, device: int = 0):
    """Seeded batch: tile t keeps min(available, round(exp(U(ln lo, ln hi)))) of
    its segments (chosen without replacement).  Returns o, d, tile (CUDA,
    grouped by tile, tile ids non-decreasing) and the per-tile counts."""
    import torch
    o, d, t = tile_segments(synth, views, device)
    rng = np.random.default_rng(seed)
    t_host = t.cpu().numpy()
    order = np.argsort(t_host, kind="stable")
    bounds = np.searchsorted(t_host[order], np.arange(synth.desc.num_tiles + 1))
    keep, counts = [], []
    for tile in range(synth.desc.num_tiles):
        idx = order[bounds[tile]:bounds[tile + 1]]
        want = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        take = min(want, idx.size)
        sel = np.sort(rng.choice(idx, take, replace=False)) if take else idx[:0]
        keep.append(sel)
        counts.append(take)
    sel = torch.from_numpy(np.concatenate(keep).astype(np.int64)).to(o.device)
    return o[sel].contiguous(), d[sel].contiguous(), t[sel].contiguous(), np.array(counts)
