"""Occupancy pruning of one tile after a training epoch (Tile.pruning,
training/scripts/tile/tile.py:297-395), on the device:

1. transparency statistic of the training rays over the dilated density
   grid (CUDA_EXT.transparency_statistic, Helper_kernel.cu:108-172);
2. the flag update: 3^3 max filter of the statistic, block maxima of the
   density at the voxel centres, the geometry threshold th on exp(-sigma)
   and the transparency threshold T_th, border dilation
   (dilate_boundary, Helper_kernel.cu:174-226);
3. the new occupancy as this library's 64-bit words.

Grids are [x][y][z] (the reference keeps its tensors [z][y][x] and permutes
them before the CUDA calls).  The reference evaluates the tile's model for
the densities; here the caller passes them: `sigma_voxels` [D^3] at the
dilated cell centres (D = N + 2) and `voxel_sigma` [N^3] at the voxel
centres.  `grids_from_arrays` builds both from this library's scene arrays
(density = softplus of the trilinear vertex logit, per unit length).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import ops


@dataclass
class PruneResult:
    nodes_flag: "object"      # int16 [D,D,D]: 1 kept, 0 dilated border, -1 empty
    T_voxels: "object"        # float32 [D,D,D] statistic before the max filter
    words: "object"           # int64 [ceil(N^3/64)] occupancy words
    occupied: int             # voxels kept
    info: str                 # the reference's summary text


def pruning(rays_o, rays_d, tile_center, tile_size: float, voxel_size: float, sigma_voxels, nodes_flag,
            voxel_sigma, init_flags=None, block: int = 4, th: float = 0.5, T_th: float = 0.0,
            rate: float = 0.1, batch: int | None = None) -> PruneResult:
    """One tile's pruning.  rays_o / rays_d [B,3] float32 CUDA (the tile's
    training rays; rays that miss the tile add nothing), tile_center [3],
    sigma_voxels [D,D,D] (negative values count as 0, as the reference's
    ReLU), nodes_flag [D,D,D] int16 (the current flags; samples only where
    1), voxel_sigma [N,N,N], init_flags [N,N,N] int16 or None."""
    import torch
    D = nodes_flag.shape[0]
    N = D - 2
    dev = nodes_flag.device
    T_voxels = torch.zeros(D, D, D, dtype=torch.float32, device=dev)
    sigma = torch.relu(sigma_voxels).contiguous()
    step = voxel_size * rate
    B = rays_o.shape[0]
    bs = B if not batch else int(batch)
    for i in range(0, B, max(bs, 1)):
        ops.transparency_statistic(rays_o[i:i + bs].contiguous(), rays_d[i:i + bs].contiguous(), D,
                                   tile_center, tile_size, voxel_size, step, sigma, nodes_flag, T_voxels)
    new_flags = torch.empty_like(nodes_flag)
    ops.prune_flags(T_voxels, voxel_sigma.contiguous(), init_flags, block, th, T_th, new_flags)
    words, count = ops.pack_occupancy(new_flags)
    occupied = int(count)
    info = (f"Transparency info:\nblock size {block}\tgeo_th: {th}\ttrans_th: {T_th}\n"
            f"min {float(T_voxels.min()):.5f}\tmax {float(T_voxels.max()):.5f}\tmean {float(T_voxels.mean()):.5f}\n"
            f"\noriginal voxel num: {N ** 3}\nafter pruning: {occupied}\n"
            f"Geometry Rate: {occupied / N ** 3 * 100:.3f} %\n")
    return PruneResult(new_flags, T_voxels, words, occupied, info)


def _softplus(x):
    return np.maximum(x, 0) + np.log1p(np.exp(-np.abs(x)))


def grids_from_arrays(desc, arrays: dict, tile: int):
    """(sigma_voxels [D^3], voxel_sigma [N^3], nodes_flag [D^3] int16) of one
    tile of this library's scene arrays: density per unit length at the
    dilated cell centres (0 outside occupied voxels) and at the voxel
    centres, flags 1 where occupied, 0 on their one-cell border, -1 else."""
    N = int(desc.res)
    D = N + 2
    voxel = float(desc.tile_size) / N
    occ = np.unpackbits(arrays["occupancy"].view(np.uint8), bitorder="little").astype(bool)
    occ = occ.reshape(-1, N ** 3)[tile].reshape(N, N, N)
    per_tile = np.unpackbits(arrays["occupancy"].view(np.uint8), bitorder="little").reshape(-1, N ** 3).sum(1)
    first = int(per_tile[:tile].sum())
    corners = arrays["voxel_corners"][first:first + int(per_tile[tile])]
    dens = arrays["vertex_density"].astype(np.float32)
    s = (_softplus(dens[corners].mean(axis=1)) / voxel).astype(np.float32)
    voxel_sigma = np.zeros((N, N, N), np.float32)
    voxel_sigma[occ] = s
    sigma_voxels = np.zeros((D, D, D), np.float32)
    sigma_voxels[1:-1, 1:-1, 1:-1] = voxel_sigma
    one = np.zeros((D, D, D), bool)
    one[1:-1, 1:-1, 1:-1] = occ
    pad = np.pad(one, 1)
    near = np.zeros_like(one)
    for dx in (0, 1, 2):
        for dy in (0, 1, 2):
            for dz in (0, 1, 2):
                near |= pad[dx:dx + D, dy:dy + D, dz:dz + D]
    flags = np.where(one, 1, np.where(near, 0, -1)).astype(np.int16)
    return sigma_voxels, voxel_sigma, flags


def tile_centers(desc, arrays: dict) -> np.ndarray:
    """[NT,3] float32 centre of every sparse tile."""
    gx, gy, gz = int(desc.grid[0]), int(desc.grid[1]), int(desc.grid[2])
    idx = np.asarray(arrays["tile_index"], np.int32).reshape(gx, gy, gz)
    out = np.zeros((int(desc.num_tiles), 3), np.float32)
    smin = np.array(list(desc.scene_min), np.float32)
    for x in range(gx):
        for y in range(gy):
            for z in range(gz):
                if idx[x, y, z] >= 0:
                    out[idx[x, y, z]] = smin + (np.array([x, y, z], np.float32) + 0.5) * np.float32(desc.tile_size)
    return out
