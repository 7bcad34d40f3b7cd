"""The reference's scene format (renderData.npz) for its diffuse octree
renderer: load / save it, move it to the device with the reference's
dtypes (rendering/src/__init__.py:98-136), and build it from a seeded
synthetic scene.

Layout (rendering/src/raydiffuse_render_octree_fp16.cu:20-139,
half_ope.h:409-471): each 64^3 tile is split into 4^3 blocks of 16^3 voxels;
a non-empty block is a node holding an 18^3 dilated grid (one voxel of
border): nodes_IndexMap [Nn][18^3] int16 indexes the node's rows of
data_voxels [Nv][4] (FP16 RGBA: post-sigmoid colour, density per unit
length), nodes_sampleFlag [Nn][18^3] marks the voxels where samples are
taken, voxels_start [Nn] is the node's first row, block_IndexMap [NT][64]
maps blocks to nodes (-1 = empty).
"""
from __future__ import annotations

import numpy as np

OCTREE_DEPTH = 2
NUM_BLOCK = 4
NUM_VOXEL = 64
DILATED = NUM_VOXEL // NUM_BLOCK + 2  # 18

KEYS = ("octree_depth", "num_voxel", "voxel_size", "scene_min_corner", "tile_shape", "net_params", "group_centers",
        "centers", "tile2group", "tile_IndexMap", "block_IndexMap", "nodes_IndexMap", "nodes_sampleFlag",
        "voxels_start", "data_voxels", "group_names")


def load(path: str) -> dict:
    """renderData.npz -> dict of numpy arrays (the reference's keys)."""
    z = np.load(path, allow_pickle=True)
    return {k: z[k] for k in z.files}


def save(path: str, data: dict) -> None:
    np.savez(path, **{k: data[k] for k in KEYS if k in data})


def derived(data: dict, sample_step_scale: float = 0.2) -> dict:
    """The renderer's scalar parameters (rendering/src/__init__.py:129-140)."""
    num_voxel = int(data["num_voxel"][0])
    voxel_size = float(data["voxel_size"][0])
    depth = int(data["octree_depth"][0])
    tile_size = num_voxel * voxel_size
    shape = np.asarray(data["tile_shape"])
    return {"tile_size": tile_size, "voxel_size": voxel_size,
            "block_num_voxel": num_voxel // (2 ** depth) + 2, "sample_step": sample_step_scale * voxel_size,
            "far": float(np.linalg.norm(tile_size * shape)), "scene_size": shape * tile_size}


def to_device(data: dict, device="cuda") -> dict:
    """Device tensors with the reference's dtypes."""
    import torch
    dt = {"scene_min_corner": torch.float32, "tile_shape": torch.int32, "net_params": torch.float16,
          "group_centers": torch.float32, "centers": torch.float32, "tile2group": torch.int32,
          "tile_IndexMap": torch.int32, "block_IndexMap": torch.int32, "nodes_IndexMap": torch.int16,
          "nodes_sampleFlag": torch.bool, "voxels_start": torch.int64, "data_voxels": torch.float16}
    return {k: torch.from_numpy(np.ascontiguousarray(data[k])).to(dtype=v, device=device).contiguous()
            for k, v in dt.items()}


def _sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def _softplus(x):
    return np.maximum(x, 0) + np.log1p(np.exp(-np.abs(x)))


def from_synth(synth, groups: int | None = None, seed: int = 0) -> dict:
    """Reference-format scene from a seeded synthetic scene with 64^3 tiles.
    Occupied voxels get baked RGBA from their trilinear centre values:
    colour = sigmoid(4 x the first three features), density per unit length
    = softplus(density logit) / voxel; the voxels within one voxel of an
    occupied one are stored (RGBA 0 where unoccupied), sampled where occupied.
    One group per tile unless `groups` is given (tiles split evenly)."""
    from .spec_synth import spec_params
    d = synth.desc
    a = synth.arrays()
    N = int(d.res)
    if N != NUM_VOXEL:
        raise ValueError("the reference format needs 64^3 tiles")
    NT = int(d.num_tiles)
    gx, gy, gz = int(d.grid[0]), int(d.grid[1]), int(d.grid[2])
    tile = float(d.tile_size)
    voxel = tile / N
    bits = np.unpackbits(a["occupancy"].view(np.uint8), bitorder="little").astype(bool).reshape(NT, N, N, N)
    # per-voxel centre values (voxels in (tile, v) order)
    corners = a["voxel_corners"]
    feat = a["vertex_feat"].astype(np.float32)
    dens = a["vertex_density"].astype(np.float32)
    cf = feat[corners].mean(axis=1)
    cd = dens[corners].mean(axis=1)
    rgba_occ = np.concatenate([_sigmoid(4.0 * cf[:, :3]), (_softplus(cd) / voxel)[:, None]], 1).astype(np.float32)
    dense = np.zeros((NT, N, N, N, 4), np.float32)
    dense[bits] = rgba_occ  # boolean indexing walks (tile, x, y, z) in C order = global voxel order
    # voxels whose data are needed: occupied dilated by one voxel (3^3)
    pad = np.pad(bits, ((0, 0), (1, 1), (1, 1), (1, 1)))
    need = np.zeros_like(pad)
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                need[:, 1:-1, 1:-1, 1:-1] |= pad[:, 1 + dx:N + 1 + dx, 1 + dy:N + 1 + dy, 1 + dz:N + 1 + dz]
    occ_p = pad
    dense_p = np.pad(dense, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    B = N // NUM_BLOCK
    block_map = -np.ones((NT, NUM_BLOCK ** 3), np.int32)
    node_maps, flags, starts, datas = [], [], [], []
    row = 0
    for t in range(NT):
        for bx in range(NUM_BLOCK):
            for by in range(NUM_BLOCK):
                for bz in range(NUM_BLOCK):
                    core = bits[t, B * bx:B * bx + B, B * by:B * by + B, B * bz:B * bz + B]
                    if not core.any():
                        continue
                    sl = (t, slice(B * bx, B * bx + DILATED), slice(B * by, B * by + DILATED),
                          slice(B * bz, B * bz + DILATED))  # padded coordinates: block start - 1 + 1
                    nd = need[sl]
                    idx = np.zeros(nd.shape, np.int32)
                    m = int(nd.sum())
                    idx[nd] = np.arange(1, m + 1, dtype=np.int32)
                    block_map[t, (bx * NUM_BLOCK + by) * NUM_BLOCK + bz] = len(node_maps)
                    node_maps.append(idx.reshape(-1).astype(np.int16))
                    flags.append(occ_p[sl].reshape(-1))
                    starts.append(row)
                    datas.append(np.concatenate([np.zeros((1, 4), np.float32), dense_p[sl][nd]], 0))
                    row += m + 1
    tile_index = np.asarray(a["tile_index"], np.int32).reshape(gx, gy, gz)
    centers = np.zeros((NT, 3), np.float32)
    smin = np.array(list(d.scene_min), np.float32)
    for x in range(gx):
        for y in range(gy):
            for z in range(gz):
                t = tile_index[x, y, z]
                if t >= 0:
                    centers[t] = smin + (np.array([x, y, z], np.float32) + 0.5) * tile
    G = NT if groups is None else int(groups)
    tile2group = (np.arange(NT) * G // NT).astype(np.int32)
    group_centers = np.stack([centers[tile2group == g].mean(0) if (tile2group == g).any() else np.zeros(3)
                              for g in range(G)]).astype(np.float32)
    rng = np.random.default_rng(seed)
    return {
        "octree_depth": np.array([OCTREE_DEPTH]), "num_voxel": np.array([NUM_VOXEL]),
        "voxel_size": np.array([voxel], np.float32), "scene_min_corner": smin,
        "tile_shape": np.array([gx, gy, gz], np.int32), "net_params": spec_params(G, rng),
        "group_centers": group_centers, "centers": centers, "tile2group": tile2group, "tile_IndexMap": tile_index,
        "block_IndexMap": block_map, "nodes_IndexMap": np.stack(node_maps),
        "nodes_sampleFlag": np.stack(flags), "voxels_start": np.array(starts, np.int64),
        "data_voxels": np.concatenate(datas, 0).astype(np.float16),
        "group_names": np.array([f"group{g}" for g in range(G)]),
    }
