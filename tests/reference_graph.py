"""PyTorch restatement of the reference's training graph for one tile
(test infrastructure; float64 on the CPU).

The reference trains with plain autograd: it looks features and density up
with grid_sample(align_corners=True) in query_voxel
(training/scripts/tile/tile.py:225-236), encodes the view direction with
Positional_Encoding (training/scripts/networks.py:4-15), runs a Linear/ReLU
MLP and composites with the cumprod of volume_rendering
(training/scripts/utils.py:823-837), T = cumprod([1, 1 - alpha + 1e-10])[:-1].
It has no custom backward op, so its gradients are autograd of this graph.
Here the lookup grid is the tile's dense grid of trilinear corners (vertex
values scattered to corner positions), sampled at the sample positions the
oracle's training forward takes; the MLP reads the looked-up features
directly.  Autograd of this graph is the gradient reference for the
hand-written adjoint.
"""
from __future__ import annotations

import numpy as np


def voxel_coords(desc, arrays):
    """Per global voxel id: (tile, x, y, z), from the occupancy bitfields
    (bit v & 63 of word v >> 6, v = (x*N + y)*N + z, voxels in (tile, v) order)."""
    N = int(desc.res)
    bits = np.unpackbits(arrays["occupancy"].view(np.uint8), bitorder="little")
    ids = np.nonzero(bits)[0]
    tile = ids // (N ** 3)
    v = ids % (N ** 3)
    return np.stack([tile, v // (N * N), (v // N) % N, v % N], 1)


def corner_index_grid(desc, arrays, tile: int = 0):
    """[(N+1)^3] vertex id of each corner position of `tile` (-1: no vertex)."""
    N = int(desc.res)
    vc = voxel_coords(desc, arrays)
    sel = np.nonzero(vc[:, 0] == tile)[0]
    grid = -np.ones((N + 1,) * 3, np.int64)
    corners = arrays["voxel_corners"]
    for k in range(8):
        dx, dy, dz = (k >> 2) & 1, (k >> 1) & 1, k & 1
        grid[vc[sel, 1] + dx, vc[sel, 2] + dy, vc[sel, 3] + dz] = corners[sel, k]
    return grid.reshape(-1)


def positional_encoding(d, freqs: int = 4):
    import torch
    parts = [d]
    for i in range(freqs):
        parts += [torch.sin((2.0 ** i) * d), torch.cos((2.0 ** i) * d)]
    return torch.cat(parts, -1)


def render(vf, vd, W, desc, idx_grid, samples, dirs):
    """rgb [n,3] of the rays (float64 torch tensors vf [NV,F], vd [NV], W [P])."""
    import torch
    import torch.nn.functional as Fn
    off, _, pos, dv = samples
    N, F, H, L = int(desc.res), int(desc.feat_dim), int(desc.mlp_hidden), int(desc.mlp_layers)
    n = off.size - 1
    S = int(off[-1])
    gi = torch.from_numpy(np.maximum(idx_grid, 0))
    mask = torch.from_numpy(idx_grid >= 0).to(vf.dtype)
    Gf = (vf[gi] * mask[:, None]).reshape(N + 1, N + 1, N + 1, F).permute(3, 0, 1, 2)[None]
    Gd = (vd[gi] * mask).reshape(1, 1, N + 1, N + 1, N + 1)
    g = torch.from_numpy(pos) / N * 2.0 - 1.0
    grid = torch.stack([g[:, 2], g[:, 1], g[:, 0]], -1).reshape(1, S, 1, 1, 3)
    feat = Fn.grid_sample(Gf, grid, mode="bilinear", align_corners=True).reshape(F, S).t()
    dens = Fn.grid_sample(Gd, grid, mode="bilinear", align_corners=True).reshape(S)
    cnt = np.diff(off)
    ray = torch.from_numpy(np.repeat(np.arange(n), cnt))
    enc = positional_encoding(torch.from_numpy(np.asarray(dirs, np.float64)))[ray]
    x = torch.cat([feat, enc], 1)
    o = 0
    for l in range(L + 1):
        fi = F + 27 if l == 0 else H
        fo = 3 if l == L else H
        Wl = W[o:o + fi * fo].reshape(fo, fi)
        bl = W[o + fi * fo:o + fi * fo + fo]
        x = x @ Wl.t() + bl
        if l < L:
            x = torch.relu(x)
        o += fi * fo + fo
    c = torch.sigmoid(x)
    sigma = Fn.softplus(dens)
    alpha = 1.0 - torch.exp(-sigma * torch.from_numpy(dv))
    slot = torch.from_numpy(np.arange(S) - np.repeat(off[:-1], cnt))
    smax = int(cnt.max()) if n and S else 1
    A = torch.zeros(n, smax, dtype=vf.dtype).index_put((ray, slot), alpha)
    Cp = torch.zeros(n, smax, 3, dtype=vf.dtype).index_put((ray, slot), c)
    T = torch.cumprod(torch.cat([torch.ones(n, 1, dtype=vf.dtype), 1.0 - A + 1e-10], 1), 1)[:, :-1]
    return ((A * T)[..., None] * Cp).sum(1)
