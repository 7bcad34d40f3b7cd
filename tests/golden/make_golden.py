"""Generates tests/golden/reference_python.npz by running the reference's own
Python code on seeded inputs (CPU, float64):

  volume_rendering  training/scripts/utils.py:823-837   (cumprod compositing)
  query_voxel       training/scripts/tile/tile.py:225-236 (grid_sample lookup)
  Positional_Encoding  training/scripts/networks.py:4-15
  eval_sh           training/scripts/sh.py:55-111 (degree 2)
  Tile.pruning      training/scripts/tile/tile.py:297-395 (host flow; its
                    CUDA helpers run as the oracle's restatements)

utils.py and tile.py import compiled extensions at module level, so only the
needed function definitions are extracted (ast) and executed; networks.py
imports only torch and is loaded as a module.  Needs the reference tree
(default /root/reference); the fixture it writes is committed, so the tests
themselves never read the reference.

    python tests/golden/make_golden.py [--reference PATH]
"""
from __future__ import annotations

import argparse
import ast
import importlib.util
import os
import types

import numpy as np
import torch
import torch.nn.functional as F

HERE = os.path.dirname(os.path.abspath(__file__))


def _extract(path: str, name: str, cls: str | None = None) -> str:
    tree = ast.parse(open(path).read())
    nodes = tree.body
    if cls is not None:
        nodes = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls).body
    fn = next(n for n in nodes if isinstance(n, ast.FunctionDef) and n.name == name)
    return ast.unparse(fn)


def _pruning_case(ref: str, rng) -> dict:
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import oracle

    N, block = 16, 4
    D = N + 2
    vs, center = 0.0625, np.array([0.3, -0.1, 0.2], np.float32)
    tile = N * vs
    # density at the voxel centres [x][y][z]: an opaque ball plus noise, zero in a slab
    g = (np.arange(N) + 0.5) / N - 0.5
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    voxel_sigma = np.where(X ** 2 + Y ** 2 + Z ** 2 < 0.09, 1000.0, 0.0) + rng.random((N, N, N)) * 0.6
    voxel_sigma[:, :, :3] = 0.0
    voxel_sigma = voxel_sigma.astype(np.float32)
    sig_d = np.zeros((D, D, D), np.float32)
    sig_d[1:-1, 1:-1, 1:-1] = voxel_sigma
    flags_xyz = -np.ones((D, D, D), np.int16)
    flags_xyz[1:-1, 1:-1, 1:-1] = np.where(rng.random((N, N, N)) < 0.8, 1, 0)
    init_xyz = np.where(rng.random((N, N, N)) < 0.9, 1, -1).astype(np.int16)
    # rays from a ring of origins outside the tile towards points inside it
    n = 768
    ang = rng.random(n) * 2 * np.pi
    ro = center + np.stack([np.cos(ang), np.sin(ang), rng.random(n) - 0.5], 1) * 1.5 * tile
    tgt = center + (rng.random((n, 3)) - 0.5) * tile * 0.9
    rd = tgt - ro
    rd /= np.linalg.norm(rd, axis=1, keepdims=True)
    ro, rd = ro.astype(np.float32), rd.astype(np.float32)

    captured = {}

    def transparency_statistic(o, d, nv, c, tsize, vsz, step, voxels, nodes, T):
        t = T.numpy()
        oracle.op_transparency_statistic(o.numpy(), d.numpy(), nv, c.numpy(), tsize, vsz, step,
                                         voxels.numpy(), nodes.numpy(), t)
        captured["T"] = t.copy()

    def dilate_boundary(f, nv):
        a = f.numpy()
        oracle.op_dilate_boundary(a)

    ns = {"torch": torch, "np": np, "os": os, "datetime": None, "transparency_statistic": transparency_statistic,
          "dilate_boundary": dilate_boundary}
    exec(_extract(os.path.join(ref, "training/scripts/tile/tile.py"), "pruning", cls="Tile"), ns)
    exec(_extract(os.path.join(ref, "training/scripts/tile/tile.py"), "create_meshgrid", cls="Tile"), ns)
    corner = torch.from_numpy(center) - tile / 2.0

    def inference_diffuse(model, x):  # the model density at voxel centres, [x][y][z] lookup
        idx = torch.floor((x.reshape(-1, 3) - corner) / vs).long().clamp(0, N - 1)
        s = torch.from_numpy(voxel_sigma)[idx[:, 0], idx[:, 1], idx[:, 2]]
        return None, torch.relu(s).reshape(*x.shape[:-1], 1)

    results = {}
    for init in (False, True):
        st = types.SimpleNamespace(
            dilate_num_voxel=D, num_voxel=N, tile_size=tile, voxel_size=vs, tileIdx=0, logdir=".",
            tile_center=torch.from_numpy(center), tile_center_np=center, device="cpu", relu=torch.nn.ReLU(),
            min_corner=torch.from_numpy(center) - tile / 2.0 - vs,
            voxels=torch.from_numpy(np.stack([np.zeros_like(sig_d)] * 3 + [sig_d])).permute(0, 3, 2, 1)[None],
            nodes_flag=torch.from_numpy(flags_xyz.transpose(2, 1, 0).copy()),
            init_nodes_flag=torch.from_numpy(init_xyz.transpose(2, 1, 0).copy()),
            cfg=types.SimpleNamespace(PATCH_SIZE=16, PATCH_TRAIN=False, INIT_VOXEL=init),
            create_meshgrid=ns["create_meshgrid"], inference_diffuse=inference_diffuse)
        data = torch.from_numpy(np.concatenate([ro, rd, np.zeros((n, 8), np.float32)], 1))
        ns["pruning"](st, None, data, block=block, th=0.5, T_th=0.02, rate=0.1)
        results[init] = st.nodes_flag.numpy().transpose(2, 1, 0).copy()
    return dict(pr_ro=ro, pr_rd=rd, pr_center=center, pr_vs=np.float32(vs), pr_N=np.int64(N),
                pr_block=np.int64(block), pr_th=np.float32(0.5), pr_T_th=np.float32(0.02), pr_rate=np.float32(0.1),
                pr_sigma_d=sig_d, pr_voxel_sigma=voxel_sigma, pr_flags=flags_xyz, pr_init=init_xyz,
                pr_T=captured["T"], pr_out=results[False], pr_out_init=results[True])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    a = ap.parse_args()
    ref = a.reference
    rng = np.random.default_rng(2024)
    out = {}

    # volume_rendering
    ns = {"torch": torch}
    exec(_extract(os.path.join(ref, "training/scripts/utils.py"), "volume_rendering"), ns)
    vr = ns["volume_rendering"]
    B, S = 64, 24
    rgb = rng.random((B, S, 3)).astype(np.float32)
    sigma = (rng.random((B, S, 1)) * 3).astype(np.float32)
    dists = (rng.random((B, S, 1)) * 0.5).astype(np.float32)
    init_T = 0.75
    o, t, al = vr(torch.from_numpy(rgb).double(), torch.from_numpy(sigma).double(),
                  torch.from_numpy(dists).double(), init_T)
    out.update(vr_rgb=rgb, vr_sigma=sigma[..., 0], vr_dists=dists[..., 0], vr_init_T=np.float64(init_T),
               vr_out=o.numpy(), vr_T=t[..., 0].numpy(), vr_alpha=al[..., 0].numpy())

    # query_voxel (grid_sample, align_corners=True, zero padding)
    ns = {"torch": torch, "F": F}
    exec(_extract(os.path.join(ref, "training/scripts/tile/tile.py"), "query_voxel", cls="Tile"), ns)
    qv = ns["query_voxel"]
    D = 10
    self_ = types.SimpleNamespace(min_corner=torch.tensor([0.1, -0.2, 0.3], dtype=torch.float64),
                                  voxel_size=0.05, dilate_num_voxel=D,
                                  voxels=torch.from_numpy(rng.standard_normal((1, 4, D, D, D))).double())
    x = (self_.min_corner.numpy() + rng.random((48, 5, 3)) * D * 0.05).astype(np.float64)
    q_rgb, q_sigma = qv(self_, torch.from_numpy(x))
    out.update(qv_min_corner=self_.min_corner.numpy(), qv_voxel=np.float64(0.05), qv_D=np.int64(D),
               qv_voxels=self_.voxels.numpy()[0], qv_x=x, qv_rgb=q_rgb.numpy(), qv_sigma=q_sigma.numpy())

    # Positional_Encoding
    spec = importlib.util.spec_from_file_location("ref_networks", os.path.join(ref, "training/scripts/networks.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    pe = mod.Positional_Encoding(4)
    xp = rng.standard_normal((128, 3)).astype(np.float32)
    out.update(pe_x=xp, pe_out=pe(torch.from_numpy(xp).double()).numpy())

    # SH degree 2 (training/scripts/sh.py eval_sh; sh [..., C, 9], unit dirs)
    spec = importlib.util.spec_from_file_location("ref_sh", os.path.join(ref, "training/scripts/sh.py"))
    shm = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(shm)
    coeff = rng.standard_normal((256, 3, 9))
    dirs = rng.standard_normal((256, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    out.update(sh_coeff=coeff, sh_dirs=dirs,
               sh_out=shm.eval_sh(2, torch.from_numpy(coeff), torch.from_numpy(dirs)).numpy())

    # Tile.pruning (training/scripts/tile/tile.py:297-395) on a 16^3 tile: the
    # reference's host flow (max filter, block maxima of the model density,
    # thresholds, permutes) with its two CUDA helpers replaced by the oracle.
    out.update(_pruning_case(ref, rng))

    path = os.path.join(HERE, "reference_python.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
