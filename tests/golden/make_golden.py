"""Generates tests/golden/reference_python.npz by running the reference's own
Python code on seeded inputs (CPU, float64):

  volume_rendering  training/scripts/utils.py:823-837   (cumprod compositing)
  query_voxel       training/scripts/tile/tile.py:225-236 (grid_sample lookup)
  Positional_Encoding  training/scripts/networks.py:4-15
  eval_sh           training/scripts/sh.py:55-111 (degree 2)

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

    path = os.path.join(HERE, "reference_python.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
