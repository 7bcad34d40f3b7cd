"""Golden vectors from the reference's own CUDA kernels, for the CPU tests.

Runs on a GPU host after the library build (the reference's kernels come
from the cubins of oracle/build_ref.py, launched by tests/refgpu.py) and
writes tests/golden/reference_kernels.npz: the outputs of compute_rays,
tracing_tiles, rendering_diffuse_octree_fp16, inverse_z_sampling,
integrate_points, Sample_sparse, Sample_bg, transparency_statistic and
dilate_boundary on small seeded inputs.  The inputs are rebuilt on the CPU
from the same seeds (tests/test_oracle_refgpu_golden.py), so only outputs
are stored (the octree case also stores its rays and visited lists, which
come from the reference's compute_rays and tracing_tiles).

    python tests/golden/make_refgpu_golden.py [--out PATH]
"""
from __future__ import annotations

import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "scalable-neural-indoor-scene-rendering_gb300"), os.path.dirname(HERE)]

import numpy as np  # noqa: E402

import refgpu_cases as cases  # noqa: E402


def main():
    import torch

    import refgpu

    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "reference_kernels.npz"))
    args = ap.parse_args()

    def t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    def n(x):
        torch.cuda.synchronize()
        return x.cpu().numpy()

    out = {}
    # compute_rays
    c = cases.camera_case()
    rays = torch.full((c["H"], c["W"], 3), -1.0, device="cuda")
    refgpu.compute_rays(c["intr"], c["rot"], 256, rays)
    out["cr_rays"] = n(rays)
    # tracing_tiles, camera inside and outside the scene box
    for tag, origin in (("in", c["origin"]), ("out", cases.OUTSIDE_ORIGIN)):
        tc = cases.tracing_case()
        vis = torch.empty((c["H"], c["W"], tc["K"]), dtype=torch.int32, device="cuda")
        refgpu.tracing_tiles(rays, t(tc["imap"]), origin, tc["shape"], tc["smin"], tc["ssize"], tc["tile"], 256, vis)
        out[f"tt_vis_{tag}"] = n(vis)
    # octree renderer (its rays and visited lists from the reference ops above)
    from snisr import octree
    o = cases.octree_case()
    T = octree.to_device(o["D"])
    orays = torch.empty((o["H"], o["W"], 3), device="cuda")
    refgpu.compute_rays(o["intr"], o["rot"], 256, orays)
    ovis = torch.empty((o["H"], o["W"], o["K"]), dtype=torch.int32, device="cuda")
    refgpu.tracing_tiles(orays, T["tile_IndexMap"], o["origin"], o["tile_shape"], o["scene_min_corner"],
                         o["scene_size"], o["tile_size"], 256, ovis)
    out["oc_rays"], out["oc_vis"] = n(orays), n(ovis)
    for soft in (False, True):
        frame = torch.full((o["H"], o["W"], 3), -1.0, device="cuda")
        inv = torch.full((o["H"], o["W"]), 1e-8, device="cuda")
        net = torch.full((o["H"], o["W"]), -1, dtype=torch.int16, device="cuda")
        refgpu.rendering_diffuse_octree_fp16(orays, ovis, o["origin"], T["tile2group"], T["data_voxels"],
                                             T["block_IndexMap"], T["nodes_IndexMap"], T["nodes_sampleFlag"],
                                             T["voxels_start"], T["centers"], o["tile_size"], o["voxel_size"],
                                             o["sample_step"], o["block_num_voxel"], 256, 0.0 if soft else 0.8, 0.01,
                                             soft, frame, inv, net)
        k = "soft" if soft else "hard"
        out[f"oc_frame_{k}"], out[f"oc_inv_{k}"], out[f"oc_net_{k}"] = n(frame), n(inv), n(net)
    # inverse-z sampling
    z = cases.inverse_z_case()
    for off in z["offsets"]:
        pts = torch.full(z["pts_shape"], -1.0, device="cuda")
        steps = torch.zeros(z["steps_shape"], device="cuda")
        refgpu.inverse_z_sampling(z["origin"], t(z["rays_d"]), t(z["inv_near"]), t(z["inv_bound"]), 256, off,
                                  z["spr"], pts, steps)
        out[f"iz_pts_{off}"], out[f"iz_steps_{off}"] = n(pts), n(steps)
    # integrate_points
    ip = cases.integrate_case()
    tr, fr = t(ip["trans"]), t(ip["frame"])
    refgpu.integrate_points(t(ip["rgba"]), t(ip["dz"]), 512, ip["early"], tr, fr)
    out["ip_trans"], out["ip_frame"] = n(tr), n(fr)
    # Sample_sparse
    ss = cases.sample_sparse_case()
    zv = torch.full((ss["B"], ss["ns"]), -1.0, device="cuda")
    dv = torch.full((ss["B"], ss["ns"]), -1.0, device="cuda")
    refgpu.Sample_sparse(t(ss["ro"]), t(ss["rd"]), t(ss["flags"]), *ss["center"], ss["tile"], ss["N"], zv, dv)
    out["ss_z"], out["ss_d"] = n(zv), n(dv)
    # Sample_bg
    bg = cases.sample_bg_case()
    zb = torch.full((bg["n"], bg["ns"]), -1.0, device="cuda")
    refgpu.Sample_bg(t(bg["ro"]), t(bg["rd"]), t(bg["bg"]), t(bg["center"]), bg["tile"], bg["range"], zb)
    out["bg_z"] = n(zb)
    # transparency statistic (stored sparse: the touched cells)
    ts = cases.transparency_case()
    Tv = torch.zeros((ts["D"],) * 3, device="cuda")
    refgpu.transparency_statistic(t(ts["ro"]), t(ts["rd"]), ts["D"], t(ts["center"]), ts["tile"], ts["vs"],
                                  ts["step"], t(ts["sigma"]), t(ts["flags"]), Tv)
    Tn = n(Tv).reshape(-1)
    nz = np.nonzero(Tn)[0].astype(np.int32)
    out["ts_idx"], out["ts_val"] = nz, Tn[nz]
    # dilate_boundary
    db = cases.dilate_case()
    g = t(db["flags"])
    refgpu.dilate_boundary(g, db["D"])
    out["db_flags"] = n(g)
    np.savez_compressed(args.out, **out)
    print("wrote", args.out, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
