"""The drop-in for the reference's FP16 diffuse renderer on its own scene
format (FASTRENDERING.rendering_diffuse_octree_fp16) against the oracle's
restatement, on synthetic scenes converted to renderData format (1 tile and
16 tiles of 64^3), called with the reference's arguments after the
compute_rays and tracing_tiles drop-ins, with soft_hit off (the reference
renderer's setting, first-hit threshold 0.8) and on (threshold 0, so every
pixel takes the soft-hit path).

Both round every FP16 and FP32 operation on its own, and CUDA's hexp equals
exp rounded to FP16 on the inputs used: colour, first-hit inverse depth and
network id are bit-identical."""
import numpy as np
import pytest

import oracle
import snisr
from snisr import octree, ops

pytestmark = pytest.mark.gpu


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("soft", [False, True], ids=["hard", "soft"])
@pytest.mark.parametrize("cfg", [snisr.CFG1, snisr.CFG2.replace(res=64, with_mesh=False)], ids=["1tile", "16tiles"])
def test_octree_diffuse_vs_oracle(cuda, cfg, soft):
    import torch
    th = 0.0 if soft else 0.8
    s = snisr.SynthScene(cfg)
    D = octree.from_synth(s, groups=min(4, s.desc.num_tiles))
    der = octree.derived(D)
    T = octree.to_device(D)
    cam = s.camera(1, 320, 240)
    H, W = cam.height, cam.width
    intr = _t(np.array([cam.cx, cam.cy, cam.inv_focal], np.float32))
    rot = _t(np.array([[cam.c2w[0], cam.c2w[1], cam.c2w[2]], [cam.c2w[4], cam.c2w[5], cam.c2w[6]],
                       [cam.c2w[8], cam.c2w[9], cam.c2w[10]]], np.float32))
    origin = _t(np.array([cam.c2w[3], cam.c2w[7], cam.c2w[11]], np.float32))
    rays_d = torch.full((H, W, 3), -1.0, device="cuda")
    ops.compute_rays(intr, rot, 0, rays_d)
    visited = torch.full((H, W, 30), -1, dtype=torch.int32, device="cuda")
    ops.tracing_tiles(rays_d, T["tile_IndexMap"], origin, T["tile_shape"], T["scene_min_corner"],
                      _t(der["scene_size"].astype(np.float32)), der["tile_size"], 0, visited)
    frame = torch.full((H, W, 3), -1.0, device="cuda")
    inv = torch.full((H, W), 1e-8, device="cuda")
    net = torch.full((H, W), -1, dtype=torch.int16, device="cuda")
    ops.rendering_diffuse_octree_fp16(rays_d, visited, origin, T["tile2group"], T["data_voxels"],
                                      T["block_IndexMap"], T["nodes_IndexMap"], T["nodes_sampleFlag"],
                                      T["voxels_start"], T["centers"], der["tile_size"], der["voxel_size"],
                                      der["sample_step"], der["block_num_voxel"], 256, th, 0.01, soft,
                                      frame, inv, net)
    torch.cuda.synchronize()
    n = H * W
    rd = rays_d.cpu().numpy().reshape(n, 3)
    vis = visited.cpu().numpy().reshape(n, 30)
    fo = np.zeros((n, 3), np.float32)
    io = np.full(n, 1e-8, np.float32)
    no = np.full(n, -1, np.int16)
    oracle.op_rendering_diffuse_octree(rd, vis, origin.cpu().numpy(), D, der["sample_step"], th, 0.01, fo, io, no,
                                       soft_hit=soft)
    fg, ig, ng = frame.cpu().numpy().reshape(n, 3), inv.cpu().numpy().reshape(n), net.cpu().numpy().reshape(n)
    diff = np.abs(fg - fo).max(axis=1)
    same = (ig == io) & (ng == no)
    print(f"{cfg.name}: hit {float((no >= 0).mean()):.3f}, colour max-abs {float(diff.max()):.3g}, "
          f"identical {float((diff == 0).mean()):.5f}, first-hit identical {float(same.mean()):.5f}")
    assert (no >= 0).mean() > 0.3
    assert np.array_equal(fg, fo)
    assert np.array_equal(ig, io) and np.array_equal(ng, no)
