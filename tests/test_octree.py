"""The reference's scene format (renderData.npz) built from seeded synthetic
scenes (CPU): format invariants, save/load round trip, derived parameters,
and a non-trivial oracle render of it."""
import os

import numpy as np

import oracle
import snisr
from snisr import octree


def _scene():
    s = snisr.SynthScene(snisr.CFG2.replace(res=64, with_mesh=False))
    return s, octree.from_synth(s, groups=4)


def test_format_invariants():
    s, D = _scene()
    NT = s.desc.num_tiles
    assert D["block_IndexMap"].shape == (NT, 64)
    nn = D["nodes_IndexMap"].shape[0]
    assert D["nodes_IndexMap"].shape == (nn, 18 ** 3) and D["nodes_sampleFlag"].shape == (nn, 18 ** 3)
    assert D["nodes_IndexMap"].dtype == np.int16 and D["data_voxels"].dtype == np.float16
    assert sorted(D["block_IndexMap"][D["block_IndexMap"] >= 0].tolist()) == list(range(nn))
    starts = D["voxels_start"]
    assert starts[0] == 0 and (np.diff(starts) > 0).all()
    sizes = np.diff(np.concatenate([starts, [D["data_voxels"].shape[0]]]))
    assert (D["nodes_IndexMap"].max(axis=1) < sizes).all() and D["nodes_IndexMap"].min() >= 0
    # sampled voxels have data; entry 0 of every node is the zero row
    assert (D["nodes_IndexMap"][D["nodes_sampleFlag"]] > 0).all()
    assert not D["data_voxels"][starts].astype(np.float32).any()
    # occupied voxels counted once in node cores (interior 16^3 of the 18^3 grid)
    core = D["nodes_sampleFlag"].reshape(nn, 18, 18, 18)[:, 1:17, 1:17, 1:17]
    assert int(core.sum()) == s.desc.num_voxels
    assert set(np.unique(D["tile2group"]).tolist()) == set(range(4))
    der = octree.derived(D)
    assert der["block_num_voxel"] == 18 and abs(der["tile_size"] - s.desc.tile_size) < 1e-6


def test_save_load_round_trip(tmp_path):
    _, D = _scene()
    p = os.path.join(tmp_path, "renderData.npz")
    octree.save(p, D)
    E = octree.load(p)
    for k in octree.KEYS:
        assert np.array_equal(np.asarray(D[k]), np.asarray(E[k])), k


def test_oracle_renders_converted_scene():
    s, D = _scene()
    cam = s.camera(2, 160, 90)
    d = oracle.camera_dirs(cam)
    o = np.array([cam.c2w[3], cam.c2w[7], cam.c2w[11]], np.float32)
    der = octree.derived(D)
    vis = oracle.op_tracing_tiles(d, D["tile_IndexMap"].reshape(-1), o, D["tile_shape"], D["scene_min_corner"],
                                  der["scene_size"].astype(np.float32), der["tile_size"], 30)
    n = d.shape[0]
    frame = np.zeros((n, 3), np.float32)
    inv = np.full(n, 1e-8, np.float32)
    net = np.full(n, -1, np.int16)
    oracle.op_rendering_diffuse_octree(d, vis, o, D, der["sample_step"], 0.8, 0.01, frame, inv, net)
    assert (net >= 0).mean() > 0.5 and frame.max() > 0.3
    hit = net >= 0
    assert (inv[hit] > 0).all() and (inv[hit] < 10).all()
    # soft_hit: first hits unchanged
    f2, i2 = np.zeros((n, 3), np.float32), np.full(n, 1e-8, np.float32)
    n2 = np.full(n, -1, np.int16)
    oracle.op_rendering_diffuse_octree(d, vis, o, D, der["sample_step"], 0.8, 0.01, f2, i2, n2, soft_hit=True)
    assert np.array_equal(f2, frame) and np.array_equal(n2[hit], net[hit]) and np.array_equal(i2[hit], inv[hit])
    # trans_th 0 (no first hits): with soft_hit every pixel that examined a tile gets a network
    f3, i3 = np.zeros((n, 3), np.float32), np.full(n, 1e-8, np.float32)
    n3 = np.full(n, -1, np.int16)
    oracle.op_rendering_diffuse_octree(d, vis, o, D, der["sample_step"], 0.0, 0.01, f3, i3, n3, soft_hit=True)
    some = vis[:, 0] >= 0
    assert some.sum() > n // 2 and np.array_equal(f3, frame)
    assert (n3[some] >= 0).all() and (i3[some] != 1e-8).all() and (n3[~some] == -1).all()
