"""Pruning after a training epoch, CPU side: the oracle's restatements
against the reference's own host flow of Tile.pruning
(training/scripts/tile/tile.py:297-395, run by tests/golden/make_golden.py on
a 16^3 tile with its CUDA helpers as the oracle's restatements), the
dilation against a direct numpy statement, and the occupancy-word layout
against the scene format.

* prune_flags: bit-exact with the reference flow's nodes_flag (with and
  without initial flags);
* transparency_statistic: the fixture's statistic reproduced exactly;
  the transparency threshold removes voxels the geometry threshold keeps;
* dilate_boundary: equals the numpy 3^3 neighbourhood rule;
* pack_occupancy: equals numpy packbits (little bit order) of flags == 1.
"""
import os

import numpy as np

import oracle
import snisr
from snisr import prune

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_python.npz"))


def test_prune_flags_matches_reference_flow():
    N, block = int(G["pr_N"]), int(G["pr_block"])
    out = oracle.op_prune_flags(G["pr_T"], G["pr_voxel_sigma"], None, N, block, G["pr_th"], G["pr_T_th"])
    assert np.array_equal(out, G["pr_out"])
    out = oracle.op_prune_flags(G["pr_T"], G["pr_voxel_sigma"], G["pr_init"], N, block, G["pr_th"], G["pr_T_th"])
    assert np.array_equal(out, G["pr_out_init"])
    kept = (G["pr_out"][1:-1, 1:-1, 1:-1] == 1).sum()
    assert 0 < kept < N ** 3 // 2
    # the transmittance threshold does work here: without it more voxels stay
    loose = oracle.op_prune_flags(G["pr_T"], G["pr_voxel_sigma"], None, N, block, G["pr_th"], -1.0)
    assert (loose[1:-1, 1:-1, 1:-1] == 1).sum() > kept


def test_transparency_statistic_reproduces_fixture():
    N = int(G["pr_N"])
    D = N + 2
    vs = float(G["pr_vs"])
    T = np.zeros((D, D, D), np.float32)
    oracle.op_transparency_statistic(G["pr_ro"], G["pr_rd"], D, G["pr_center"], N * vs, vs,
                                     vs * float(G["pr_rate"]), G["pr_sigma_d"], G["pr_flags"], T)
    assert np.array_equal(T, G["pr_T"])
    assert T.max() <= 1.0 and (T > 0).mean() > 0.3


def _dilate_numpy(f):
    D = f.shape[0]
    pad = np.pad(f == 1, 1)
    near = np.zeros(f.shape, bool)
    for dx in range(3):
        for dy in range(3):
            for dz in range(3):
                near |= pad[dx:dx + D, dy:dy + D, dz:dz + D]
    return np.where((f == -1) & near, 0, f).astype(np.int16)


def test_dilate_boundary_rule():
    rng = np.random.default_rng(4)
    for D, p in ((6, 0.05), (19, 0.02), (34, 0.2)):
        f = rng.choice(np.array([-1, 0, 1], np.int16), size=(D, D, D), p=[1 - p - 0.1, 0.1, p])
        g = f.copy()
        oracle.op_dilate_boundary(g)
        assert np.array_equal(g, _dilate_numpy(f))


def test_pack_occupancy_layout():
    rng = np.random.default_rng(5)
    N = 20
    f = rng.choice(np.array([-1, 0, 1], np.int16), size=(N + 2,) * 3)
    words, count = oracle.op_pack_occupancy(f, N)
    bits = (f[1:-1, 1:-1, 1:-1] == 1).reshape(-1)
    ref = np.packbits(np.concatenate([bits, np.zeros(-len(bits) % 64, bool)]), bitorder="little").view(np.uint64)
    assert np.array_equal(words, ref) and count == bits.sum()


def test_grids_from_scene_arrays():
    s = snisr.SynthScene(snisr.CFG1)
    a = s.arrays()
    sig_d, vsig, flags = prune.grids_from_arrays(s.desc, a, 0)
    N = s.desc.res
    words, count = oracle.op_pack_occupancy(flags, N)
    assert np.array_equal(words, a["occupancy"].reshape(-1)[:words.size].view(np.uint64))
    assert (vsig[flags[1:-1, 1:-1, 1:-1] == 1] > 0).all() and (vsig[flags[1:-1, 1:-1, 1:-1] != 1] == 0).all()
    assert np.array_equal(_dilate_numpy(np.where(flags == 0, -1, flags).astype(np.int16)), flags)
