"""Pruning after a training epoch on the GPU (transparency_statistic,
dilate_boundary, prune_flags, pack_occupancy and the snisr.prune.pruning
routine) against the oracle and the reference-flow fixture.

* dilate_boundary, prune_flags, pack_occupancy: bit-exact (integer and
  comparison work); prune_flags also equals the reference flow's output on
  the 16^3 fixture;
* transparency_statistic: max-abs <= 1e-5 against the oracle (CUDA's expf
  against the host's exp changes the transmittance by ulps; the maxima
  themselves are order-free), on the fixture and on a 128^3 tile of the
  4x4x1-tile scene with 24,576 camera rays that cross it;
* pruning(): equals the oracle's flag update applied to the GPU statistic.
"""
import os

import numpy as np
import pytest

import oracle
import snisr
from snisr import ops, prune

pytestmark = pytest.mark.gpu
G = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_python.npz"))


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_dilate_boundary_bitexact(cuda):
    import torch
    rng = np.random.default_rng(11)
    for D, p in ((6, 0.05), (34, 0.05), (130, 0.01)):
        f = rng.choice(np.array([-1, 0, 1], np.int16), size=(D, D, D), p=[0.9 - p, 0.1, p])
        g = _t(f)
        ops.dilate_boundary(g, D)
        ref = f.copy()
        oracle.op_dilate_boundary(ref)
        torch.cuda.synchronize()
        assert np.array_equal(g.cpu().numpy(), ref)


def test_prune_flags_and_pack_on_fixture(cuda):
    import torch
    N, block = int(G["pr_N"]), int(G["pr_block"])
    for init, key in ((None, "pr_out"), (G["pr_init"], "pr_out_init")):
        out = torch.empty((N + 2,) * 3, dtype=torch.int16, device="cuda")
        ops.prune_flags(_t(G["pr_T"]), _t(G["pr_voxel_sigma"]), None if init is None else _t(init), block,
                        float(G["pr_th"]), float(G["pr_T_th"]), out)
        assert np.array_equal(out.cpu().numpy(), G[key])
        words, count = ops.pack_occupancy(out)
        ref_w, ref_n = oracle.op_pack_occupancy(G[key], N)
        assert np.array_equal(words.cpu().numpy().view(np.uint64), ref_w) and int(count) == ref_n


def test_transparency_statistic_fixture(cuda):
    N = int(G["pr_N"])
    vs = float(G["pr_vs"])
    T = _t(np.zeros((N + 2,) * 3, np.float32))
    ops.transparency_statistic(_t(G["pr_ro"]), _t(G["pr_rd"]), N + 2, _t(G["pr_center"]), N * vs, vs,
                               vs * float(G["pr_rate"]), _t(G["pr_sigma_d"]), _t(G["pr_flags"]), T)
    got = T.cpu().numpy()
    err = float(np.abs(got - G["pr_T"]).max())
    print(f"fixture statistic: max-abs {err:.3g}, identical {float((got == G['pr_T']).mean()):.4f}")
    assert err <= 1e-5


def _crosses(o, d, c, h):
    """Rays that cross the box (float64 slab test; selection only)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d.astype(np.float64)
        t0 = (c - h - o) * inv
        t1 = (c + h - o) * inv
    lo = np.nanmax(np.minimum(t0, t1), axis=1)
    hi = np.nanmin(np.maximum(t0, t1), axis=1)
    return (hi > np.maximum(lo, 0)) & np.isfinite(hi)


@pytest.fixture(scope="module")
def tile_problem():
    s = snisr.SynthScene(snisr.CFG2)
    a = s.arrays()
    t = 5
    sig_d, vsig, flags = prune.grids_from_arrays(s.desc, a, t)
    center = prune.tile_centers(s.desc, a)[t]
    tile = float(s.desc.tile_size)
    N = int(s.desc.res)
    rng = np.random.default_rng(8)
    ro, rd = [], []
    for v in range(4):
        cam = s.camera(v, 320, 180)
        d = oracle.camera_dirs(cam)
        o = oracle.camera_origins(cam, d.shape[0])
        hit = _crosses(o, d, center, tile / 2)
        ro.append(o[hit])
        rd.append(d[hit])
    ro, rd = np.concatenate(ro), np.concatenate(rd)
    pick = np.sort(rng.choice(ro.shape[0], min(24576, ro.shape[0]), replace=False))
    return dict(N=N, tile=tile, vs=tile / N, center=center, sig_d=sig_d, vsig=vsig, flags=flags,
                ro=np.ascontiguousarray(ro[pick]), rd=np.ascontiguousarray(rd[pick]))


def test_transparency_statistic_scene_tile(cuda, tile_problem):
    P = tile_problem
    D = P["N"] + 2
    step = P["vs"] * 0.1
    ref = np.zeros((D, D, D), np.float32)
    oracle.op_transparency_statistic(P["ro"], P["rd"], D, P["center"], P["tile"], P["vs"], step, P["sig_d"],
                                     P["flags"], ref)
    T = _t(np.zeros((D, D, D), np.float32))
    ops.transparency_statistic(_t(P["ro"]), _t(P["rd"]), D, _t(P["center"]), P["tile"], P["vs"], step,
                               _t(P["sig_d"]), _t(P["flags"]), T)
    got = T.cpu().numpy()
    err = float(np.abs(got - ref).max())
    print(f"128^3 tile statistic: {P['ro'].shape[0]} rays, touched {float((ref > 0).mean()):.4f}, "
          f"max-abs {err:.3g}, identical {float((got == ref).mean()):.5f}")
    assert (ref > 0).sum() > 10000
    assert err <= 1e-5


@pytest.mark.parametrize("with_init", [False, True], ids=["all-on", "init-flags"])
def test_pruning_routine(cuda, tile_problem, with_init):
    """Without initial flags the reference starts from every voxel on and
    keeps whole 4^3 blocks whose densest voxel passes the geometry
    threshold; with the current occupancy as initial flags (its INIT_VOXEL
    form) voxels can only be removed."""
    P = tile_problem
    init = np.where(P["flags"][1:-1, 1:-1, 1:-1] == 1, 1, -1).astype(np.int16) if with_init else None
    r = prune.pruning(_t(P["ro"]), _t(P["rd"]), _t(P["center"]), P["tile"], P["vs"], _t(P["sig_d"]),
                      _t(P["flags"]), _t(P["vsig"]), None if init is None else _t(init), block=4, th=0.5,
                      T_th=0.01)
    T = r.T_voxels.cpu().numpy()
    ref = oracle.op_prune_flags(T, P["vsig"], init, P["N"], 4, 0.5, 0.01)
    assert np.array_equal(r.nodes_flag.cpu().numpy(), ref)
    words, count = oracle.op_pack_occupancy(ref, P["N"])
    assert r.occupied == count and np.array_equal(r.words.cpu().numpy().view(np.uint64), words)
    before = int((P["flags"] == 1).sum())
    print(f"pruning ({'init flags' if with_init else 'all on'}): {before} -> {r.occupied} voxels")
    assert r.occupied > 0
    if with_init:
        assert r.occupied < before
