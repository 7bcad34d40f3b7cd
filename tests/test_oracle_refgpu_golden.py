"""The oracle against golden vectors of the reference's own CUDA kernels
(tests/golden/reference_kernels.npz, written on a GB300 by
tests/golden/make_refgpu_golden.py from the kernels compiled out of the
reference's sources).  Inputs are rebuilt from the same seeds
(tests/refgpu_cases.py).

* compute_rays, tracing_tiles (camera inside and outside the scene box),
  inverse_z_sampling, Sample_sparse, Sample_bg, dilate_boundary: identical.
* rendering_diffuse_octree_fp16: inverse near depth and network ids
  identical; colours identical but where the oracle's FP16 exponential
  (exp rounded once) and CUDA's hexp round differently (at most 1 % of the
  pixels, by at most two FP16 ulps).
* integrate_points (the reference's __expf against std::exp) and
  transparency_statistic (CUDA's expf against the host's): within 1e-6 and
  1e-5."""
import os

import numpy as np
import pytest

import oracle
import refgpu_cases as cases

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_kernels.npz")
pytestmark = pytest.mark.skipif(not os.path.exists(GOLD), reason="reference-kernel golden vectors not generated")


@pytest.fixture(scope="module")
def G():
    return np.load(GOLD)


def test_compute_rays_and_tracing(G):
    c = cases.camera_case()
    rays = oracle.op_compute_rays(c["intr"], c["rot"], c["H"], c["W"]).reshape(c["H"], c["W"], 3)
    assert np.array_equal(rays, G["cr_rays"])
    tc = cases.tracing_case()
    for tag, origin in (("in", c["origin"]), ("out", cases.OUTSIDE_ORIGIN)):
        vis = oracle.op_tracing_tiles(G["cr_rays"].reshape(-1, 3), tc["imap"], origin, tc["shape"], tc["smin"],
                                      tc["ssize"], np.float32(tc["tile"]), tc["K"])
        assert np.array_equal(vis, G[f"tt_vis_{tag}"].reshape(-1, tc["K"])), tag


@pytest.mark.parametrize("soft", [False, True], ids=["hard", "soft"])
def test_octree_renderer(G, soft):
    o = cases.octree_case()
    n = o["H"] * o["W"]
    k = "soft" if soft else "hard"
    fo = np.zeros((n, 3), np.float32)
    io = np.full(n, 1e-8, np.float32)
    no = np.full(n, -1, np.int16)
    oracle.op_rendering_diffuse_octree(G["oc_rays"].reshape(n, 3), G["oc_vis"].reshape(n, o["K"]), o["origin"],
                                       o["D"], o["sample_step"], 0.0 if soft else 0.8, 0.01, fo, io, no,
                                       soft_hit=soft)
    fr = G[f"oc_frame_{k}"].reshape(n, 3)
    assert (G[f"oc_net_{k}"] >= 0).mean() > 0.3
    assert np.array_equal(io, G[f"oc_inv_{k}"].reshape(n)) and np.array_equal(no, G[f"oc_net_{k}"].reshape(n))
    same = (fo == fr).all(1)
    assert same.mean() >= 0.99
    assert np.abs(fo - fr).max() <= 2 * 2.0 ** -11


def test_inverse_z_and_integrate(G):
    z = cases.inverse_z_case()
    for off in z["offsets"]:
        pts, steps = oracle.op_inverse_z(z["rays_d"].reshape(-1, 3), z["origin"], z["inv_near"].reshape(-1),
                                         z["inv_bound"].reshape(-1), off, z["spr"])
        assert np.array_equal(pts.reshape(z["pts_shape"]), G[f"iz_pts_{off}"])
        assert np.array_equal(steps.reshape(z["steps_shape"]), G[f"iz_steps_{off}"])
    ip = cases.integrate_case()
    n = ip["frame"].shape[0] * ip["frame"].shape[1]
    fr, tr = oracle.op_integrate(ip["rgba"].reshape(n, 16, 4), ip["dz"].reshape(n, 16), np.float32(ip["early"]),
                                 ip["frame"].reshape(n, 3).copy(), ip["trans"].reshape(n).copy())
    np.testing.assert_allclose(fr, G["ip_frame"].reshape(n, 3), atol=1e-6)
    np.testing.assert_allclose(tr, G["ip_trans"].reshape(n), atol=1e-6)


def test_training_ops(G):
    ss = cases.sample_sparse_case()
    zv, dv = oracle.op_sample_sparse(ss["ro"], ss["rd"], ss["flags"], np.array(ss["center"], np.float32),
                                     np.float32(ss["tile"]), ss["N"], ss["ns"])
    assert np.array_equal(zv, G["ss_z"]) and np.array_equal(dv, G["ss_d"])
    assert (G["ss_z"][:, 0] != -1).sum() > 20
    bg = cases.sample_bg_case()
    zb = np.full((bg["n"], bg["ns"]), -1, np.float32)
    oracle.sample_bg(bg["ro"], bg["rd"], bg["bg"], bg["ns"], bg["range"], bg["center"], bg["tile"], zb)
    assert np.array_equal(zb, G["bg_z"])
    ts = cases.transparency_case()
    T = np.zeros((ts["D"],) * 3, np.float32)
    oracle.op_transparency_statistic(ts["ro"], ts["rd"], ts["D"], ts["center"], np.float32(ts["tile"]),
                                     np.float32(ts["vs"]), np.float32(ts["step"]), ts["sigma"], ts["flags"], T)
    ref = np.zeros(T.size, np.float32)
    ref[G["ts_idx"]] = G["ts_val"]
    assert G["ts_idx"].size > 100
    assert float(np.abs(T.reshape(-1) - ref).max()) <= 1e-5
    db = cases.dilate_case()
    f = db["flags"].copy()
    oracle.op_dilate_boundary(f)
    assert np.array_equal(f, G["db_flags"])
