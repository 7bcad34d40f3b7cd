"""Training-ray preparation (get_trainData_v3's device chain and
CUDA_EXT.Sample_bg) on the GPU against the oracle, on the 4x4x1-tile scene
with its ~205k-triangle proxy mesh, three 192x108 views:

* train_rays, train_tracing_tiles, double_hits, train_bgdepth, Sample_bg,
  patch_rows: bit-exact (the same operations, fused where the reference's
  build fuses them; the double hits use the same two-sided triangle test);
* gen_diffuse: bit-exact except where CUDA's rsqrtf (the kernel, as the
  reference) and the oracle's correctly rounded 1/sqrt differ: values within
  2e-7, and pixels whose only contributing view is their own training view,
  where the view-angle weight is a rounding residue -- one side keeps 0, the
  other takes the pixel's own colour (its row's ground-truth colour);
* TrainPrep.view / get_train_data: the rows equal the oracle chain's rows
  under the same rule for the diffuse columns.

Depth maps are the proxy mesh's first-hit depth of each view (camera z),
images seeded noise in [0, 1].
"""
import numpy as np
import pytest

import oracle
import snisr
from snisr import trainprep

pytestmark = pytest.mark.gpu
H, W, KT, P = 108, 192, 30, 7


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def prep(cuda):
    s = snisr.SynthScene(snisr.CFG2)
    a = s.arrays()
    d = s.desc
    sc = snisr.Scene(d)
    osc = oracle.OracleScene(d)
    views = [0, 3, 5]
    Ks, C2Ws = [], []
    for v in views:
        cam = s.camera(v, W, H)
        f = 1.0 / cam.inv_focal
        Ks.append(np.array([f, 0, cam.cx, 0, f, cam.cy, 0, 0, 1], np.float32))
        C2Ws.append(np.array(list(cam.c2w), np.float32))
    Ks, C2Ws = np.stack(Ks), np.stack(C2Ws)
    rng = np.random.default_rng(3)
    images = rng.random((len(views), H * W, 3), dtype=np.float32)
    depths = np.zeros((len(views), H * W), np.float32)
    for j in range(len(views)):
        ro, rd = oracle.train_rays(Ks[j], C2Ws[j], H, W)
        t, _ = sc.proxy_hit(_t(ro), _t(rd))
        tt = t.cpu().numpy()
        depths[j] = np.where(tt > 0, tt, 1e4)
    grid = (int(d.grid[0]), int(d.grid[1]), int(d.grid[2]))
    yield dict(s=s, a=a, d=d, sc=sc, osc=osc, Ks=Ks, C2Ws=C2Ws, images=images, depths=depths, grid=grid,
               imap=np.asarray(a["tile_index"], np.int32).reshape(-1), smin=np.array(list(d.scene_min), np.float32),
               tile=float(d.tile_size))
    sc.close()


def _diffuse_agrees(got, ref, own):
    """Per pixel: the same diffuse colour up to 2e-7, or (the training view's
    own weight being a rounding residue on one side only) one side 0 and the
    other the pixel's own colour within 1e-3."""
    close = (np.abs(got - ref) <= 2e-7).all(1)
    zero_g, zero_r = (got == 0).all(1), (ref == 0).all(1)
    own_g = (np.abs(got - own) <= 1e-3).all(1)
    own_r = (np.abs(ref - own) <= 1e-3).all(1)
    return close | (zero_g & own_r) | (zero_r & own_g)


def _rows_agree(got, ref):
    """Patch rows [n, P*P, 14] = ray origin, direction, bg depth, gt colour,
    diffuse, valid: every column but the diffuse one identical, the diffuse
    columns under _diffuse_agrees (own colour = the row's gt colour)."""
    other = np.r_[0:10, 13]
    assert np.array_equal(got[..., other], ref[..., other])
    g, r = got[..., 10:13].reshape(-1, 3), ref[..., 10:13].reshape(-1, 3)
    ok = _diffuse_agrees(g, r, ref[..., 7:10].reshape(-1, 3))
    return bool(ok.all()), float((g == r).all(1).mean())


def _chain_oracle(P_, j, train_tile):
    ro, rd = oracle.train_rays(P_["Ks"][j], P_["C2Ws"][j], H, W)
    vis = oracle.train_tracing(ro, rd, P_["imap"], P_["grid"], P_["smin"], P_["tile"], KT)
    hits = P_["osc"].double_hits(ro, rd, vis)
    bg, valid = oracle.train_bgdepth(train_tile, vis, hits)
    ms = np.stack([oracle.project_matrix(P_["Ks"][i], P_["C2Ws"][i]) for i in range(len(P_["Ks"]))])
    origins = P_["C2Ws"][:, [3, 7, 11]].copy()
    diffuse = oracle.gen_diffuse(origins, train_tile, ro, rd, hits, vis, P_["images"], P_["depths"], ms, H, W, bg)
    rows = oracle.patch_rows(valid, H, W, P, ro, rd, bg, P_["images"][j], diffuse)
    return dict(ro=ro, rd=rd, vis=vis, hits=hits, bg=bg, valid=valid, diffuse=diffuse, rows=rows, ms=ms)


def test_project_matrix_matches_oracle(prep):
    for K, c in zip(prep["Ks"], prep["C2Ws"]):
        assert np.array_equal(trainprep.project_matrix(K, c), oracle.project_matrix(K, c))


def test_chain_bitexact(prep):
    import torch
    P_ = prep
    j = 0
    # training tile: the tile of most first hits in view 0 (oracle)
    ro, rd = oracle.train_rays(P_["Ks"][j], P_["C2Ws"][j], H, W)
    vis = oracle.train_tracing(ro, rd, P_["imap"], P_["grid"], P_["smin"], P_["tile"], KT)
    hits = P_["osc"].double_hits(ro, rd, vis)
    first = np.array([vis[i][np.argmax(hits[i, :, 0] != -1)] if (hits[i, :, 0] != -1).any() else -1
                      for i in range(vis.shape[0])])
    train_tile = int(np.bincount(first[first >= 0]).argmax())
    ref = _chain_oracle(P_, j, train_tile)

    tp = trainprep.TrainPrep(P_["sc"], H, W, P_["imap"], P_["grid"], P_["smin"], P_["tile"], KT, P)
    proj = _t(ref["ms"])
    origins = _t(P_["C2Ws"][:, [3, 7, 11]])
    rows, count = tp.view(train_tile, _t(P_["Ks"][j]), _t(P_["C2Ws"][j]), _t(P_["images"][j]), origins,
                          _t(P_["images"]), _t(P_["depths"]), proj)
    torch.cuda.synchronize()
    P_["sc"].check()
    g = lambda t: t.cpu().numpy()
    assert np.array_equal(g(tp.ro), ref["ro"]) and np.array_equal(g(tp.rd), ref["rd"])
    assert np.array_equal(g(tp.visited), ref["vis"])
    hit_eq = g(tp.hits) == ref["hits"]
    print(f"tile {train_tile}: pairs with a hit {int((ref['hits'][..., 0] != -1).sum())}, "
          f"second hits {int((ref['hits'][..., 1] != -1).sum())}, hits identical {float(hit_eq.mean()):.6f}, "
          f"valid {int(ref['valid'].sum())}, patches {ref['rows'].shape[0]}")
    assert hit_eq.all()
    assert np.array_equal(g(tp.valid), ref["valid"]) and np.array_equal(g(tp.bg), ref["bg"])
    dif = g(tp.diffuse)
    own = P_["images"][j]
    assert _diffuse_agrees(dif, ref["diffuse"], own).all()
    print(f"diffuse identical {float((dif == ref['diffuse']).all(1).mean()):.4f}")
    n = int(count)
    assert n == ref["rows"].shape[0] and n > 0
    ok, _ = _rows_agree(g(rows[:n * P * P]).reshape(n, P * P, 14), ref["rows"])
    assert ok
    assert int(ref["valid"].sum()) > 100 and (ref["diffuse"].sum(1) > 0).sum() > 100


def test_get_train_data_all_views(prep):
    import torch
    P_ = prep
    train_tile = 5
    out = trainprep.get_train_data(P_["sc"], train_tile, P_["Ks"], P_["C2Ws"], [0, 1, 2],
                                   _t(P_["images"].reshape(3, H, W, 3)), _t(P_["depths"].reshape(3, H, W)),
                                   P_["imap"], P_["grid"], P_["smin"], P_["tile"], KT, P)
    torch.cuda.synchronize()
    ref = np.concatenate([_chain_oracle(P_, j, train_tile)["rows"] for j in range(3)])
    assert out.shape == ref.shape
    ok, _ = _rows_agree(out.cpu().numpy(), ref)
    assert ok


def test_sample_bg_bitexact(prep):
    import torch
    from snisr import ops
    P_ = prep
    rng = np.random.default_rng(9)
    n, ns = 4096, 16
    center = np.array([1.5, 4.5, 1.5], np.float32)
    ro = (center + rng.uniform(-6, 6, (n, 3))).astype(np.float32)
    rd = rng.standard_normal((n, 3)).astype(np.float32)
    bg = rng.uniform(0.0, 12.0, (n, 1)).astype(np.float32)
    bg[::7] = -1.0
    ref = np.full((n, ns), -1, np.float32)
    oracle.sample_bg(ro, rd, bg, ns, 0.6, center, P_["tile"], ref)
    z = ops.sampling_background(_t(ro), _t(rd), _t(bg), _t(center), P_["tile"], ns, 0.6)
    torch.cuda.synchronize()
    assert np.array_equal(z.cpu().numpy(), ref)
    assert (ref[::7] == -1).all() and (ref[1::7] != -1).all()
