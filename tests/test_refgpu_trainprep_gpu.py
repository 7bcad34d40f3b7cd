"""Training-data preparation against the reference's own kernels
(training/src/cuda_func.cu, compiled from its source into a cubin by
oracle/build_ref.py and launched by tests/refgpu.py as get_trainData_v3
launches them), on the 4x4x1-tile scene and its proxy mesh, three 192x108
views.  Each stage gets the same inputs on both sides:

* rays (computing_rays_kernel) and the tile DDA (tracingTile_kernel);
* the two nearest proxy hits per (ray, visited tile): the reference walks
  per-tile 16^3 block face lists (BConFaceNum / BConFaceIdx, built here from
  the mesh, every triangle listed in every block its padded bounding box
  touches) with its winding-flipped one-sided test; the library walks its
  BVH with the two-sided test;
* background depth and validity (get_trainData_kernel);
* the multi-view diffuse estimate (gen_diffuse_in_tile_kernel).

The reference's FP32 sparse-voxel renderer of the second training
iteration (render_diffuse_kernel) is timed beside the plain FP32 form of the
library's renderer on one 1280x720 frame (test_timing_*).
"""
import numpy as np
import pytest

import oracle
import refgpu
import snisr
from snisr import trainprep

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refgpu.available("cuda_func"),
                                 reason="the reference's cuda_func.cu cubin was not built (no reference tree)")]
H, W, KT, P = 108, 192, 30, 7
NUM_BLOCK = 16


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def block_face_lists(desc, arrays, num_block, pad=1e-4):
    """The reference's per-tile block face lists: for sparse tile t and block
    b = z + y*nb + x*nb*nb, BConFaceNum[t*nb^3 + b] = (start, count) into
    BConFaceIdx, faces in increasing id order."""
    V = arrays["mesh_vertices"].astype(np.float64)
    Fc = arrays["mesh_faces"].astype(np.int64)
    tri = V[Fc]  # [nt, 3, 3]
    lo, hi = tri.min(1) - pad, tri.max(1) + pad
    ts = float(desc.tile_size)
    bs = ts / num_block
    imap = arrays["tile_index"].reshape(desc.grid[0], desc.grid[1], desc.grid[2])
    smin = np.array(list(desc.scene_min), np.float64)
    nb3 = num_block ** 3
    keys, faces = [], []
    for x in range(desc.grid[0]):
        for y in range(desc.grid[1]):
            for z in range(desc.grid[2]):
                t = int(imap[x, y, z])
                if t < 0:
                    continue
                corner = smin + np.array([x, y, z]) * ts
                l = np.floor((lo - corner) / bs).astype(np.int64)
                h = np.floor((hi - corner) / bs).astype(np.int64)
                sel = np.nonzero(((h >= 0) & (l < num_block)).all(1))[0]
                l = np.clip(l[sel], 0, num_block - 1)
                h = np.clip(h[sel], 0, num_block - 1)
                for f, a, b in zip(sel, l, h):
                    for bx in range(a[0], b[0] + 1):
                        for by in range(a[1], b[1] + 1):
                            for bz in range(a[2], b[2] + 1):
                                keys.append(t * nb3 + bz + by * num_block + bx * num_block * num_block)
                                faces.append(f)
    keys = np.array(keys, np.int64)
    faces = np.array(faces, np.int32)
    order = np.lexsort((faces, keys))
    keys, faces = keys[order], faces[order]
    total = desc.num_tiles * nb3
    counts = np.bincount(keys, minlength=total).astype(np.int32)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int32)
    return np.stack([starts, counts], 1).astype(np.int32), faces


@pytest.fixture(scope="module")
def prep(cuda):
    s = snisr.SynthScene(snisr.CFG2)
    a = s.arrays()
    d = s.desc
    sc = snisr.Scene(d)
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
    bnum, bidx = block_face_lists(d, a, NUM_BLOCK)
    grid = (int(d.grid[0]), int(d.grid[1]), int(d.grid[2]))
    imap = np.asarray(a["tile_index"], np.int32).reshape(-1)
    centers = np.zeros((d.num_tiles, 3), np.float32)
    for x in range(grid[0]):
        for y in range(grid[1]):
            for z in range(grid[2]):
                tid = imap[(x * grid[1] + y) * grid[2] + z]
                if tid >= 0:
                    centers[tid] = [d.scene_min[0] + (x + 0.5) * d.tile_size, d.scene_min[1] + (y + 0.5) * d.tile_size,
                                    d.scene_min[2] + (z + 0.5) * d.tile_size]
    yield dict(s=s, a=a, d=d, sc=sc, Ks=Ks, C2Ws=C2Ws, images=images, depths=depths, grid=grid, imap=imap,
               smin=np.array(list(d.scene_min), np.float32), tile=float(d.tile_size), bnum=bnum, bidx=bidx,
               centers=centers)
    sc.close()


def test_block_face_lists_cover_the_mesh(prep):
    bnum, bidx = prep["bnum"], prep["bidx"]
    assert bnum[:, 1].sum() == bidx.size and bidx.max() < prep["d"].num_triangles
    assert np.unique(bidx).size == prep["d"].num_triangles  # every triangle lies in some block


def test_trainprep_stages_against_reference_kernels(prep):
    import torch
    P_ = prep
    g = lambda x: x.cpu().numpy()
    tp = trainprep.TrainPrep(P_["sc"], H, W, P_["imap"], P_["grid"], P_["smin"], P_["tile"], KT, P)
    ms = np.stack([trainprep.project_matrix(P_["Ks"][i], P_["C2Ws"][i]) for i in range(3)])
    origins = _t(P_["C2Ws"][:, [3, 7, 11]])
    # device copies held for the whole test: the launches are asynchronous
    images, depths, ms_d = _t(P_["images"]), _t(P_["depths"]), _t(ms)
    verts, faces = _t(P_["a"]["mesh_vertices"]), _t(P_["a"]["mesh_faces"])
    centers, bnum, bidx = _t(P_["centers"]), _t(P_["bnum"]), _t(P_["bidx"])
    imap = _t(P_["imap"])
    n = H * W
    train_tile = 5
    stats = {}
    for j in range(3):
        # the library's chain for view j
        K_d, C2W_d, gt_d = _t(P_["Ks"][j]), _t(P_["C2Ws"][j]), _t(P_["images"][j])
        tp.view(train_tile, K_d, C2W_d, gt_d, origins, images, depths, ms_d)
        torch.cuda.synchronize()
        P_["sc"].check()
        # rays
        ro = torch.empty(n, 3, device="cuda")
        rd = torch.empty(n, 3, device="cuda")
        refgpu.computing_rays(H, W, K_d, C2W_d, ro, rd)
        torch.cuda.synchronize()
        stats.setdefault("rays_identical", []).append(float((g(rd) == g(tp.rd)).all(1).mean()))
        stats.setdefault("rays_max_abs", []).append(float(np.abs(g(rd) - g(tp.rd)).max()))
        assert np.array_equal(g(ro), g(tp.ro))
        # tile DDA on the library's rays
        vis = torch.empty(n, KT, dtype=torch.int32, device="cuda")
        refgpu.tracing_tile(H, W, tp.ro, tp.rd, imap, P_["grid"], P_["tile"], KT, vis, P_["smin"])
        torch.cuda.synchronize()
        stats.setdefault("visited_identical", []).append(float((g(vis) == g(tp.visited)).all(1).mean()))
        # double hits on the library's rays and visited tiles
        hits = torch.full((n, KT, 2), -7.0, device="cuda")
        refgpu.ray_double_hit_in_tile(H, W, tp.ro, tp.rd, verts, faces, centers, bidx, bnum, P_["tile"], KT,
                                      NUM_BLOCK, tp.visited, hits)
        torch.cuda.synchronize()
        rh, mh = g(hits), g(tp.hits)
        has = (mh[..., 0] != -1) | (rh[..., 0] != -1)
        stats.setdefault("pairs_with_hit", []).append(int(has.sum()))
        stats.setdefault("first_hit_identical", []).append(float((rh[..., 0] == mh[..., 0])[has].mean()))
        stats.setdefault("second_hit_identical", []).append(float((rh[..., 1] == mh[..., 1])[has].mean()))
        close1 = np.abs(rh[..., 0] - mh[..., 0]) <= 1e-5 * np.maximum(1.0, np.abs(mh[..., 0]))
        stats.setdefault("first_hit_within_1e-5", []).append(float(close1[has].mean()))
        dup = (rh[..., 1] == rh[..., 0]) & (rh[..., 0] != -1) & (mh[..., 1] != mh[..., 0])
        stats.setdefault("reference_duplicate_second_hits", []).append(int(dup.sum()))
        # background depth and validity: both sides on the reference's hits
        bg_r = torch.full((n,), -1.0, device="cuda")
        va_r = torch.zeros(n, dtype=torch.int32, device="cuda")
        refgpu.get_train_data(train_tile, tp.ro, tp.rd, verts, faces, tp.visited, hits, KT, bg_r, va_r)
        bg_m = torch.empty(n, device="cuda")
        va_m = torch.empty(n, dtype=torch.int32, device="cuda")
        snisr._lib.check(snisr.lib().snisr_op_train_bgdepth(train_tile, tp.visited.data_ptr(), hits.data_ptr(), n, KT,
                                                            bg_m.data_ptr(), va_m.data_ptr(),
                                                            torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        assert np.array_equal(g(va_r), g(va_m)) and np.array_equal(g(bg_r), g(bg_m))
        stats.setdefault("valid_rays", []).append(int(g(va_m).sum()))
        # diffuse estimate: both sides on the same hits and background depths
        dif_r = torch.full((n, 3), -7.0, device="cuda")
        bgd_r = bg_r.clone()
        refgpu.gen_diffuse_in_tile(origins, train_tile, tp.ro, tp.rd, hits, tp.visited, images, depths, ms_d, KT, 3,
                                   H, W, dif_r, bgd_r)
        dif_m = torch.full((n, 3), -7.0, device="cuda")
        bgd_m = bg_r.clone()
        L = snisr.lib()
        snisr._lib.check(L.snisr_op_gen_diffuse(origins.data_ptr(), train_tile, tp.ro.data_ptr(), tp.rd.data_ptr(),
                                                hits.data_ptr(), tp.visited.data_ptr(), images.data_ptr(),
                                                depths.data_ptr(), ms_d.data_ptr(), KT, 3, H, W,
                                                dif_m.data_ptr(), bgd_m.data_ptr(),
                                                torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        stats.setdefault("bg_after_visibility_identical", []).append(float((g(bgd_r) == g(bgd_m)).mean()))
        stats.setdefault("diffuse_identical", []).append(float((g(dif_r) == g(dif_m)).all(1).mean()))
        stats.setdefault("diffuse_max_abs", []).append(float(np.abs(g(dif_r) - g(dif_m)).max()))
        stats.setdefault("diffuse_nonzero", []).append(int((g(dif_m).sum(1) > 0).sum()))
    print("training-data preparation vs the reference's kernels:", stats)
    assert min(stats["visited_identical"]) == 1.0
    assert min(stats["pairs_with_hit"]) > 1000 and sum(stats["valid_rays"]) > 1000
    assert min(stats["rays_identical"]) == 1.0
    assert min(stats["first_hit_within_1e-5"]) > 0.99
    # same inputs on both sides: background depth, validity and the diffuse
    # estimate are identical to the reference's kernels
    assert min(stats["bg_after_visibility_identical"]) == 1.0
    assert min(stats["diffuse_identical"]) == 1.0


def _dense_reference_grid(s, res):
    """The reference's second-iteration tile data from the synthetic scene:
    per tile a dilated (res+2)^3 grid of RGBA (RGB in (0, 1), density per
    world length = softplus of the voxel's mean corner logit / voxel size) and
    int16 sample flags (1 on occupied voxels), index (x+1, y+1, z+1)."""
    d = s.desc
    a = s.arrays()
    N = res
    D = N + 2
    words = a["occupancy"].reshape(d.num_tiles, -1)
    bits = np.unpackbits(words.view(np.uint8), axis=1, bitorder="little").astype(bool)
    logit = a["vertex_density"].astype(np.float32)[a["voxel_corners"]].mean(1)
    sigma = np.logaddexp(0.0, logit).astype(np.float32) / np.float32(d.tile_size / N)
    rng = np.random.default_rng(17)
    rgb = rng.random((d.num_voxels, 3), dtype=np.float32)
    vox = np.zeros((d.num_tiles, D, D, D, 4), np.float32)
    nodes = np.zeros((d.num_tiles, D, D, D), np.int16)
    k = 0
    for t in range(d.num_tiles):
        ids = np.nonzero(bits[t])[0]
        x, y, z = ids // (N * N), (ids // N) % N, ids % N
        m = ids.size
        vox[t, x + 1, y + 1, z + 1, :3] = rgb[k:k + m]
        vox[t, x + 1, y + 1, z + 1, 3] = sigma[k:k + m]
        nodes[t, x + 1, y + 1, z + 1] = 1
        k += m
    return vox.reshape(-1), nodes.reshape(-1)


def test_timing_render_diffuse_vs_plain_form(prep):
    """One 1280x720 frame of the 4x4x1 scene: the reference's FP32 renderer
    (baked per-voxel RGBA, no MLP, samples every half voxel, early stop at
    T < 1e-5) against the library's plain FP32 form (per-sample MLP 59-64x3-3
    on the CUDA cores) and tensor-core form, CUDA events, L2 flushed."""
    import torch
    P_ = prep
    s, d = P_["s"], P_["d"]
    cam = s.camera(0)
    Wf, Hf = cam.width, cam.height
    n = Wf * Hf
    vox, nodes = _dense_reference_grid(s, int(d.res))
    vox_d, nodes_d = _t(vox), _t(nodes)
    del vox, nodes
    f = 1.0 / cam.inv_focal
    K = _t(np.array([f, 0, cam.cx, 0, f, cam.cy, 0, 0, 1], np.float32))
    C2W = _t(np.array(list(cam.c2w), np.float32))
    ro = torch.empty(n, 3, device="cuda")
    rd = torch.empty(n, 3, device="cuda")
    refgpu.computing_rays(Hf, Wf, K, C2W, ro, rd)
    vis = torch.empty(n, KT, dtype=torch.int32, device="cuda")
    imap, centers = _t(P_["imap"]), _t(P_["centers"])  # held: the launches are asynchronous
    refgpu.tracing_tile(Hf, Wf, ro, rd, imap, P_["grid"], P_["tile"], KT, vis, P_["smin"])
    s2g = _t(np.arange(d.num_tiles, dtype=np.int32))
    dif = torch.empty(n, 3, device="cuda")
    dep = torch.empty(n, device="cuda")
    val = torch.empty(n, dtype=torch.int32, device="cuda")
    voxel = P_["tile"] / int(d.res)
    flush = torch.empty(64 * 1024 * 1024, device="cuda")
    stream = torch.cuda.current_stream()

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return min(ms)

    ref_ms = timed(lambda: refgpu.render_diffuse(5, ro, rd, vis, s2g, KT, P_["tile"], int(d.res) + 2, voxel,
                                                 0.5 * voxel, centers, vox_d, nodes_d, dif, dep, val))
    assert int(val.sum()) > n // 2  # most rays reach an occupied voxel
    out = (torch.empty(n, 3, device="cuda"), torch.empty(n, device="cuda"), torch.empty(n, device="cuda"))
    plain_ms = timed(lambda: P_["sc"].render(cam, snisr.FORM_PLAIN_FP32, out))
    tc_ms = timed(lambda: P_["sc"].render(cam, snisr.FORM_TC, out))
    P_["sc"].check()
    print(f"1280x720 frame: reference render_diffuse_kernel (FP32, baked RGBA) {ref_ms:.3f} ms; library plain "
          f"FP32 form (per-sample MLP) {plain_ms:.3f} ms; tensor-core form {tc_ms:.3f} ms")
    assert ref_ms > 0 and plain_ms > 0 and tc_ms > 0
