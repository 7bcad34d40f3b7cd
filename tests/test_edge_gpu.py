"""Edge cases of the drop-in ops on the GPU, against the oracle or the
reference's documented no-op behaviour: empty and ragged inputs, networks
with fewer pixels than blocks, skipped (-1) networks, rays that miss, tiles
no ray visits, images smaller than one patch, grids whose voxel count is not
a multiple of 64."""
import numpy as np
import pytest

import oracle
import snisr
from snisr import ops, prune, trainprep

pytestmark = pytest.mark.gpu
SENT = -7.0


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_assign_pixels_more_blocks_than_pixels(cuda):
    import torch
    net = np.array([3, -1, 7, 9], np.int16)
    ps = np.array([0, 2, 3, 10, 11], np.int32)         # 2, 1, 7, 1 pixels
    bs = np.array([0, 4, 5, 8, 11], np.int32)          # 4, 1, 3, 3 blocks
    nn_g, np_g = torch.zeros(11, dtype=torch.int16, device="cuda"), torch.zeros(11, dtype=torch.int32, device="cuda")
    ops.assign_pixels(_t(net), _t(ps), _t(bs), 0, nn_g, np_g)
    nn_o, np_o = np.zeros(11, np.int16), np.zeros(11, np.int32)
    oracle.op_assign_pixels(net, ps, bs, nn_o, np_o)
    assert np.array_equal(nn_g.cpu().numpy(), nn_o) and np.array_equal(np_g.cpu().numpy(), np_o)


def test_inference_mlp_skips_unassigned_network(cuda):
    from snisr import spec_synth as sp
    P = sp.problem(5, G=4, H=8, W=16)
    npix, spr = P["npix"], P["spr"]
    net = np.array([-1, 2], np.int16)
    ps = np.array([0, 64, npix], np.int32)
    q = np.arange(npix, dtype=np.int32)
    samples = np.repeat(P["rays_d"][:, None, :], spr, 1).astype(np.float32)
    res_g = _t(np.full((npix, spr, 4), SENT, np.float32))
    ops.inference_mlp(spr, 2, 0, float(P["inverse_far"]), float(P["trans_stop"]), _t(net),
                      _t(np.ones(npix, np.float32)), _t(q), _t(ps), _t(P["centers"]), _t(samples), _t(P["rays_d"]),
                      _t(P["params"]), res_g)
    ops.check_errors()
    got = res_g.cpu().numpy()
    assert (got[:64] == SENT).all()          # network -1: untouched, as the reference returns
    assert (got[64:] != SENT).all()


def test_octree_rays_without_tiles(cuda):
    import torch
    s = snisr.SynthScene(snisr.CFG1)
    from snisr import octree
    D = octree.from_synth(s)
    der = octree.derived(D)
    T = octree.to_device(D)
    n, K = 1000, 30
    rays = torch.randn(n, 3, device="cuda")
    visited = torch.full((n, K), -1, dtype=torch.int32, device="cuda")
    frame = torch.full((n, 3), SENT, device="cuda")
    inv = torch.full((n,), SENT, device="cuda")
    net = torch.full((n,), 5, dtype=torch.int16, device="cuda")
    origin = _t(np.zeros(3, np.float32))
    ops.rendering_diffuse_octree_fp16(rays, visited, origin, T["tile2group"], T["data_voxels"], T["block_IndexMap"],
                                      T["nodes_IndexMap"], T["nodes_sampleFlag"], T["voxels_start"], T["centers"],
                                      der["tile_size"], der["voxel_size"], der["sample_step"], der["block_num_voxel"],
                                      0, 0.8, 0.01, True, frame, inv, net)
    torch.cuda.synchronize()
    assert (frame.cpu().numpy() == 0).all()
    assert (inv.cpu().numpy() == SENT).all() and (net.cpu().numpy() == 5).all()


def test_transparency_statistic_missing_rays_and_single_ray(cuda):
    import torch
    D = 18
    sig = np.full((D, D, D), 5.0, np.float32)
    flags = -np.ones((D, D, D), np.int16)
    flags[1:-1, 1:-1, 1:-1] = 1
    center = np.zeros(3, np.float32)
    # rays far away pointing away from the tile: nothing changes
    ro = np.tile(np.array([[10.0, 10.0, 10.0]], np.float32), (64, 1))
    rd = np.tile(np.array([[1.0, 0.0, 0.0]], np.float32), (64, 1))
    T = _t(np.zeros((D, D, D), np.float32))
    ops.transparency_statistic(_t(ro), _t(rd), D, _t(center), 1.0, 1.0 / 16, 1.0 / 160, _t(sig), _t(flags), T)
    torch.cuda.synchronize()
    assert (T.cpu().numpy() == 0).all()
    # one ray through the tile
    ro1, rd1 = np.array([[-2.0, 0.01, 0.02]], np.float32), np.array([[1.0, 0.0, 0.0]], np.float32)
    ref = np.zeros((D, D, D), np.float32)
    oracle.op_transparency_statistic(ro1, rd1, D, center, 1.0, 1.0 / 16, 1.0 / 160, sig, flags, ref)
    T1 = _t(np.zeros((D, D, D), np.float32))
    ops.transparency_statistic(_t(ro1), _t(rd1), D, _t(center), 1.0, 1.0 / 16, 1.0 / 160, _t(sig), _t(flags), T1)
    torch.cuda.synchronize()
    assert (ref > 0).sum() > 16 and np.abs(T1.cpu().numpy() - ref).max() <= 1e-6


def test_dilate_and_pack_degenerate_grids(cuda):
    import torch
    for fill in (-1, 1, 0):
        f = np.full((7, 7, 7), fill, np.int16)
        g = _t(f)
        ops.dilate_boundary(g, 7)
        torch.cuda.synchronize()
        assert np.array_equal(g.cpu().numpy(), f)
    rng = np.random.default_rng(2)
    f = rng.choice(np.array([-1, 0, 1], np.int16), size=(7, 7, 7))  # N = 5: 125 voxels, two words
    words, count = ops.pack_occupancy(_t(f))
    ref_w, ref_n = oracle.op_pack_occupancy(f, 5)
    assert np.array_equal(words.cpu().numpy().view(np.uint64), ref_w) and int(count) == ref_n


def test_trainprep_tile_not_visited_and_tiny_view(cuda):
    import torch
    s = snisr.SynthScene(snisr.CFG2)
    a = s.arrays()
    d = s.desc
    sc = snisr.Scene(d)
    try:
        imap = np.asarray(a["tile_index"], np.int32).reshape(-1)
        grid = (int(d.grid[0]), int(d.grid[1]), int(d.grid[2]))
        smin = np.array(list(d.scene_min), np.float32)
        for H, W in ((36, 64), (5, 5)):
            cam = s.camera(0, W, H)
            f = 1.0 / cam.inv_focal
            K = np.array([f, 0, cam.cx, 0, f, cam.cy, 0, 0, 1], np.float32)
            C2W = np.array(list(cam.c2w), np.float32)
            tp = trainprep.TrainPrep(sc, H, W, imap, grid, smin, float(d.tile_size), 30, 7)
            img = _t(np.zeros((1, H * W, 3), np.float32))
            dep = _t(np.full((1, H * W), 1e4, np.float32))
            proj = _t(trainprep.project_matrix(K, C2W)[None])
            org = _t(C2W[[3, 7, 11]][None])
            rows, count = tp.view(int(d.num_tiles) + 3, _t(K), _t(C2W), img[0], org, img, dep, proj)
            torch.cuda.synchronize()
            assert int(count) == 0
            assert (tp.valid.cpu().numpy() == 0).all() and (tp.bg.cpu().numpy() == -1).all()
        sc.check()
    finally:
        sc.close()


def test_sample_bg_all_background_missing(cuda):
    import torch
    n, ns = 100, 8
    ro = np.random.default_rng(1).standard_normal((n, 3)).astype(np.float32)
    rd = np.random.default_rng(2).standard_normal((n, 3)).astype(np.float32)
    bg = np.full((n, 1), -1.0, np.float32)
    z = ops.sampling_background(_t(ro), _t(rd), _t(bg), _t(np.zeros(3, np.float32)), 3.0, ns, 0.5)
    torch.cuda.synchronize()
    assert (z.cpu().numpy() == -1).all()


def test_bounded_wait_reports_timeout_and_context_stays_usable(cuda):
    """A kernel wait on an mbarrier that nothing completes gives up after its
    time limit and reports it (no fault, no hang); the context is usable
    afterwards: a render right after it matches the oracle."""
    import ctypes as C
    import torch
    from snisr import _lib
    waited = C.c_int64()
    assert snisr.lib().snisr_diag_wait_timeout(20_000_000, C.byref(waited), None) == _lib.DEVICE_TIMEOUT
    assert 20_000_000 <= waited.value < 1_000_000_000, waited.value
    s = snisr.SynthScene(snisr.CFG1)
    sc = snisr.Scene(s.desc)
    cam = s.camera(0, 64, 48)
    rgb, depth, opac = sc.render(cam, snisr.FORM_PLAIN_FP32)
    torch.cuda.synchronize()
    sc.check()
    d = oracle.camera_dirs(cam)
    o = oracle.camera_origins(cam, d.shape[0])
    osc = oracle.OracleScene(s.desc)
    _, _, oop, _ = osc.render(o, d, None, 0)
    assert np.abs(opac.cpu().numpy() - oop).max() <= 1e-5
    sc.close()


@pytest.mark.parametrize("case", ["all_miss", "one_ray", "mixed"])
def test_render_tc_frames_without_or_with_few_samples(cuda, case):
    """The tensor-core render on frames that give the MLP no chunk at all
    (every ray misses the scene), one ray, and a ragged mix of misses and
    hits: colour, depth and opacity against the oracle, and an error word
    that stays clear."""
    import torch
    s = snisr.SynthScene(snisr.CFG1)
    sc = snisr.Scene(s.desc)
    osc = oracle.OracleScene(s.desc)
    cam = s.camera(0)
    d_all = oracle.camera_dirs(cam)
    o_all = oracle.camera_origins(cam, d_all.shape[0])
    rng = np.random.default_rng(4)
    away_o = np.tile(np.array([[-10.0, -10.0, -10.0]], np.float32), (300, 1))
    away_d = np.tile(np.array([[-1.0, 0.0, 0.0]], np.float32), (300, 1))
    if case == "all_miss":
        o, d = away_o, away_d
    elif case == "one_ray":
        k = d_all.shape[0] // 2 + cam.width // 2  # the centre pixel
        o, d = o_all[k:k + 1], d_all[k:k + 1]
    else:
        pick = rng.choice(d_all.shape[0], 333, replace=False)
        o = np.concatenate([o_all[pick], away_o[:77]])
        d = np.concatenate([d_all[pick], away_d[:77]])
    o, d = np.ascontiguousarray(o, np.float32), np.ascontiguousarray(d, np.float32)
    rgb, depth, opac = sc.render_rays(_t(o), _t(d), snisr.FORM_TC)
    torch.cuda.synchronize()
    sc.check()
    orgb, odep, oop, _ = osc.render(o, d, None, 1)
    assert np.abs(opac.cpu().numpy() - oop).max() <= 1e-5
    assert float(np.sqrt(((rgb.cpu().numpy() - orgb) ** 2).mean())) <= 1e-3
    assert np.abs(rgb.cpu().numpy() - orgb).max() <= 1e-2
    if case == "all_miss":
        assert (opac.cpu().numpy() == 0).all() and (rgb.cpu().numpy() == 0).all()
    sc.close()


def test_march_math_bits_match_the_oracle(cuda):
    """The kernels' e^x, log1p and softplus give the host restatement's bits,
    so transmittance and the early-stop decision agree exactly."""
    import torch
    from test_oracle import _march_math_inputs
    L = snisr.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for fn, v in zip((oracle.MATH_EXP, oracle.MATH_LOG1P, oracle.MATH_SOFTPLUS), _march_math_inputs()):
        xd = torch.from_numpy(v).cuda()
        out = torch.empty_like(xd)
        snisr._lib.check(L.snisr_diag_march_math(fn, xd.data_ptr(), v.size, out.data_ptr(), stream))
        got = out.cpu().numpy()
        ref = oracle.march_math(fn, v)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), fn
