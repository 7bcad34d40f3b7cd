"""GPU parity of the render path against the oracle (through the C ABI).

Tolerances (stated by the benchmark contract):
  plain FP32 form vs oracle FP32: colour/opacity max-abs <= 1e-5, depth rel <= 1e-5
  tensor-core form vs oracle FP64: colour RMSE <= 1e-3
  visited occupied-voxel sequences and proxy-hit triangle ids: bit-exact
"""
import numpy as np
import pytest

import oracle
import snisr

pytestmark = pytest.mark.gpu

PLAIN_MAX_ABS = 1e-5
TC_RMSE = 1e-3


@pytest.fixture(scope="module")
def cfg1(cuda):
    s = snisr.SynthScene(snisr.CFG1)
    sc = snisr.Scene(s.desc)
    yield s, sc, oracle.OracleScene(s.desc)
    sc.close()


@pytest.fixture(scope="module")
def cfg2(cuda):
    s = snisr.SynthScene(snisr.CFG2)
    sc = snisr.Scene(s.desc)
    yield s, sc, oracle.OracleScene(s.desc)
    sc.close()


def _torch(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("mode", [0, 3])  # A from shared memory / from tensor memory
def test_diag_mma_fp16_bf16(cuda, mode):
    import torch
    g = torch.Generator().manual_seed(0)
    for bf16 in (0, 1):
        for N in (32, 64):
            A = torch.randn(128, 64, generator=g)
            B = torch.randn(N, 64, generator=g)
            dt = torch.bfloat16 if bf16 else torch.float16
            Ah, Bh = A.to(dt), B.to(dt)
            # keep the device copies referenced for the duration of the call
            Ad, Bd = Ah.cuda().view(torch.int16), Bh.cuda().view(torch.int16)
            D = torch.empty(128, N, device=cuda)
            snisr._lib.check(snisr.lib().snisr_diag_mma(Ad.data_ptr(), Bd.data_ptr(), D.data_ptr(), N, bf16, mode,
                                                        torch.cuda.current_stream().cuda_stream))
            ref = Ah.double() @ Bh.double().T
            err = (D.cpu().double() - ref).abs().max().item()
            assert err < 1e-4, (bf16, N, err)


def test_camera_rays_bitexact(cfg1):
    s, sc, _ = cfg1
    cam = s.camera(0)
    d = _np(snisr.camera_rays(cam))
    assert np.array_equal(d, oracle.camera_dirs(cam))


def test_trace_voxels_bitexact_cfg1(cfg1):
    s, sc, osc = cfg1
    cam = s.camera(0)
    d = oracle.camera_dirs(cam)
    o = oracle.camera_origins(cam, d.shape[0])
    K = 192
    vis, cnt = sc.trace_voxels(_torch(o), _torch(d), K)
    ovis, ocnt = osc.trace(o, d, None, K)
    assert np.array_equal(_np(cnt), ocnt)
    assert np.array_equal(_np(vis), ovis)
    assert ocnt.sum() > 0


@pytest.mark.parametrize("pose", [0, 3])
def test_render_plain_cfg1(cfg1, pose):
    s, sc, osc = cfg1
    cam = s.camera(pose)
    rgb, depth, opac = sc.render(cam, snisr.FORM_PLAIN_FP32)
    sc.check()
    d = oracle.camera_dirs(cam)
    o = oracle.camera_origins(cam, d.shape[0])
    orgb, odep, oop, stats = osc.render(o, d, None, 0)
    assert stats[0] > 0
    assert np.abs(_np(rgb) - orgb).max() <= PLAIN_MAX_ABS
    assert np.abs(_np(opac) - oop).max() <= PLAIN_MAX_ABS
    assert np.abs(_np(depth) - odep).max() <= PLAIN_MAX_ABS * max(1.0, float(np.abs(odep).max()))


@pytest.mark.parametrize("pose", [0, 5])
def test_render_tc_cfg1(cfg1, pose):
    s, sc, osc = cfg1
    cam = s.camera(pose)
    rgb, depth, opac = sc.render(cam, snisr.FORM_TC)
    sc.check()
    d = oracle.camera_dirs(cam)
    o = oracle.camera_origins(cam, d.shape[0])
    orgb, odep, oop, _ = osc.render(o, d, None, 1)
    rmse = float(np.sqrt(((_np(rgb) - orgb) ** 2).mean()))
    assert rmse <= TC_RMSE, rmse
    # depth/opacity are computed without the MLP: FP32-exact semantics
    assert np.abs(_np(opac) - oop).max() <= PLAIN_MAX_ABS
    # tighter: against the oracle's emulation of FP16 MLP inputs
    trgb, _, _, _ = osc.render(o, d, None, 2)
    assert float(np.sqrt(((_np(rgb) - trgb) ** 2).mean())) <= 2e-4


def test_frame_footprint_cfg1(cfg1):
    """Distinct voxels / vertices read by a tensor-core frame (the compulsory-
    bytes roofline counter) match the oracle's sampled voxels exactly."""
    s, sc, osc = cfg1
    cam = s.camera(2)
    sc.render(cam, snisr.FORM_TC)
    fp = sc.frame_footprint()
    d = oracle.camera_dirs(cam)
    o = oracle.camera_origins(cam, d.shape[0])
    touched = osc.touched_voxels(o, d)
    corners = s.arrays()["voxel_corners"]
    assert fp["voxels"] == int(touched.sum()) > 0
    assert fp["vertices"] == len(np.unique(corners[touched]))


def _subset(cam, n, seed):
    d = oracle.camera_dirs(cam)
    idx = np.random.default_rng(seed).choice(d.shape[0], n, replace=False)
    d = np.ascontiguousarray(d[np.sort(idx)])
    return oracle.camera_origins(cam, n), d


def test_proxy_hit_bitexact_cfg2(cfg2):
    s, sc, osc = cfg2
    o, d = _subset(s.camera(1), 1024, 7)
    t, tri = sc.proxy_hit(_torch(o), _torch(d))
    _, oth, otri = osc.proxy(o, d)
    assert np.array_equal(_np(tri), otri)
    assert np.array_equal(_np(t), oth)
    assert (otri >= 0).mean() > 0.95


def test_render_cfg2_subset(cfg2):
    s, sc, osc = cfg2
    o, d = _subset(s.camera(2), 2048, 11)
    ts, _, _ = osc.proxy(o, d)
    vis, cnt = sc.trace_voxels(_torch(o), _torch(d), 256)
    ovis, ocnt = osc.trace(o, d, ts, 256)
    assert np.array_equal(_np(cnt), ocnt) and np.array_equal(_np(vis), ovis)
    rgb, depth, opac = sc.render_rays(_torch(o), _torch(d), snisr.FORM_PLAIN_FP32)
    orgb, odep, oop, _ = osc.render(o, d, ts, 0)
    assert np.abs(_np(rgb) - orgb).max() <= PLAIN_MAX_ABS
    assert np.abs(_np(opac) - oop).max() <= PLAIN_MAX_ABS
    trgb, tdep, top = sc.render_rays(_torch(o), _torch(d), snisr.FORM_TC)
    sc.check()
    o64, _, _, _ = osc.render(o, d, ts, 1)
    assert float(np.sqrt(((_np(trgb) - o64) ** 2).mean())) <= TC_RMSE


def test_render_cfg2_full_frame_forms_agree(cfg2):
    """Full 1280x720 frame: both GPU forms against each other (size-independent
    property; the oracle covers the subsets above)."""
    s, sc, _ = cfg2
    cam = s.camera(0)
    p = sc.render(cam, snisr.FORM_PLAIN_FP32)
    t = sc.render(cam, snisr.FORM_TC)
    sc.check()
    prgb, trgb = _np(p[0]), _np(t[0])
    assert float(np.sqrt(((prgb - trgb) ** 2).mean())) <= TC_RMSE
    assert np.abs(_np(p[2]) - _np(t[2])).max() <= PLAIN_MAX_ABS
    assert (_np(t[2]) > 0.5).mean() > 0.5  # most rays hit a surface


def test_render_host_async_matches_device_render(cuda):
    """The pipelined host-output render writes the same frames as snisr_render."""
    import torch
    s = snisr.SynthScene(snisr.CFG1)
    sc = snisr.Scene(s.desc)
    try:
        cams = [s.camera(p) for p in range(4)]
        n = cams[0].width * cams[0].height
        hb = [tuple(torch.empty(*shape, pin_memory=True) for shape in ((n, 3), (n,), (n,))) for _ in range(4)]
        for cam, bufs in zip(cams, hb):
            sc.render_host_async(cam, snisr.FORM_TC, *bufs)
        sc.render_host_wait()
        for cam, bufs in zip(cams, hb):
            ref = [t.cpu() for t in sc.render(cam, snisr.FORM_TC)]
            assert float((bufs[0] - ref[0]).abs().max()) <= 1e-6  # colour: atomics in any order
            assert torch.equal(bufs[1], ref[1]) and torch.equal(bufs[2], ref[2])
        sc.check()
    finally:
        sc.close()


def test_sample_buffer_overflow_is_reported_and_contained(cuda):
    """A frame with more samples than the buffer holds (one slot per ray here)
    is flagged by snisr_scene_check; the stages after the traversal skip the
    frame instead of indexing past the buffers, and the scene stays usable."""
    import torch
    s = snisr.SynthScene(snisr.CFG2, max_pixels=320 * 180, max_samples_per_ray=1)
    sc = snisr.Scene(s.desc)
    try:
        cam = s.camera(0, 320, 180)
        sc.render(cam, snisr.FORM_TC)
        with pytest.raises(snisr.SnisrError):
            sc.check()
        torch.cuda.synchronize()
        sc.render(cam, snisr.FORM_PLAIN_FP32)  # the plain form needs no sample buffer
        sc.check()
    finally:
        sc.close()
