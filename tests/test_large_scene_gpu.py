"""The large scene (8x8x2 tiles of 128^3 over 24x24x6 m, multi-room,
~1.0M-triangle proxy mesh, 1920x1080 at 75 degrees): proxy hits bit-exact
on a ray subset, and a 256x256 centre crop of the full-frame tensor-core
render against the FP64 oracle (colour RMSE <= 1e-3) with the plain FP32 form
on the same rays against the oracle's FP32 evaluation (max-abs <= 1e-5)."""
import numpy as np
import pytest

import oracle
import snisr

pytestmark = pytest.mark.gpu


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def cfg5(cuda):
    s = snisr.SynthScene(snisr.CFG5)
    sc = snisr.Scene(s.desc)
    yield s, sc, oracle.OracleScene(s.desc)
    sc.close()


def test_cfg5_sizes(cfg5):
    s, sc, _ = cfg5
    assert s.desc.num_tiles == 128 and 0.9e6 < s.desc.num_triangles < 1.2e6
    assert 0.02 < s.occupancy_fraction() < 0.06


def test_cfg5_proxy_hit_bitexact(cfg5):
    s, sc, osc = cfg5
    cam = s.camera(3)
    d = oracle.camera_dirs(cam)
    d = np.ascontiguousarray(d[np.sort(np.random.default_rng(5).choice(d.shape[0], 512, replace=False))])
    o = oracle.camera_origins(cam, d.shape[0])
    t, tri = sc.proxy_hit(_t(o), _t(d))
    _, oth, otri = osc.proxy(o, d)
    assert np.array_equal(tri.cpu().numpy(), otri)
    assert np.array_equal(t.cpu().numpy(), oth)


def test_cfg5_full_frame_crop_vs_fp64(cfg5):
    s, sc, osc = cfg5
    cam = s.camera(0)
    W, H = cam.width, cam.height
    assert (W, H) == (1920, 1080)
    rgb, depth, opac = sc.render(cam, snisr.FORM_TC)
    sc.check()
    y0, x0 = H // 2 - 128, W // 2 - 128
    pix = (np.arange(y0, y0 + 256)[:, None] * W + np.arange(x0, x0 + 256)[None, :]).reshape(-1)
    d = np.ascontiguousarray(oracle.camera_dirs(cam)[pix])
    o = oracle.camera_origins(cam, d.shape[0])
    th, _ = sc.proxy_hit(_t(o), _t(d))
    ts = osc.start_from_hit(th.cpu().numpy())
    o64, _, _, _ = osc.render(o, d, ts, 1)
    crop = rgb.cpu().numpy()[pix]
    assert float(np.sqrt(((crop - o64) ** 2).mean())) <= 1e-3
    assert (opac.cpu().numpy()[pix] > 0.5).mean() > 0.5
    prgb, _, popac = sc.render_rays(_t(o), _t(d), snisr.FORM_PLAIN_FP32)
    o32, _, oop, _ = osc.render(o, d, ts, 0)
    assert np.abs(prgb.cpu().numpy() - o32).max() <= 1e-5
    assert np.abs(popac.cpu().numpy() - oop).max() <= 1e-5
    assert np.abs(opac.cpu().numpy()[pix] - oop).max() <= 1e-5
