"""Render parity on every benchmark pose, with colour, depth and opacity
errors stated for both forms.

Full-frame scene (4x4x1 tiles of 128^3, ~5 % occupied, ~205k-triangle proxy
mesh, 1280x720): each of the 8 seeded poses on 65,536 random pixels, and the
whole 1280x720 frame of pose 0.  Large scene (8x8x2 tiles, ~1.0M-triangle
mesh, 1920x1080): each of the 16 poses on the 256x256 centre crop.

Rays start 2 voxels before the proxy hit.  The GPU's hits are checked
bit-exact against the oracle's brute-force nearest hit on 512 rays per pose
and then used as the oracle's start distances for all rays.

Tolerances:
* plain FP32 form against the oracle's FP32 evaluation: colour and opacity
  max-abs <= 1e-5, depth max-abs <= 1e-5 * max(1, max depth);
* tensor-core form (FP16 features and weights, FP32 accumulation) against the
  FP64 oracle: colour RMSE <= 1e-3.  Its depth and opacity come from the FP32
  traversal (weights T * alpha, no MLP): against the oracle's FP32
  evaluation with the plain form's tolerances, and against FP64 depth
  max-abs <= 1e-3 m, opacity max-abs <= 1e-4.
"""
import numpy as np
import pytest

import oracle
import snisr

pytestmark = pytest.mark.gpu

PLAIN_MAX_ABS = 1e-5
TC_RMSE = 1e-3


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _np(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def frame_scene(cuda):
    s = snisr.SynthScene(snisr.CFG2)
    sc = snisr.Scene(s.desc)
    yield s, sc, oracle.OracleScene(s.desc)
    sc.close()


@pytest.fixture(scope="module")
def large_scene(cuda):
    s = snisr.SynthScene(snisr.CFG5)
    sc = snisr.Scene(s.desc)
    yield s, sc, oracle.OracleScene(s.desc)
    sc.close()


def _starts(sc, osc, o, d, check):
    """GPU proxy hits (checked bit-exact on the first `check` rays) -> start distances."""
    th, tri = sc.proxy_hit(_t(o), _t(d))
    th, tri = _np(th), _np(tri)
    _, oth, otri = osc.proxy(o[:check], d[:check])
    assert np.array_equal(tri[:check], otri) and np.array_equal(th[:check], oth)
    return osc.start_from_hit(th)


def _compare(label, sc, osc, o, d, ts, tc_frame=None, pix=None):
    """Both forms on rays (o, d) against the oracle; tc_frame = (rgb, depth,
    opacity) of a full-frame TC render to compare at pixels `pix` instead of
    rendering the rays again."""
    o32 = osc.render(o, d, ts, 0)
    o64 = osc.render(o, d, ts, 1)
    assert o32[3][0] > 0
    prgb, pdep, pop = (_np(x) for x in sc.render_rays(_t(o), _t(d), snisr.FORM_PLAIN_FP32))
    if tc_frame is None:
        trgb, tdep, top = (_np(x) for x in sc.render_rays(_t(o), _t(d), snisr.FORM_TC))
    else:
        trgb, tdep, top = (_np(x)[pix] for x in tc_frame)
    sc.check()
    dscale = max(1.0, float(np.abs(o32[1]).max()))
    e = dict(
        plain_rgb=float(np.abs(prgb - o32[0]).max()), plain_dep=float(np.abs(pdep - o32[1]).max()),
        plain_op=float(np.abs(pop - o32[2]).max()),
        tc_rmse=float(np.sqrt(((trgb - o64[0]) ** 2).mean())), tc_rgb_max=float(np.abs(trgb - o64[0]).max()),
        tc_dep32=float(np.abs(tdep - o32[1]).max()), tc_op32=float(np.abs(top - o32[2]).max()),
        tc_dep64=float(np.abs(tdep - o64[1]).max()), tc_op64=float(np.abs(top - o64[2]).max()),
        hit=float((o64[2] > 0.5).mean()))
    print(f"{label}: plain vs FP32 oracle max-abs rgb {e['plain_rgb']:.1e} depth {e['plain_dep']:.1e} "
          f"opacity {e['plain_op']:.1e} | TC vs FP64 colour RMSE {e['tc_rmse']:.2e} (max {e['tc_rgb_max']:.1e}), "
          f"depth {e['tc_dep64']:.1e} m, opacity {e['tc_op64']:.1e} | TC depth/opacity vs FP32 "
          f"{e['tc_dep32']:.1e}/{e['tc_op32']:.1e} | opaque {e['hit']:.2f}")
    assert e["plain_rgb"] <= PLAIN_MAX_ABS and e["plain_op"] <= PLAIN_MAX_ABS
    assert e["plain_dep"] <= PLAIN_MAX_ABS * dscale
    assert e["tc_rmse"] <= TC_RMSE
    assert e["tc_op32"] <= PLAIN_MAX_ABS and e["tc_dep32"] <= PLAIN_MAX_ABS * dscale
    assert e["tc_dep64"] <= 1e-3 and e["tc_op64"] <= 1e-4
    return e


@pytest.mark.parametrize("pose", range(8))
def test_frame_scene_pose(frame_scene, pose):
    s, sc, osc = frame_scene
    cam = s.camera(pose)
    d = oracle.camera_dirs(cam)
    idx = np.sort(np.random.default_rng(100 + pose).choice(d.shape[0], 65536, replace=False))
    d = np.ascontiguousarray(d[idx])
    o = oracle.camera_origins(cam, d.shape[0])
    ts = _starts(sc, osc, o, d, 512)
    e = _compare(f"1280x720 scene pose {pose} (65,536 rays)", sc, osc, o, d, ts)
    assert e["hit"] > 0.5


def test_frame_scene_whole_frame(frame_scene):
    """Every pixel of one 1280x720 frame through the public frame entry
    (snisr_render), TC form, against the FP64 oracle."""
    s, sc, osc = frame_scene
    cam = s.camera(0)
    frame = sc.render(cam, snisr.FORM_TC)
    d = oracle.camera_dirs(cam)
    o = oracle.camera_origins(cam, d.shape[0])
    ts = _starts(sc, osc, o, d, 256)
    pix = np.arange(d.shape[0])
    _compare("1280x720 scene pose 0, whole frame", sc, osc, o, d, ts, tc_frame=frame, pix=pix)


@pytest.mark.parametrize("pose", range(16))
def test_large_scene_pose_crop(large_scene, pose):
    s, sc, osc = large_scene
    cam = s.camera(pose)
    W, H = cam.width, cam.height
    frame = sc.render(cam, snisr.FORM_TC)
    y0, x0 = H // 2 - 128, W // 2 - 128
    pix = (np.arange(y0, y0 + 256)[:, None] * W + np.arange(x0, x0 + 256)[None, :]).reshape(-1)
    d = np.ascontiguousarray(oracle.camera_dirs(cam)[pix])
    o = oracle.camera_origins(cam, d.shape[0])
    ts = _starts(sc, osc, o, d, 256)
    _compare(f"1920x1080 large scene pose {pose} (256x256 crop)", sc, osc, o, d, ts, tc_frame=frame, pix=pix)
