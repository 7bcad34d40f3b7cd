"""Launch-shape knobs and their autotuner: results do not depend on the
launch shapes (depth and opacity bit-exact, colours and gradients to the
summation order of atomics), out-of-range knobs are rejected, and the
autotuners return a valid configuration and keep it in the scene."""
import numpy as np
import pytest

import oracle
import snisr
from snisr.train import tile_field

pytestmark = pytest.mark.gpu

SHAPES = [dict(traverse_threads=64, scatter_blocks_per_sm=8, mlp_ctas_per_sm=1),
          dict(traverse_threads=256, scatter_blocks_per_sm=32, mlp_ctas_per_sm=3),
          dict(traverse_threads=96, scatter_blocks_per_sm=1, mlp_ctas_per_sm=2)]


@pytest.fixture(scope="module")
def cfg1(cuda):
    s = snisr.SynthScene(snisr.CFG1)
    sc = snisr.Scene(s.desc)
    yield s, sc
    sc.close()


def test_render_independent_of_launch_shapes(cfg1):
    import torch
    s, sc = cfg1
    cam = s.camera(2)
    default = sc.tuning()
    ref = [t.clone() for t in sc.render(cam, snisr.FORM_TC)]
    for shape in SHAPES:
        sc.set_tuning(**shape)
        got = sc.render(cam, snisr.FORM_TC)
        sc.check()
        assert torch.equal(got[1], ref[1]) and torch.equal(got[2], ref[2])
        assert float((got[0] - ref[0]).abs().max()) <= 1e-6
    sc.set_tuning(**default)


def test_training_independent_of_launch_shapes(cfg1):
    import torch
    s, sc = cfg1
    a = s.arrays()
    cam = s.camera(1)
    d = oracle.camera_dirs(cam)
    d = torch.from_numpy(np.ascontiguousarray(d[::4])).cuda()
    o = torch.from_numpy(oracle.camera_origins(cam, d.shape[0])).cuda()
    rt = torch.zeros(d.shape[0], dtype=torch.int32, device="cuda")
    g = torch.randn(d.shape[0], 3, device="cuda", generator=torch.Generator(device="cuda").manual_seed(2))
    default = sc.tuning()

    def grads():
        leaves = [torch.from_numpy(x).cuda().requires_grad_(True)
                  for x in (a["vertex_feat"].astype(np.float32), a["vertex_density"].astype(np.float32),
                            a["mlp_params"].copy())]
        (tile_field(*leaves, sc, o, d, rt, snisr.FORM_TC) * g).sum().backward()
        return [x.grad for x in leaves]

    ref = grads()
    for march, fwd in ((64, 4), (256, 8), (160, 4)):
        sc.set_tuning(train_march_threads=march, train_fwd_warps=fwd)
        for x, r in zip(grads(), ref):
            assert float((x - r).norm() / r.norm()) <= 1e-5
    sc.set_tuning(**default)


def test_bad_tuning_rejected(cfg1):
    _, sc = cfg1
    for bad in (dict(traverse_threads=48), dict(traverse_threads=512), dict(scatter_blocks_per_sm=0),
                dict(mlp_ctas_per_sm=9), dict(train_fwd_warps=6)):
        with pytest.raises(snisr.SnisrError):
            sc.set_tuning(**bad)


def test_autotune_render_and_train(cfg1):
    import torch
    s, sc = cfg1
    cam = s.camera(3)
    cfg, ms = sc.autotune_render(cam, reps=2)
    assert ms > 0 and cfg == sc.tuning()
    assert cfg["traverse_threads"] in (64, 128, 256) and cfg["mlp_ctas_per_sm"] in (0, 2, 3)
    a = s.arrays()
    d = torch.from_numpy(np.ascontiguousarray(oracle.camera_dirs(cam)[::8])).cuda()
    o = torch.from_numpy(oracle.camera_origins(cam, d.shape[0])).cuda()
    rt = torch.zeros(d.shape[0], dtype=torch.int32, device="cuda")
    vf, vd, W = (torch.from_numpy(x).cuda() for x in (a["vertex_feat"].astype(np.float32),
                                                       a["vertex_density"].astype(np.float32),
                                                       a["mlp_params"].copy()))
    cfg2, ms2 = sc.autotune_train(vf, vd, W, o, d, rt, reps=2)
    assert ms2 > 0 and cfg2 == sc.tuning()
    assert cfg2["train_march_threads"] in (64, 128, 256) and cfg2["train_fwd_warps"] in (4, 8)
