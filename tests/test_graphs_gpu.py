"""CUDA-graph capture of the hot path: after one warm-up call (workspace and
per-device kernel attributes in place) a render frame and a whole training
step (forward, loss, hand-written backward) capture into a CUDA graph and
replay with the same results as eager calls.  Colour and gradient sums use
atomics, so replays agree with eager runs to summation order (1e-6 relative);
depth and opacity are bit-exact."""
import numpy as np
import pytest

import oracle
import snisr
from snisr.train import tile_field

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg1(cuda):
    s = snisr.SynthScene(snisr.CFG1)
    sc = snisr.Scene(s.desc)
    yield s, sc
    sc.close()


@pytest.mark.parametrize("form", [snisr.FORM_TC, snisr.FORM_PLAIN_FP32])
def test_render_graph_replay(cfg1, form):
    import torch
    s, sc = cfg1
    cam = s.camera(4)
    n = cam.width * cam.height
    out = tuple(torch.empty(n, 3 if i == 0 else 1, device="cuda").squeeze(-1) for i in range(3))
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        sc.render(cam, form, out)  # warm-up outside capture
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    ref = [t.clone() for t in out]
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        sc.render(cam, form, out)
    for t in out:
        t.fill_(-7.0)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    sc.check()
    assert torch.equal(out[1], ref[1]) and torch.equal(out[2], ref[2])
    assert float((out[0] - ref[0]).abs().max()) <= 1e-6
    assert float(ref[0].abs().sum()) > 0


def test_training_step_graph_replay(cfg1):
    import torch
    s, sc = cfg1
    a = s.arrays()
    dev = torch.device("cuda")
    vf = torch.from_numpy(a["vertex_feat"].astype(np.float32)).to(dev).requires_grad_(True)
    vd = torch.from_numpy(a["vertex_density"].astype(np.float32)).to(dev).requires_grad_(True)
    W = torch.from_numpy(a["mlp_params"].copy()).to(dev).requires_grad_(True)
    cam = s.camera(1)
    d = oracle.camera_dirs(cam)
    idx = np.sort(np.random.default_rng(4).choice(d.shape[0], 8192, replace=False))
    d = torch.from_numpy(np.ascontiguousarray(d[idx])).to(dev)
    o = torch.from_numpy(oracle.camera_origins(cam, d.shape[0])).to(dev)
    rt = torch.zeros(d.shape[0], dtype=torch.int32, device=dev)
    target = torch.rand(d.shape[0], 3, device=dev, generator=torch.Generator(device=dev).manual_seed(1))

    def step():
        rgb = tile_field(vf, vd, W, sc, o, d, rt, snisr.FORM_TC)
        loss = ((rgb - target) ** 2).mean()
        loss.backward()
        return loss

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            vf.grad = vd.grad = W.grad = None
            step()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    ref = [t.grad.clone() for t in (vf, vd, W)]
    vf.grad = vd.grad = W.grad = None
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        loss = step()
    g.replay()
    torch.cuda.synchronize()
    sc.check()
    for t, r in zip((vf, vd, W), ref):
        assert float(r.abs().sum()) > 0
        err = float((t.grad - r).norm() / r.norm())
        assert err <= 1e-6, err
    assert np.isfinite(float(loss.detach()))
