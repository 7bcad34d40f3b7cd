"""The hand-written training adjoint against PyTorch autograd of the
reference-style graph (grid_sample lookup, Positional_Encoding, Linear/ReLU
MLP, cumprod compositing with +1e-10; see reference_graph.py), float64 on
the CPU.

CPU test: the FP64 oracle adjoint and forward agree with the graph to 1e-6
relative (the graph's +1e-10 in the cumprod is the only difference).
GPU test (marked gpu): libsnisr's gradients through tile_field agree with the
graph -- plain FP32 form <= 1e-3, tensor-core form <= 1e-2 relative per
parameter group (||g - g_ref|| / ||g_ref||).
"""
import numpy as np
import pytest
import torch

import oracle
import snisr

import reference_graph as rg


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def problem():
    s = snisr.SynthScene(snisr.CFG1)
    a = s.arrays()
    rng = np.random.default_rng(21)
    vf = a["vertex_feat"].astype(np.float32).copy()
    vd = a["vertex_density"].astype(np.float32).copy()
    W = a["mlp_params"].copy()
    W += rng.normal(0, 0.05, W.shape).astype(np.float32)
    cam = s.camera(1)
    d = oracle.camera_dirs(cam)
    idx = np.sort(rng.choice(d.shape[0], 8192, replace=False))
    d = np.ascontiguousarray(d[idx])
    o = oracle.camera_origins(cam, d.shape[0])
    rt = np.zeros(d.shape[0], np.int32)
    osc = oracle.OracleScene(s.desc)
    samples = osc.train_samples(vf, vd, W, o, d, rt)
    g = np.random.default_rng(5).standard_normal((d.shape[0], 3))
    grid = rg.corner_index_grid(s.desc, a, 0)
    # reference-style graph, float64 autograd
    tv = [torch.tensor(x.astype(np.float64).reshape(-1) if x is W else x.astype(np.float64), requires_grad=True)
          for x in (vf, vd, W)]
    rgb = rg.render(tv[0], tv[1], tv[2], s.desc, grid, samples, d)
    (rgb * torch.from_numpy(g)).sum().backward()
    ref = dict(rgb=rgb.detach().numpy(), gF=tv[0].grad.numpy(), gG=tv[1].grad.numpy(),
               gW=tv[2].grad.numpy().reshape(W.shape))
    return dict(s=s, osc=osc, vf=vf, vd=vd, W=W, o=o, d=d, rt=rt, g=g, samples=samples, ref=ref)


def test_graph_has_work(problem):
    off = problem["samples"][0]
    assert off[-1] > 2000 and (np.diff(off) > 0).sum() > 300


def test_oracle_matches_reference_graph(problem):
    P = problem
    rgb, _ = P["osc"].train_forward(P["vf"], P["vd"], P["W"], P["o"], P["d"], P["rt"])
    assert np.abs(rgb - P["ref"]["rgb"]).max() <= 1e-8
    gF, gG, gW = P["osc"].train_backward(P["vf"], P["vd"], P["W"], P["o"], P["d"], P["rt"], P["g"])
    assert _rel(gF, P["ref"]["gF"]) <= 1e-6
    assert _rel(gG, P["ref"]["gG"]) <= 1e-6
    assert _rel(gW, P["ref"]["gW"]) <= 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("form,tol", [(snisr.FORM_PLAIN_FP32, 1e-3), (snisr.FORM_TC, 1e-2)])
def test_gpu_gradients_match_reference_graph(problem, cuda, form, tol):
    from snisr.train import tile_field
    P = problem
    sc = snisr.Scene(P["s"].desc)
    try:
        T = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
        vf, vd, W = (T(P[k]).requires_grad_(True) for k in ("vf", "vd", "W"))
        rgb = tile_field(vf, vd, W, sc, T(P["o"]), T(P["d"]), T(P["rt"]), form)
        (rgb * torch.from_numpy(P["g"]).float().cuda()).sum().backward()
        sc.check()
        assert _rel(vf.grad.cpu().numpy(), P["ref"]["gF"]) <= tol
        assert _rel(vd.grad.cpu().numpy(), P["ref"]["gG"]) <= tol
        assert _rel(W.grad.cpu().numpy(), P["ref"]["gW"]) <= tol
    finally:
        sc.close()
