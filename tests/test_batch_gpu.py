"""Batched multi-tile training (one forward/backward over the segments of
many tiles, each tile with its own MLP) against per-tile calls and the
oracle, on a reduced copy of the 32-tile configuration (64^3 per tile).

* segments come back grouped by tile with the requested per-tile counts;
* plain FP32 form: batched colours match the oracle (max-abs <= 1e-5);
* both forms: one batched call equals the 32 per-tile calls (colours
  max-abs <= 1e-6, gradients relative <= 1e-5: atomics order only).
"""
import numpy as np
import pytest

import oracle
import snisr
from snisr import batch
from snisr.train import tile_field

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def problem(cuda):
    import torch
    cfg = snisr.CFG4.replace(res=64)
    s = snisr.SynthScene(cfg)
    sc = snisr.Scene(s.desc)
    o, d, t, counts = batch.tile_batch(s, views=2, lo=64, hi=1024, seed=3)
    a = s.arrays()
    rng = np.random.default_rng(1)
    W = a["mlp_params"].copy()
    W += rng.normal(0, 0.05, W.shape).astype(np.float32)
    g = torch.from_numpy(rng.standard_normal((o.shape[0], 3)).astype(np.float32)).cuda()
    yield dict(s=s, sc=sc, o=o, d=d, t=t, counts=counts, vf=a["vertex_feat"].astype(np.float32),
               vd=a["vertex_density"].astype(np.float32), W=W, g=g)
    sc.close()


def test_segments_grouped_by_tile(problem):
    t = problem["t"].cpu().numpy()
    counts = problem["counts"]
    assert (np.diff(t) >= 0).all()
    assert np.array_equal(np.bincount(t, minlength=counts.size), counts)
    assert (counts > 0).sum() >= 10 and counts.max() <= 1024
    assert problem["s"].desc.num_tiles == 32


def test_batched_plain_matches_oracle(problem):
    P = problem
    import torch
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    rgb = tile_field(T(P["vf"]), T(P["vd"]), T(P["W"]), P["sc"], P["o"], P["d"], P["t"], snisr.FORM_PLAIN_FP32)
    P["sc"].check()
    osc = oracle.OracleScene(P["s"].desc)
    ref, cnt = osc.train_forward(P["vf"], P["vd"], P["W"], P["o"].cpu().numpy(), P["d"].cpu().numpy(),
                                 P["t"].cpu().numpy())
    assert cnt.sum() > 10000
    assert np.abs(rgb.cpu().numpy() - ref).max() <= 1e-5


@pytest.mark.parametrize("form", [snisr.FORM_PLAIN_FP32, snisr.FORM_TC])
def test_batched_equals_per_tile_calls(problem, form):
    import torch
    P = problem
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()

    def leaves():
        return [T(x).requires_grad_(True) for x in (P["vf"], P["vd"], P["W"])]

    vf, vd, W = leaves()
    rgb = tile_field(vf, vd, W, P["sc"], P["o"], P["d"], P["t"], form)
    (rgb * P["g"]).sum().backward()
    batched = [rgb.detach().clone()] + [x.grad.clone() for x in (vf, vd, W)]

    vf2, vd2, W2 = leaves()
    parts = []
    start = 0
    for c in P["counts"]:
        if c == 0:
            continue
        sl = slice(start, start + int(c))
        r = tile_field(vf2, vd2, W2, P["sc"], P["o"][sl].contiguous(), P["d"][sl].contiguous(),
                       P["t"][sl].contiguous(), form)
        (r * P["g"][sl]).sum().backward()
        parts.append(r.detach())
        start += int(c)
    P["sc"].check()
    assert float((torch.cat(parts) - batched[0]).abs().max()) <= 1e-6
    for x, ref in zip((vf2, vd2, W2), batched[1:]):
        assert _rel(x.grad.cpu().numpy(), ref.cpu().numpy()) <= 1e-5
