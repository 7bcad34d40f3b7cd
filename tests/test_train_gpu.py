"""Training forward and hand-written adjoint on the GPU against the FP64
oracle (forward colours, analytic gradients) and FP64 central finite
differences (h = 1e-4, 64 random parameters).

Tolerances (relative error = ||g - g_ref|| / ||g_ref|| per parameter group):
plain FP32 form colours max-abs <= 1e-5 and gradient relative error <= 1e-3;
tensor-core form (three-part split BF16 forward operands, BF16 backward
operands) colour max-abs <= 1e-5 and gradient relative error <= 1e-2
against the exact FP64 oracle, and -- against the oracle emulating the
tensor-core operand rounding -- colour max-abs <= 1e-5 and gradient
relative error <= 2e-3."""
import numpy as np
import pytest

import oracle
import snisr
from snisr.train import tile_field

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def setup(cuda):
    import torch
    cfg = snisr.CFG1
    s = snisr.SynthScene(cfg)
    sc = snisr.Scene(s.desc)
    a = s.arrays()
    rng = np.random.default_rng(9)
    vf = a["vertex_feat"].astype(np.float32).copy()
    vd = a["vertex_density"].astype(np.float32).copy()
    W = a["mlp_params"].copy()
    W += rng.normal(0, 0.05, W.shape).astype(np.float32)  # non-zero biases, off the init
    cam = s.camera(1)
    d = oracle.camera_dirs(cam)
    idx = np.sort(rng.choice(d.shape[0], 4096, replace=False))
    d = np.ascontiguousarray(d[idx])
    o = oracle.camera_origins(cam, d.shape[0])
    rt = np.zeros(d.shape[0], np.int32)
    osc = oracle.OracleScene(s.desc)
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    yield dict(s=s, sc=sc, osc=osc, vf=vf, vd=vd, W=W, o=o, d=d, rt=rt, T=T)
    sc.close()


@pytest.mark.parametrize("form", [snisr.FORM_PLAIN_FP32, snisr.FORM_TC])
def test_train_forward_matches_oracle(setup, form):
    S = setup
    T = S["T"]
    rgb = tile_field(T(S["vf"]), T(S["vd"]), T(S["W"]), S["sc"], T(S["o"]), T(S["d"]), T(S["rt"]), form)
    ref, cnt = S["osc"].train_forward(S["vf"], S["vd"], S["W"], S["o"], S["d"], S["rt"])
    assert cnt.sum() > 1000
    got = rgb.detach().cpu().numpy()
    if form == snisr.FORM_PLAIN_FP32:
        assert np.abs(got - ref).max() <= 1e-5
    else:
        assert np.abs(got - ref).max() <= 1e-5
        emu, _ = S["osc"].train_forward(S["vf"], S["vd"], S["W"], S["o"], S["d"], S["rt"], emulate="tc")
        assert np.abs(got - emu).max() <= 1e-5


@pytest.mark.parametrize("form", [snisr.FORM_PLAIN_FP32, snisr.FORM_TC])
def test_train_backward_matches_oracle_adjoint(setup, form):
    import torch
    S = setup
    T = S["T"]
    vf, vd, W = (T(S[k]).requires_grad_(True) for k in ("vf", "vd", "W"))
    g = np.random.default_rng(3).standard_normal((S["d"].shape[0], 3))
    rgb = tile_field(vf, vd, W, S["sc"], T(S["o"]), T(S["d"]), T(S["rt"]), form)
    (rgb * torch.from_numpy(g).float().cuda()).sum().backward()
    gF, gG, gW = S["osc"].train_backward(S["vf"], S["vd"], S["W"], S["o"], S["d"], S["rt"], g)
    tol = 1e-3 if form == snisr.FORM_PLAIN_FP32 else 1e-2
    errs = (_rel(vf.grad.cpu().numpy(), gF), _rel(vd.grad.cpu().numpy(), gG), _rel(W.grad.cpu().numpy(), gW))
    print(f"form {form}: gradient relative errors (features, density, mlp) = {errs}")
    assert _rel(vf.grad.cpu().numpy(), gF) <= tol
    assert _rel(vd.grad.cpu().numpy(), gG) <= tol
    assert _rel(W.grad.cpu().numpy(), gW) <= tol
    if form == snisr.FORM_TC:
        eF, eG, eW = S["osc"].train_backward(S["vf"], S["vd"], S["W"], S["o"], S["d"], S["rt"], g, emulate="tc")
        emu = (_rel(vf.grad.cpu().numpy(), eF), _rel(vd.grad.cpu().numpy(), eG), _rel(W.grad.cpu().numpy(), eW))
        print(f"form {form}: relative errors against the tensor-core emulation = {emu}")
        assert max(emu) <= 2e-3
    if form == snisr.FORM_PLAIN_FP32:
        S["grads"] = (vf.grad.cpu().numpy(), vd.grad.cpu().numpy(), W.grad.cpu().numpy(), g)


def test_train_gradients_vs_fp64_finite_differences(setup):
    """64 random parameters with non-negligible gradient; FP64 oracle forward,
    central differences with h = 1e-4."""
    S = setup
    if "grads" not in S:
        pytest.skip("needs the backward test's gradients")
    gF, gG, gW, g = S["grads"]
    rng = np.random.default_rng(11)
    osc = S["osc"]

    def loss(vf, vd, W):
        r, _ = osc.train_forward(vf, vd, W, S["o"], S["d"], S["rt"])
        return float((r * g).sum())

    picks = []
    for name, grad in (("vf", gF), ("vd", gG), ("W", gW)):
        flat = np.abs(grad.reshape(-1))
        cand = np.nonzero(flat > 1e-3 * flat.max())[0]
        for i in rng.choice(cand, 22 if name != "vd" else 20, replace=False):
            picks.append((name, int(i)))
    errs = []
    h = 1e-4
    for name, i in picks[:64]:
        args = {"vf": S["vf"], "vd": S["vd"], "W": S["W"]}
        p = args[name].copy()
        flat = p.reshape(-1)
        orig = float(flat[i])
        flat[i] = np.float32(orig + h)
        lp = loss(**{**args, name: p})
        flat[i] = np.float32(orig - h)
        lm = loss(**{**args, name: p})
        hp = float(np.float32(orig + h)) - float(np.float32(orig - h))
        fd = (lp - lm) / hp
        an = {"vf": gF, "vd": gG, "W": gW}[name].reshape(-1)[i]
        errs.append(abs(an - fd) / max(abs(fd), 1e-6))
    errs = np.array(errs)
    # ReLU kinks and the early-stop cut make a few parameters non-smooth at
    # this step size; the bulk must agree to 1e-2
    assert np.median(errs) <= 1e-3
    assert (errs <= 1e-2).mean() >= 0.9


@pytest.mark.parametrize("form", [snisr.FORM_PLAIN_FP32, snisr.FORM_TC])
def test_train_long_segments_match_oracle(setup, form):
    """Low density (logit -3): segments of up to 56 samples, longer than the
    march's single-pass staging of 32 records per ray, so the second march
    over the long rays runs; results must not change."""
    import torch
    S = setup
    T = S["T"]
    vd_np = np.full_like(S["vd"], -3.0)
    ref, cnt = S["osc"].train_forward(S["vf"], vd_np, S["W"], S["o"], S["d"], S["rt"], emulate=None
                                      if form == snisr.FORM_PLAIN_FP32 else "tc")
    assert (cnt > 32).sum() > 50
    vf, vd, W = (T(x).requires_grad_(True) for x in (S["vf"], vd_np, S["W"]))
    rgb = tile_field(vf, vd, W, S["sc"], T(S["o"]), T(S["d"]), T(S["rt"]), form)
    g = np.random.default_rng(8).standard_normal((S["d"].shape[0], 3))
    (rgb * torch.from_numpy(g).float().cuda()).sum().backward()
    S["sc"].check()
    assert np.abs(rgb.detach().cpu().numpy() - ref).max() <= 1e-5
    gF, gG, gW = S["osc"].train_backward(S["vf"], vd_np, S["W"], S["o"], S["d"], S["rt"], g,
                                         emulate=None if form == snisr.FORM_PLAIN_FP32 else "tc")
    tol = 1e-3 if form == snisr.FORM_PLAIN_FP32 else 2e-3
    assert _rel(vf.grad.cpu().numpy(), gF) <= tol
    assert _rel(vd.grad.cpu().numpy(), gG) <= tol
    assert _rel(W.grad.cpu().numpy(), gW) <= tol


def test_backward_of_a_replaced_forward_is_rejected(setup):
    """Two forwards of equal batch size on one scene, then the first one's
    backward: the records of the first were replaced by the second, so the
    backward must fail with a clear error; the second's backward still gives
    the oracle's gradients."""
    import torch
    S = setup
    T = S["T"]
    form = snisr.FORM_PLAIN_FP32
    vf, vd, W = (T(S[k]).requires_grad_(True) for k in ("vf", "vd", "W"))
    g = np.random.default_rng(5).standard_normal((S["d"].shape[0], 3))
    gt = torch.from_numpy(g).float().cuda()
    first = tile_field(vf, vd, W, S["sc"], T(S["o"]), T(S["d"]), T(S["rt"]), form)
    vf2, vd2, W2 = (T(S[k]).requires_grad_(True) for k in ("vf", "vd", "W"))
    second = tile_field(vf2, vd2, W2, S["sc"], T(S["o"]), T(S["d"]), T(S["rt"]), form)
    with pytest.raises(snisr.SnisrError, match="generation"):
        (first * gt).sum().backward()
    (second * gt).sum().backward()
    gF, gG, gW = S["osc"].train_backward(S["vf"], S["vd"], S["W"], S["o"], S["d"], S["rt"], g)
    assert _rel(vf2.grad.cpu().numpy(), gF) <= 1e-3
    assert _rel(vd2.grad.cpu().numpy(), gG) <= 1e-3
    assert _rel(W2.grad.cpu().numpy(), gW) <= 1e-3
