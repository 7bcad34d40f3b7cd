"""The oracle's emulation of the tensor-core training form (emulate="tc":
three-part split BF16 forward operands with exact biases, the forward's
activations reused by the backward, single BF16 backward operands) and its
attribution modes, on the CPU: the three-part forward keeps the colours at
FP32-level accuracy, the two-part split does not; the modes differ from each
other only where their definitions differ; every emulated gradient stays
within the 1e-2 bound of the exact FP64 adjoint."""
import numpy as np
import pytest

import oracle
import snisr


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def problem():
    s = snisr.SynthScene(snisr.CFG1)
    a = s.arrays()
    rng = np.random.default_rng(11)
    W = a["mlp_params"].copy()
    W += rng.normal(0, 0.05, W.shape).astype(np.float32)
    cam = s.camera(1)
    d = oracle.camera_dirs(cam)
    idx = np.sort(rng.choice(d.shape[0], 512, replace=False))
    d = np.ascontiguousarray(d[idx])
    o = oracle.camera_origins(cam, d.shape[0])
    rt = np.zeros(d.shape[0], np.int32)
    g = rng.standard_normal((d.shape[0], 3))
    osc = oracle.OracleScene(s.desc)
    vf, vd = a["vertex_feat"].astype(np.float32), a["vertex_density"].astype(np.float32)
    out = {}
    for mode in (None, "tc", "tc_split2", "tc_split3"):
        rgb, cnt = osc.train_forward(vf, vd, W, o, d, rt, emulate=mode)
        grads = osc.train_backward(vf, vd, W, o, d, rt, g, emulate=mode)
        out[mode] = (rgb, grads)
    assert cnt.sum() > 300
    return out


def test_three_part_forward_keeps_fp32_colours(problem):
    exact = problem[None][0]
    assert np.abs(problem["tc"][0] - exact).max() <= 1e-6
    assert np.abs(problem["tc_split3"][0] - exact).max() <= 1e-6
    two = np.abs(problem["tc_split2"][0] - exact).max()
    assert 1e-7 < two <= 1e-4  # the two-part split is visibly coarser


def test_modes_differ_only_where_defined(problem):
    # tc and tc_split3 differ only in the biases (exact vs three-part): the
    # three-part split of an FP32 value is the value itself
    for a, b in zip(problem["tc"][1], problem["tc_split3"][1]):
        assert _rel(a, b) <= 1e-6


def test_emulated_gradients_within_the_bound(problem):
    for mode in ("tc", "tc_split2", "tc_split3"):
        errs = [_rel(a, b) for a, b in zip(problem[mode][1], problem[None][1])]
        assert max(errs) <= 1e-2, (mode, errs)
        assert max(errs) > 0.0  # the backward operands are rounded to BF16
