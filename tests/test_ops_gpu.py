"""GPU parity of the reference-op drop-ins (FASTRENDERING / CUDA_EXT argument
meaning) against the oracle, through the C ABI.  Integer outputs and the
IEEE-exact float ops are compared bit-for-bit; integrate_points (exp) within
1e-6."""
import numpy as np
import pytest

import oracle
import snisr
from snisr import ops

pytestmark = pytest.mark.gpu


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _n(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def cfg2(cuda):
    return snisr.SynthScene(snisr.CFG2.replace(res=32))


def _intrinsic_rot(cam):
    intr = np.array([cam.cx, cam.cy, cam.inv_focal], np.float32)
    rot = np.array([[cam.c2w[4 * r + c] for c in range(3)] for r in range(3)], np.float32)
    return intr, rot


def test_compute_rays_bitexact(cfg2):
    import torch
    cam = cfg2.camera(0, 320, 180)
    intr, rot = _intrinsic_rot(cam)
    rays_d = torch.full((180, 320, 3), -1.0, device="cuda")
    ops.compute_rays(_t(intr), _t(rot), 256, rays_d)
    assert np.array_equal(_n(rays_d), oracle.op_compute_rays(intr, rot, 180, 320))


@pytest.mark.parametrize("inside", [True, False])
def test_tracing_tiles_bitexact(cfg2, inside):
    import torch
    cam = cfg2.camera(1, 256, 144)
    intr, rot = _intrinsic_rot(cam)
    rd = oracle.op_compute_rays(intr, rot, 144, 256).reshape(-1, 3)
    d = cfg2.desc
    imap = cfg2.arrays()["tile_index"].copy()
    origin = np.array([cam.c2w[3], cam.c2w[7], cam.c2w[11]], np.float32)
    if not inside:
        origin = np.array([-2.0, 5.5, 1.4], np.float32)  # outside the scene box
    shape = np.array(list(d.grid), np.int32)
    smin = np.zeros(3, np.float32)
    ssize = shape.astype(np.float32) * np.float32(d.tile_size)
    K = 30
    vis = torch.empty((144, 256, K), dtype=torch.int32, device="cuda")
    ops.tracing_tiles(_t(rd.reshape(144, 256, 3)), _t(imap), _t(origin), _t(shape), _t(smin), _t(ssize),
                      float(d.tile_size), 256, vis)
    ref = oracle.op_tracing_tiles(rd, imap, origin, shape, smin, ssize, np.float32(d.tile_size), K)
    assert np.array_equal(_n(vis).reshape(-1, K), ref)
    assert (ref[:, 0] >= 0).mean() > 0.5


def test_sample_sparse_bitexact(cuda):
    import torch
    s = snisr.SynthScene(snisr.CFG1)
    a = s.arrays()
    N = s.desc.res
    bits = np.unpackbits(a["occupancy"].view(np.uint8), bitorder="little")[: N ** 3]
    flags = bits.astype(np.int16).reshape(N, N, N)  # x-major, 1 = occupied
    rng = np.random.default_rng(5)
    B, ns = 4096, 64
    ro = np.ascontiguousarray(np.concatenate([rng.uniform(0.2, 1.8, (B // 2, 3)),
                                              rng.uniform(-1.0, 3.0, (B // 2, 3))]).astype(np.float32))
    rd = rng.standard_normal((B, 3)).astype(np.float32)
    rd /= np.linalg.norm(rd, axis=1, keepdims=True)
    rd[::17, 1] = 0.0  # axis-parallel components
    center = np.array([1.0, 1.0, 1.0], np.float32)
    z = torch.full((B, ns), -1.0, device="cuda")
    dd = torch.full((B, ns), -1.0, device="cuda")
    ops.Sample_sparse(_t(ro), _t(rd), _t(flags), float(center[0]), float(center[1]), float(center[2]), 2.0, N, z, dd)
    rz, rdist = oracle.op_sample_sparse(ro, rd, flags, center, np.float32(2.0), N, ns)
    assert np.array_equal(_n(z), rz) and np.array_equal(_n(dd), rdist)
    assert (rz[:, 0] != -1).sum() > 100


def test_inverse_z_sampling_bitexact(cuda):
    import torch
    rng = np.random.default_rng(6)
    H, W, spr = 60, 80, 16
    rays_d = rng.standard_normal((H, W, 3)).astype(np.float32)
    inv_near = (1.0 / rng.uniform(0.3, 4.0, (H, W))).astype(np.float32)
    far = np.float32(8.0)
    inv_bound = ((1.0 / (1.0 / inv_near + far) - inv_near) / 63).astype(np.float32)
    origin = np.array([0.3, -0.2, 1.1], np.float32)
    pts = torch.full((H, W, spr, 3), -1.0, device="cuda")
    steps = torch.zeros((H, W, spr), device="cuda")
    ops.inverse_z_sampling(_t(origin), _t(rays_d), _t(inv_near), _t(inv_bound), 256, 16, spr, pts, steps)
    rp, rs = oracle.op_inverse_z(rays_d.reshape(-1, 3), origin, inv_near.reshape(-1), inv_bound.reshape(-1), 16, spr)
    assert np.array_equal(_n(pts).reshape(-1, spr, 3), rp)
    assert np.array_equal(_n(steps).reshape(-1, spr), rs)


def test_integrate_points(cuda):
    import torch
    rng = np.random.default_rng(7)
    H, W = 40, 50
    rgba = rng.random((H, W, 16, 4)).astype(np.float32)
    rgba[..., 3] *= 5
    dz = (rng.random((H, W, 16)) * 0.3).astype(np.float32)
    trans = np.ones((H, W, 1), np.float32)
    trans.reshape(-1)[::11] = 1e-4  # below early stop: skipped
    frame = (rng.random((H, W, 3)) * 0.1).astype(np.float32)
    tt, tf = _t(trans), _t(frame)
    ops.integrate_points(_t(rgba), _t(dz), 512, 1e-3, tt, tf)
    rf, rt = oracle.op_integrate(rgba.reshape(-1, 16, 4), dz.reshape(-1, 16), np.float32(1e-3), frame.reshape(-1, 3).copy(),
                                 trans.reshape(-1).copy())
    np.testing.assert_allclose(_n(tf).reshape(-1, 3), rf, atol=1e-6)
    np.testing.assert_allclose(_n(tt).reshape(-1), rt, atol=1e-6)
