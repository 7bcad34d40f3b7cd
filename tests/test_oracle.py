"""CPU checks of the oracle itself (no GPU).

1. Against the reference's own Python code: golden vectors in
   tests/golden/reference_python.npz (made by tests/golden/make_golden.py).
2. Against the reference's own header functions compiled for the host
   (oracle/_ref/libref.so, built by oracle/build_ref.py where the reference
   tree exists; skipped elsewhere).
3. Known-answer tests of the traversal (DDA ties, axis-aligned rays, empty
   and boundary cases) and internal consistency (FP32 vs FP64 shading).
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
import snisr

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_python.npz")


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- golden vectors
def test_volume_rendering_matches_reference_python():
    g = np.load(GOLD)
    out, T, alpha = oracle.volume_rendering(g["vr_rgb"], g["vr_sigma"], g["vr_dists"], float(g["vr_init_T"]))
    np.testing.assert_allclose(out, g["vr_out"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(T, g["vr_T"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(alpha, g["vr_alpha"], rtol=1e-12, atol=1e-12)


def test_query_voxel_matches_reference_python():
    g = np.load(GOLD)
    idx = (g["qv_x"] - g["qv_min_corner"]) / g["qv_voxel"] - 0.5
    res = oracle.grid_sample(g["qv_voxels"].astype(np.float32), idx.reshape(-1, 3).astype(np.float32))
    ref = np.concatenate([g["qv_rgb"], g["qv_sigma"]], -1).reshape(-1, 4)
    # inputs rounded to float32 for the oracle; compare at float32 resolution
    np.testing.assert_allclose(res, ref, rtol=1e-5, atol=1e-5)


def test_positional_encoding_matches_reference_python():
    g = np.load(GOLD)
    res = oracle.positional_encoding(g["pe_x"], 4)
    np.testing.assert_allclose(res, g["pe_out"], rtol=1e-12, atol=1e-12)


# ----------------------------------------------------- reference header harness
@pytest.fixture(scope="module")
def ref():
    import importlib.util
    spec = importlib.util.spec_from_file_location("build_ref", os.path.join(oracle.HERE, "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.build()
    if path is None or not os.path.exists(path):
        pytest.skip("reference tree not present: header harness unavailable")
    L = C.CDLL(path)
    P = C.c_void_p
    L.ref_ray_aabb.argtypes = [P, P, P, C.c_float, P]
    L.ref_voxel_traversal.argtypes = [P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float]
    L.ref_voxel_traversal.restype = C.c_int
    L.ref_ray_triangle.argtypes = [P, P, P, P, P]
    L.ref_ray_triangle.restype = C.c_float
    L.ref_trilinear_base.argtypes = [P, C.c_int, C.c_int, C.c_int, P, P]
    return L


def test_ray_aabb_bitexact_vs_reference(ref):
    rng = np.random.default_rng(1)
    O = oracle.lib()
    for i in range(4000):
        o = rng.uniform(-3, 3, 3).astype(np.float32)
        d = rng.standard_normal(3).astype(np.float32)
        if i % 7 == 0:
            d[rng.integers(3)] = 0.0  # axis-parallel rays (safe_divide path)
        c = rng.uniform(-1, 1, 3).astype(np.float32)
        h = np.float32(rng.uniform(0.1, 2))
        a = np.zeros(2, np.float32)
        b = np.zeros(2, np.float32)
        ref.ref_ray_aabb(_p(o), _p(d), _p(c), h, _p(a))
        O.oracle_ray_aabb(_p(o), _p(d), _p(c), h, _p(b))
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (o, d, c, h, a, b)


def test_voxel_traversal_bitexact_vs_reference(ref):
    rng = np.random.default_rng(2)
    O = oracle.lib()
    M = (6, 5, 7)
    vs = np.float32(0.37)
    for i in range(1500):
        imap = np.where(rng.random(np.prod(M)) < 0.4, rng.integers(0, 100, np.prod(M)), -1).astype(np.int32)
        o = (rng.random(3) * np.array(M) * vs * 0.999).astype(np.float32)
        if i % 5 == 0:  # start exactly on voxel boundaries (tie rules)
            o = (np.floor(o / vs) * vs).astype(np.float32)
        d = rng.standard_normal(3).astype(np.float32)
        if i % 4 == 0:
            d = np.array([1, 1, 1], np.float32) * np.sign(d)  # exact diagonal ties
        if i % 9 == 0:
            d[rng.integers(3)] = 0.0
        K = 40
        a = np.zeros(K, np.int32)
        b = np.full(K, -1, np.int32)
        na = ref.ref_voxel_traversal(_p(o), _p(d), _p(imap), _p(a), K, *M, vs)
        nb = O.oracle_voxel_traversal(_p(o), _p(d), _p(imap), _p(b), K, *M, vs)
        assert na == nb and np.array_equal(a[:na], b[:nb]), (i, o, d)


def test_ray_triangle_bitexact_vs_reference(ref):
    rng = np.random.default_rng(3)
    O = oracle.lib()
    hits = 0
    for _ in range(5000):
        o = rng.uniform(-1, 1, 3).astype(np.float32)
        A, B, Cc = (rng.uniform(-1, 1, 3).astype(np.float32) for _ in range(3))
        tgt = (A + B + Cc) / 3 + rng.normal(0, 0.3, 3)
        d = (tgt - o).astype(np.float32)
        a = ref.ref_ray_triangle(_p(o), _p(d), _p(A), _p(B), _p(Cc))
        b = O.oracle_ray_triangle_onesided(_p(o), _p(d), _p(A), _p(B), _p(Cc))
        assert np.float32(a).view(np.uint32) == np.float32(b).view(np.uint32)
        hits += a > 0
    assert hits > 100


def test_trilinear_base_bitexact_vs_reference(ref):
    rng = np.random.default_rng(4)
    O = oracle.lib()
    M = (5, 4, 6)
    vox = rng.standard_normal((np.prod(M), 4)).astype(np.float32)
    for _ in range(3000):
        p = (rng.random(3) * (np.array(M) - 0.5)).astype(np.float32)
        if rng.random() < 0.2:
            p[rng.integers(3)] = np.float32(M[rng.integers(3)] - 1)  # edge fallbacks
        p = np.minimum(p, np.array(M, np.float32) - 1)
        a = np.zeros(4, np.float32)
        b = np.zeros(4, np.float32)
        ref.ref_trilinear_base(_p(vox), *M, _p(p), _p(a))
        O.oracle_trilinear_base(_p(vox), *M, _p(p), _p(b))
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), p


# ------------------------------------------------------- traversal known answers
def _one_tile_scene(N=8, occupied=()):
    """A 1-tile scene description built in Python (numpy-owned arrays)."""
    occ = np.zeros(N ** 3 // 64, np.uint64)
    for (x, y, z) in occupied:
        v = (x * N + y) * N + z
        occ[v >> 6] |= np.uint64(1) << np.uint64(v & 63)
    nvox = int(sum(bin(int(w)).count("1") for w in occ))
    keep = {}
    desc = snisr._lib.SceneDesc()
    for i in range(3):
        desc.grid[i] = 1
        desc.scene_min[i] = 0.0
    desc.tile_size = 1.0
    desc.res = N
    desc.num_tiles = 1
    keep["ti"] = np.zeros(1, np.int32)
    keep["occ"] = occ
    keep["corners"] = np.arange(nvox * 8, dtype=np.int32) % max(nvox * 8, 1)
    keep["vf"] = np.zeros((max(nvox * 8, 1), 16), np.float32)
    keep["vd"] = np.zeros(max(nvox * 8, 1), np.float32)
    P = int(snisr.lib().snisr_mlp_param_count(16, 4, 32, 2))
    keep["mlp"] = np.zeros(P, np.float32)
    desc.tile_index = keep["ti"].ctypes.data_as(C.POINTER(C.c_int32))
    desc.occupancy = keep["occ"].ctypes.data_as(C.POINTER(C.c_uint64))
    desc.num_voxels = nvox
    desc.voxel_corners = keep["corners"].ctypes.data_as(C.POINTER(C.c_int32))
    desc.num_vertices = max(nvox * 8, 1)
    desc.feat_dim = 16
    desc.feat_type = snisr.F32
    desc.vertex_feat = keep["vf"].ctypes.data
    desc.vertex_density = keep["vd"].ctypes.data
    desc.dir_freqs = 4
    desc.mlp_hidden = 32
    desc.mlp_layers = 2
    desc.mlp_params = keep["mlp"].ctypes.data_as(C.POINTER(C.c_float))
    desc.step_vox = 0.5
    desc.early_stop = 1e-3
    desc.start_offset_vox = 2.0
    desc.max_samples_per_ray = 8
    desc.max_pixels = 1024
    return desc, keep


def test_kat_axis_ray_visits_row_in_order():
    N = 8
    occ = [(x, 3, 4) for x in range(N)]
    desc, keep = _one_tile_scene(N, occ)
    osc = oracle.OracleScene(desc)
    o = np.array([[-0.5, 3.5 / N, 4.5 / N]], np.float32)
    d = np.array([[1.0, 0.0, 0.0]], np.float32)
    vis, cnt = osc.trace(o, d, None, 16)
    ids = sorted(((x * N + 3) * N + 4) for (x, _, _) in occ)
    assert cnt[0] == N
    assert list(vis[0, :N]) == list(range(N))  # ranks follow voxel order along +x
    # reversed direction visits them backwards
    vis2, cnt2 = osc.trace(np.array([[1.5, 3.5 / N, 4.5 / N]], np.float32), -d, None, 16)
    assert list(vis2[0, :N]) == list(range(N))[::-1]
    assert len(ids) == N


def test_kat_diagonal_tie_prefers_z_then_y():
    # exact diagonal through voxel corners: ties go to z, then y (reference tie rule)
    N = 4
    occ = [(x, y, z) for x in range(N) for y in range(N) for z in range(N)]
    desc, keep = _one_tile_scene(N, occ)
    osc = oracle.OracleScene(desc)
    o = np.array([[0.0, 0.0, 0.0]], np.float32)
    d = np.array([[1, 1, 1]], np.float32) / np.float32(np.sqrt(3))
    vis, cnt = osc.trace(np.ascontiguousarray(o), np.ascontiguousarray(d.astype(np.float32)), None, 64)
    seq = []
    for r in vis[0, :cnt[0]]:
        seq.append((r // (N * N), (r // N) % N, r % N))
    # every step changes exactly one axis by +1
    for a, b in zip(seq, seq[1:]):
        diff = np.array(b) - np.array(a)
        assert sorted(diff.tolist()) == [0, 0, 1]
    assert seq[0] == (0, 0, 0) and seq[-1] == (N - 1, N - 1, N - 1)


def test_kat_empty_scene_and_miss():
    desc, keep = _one_tile_scene(8, [])
    osc = oracle.OracleScene(desc)
    o = np.array([[0.5, 0.5, 0.5], [5.0, 5.0, 5.0]], np.float32)
    d = np.array([[0.0, 0.0, 1.0], [1.0, 0.0, 0.0]], np.float32)
    vis, cnt = osc.trace(o, d, None, 4)
    assert cnt.tolist() == [0, 0] and (vis == -1).all()
    rgb, depth, opac, st = osc.render(o, d, None, 0)
    assert st[0] == 0 and np.all(rgb == 0) and np.all(opac == 0)


def test_oracle_fp32_vs_fp64_cfg1():
    s = snisr.SynthScene(snisr.CFG1)
    osc = oracle.OracleScene(s.desc)
    cam = s.camera(1)
    d = oracle.camera_dirs(cam)[::7].copy()
    o = oracle.camera_origins(cam, d.shape[0])
    r32, d32, o32, st32 = osc.render(o, d, None, 0)
    r64, d64, o64, st64 = osc.render(o, d, None, 1)
    assert st32[0] > 1000
    assert np.abs(r32 - r64).max() < 1e-5
    assert np.abs(o32 - o64).max() < 1e-5
    # FP16-input emulation of the tensor-core form stays well inside 1e-3 RMSE
    rtc, _, _, _ = osc.render(o, d, None, 2)
    assert np.sqrt(((rtc - r64) ** 2).mean()) < 2e-4


def test_oracle_start_distance_skips_voxels():
    s = snisr.SynthScene(snisr.CFG1)
    osc = oracle.OracleScene(s.desc)
    cam = s.camera(2)
    d = oracle.camera_dirs(cam)[::31].copy()
    o = oracle.camera_origins(cam, d.shape[0])
    v0, c0 = osc.trace(o, d, None, 512)
    ts = np.full(d.shape[0], 1.2, np.float32)
    v1, c1 = osc.trace(o, d, ts, 512)
    assert (c1 <= c0).all() and c1.sum() < c0.sum()
    # the later sequence is a suffix of the full one
    for i in np.nonzero(c1)[0][:200]:
        assert list(v1[i, :c1[i]]) == list(v0[i, c0[i] - c1[i]:c0[i]])


# ---------------------------------------------------------------- specular pass ops
def test_sh2_matches_reference_python():
    g = np.load(GOLD)
    coeff = g["sh_coeff"].transpose(0, 2, 1).reshape(-1, 27)  # basis-major, as the device layout
    np.testing.assert_allclose(oracle.eval_sh2(coeff, g["sh_dirs"]), g["sh_out"], rtol=0, atol=1e-12)


def test_sort_by_key_is_stable_sort_plus_unique():
    rng = np.random.default_rng(0)
    keys = rng.integers(-1, 40, 5000).astype(np.int16)
    k0 = keys.copy()
    vals = rng.integers(0, 1 << 30, 5000).astype(np.int32)
    v0 = vals.copy()
    starts = np.arange(5000, dtype=np.int32)
    n = oracle.op_sort_by_key(keys, vals, starts)
    order = np.argsort(k0, kind="stable")
    assert np.array_equal(vals, v0[order])
    u, first = np.unique(k0[order], return_index=True)
    assert n == u.size and np.array_equal(keys[:n], u) and np.array_equal(starts[:n], first)


def test_assign_pixels_known_answer():
    # net 7: 130 pixels over 3 blocks -> 44, 43, 43; net 2: 64 pixels over 1 block
    net = np.array([7, 2], np.int16)
    pixel_starts = np.array([0, 130, 194], np.int32)
    block_starts = np.array([0, 3, 4], np.int32)
    new_net = np.zeros(4, np.int16)
    new_ps = np.zeros(4, np.int32)
    oracle.op_assign_pixels(net, pixel_starts, block_starts, new_net, new_ps)
    assert new_net.tolist() == [7, 7, 7, 2]
    assert new_ps.tolist() == [0, 44, 87, 130]


def _fma32(a, b, c):
    """Correctly rounded binary32 a*b + c: the product is exact in binary64,
    the sum's rounding error is recovered exactly (two-sum) and the binary64
    sum is rounded to odd before the final rounding to binary32, which makes
    that final rounding correct."""
    a, b, c = (np.asarray(x, np.float32).astype(np.float64) for x in (a, b, c))
    p = a * b
    s = p + c
    bb = s - p
    e = (p - (s - bb)) + (c - bb)
    odd = (s.view(np.int64) & 1) == 1
    s = np.where((e != 0) & ~odd, np.nextafter(s, np.where(e > 0, np.inf, -np.inf)), s)
    return s.astype(np.float32)


def test_compute_rays_states_the_fused_operation():
    """The oracle's compute_rays is fma(c0, x, c1 * y) + c2 per component
    with one rounding in the fma (the form the reference's nvcc build
    compiles get_direction to), on random cameras: checked against an
    independent binary64 model of the same expression."""
    rng = np.random.default_rng(12)
    for _ in range(4):
        H, W = 24, 40
        intr = np.array([rng.uniform(10, 30), rng.uniform(5, 20), rng.uniform(1e-3, 5e-2)], np.float32)
        rot = rng.standard_normal((3, 3)).astype(np.float32)
        got = oracle.op_compute_rays(intr, rot, H, W).reshape(H, W, 3)
        py, px = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
        x = ((px.astype(np.float32) - intr[0]) * intr[2]).astype(np.float32)
        y = ((py.astype(np.float32) - intr[1]) * intr[2]).astype(np.float32)
        want = np.stack([(_fma32(rot[a, 0], x, (rot[a, 1] * y).astype(np.float32)) + rot[a, 2]).astype(np.float32)
                         for a in range(3)], -1)
        assert np.array_equal(got, want)
        unfused = np.stack([(((rot[a, 0] * x).astype(np.float32) + (rot[a, 1] * y).astype(np.float32))
                             .astype(np.float32) + rot[a, 2]).astype(np.float32) for a in range(3)], -1)
        assert not np.array_equal(got, unfused)  # the test can tell the two forms apart


def _march_math_inputs():
    x = -np.linspace(0, 80, 2000001).astype(np.float32)
    y = np.concatenate([np.linspace(0, 1, 2000001).astype(np.float32),
                        (10.0 ** np.linspace(-40, 0, 100000)).astype(np.float32)])
    z = np.linspace(-30, 30, 1000001).astype(np.float32)
    return x, y, z


def test_march_math_accuracy():
    """The render march's own e^x, log1p and softplus (single precision, the
    same operations on the host and the device) against float64: e^x below
    1 ulp on [-80, 0], log1p below 3 ulp on [0, 1], softplus relative error
    below 5e-7 on [-30, 30]."""
    x, y, z = _march_math_inputs()
    e = oracle.march_math(oracle.MATH_EXP, x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    assert (np.abs(e - ref) / np.spacing(ref.astype(np.float32)).astype(np.float64)).max() < 1.0
    l1 = oracle.march_math(oracle.MATH_LOG1P, y).astype(np.float64)
    ref = np.log1p(y.astype(np.float64))
    ulp = np.spacing(np.maximum(ref, 1e-45).astype(np.float32)).astype(np.float64)
    assert (np.abs(l1 - ref) / ulp).max() < 3.0
    sp = oracle.march_math(oracle.MATH_SOFTPLUS, z).astype(np.float64)
    ref = np.logaddexp(0.0, z.astype(np.float64))
    assert (np.abs(sp - ref) / ref).max() < 5e-7
    assert oracle.march_math(oracle.MATH_EXP, np.array([-100.0, 0.0, np.nan], np.float32))[:2].tolist() == [0.0, 1.0]


def test_host_bvh_proxy_equals_brute_force():
    """The oracle's hierarchy (used to time the host path) returns the brute-
    force nearest hit: same t and triangle id, on rays of two poses of the
    1280x720 scene's ~205k-triangle proxy mesh."""
    s = snisr.SynthScene(snisr.CFG2.replace(res=32))
    osc = oracle.OracleScene(s.desc)
    rng = np.random.default_rng(4)
    for pose in (0, 5):
        cam = s.camera(pose, 320, 180)
        d = oracle.camera_dirs(cam)
        d = np.ascontiguousarray(d[np.sort(rng.choice(d.shape[0], 1500, replace=False))])
        o = oracle.camera_origins(cam, d.shape[0])
        ts, th, tri = osc.proxy(o, d)
        ts2, th2, tri2 = osc.proxy_bvh(o, d)
        assert np.array_equal(tri, tri2) and np.array_equal(th, th2) and np.array_equal(ts, ts2)
        assert (tri >= 0).mean() > 0.95
