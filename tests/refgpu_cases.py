"""Seeded inputs shared by the golden-vector generator of the reference's
own kernels (tests/golden/make_refgpu_golden.py, run on a GPU host) and the
CPU test that checks the oracle against those vectors
(tests/test_oracle_refgpu_golden.py).  Everything here is numpy."""
from __future__ import annotations

import functools

import numpy as np

import snisr

OUTSIDE_ORIGIN = np.array([-2.0, 5.5, 1.4], np.float32)


@functools.lru_cache(maxsize=None)
def _scene16():
    # the scene the golden vectors were written on: 16 tiles of 64^3, 40 boxes
    # with sides U(0.3, 1.2) m (fixed here, independent of the benchmark config)
    return snisr.SynthScene(snisr.CFG2.replace(res=64, with_mesh=False, box_min=0.3, box_max=1.2))


@functools.lru_cache(maxsize=None)
def _scene1():
    return snisr.SynthScene(snisr.CFG1)


def _cam(s, pose, W, H):
    cam = s.camera(pose, W, H)
    intr = np.array([cam.cx, cam.cy, cam.inv_focal], np.float32)
    rot = np.array([[cam.c2w[4 * r + c] for c in range(3)] for r in range(3)], np.float32)
    origin = np.array([cam.c2w[3], cam.c2w[7], cam.c2w[11]], np.float32)
    return intr, rot, origin


def camera_case():
    intr, rot, origin = _cam(_scene16(), 0, 64, 48)
    return dict(H=48, W=64, intr=intr, rot=rot, origin=origin)


def tracing_case():
    s = _scene16()
    d = s.desc
    shape = np.array(list(d.grid), np.int32)
    return dict(imap=np.asarray(s.arrays()["tile_index"], np.int32), shape=shape, smin=np.zeros(3, np.float32),
                ssize=shape.astype(np.float32) * np.float32(d.tile_size), tile=float(d.tile_size), K=30)


@functools.lru_cache(maxsize=None)
def octree_case():
    from snisr import octree
    s = _scene16()
    D = octree.from_synth(s, groups=4)
    der = octree.derived(D)
    intr, rot, origin = _cam(s, 1, 64, 48)
    return dict(D=D, H=48, W=64, K=8, intr=intr, rot=rot, origin=origin, tile_shape=D["tile_shape"],
                scene_min_corner=D["scene_min_corner"], scene_size=der["scene_size"].astype(np.float32),
                tile_size=der["tile_size"], voxel_size=der["voxel_size"], sample_step=der["sample_step"],
                block_num_voxel=der["block_num_voxel"])


def inverse_z_case():
    rng = np.random.default_rng(6)
    H, W, spr = 20, 20, 16
    rays_d = rng.standard_normal((H, W, 3)).astype(np.float32)
    inv_near = (1.0 / rng.uniform(0.3, 4.0, (H, W))).astype(np.float32)
    inv_bound = ((1.0 / (1.0 / inv_near + np.float32(8.0)) - inv_near) / 63).astype(np.float32)
    return dict(rays_d=rays_d, inv_near=inv_near, inv_bound=inv_bound, spr=spr, offsets=(0, 16, 48),
                origin=np.array([0.3, -0.2, 1.1], np.float32), pts_shape=(H, W, spr, 3), steps_shape=(H, W, spr))


def integrate_case():
    rng = np.random.default_rng(7)
    H, W = 20, 25
    rgba = (rng.random((H, W, 16, 4)) * np.array([1, 1, 1, 5])).astype(np.float32)
    dz = (rng.random((H, W, 16)) * 0.3).astype(np.float32)
    trans = np.ones((H, W, 1), np.float32)
    trans.reshape(-1)[::11] = 1e-4
    frame = (rng.random((H, W, 3)) * 0.1).astype(np.float32)
    return dict(rgba=rgba, dz=dz, trans=trans, frame=frame, early=1e-3)


def sample_sparse_case():
    s = _scene1()
    N = s.desc.res
    bits = np.unpackbits(s.arrays()["occupancy"].view(np.uint8), bitorder="little")[: N ** 3]
    rng = np.random.default_rng(5)
    B = 512
    ro = np.concatenate([rng.uniform(0.2, 1.8, (B // 2, 3)), rng.uniform(-1.0, 3.0, (B // 2, 3))]).astype(np.float32)
    rd = rng.standard_normal((B, 3)).astype(np.float32)
    rd /= np.linalg.norm(rd, axis=1, keepdims=True)
    rd[::17, 1] = 0.0
    return dict(ro=ro, rd=rd, flags=bits.astype(np.int16).reshape(N, N, N), center=(1.0, 1.0, 1.0), tile=2.0,
                N=int(N), B=B, ns=64)


def sample_bg_case():
    rng = np.random.default_rng(9)
    n, ns = 512, 16
    center = np.array([1.5, 4.5, 1.5], np.float32)
    ro = (center + rng.uniform(-6, 6, (n, 3))).astype(np.float32)
    rd = rng.standard_normal((n, 3)).astype(np.float32)
    bg = rng.uniform(0.0, 12.0, (n, 1)).astype(np.float32)
    bg[::7] = -1.0
    return dict(ro=ro, rd=rd, bg=bg, center=center, tile=3.0, range=0.6, n=n, ns=ns)


def transparency_case():
    import oracle
    from snisr import prune
    s = _scene1()
    a = s.arrays()
    sigma, _, flags = prune.grids_from_arrays(s.desc, a, 0)
    center = prune.tile_centers(s.desc, a)[0].astype(np.float32)
    tile = float(s.desc.tile_size)
    N = int(s.desc.res)
    vs = tile / N
    cam = s.camera(0, 64, 48)
    rd = oracle.camera_dirs(cam).astype(np.float32)
    ro = oracle.camera_origins(cam, rd.shape[0]).astype(np.float32)
    return dict(ro=np.ascontiguousarray(ro), rd=np.ascontiguousarray(rd), D=N + 2, center=center, tile=tile, vs=vs,
                step=vs * 0.1, sigma=sigma, flags=flags)


def dilate_case():
    rng = np.random.default_rng(11)
    D = 34
    return dict(D=D, flags=rng.choice(np.array([-1, 0, 1], np.int16), size=(D, D, D), p=[0.85, 0.1, 0.05]))
