"""ORACLE — test infrastructure only (CPU restatement of the reference path).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
the checker; the product library never loads it.  See oracle.cpp for the
reference file:line each function follows.

Parity pinning: the reference has no tests or golden vectors for this path.
The restatement is pinned (a) against the reference's own header functions
compiled for the host from the reference tree by oracle/build_ref.py (only
where the reference tree is present), (b) against golden vectors made by
running the reference's Python code (training/scripts/utils.py volume_rendering,
tile.py query_voxel, networks.py PE/MLP) with tests/golden/make_golden.py, and
(c) against golden vectors written on the GPU by the reference's own CUDA
kernels, compiled from its sources into cubins by oracle/build_ref.py
(tests/golden/make_refgpu_golden.py, tests/test_oracle_refgpu_golden.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.cpp")
    hdr = os.path.join(ROOT, "include", "snisr.h")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    # -ffp-contract=off: every binary32 operation rounds separately (the
    # specification of the traversal arithmetic) on x86-64 and AArch64 alike.
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-I", os.path.join(ROOT, "include"), src, "-o", LIB + ".tmp", "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


P = C.c_void_p


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        sig = {
            "oracle_scene_create": (P, [P]),
            "oracle_scene_destroy": (None, [P]),
            "oracle_camera_dirs": (None, [P, P]),
            "oracle_march_math": (None, [C.c_int, P, C.c_int64, P]),
            "oracle_proxy": (None, [P, P, P, C.c_int64, P, P, P, C.c_int]),
            "oracle_proxy_bvh": (None, [P, P, P, C.c_int64, P, P, P, C.c_int]),
            "oracle_trace": (None, [P, P, P, P, C.c_int64, C.c_int, P, P, C.c_int]),
            "oracle_render": (None, [P, P, P, P, C.c_int64, C.c_int, P, P, P, P, C.c_int]),
            "oracle_op_compute_rays": (None, [P, P, C.c_int, C.c_int, P]),
            "oracle_op_tracing_tiles": (None, [P, C.c_int64, P, P, P, P, P, C.c_float, C.c_int, P]),
            "oracle_op_sample_sparse": (None, [P, P, C.c_int64, P, C.c_float, C.c_float, C.c_float, C.c_float,
                                               C.c_int, C.c_int, P, P]),
            "oracle_op_inverse_z": (None, [P, P, P, P, C.c_int64, C.c_int, C.c_int, P, P]),
            "oracle_op_integrate": (None, [P, P, C.c_int64, C.c_float, P, P]),
            "oracle_op_sort_by_key": (C.c_int64, [P, P, P, C.c_int64]),
            "oracle_op_rendering_diffuse_octree": (None, [P, P, C.c_int64, C.c_int, P, P, P, P, P, P, P, P, C.c_float,
                                                          C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_int,
                                                          P, P, P, C.c_int]),
            "oracle_eval_sh2": (None, [P, P, C.c_int64, P]),
            "oracle_project_matrix": (None, [P, P, P]),
            "oracle_train_rays": (None, [P, P, C.c_int, C.c_int, P, P]),
            "oracle_train_tracing": (None, [P, P, C.c_int64, P, P, P, C.c_float, C.c_int, P]),
            "oracle_double_hits": (None, [P, P, P, P, C.c_int64, C.c_int, P, C.c_int]),
            "oracle_train_bgdepth": (None, [C.c_int, P, P, C.c_int64, C.c_int, P, P]),
            "oracle_gen_diffuse": (None, [P, C.c_int, P, P, P, P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P,
                                          C.c_int]),
            "oracle_sample_bg": (None, [P, P, P, C.c_int64, C.c_int, C.c_float, P, C.c_float, P]),
            "oracle_patch_rows": (C.c_int64, [P, C.c_int, C.c_int, C.c_int, P, P, P, P, P, P]),
            "oracle_op_transparency_statistic": (None, [P, P, C.c_int64, C.c_int, P, C.c_float, C.c_float, C.c_float,
                                                        P, P, P]),
            "oracle_op_dilate_boundary": (None, [P, C.c_int]),
            "oracle_op_prune_flags": (None, [P, P, P, C.c_int, C.c_int, C.c_float, C.c_float, P]),
            "oracle_op_pack_occupancy": (C.c_int64, [P, C.c_int, P]),
            "oracle_op_assign_pixels": (None, [P, P, P, C.c_int64, P, P]),
            "oracle_op_inference_mlp": (None, [C.c_int, C.c_int64, C.c_float, C.c_float, P, P, P, P, P, P, P, P, P,
                                               C.c_int, C.c_int]),
            "oracle_ray_aabb": (None, [P, P, P, C.c_float, P]),
            "oracle_voxel_traversal": (C.c_int, [P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float]),
            "oracle_ray_triangle_onesided": (C.c_float, [P, P, P, P, P]),
            "oracle_trilinear_base": (None, [P, C.c_int, C.c_int, C.c_int, P, P]),
            "oracle_volume_rendering": (None, [P, P, P, C.c_int64, C.c_int, C.c_float, P, P, P]),
            "oracle_positional_encoding": (None, [P, C.c_int64, C.c_int, P]),
            "oracle_grid_sample": (None, [P, C.c_int, C.c_int, C.c_int, C.c_int, P, C.c_int64, P]),
            "oracle_touched_voxels": (None, [P, P, P, P, C.c_int64, P]),
            "oracle_start_from_hit": (None, [P, P, C.c_int64, P]),
            "oracle_train_samples": (None, [P, P, P, P, P, P, P, C.c_int64, P, P, P, P]),
            "oracle_train_forward": (None, [P, P, P, P, P, P, P, C.c_int64, P, P, C.c_int, C.c_int]),
            "oracle_train_backward": (None, [P, P, P, P, P, P, P, C.c_int64, P, P, P, P, C.c_int]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


# operand emulation of the tensor-core training form: "tc" is the kernels'
# (three-part split BF16 forward whose activations the backward reuses,
# exact biases, single BF16 backward products); the others attribute its
# error: the two-part split ("tc_split2"), its forward or backward rounding
# alone, the three-part split with three-part biases ("tc_split3")
_EMUL = {None: 0, "tc": 5, "tc_split2": 1, "tc_forward": 2, "tc_backward": 3, "tc_split3": 4}


def threads() -> int:
    return max(1, os.cpu_count() or 1)


class OracleScene:
    """Oracle view of a scene description (borrows the desc's host arrays)."""

    def __init__(self, desc):
        self.desc = desc
        self.num_voxels = int(desc.num_voxels)
        self._h = lib().oracle_scene_create(C.byref(desc))

    def __del__(self):
        try:
            if self._h:
                lib().oracle_scene_destroy(self._h)
        except Exception:
            pass

    def proxy(self, o: np.ndarray, d: np.ndarray, nthreads: int | None = None):
        n = o.shape[0]
        ts = np.zeros(n, np.float32)
        th = np.zeros(n, np.float32)
        tri = np.zeros(n, np.int32)
        lib().oracle_proxy(self._h, _p(o), _p(d), n, _p(ts), _p(th), _p(tri), nthreads or threads())
        return ts, th, tri

    def proxy_bvh(self, o: np.ndarray, d: np.ndarray, nthreads: int | None = None):
        """proxy() through the oracle's own hierarchy (built on first use): the
        same results, in time fit for timing the host path on a full mesh."""
        n = o.shape[0]
        ts = np.zeros(n, np.float32)
        th = np.zeros(n, np.float32)
        tri = np.zeros(n, np.int32)
        lib().oracle_proxy_bvh(self._h, _p(o), _p(d), n, _p(ts), _p(th), _p(tri), nthreads or threads())
        return ts, th, tri

    def double_hits(self, ro, rd, visited, nthreads: int | None = None):
        """[n, K, 2] two nearest proxy hits per (ray, visited tile), -1 where missing."""
        ro = np.ascontiguousarray(ro, np.float32).reshape(-1, 3)
        rd = np.ascontiguousarray(rd, np.float32).reshape(-1, 3)
        vis = np.ascontiguousarray(visited, np.int32)
        n, K = vis.shape
        out = np.zeros((n, K, 2), np.float32)
        lib().oracle_double_hits(self._h, _p(ro), _p(rd), _p(vis), n, K, _p(out), nthreads or threads())
        return out

    def trace(self, o, d, t_start, K: int, nthreads: int | None = None):
        n = o.shape[0]
        vis = np.zeros((n, K), np.int32)
        cnt = np.zeros(n, np.int32)
        lib().oracle_trace(self._h, _p(o), _p(d), _p(t_start), n, K, _p(vis), _p(cnt), nthreads or threads())
        return vis, cnt

    def train_forward(self, vfeat, vdens, mlp, o, d, ray_tile, nthreads: int | None = None, emulate: str | None = None):
        """FP64 colours [n,3] and sample counts [n] of ray segments (ray i inside tile ray_tile[i]).
        emulate: None (exact) or "tc" -- round the MLP operands as the tensor-core form does
        (split BF16 hi+mid+lo forward operands, BF16 backward operands); the other keys of
        _EMUL attribute that form's error."""
        n = o.shape[0]
        rgb = np.zeros((n, 3))
        cnt = np.zeros(n, np.int32)
        args = [np.ascontiguousarray(a, np.float32) for a in (vfeat, vdens, mlp)]
        rt = np.ascontiguousarray(ray_tile, np.int32)
        lib().oracle_train_forward(self._h, *map(_p, args), _p(o), _p(d), _p(rt), n, _p(rgb), _p(cnt),
                                   nthreads or threads(), _EMUL[emulate])
        return rgb, cnt

    def train_samples(self, vfeat, vdens, mlp, o, d, ray_tile):
        """Samples of the training forward: offsets [n+1], global voxel id [S],
        tile-local position in voxel units [S,3] (float64), delta / voxel [S]."""
        _, cnt = self.train_forward(vfeat, vdens, mlp, o, d, ray_tile)
        off = np.zeros(cnt.size + 1, np.int64)
        np.cumsum(cnt, out=off[1:])
        S = int(off[-1])
        vox = np.zeros(S, np.int32)
        pos = np.zeros((S, 3))
        dv = np.zeros(S)
        args = [np.ascontiguousarray(a, np.float32) for a in (vfeat, vdens, mlp)]
        rt = np.ascontiguousarray(ray_tile, np.int32)
        lib().oracle_train_samples(self._h, *map(_p, args), _p(o), _p(d), _p(rt), o.shape[0], _p(off), _p(vox),
                                   _p(pos), _p(dv))
        return off, vox, pos, dv

    def train_backward(self, vfeat, vdens, mlp, o, d, ray_tile, grad_rgb, emulate: str | None = None):
        """FP64 gradients of sum(grad_rgb * rgb): (d vfeat, d vdens, d mlp).  emulate as in train_forward."""
        n = o.shape[0]
        args = [np.ascontiguousarray(a, np.float32) for a in (vfeat, vdens, mlp)]
        gF = np.zeros(args[0].shape)
        gG = np.zeros(args[1].shape)
        gW = np.zeros(args[2].shape)
        rt = np.ascontiguousarray(ray_tile, np.int32)
        g = np.ascontiguousarray(grad_rgb, np.float64)
        lib().oracle_train_backward(self._h, *map(_p, args), _p(o), _p(d), _p(rt), n, _p(g), _p(gF), _p(gG),
                                    _p(gW), _EMUL[emulate])
        return gF, gG, gW

    def start_from_hit(self, t_hit):
        """Start distances for proxy-hit distances (hit - 2 voxels, 0 on a miss)."""
        t_hit = np.ascontiguousarray(t_hit, np.float32)
        out = np.zeros_like(t_hit)
        lib().oracle_start_from_hit(self._h, _p(t_hit), t_hit.size, _p(out))
        return out

    def touched_voxels(self, o, d, t_start=None):
        """Boolean mask [num_voxels] of the voxels holding samples of the rays (single-threaded)."""
        t = np.zeros(self.num_voxels, np.uint8)
        lib().oracle_touched_voxels(self._h, _p(o), _p(d), _p(t_start), o.shape[0], _p(t))
        return t.astype(bool)

    def render(self, o, d, t_start, form: int, nthreads: int | None = None):
        """form: 0 plain FP32, 1 FP64, 2 tensor-core emulation (FP16 MLP inputs, FP64 math)."""
        n = o.shape[0]
        rgb = np.zeros((n, 3), np.float32)
        depth = np.zeros(n, np.float32)
        opac = np.zeros(n, np.float32)
        stats = np.zeros(2, np.int64)
        lib().oracle_render(self._h, _p(o), _p(d), _p(t_start), n, form, _p(rgb), _p(depth), _p(opac), _p(stats),
                            nthreads or threads())
        return rgb, depth, opac, stats


def camera_dirs(cam) -> np.ndarray:
    out = np.zeros((cam.height * cam.width, 3), np.float32)
    lib().oracle_camera_dirs(C.byref(cam), _p(out))
    return out


MATH_EXP, MATH_LOG1P, MATH_SOFTPLUS = 0, 1, 2


def march_math(fn: int, x: np.ndarray) -> np.ndarray:
    """The render march's single-precision e^x (x <= 0), log1p (y in [0, 1])
    or softplus, elementwise on float32 input."""
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(x)
    lib().oracle_march_math(fn, _p(x), x.size, _p(out))
    return out


def camera_origins(cam, n: int) -> np.ndarray:
    o = np.array([cam.c2w[3], cam.c2w[7], cam.c2w[11]], np.float32)
    return np.ascontiguousarray(np.broadcast_to(o, (n, 3)))


def op_compute_rays(intr, rot, H, W):
    out = np.zeros((H, W, 3), np.float32)
    lib().oracle_op_compute_rays(_p(intr), _p(rot), H, W, _p(out))
    return out


def op_tracing_tiles(rays_d, imap, origin, shape, smin, ssize, tile, K):
    n = rays_d.shape[0]
    out = np.zeros((n, K), np.int32)
    lib().oracle_op_tracing_tiles(_p(rays_d), n, _p(imap), _p(origin), _p(shape), _p(smin), _p(ssize), tile, K,
                                  _p(out))
    return out


def op_sample_sparse(ro, rd, flags, center, tile, N, ns):
    B = ro.shape[0]
    z = np.full((B, ns), -1, np.float32)
    d = np.full((B, ns), -1, np.float32)
    lib().oracle_op_sample_sparse(_p(ro), _p(rd), B, _p(flags), center[0], center[1], center[2], tile, N, ns, _p(z),
                                  _p(d))
    return z, d


def op_inverse_z(rays_d, origin, inv_near, inv_bound, offset, spr):
    n = rays_d.shape[0]
    pts = np.zeros((n, spr, 3), np.float32)
    steps = np.zeros((n, spr), np.float32)
    lib().oracle_op_inverse_z(_p(rays_d), _p(origin), _p(inv_near), _p(inv_bound), n, offset, spr, _p(pts),
                              _p(steps))
    return pts, steps


def op_integrate(rgba, dz, early, frame, trans):
    n = frame.shape[0]
    lib().oracle_op_integrate(_p(rgba), _p(dz), n, early, _p(frame), _p(trans))
    return frame, trans


def volume_rendering(rgb, sigma, dists, init_T=1.0):
    """rgb [B,ns,3], sigma/dists [B,ns] float32 -> out [B,3], T [B,ns], alpha [B,ns] (float64)."""
    B, ns = sigma.shape
    out = np.zeros((B, 3))
    trans = np.zeros((B, ns))
    alpha = np.zeros((B, ns))
    lib().oracle_volume_rendering(_p(np.ascontiguousarray(rgb, np.float32)), _p(np.ascontiguousarray(sigma, np.float32)),
                                  _p(np.ascontiguousarray(dists, np.float32)), B, ns, init_T, _p(out), _p(trans),
                                  _p(alpha))
    return out, trans, alpha


def positional_encoding(x, L):
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros((x.shape[0], 3 + 6 * L))
    lib().oracle_positional_encoding(_p(x), x.shape[0], L, _p(out))
    return out


def grid_sample(vol, idx):
    """vol [C,D,H,W] float32, idx [n,3] (x,y,z) index-space points -> [n,C] float64."""
    vol = np.ascontiguousarray(vol, np.float32)
    idx = np.ascontiguousarray(idx, np.float32)
    C_, D, H, W = vol.shape
    out = np.zeros((idx.shape[0], C_))
    lib().oracle_grid_sample(_p(vol), C_, D, H, W, _p(idx), idx.shape[0], _p(out))
    return out


def op_sort_by_key(keys, values, starts):
    """In place, as FASTRENDERING.sort_by_key; returns the number of distinct keys."""
    assert keys.dtype == np.int16 and values.dtype == np.int32 and starts.dtype == np.int32
    return int(lib().oracle_op_sort_by_key(_p(keys), _p(values), _p(starts), keys.size))


def op_assign_pixels(net, pixel_starts, block_starts, new_net, new_pixel_starts):
    lib().oracle_op_assign_pixels(_p(net), _p(pixel_starts), _p(block_starts), net.size, _p(new_net),
                                  _p(new_pixel_starts))


def op_inference_mlp(spr, num_block, inverse_far, trans_stop, net, transparency, qpix, pstarts, centers, samples,
                     rays_d, params_f16, results, mode: int, nthreads: int | None = None):
    """FASTRENDERING.inference_mlp; mode 0: the reference's FP16 arithmetic, 1: FP64 with FP16 operands.
    params_f16: uint16 bit patterns [G][22556]; results [npix][spr][4] float32, written in place."""
    args = [np.ascontiguousarray(a) for a in (net, transparency, qpix, pstarts, centers, samples, rays_d, params_f16)]
    lib().oracle_op_inference_mlp(int(spr), int(num_block), float(inverse_far), float(trans_stop),
                                  *map(_p, args), _p(results), int(mode), nthreads or threads())


def eval_sh2(coeff_basis_major, dirs):
    """SH degree 2 (FP64): coeff [n][27] (3 * basis + channel), unit dirs [n][3] -> [n][3]."""
    c = np.ascontiguousarray(coeff_basis_major, np.float64)
    d = np.ascontiguousarray(dirs, np.float64)
    out = np.zeros((d.shape[0], 3))
    lib().oracle_eval_sh2(_p(c), _p(d), d.shape[0], _p(out))
    return out


def op_rendering_diffuse_octree(rays_d, visited, origin, data: dict, sample_step, trans_th, early_stop,
                                frame, inverse_near, net_idx, nthreads: int | None = None, soft_hit: bool = False):
    """FASTRENDERING.rendering_diffuse_octree_fp16 on reference-format scene data (numpy dict with
    tile2group, data_voxels, block_IndexMap, nodes_IndexMap, nodes_sampleFlag, voxels_start, centers,
    num_voxel, voxel_size); frame [n,3], inverse_near [n], net_idx [n] int16 written in place
    (inverse_near / net_idx only at first hits, as the reference)."""
    n = rays_d.reshape(-1, 3).shape[0]
    K = visited.reshape(n, -1).shape[1]
    voxel = float(data["voxel_size"][0])
    tile = int(data["num_voxel"][0]) * voxel
    D = int(data["num_voxel"][0]) // (2 ** int(data["octree_depth"][0])) + 2
    arr = [np.ascontiguousarray(rays_d, np.float32), np.ascontiguousarray(visited, np.int32)]
    o = np.ascontiguousarray(origin, np.float32)
    sc = [np.ascontiguousarray(data["tile2group"], np.int32), np.ascontiguousarray(data["data_voxels"], np.float16).view(np.uint16),
          np.ascontiguousarray(data["block_IndexMap"], np.int32), np.ascontiguousarray(data["nodes_IndexMap"], np.int16),
          np.ascontiguousarray(data["nodes_sampleFlag"]).astype(np.uint8),
          np.ascontiguousarray(data["voxels_start"], np.int64), np.ascontiguousarray(data["centers"], np.float32)]
    lib().oracle_op_rendering_diffuse_octree(_p(arr[0]), _p(arr[1]), n, K, _p(o), *map(_p, sc), tile, voxel,
                                             float(sample_step), D, float(trans_th), float(early_stop), int(soft_hit),
                                             _p(frame),
                                             _p(inverse_near), _p(net_idx), nthreads or threads())


def op_transparency_statistic(rays_o, rays_d, D, center, tile_size, voxel_size, sample_step, voxels, nodes, T_voxels):
    """CUDA_EXT.transparency_statistic; T_voxels [D,D,D] float32 updated in place."""
    o = np.ascontiguousarray(rays_o, np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(rays_d, np.float32).reshape(-1, 3)
    c = np.ascontiguousarray(center, np.float32)
    v = np.ascontiguousarray(voxels, np.float32)
    nd = np.ascontiguousarray(nodes, np.int16)
    assert T_voxels.dtype == np.float32 and T_voxels.flags.c_contiguous
    lib().oracle_op_transparency_statistic(_p(o), _p(d), o.shape[0], int(D), _p(c), float(tile_size),
                                           float(voxel_size), float(sample_step), _p(v), _p(nd), _p(T_voxels))


def op_dilate_boundary(flags):
    """CUDA_EXT.dilate_boundary on a contiguous int16 [D,D,D] array, in place."""
    assert flags.dtype == np.int16 and flags.flags.c_contiguous
    lib().oracle_op_dilate_boundary(_p(flags), flags.shape[0])


def op_prune_flags(T_voxels, voxel_sigma, init_flags, N, block, th, T_th):
    """Flag update of Tile.pruning; returns int16 [N+2]^3."""
    out = np.empty((N + 2,) * 3, np.int16)
    T = np.ascontiguousarray(T_voxels, np.float32)
    s = np.ascontiguousarray(voxel_sigma, np.float32)
    i = None if init_flags is None else np.ascontiguousarray(init_flags, np.int16)
    lib().oracle_op_prune_flags(_p(T), _p(s), None if i is None else _p(i), int(N), int(block), float(th),
                                float(T_th), _p(out))
    return out


def op_pack_occupancy(flags, N):
    """(words uint64 [ceil(N^3/64)], count)."""
    f = np.ascontiguousarray(flags, np.int16)
    words = np.zeros((N ** 3 + 63) // 64, np.uint64)
    n = lib().oracle_op_pack_occupancy(_p(f), int(N), _p(words))
    return words, int(n)


# --- training-ray preparation ---------------------------------------------
def _f32(a, shape=None):
    a = np.ascontiguousarray(a, np.float32)
    return a if shape is None else a.reshape(shape)


def project_matrix(K, c2w):
    m = np.zeros(12, np.float32)
    lib().oracle_project_matrix(_p(_f32(K, 9)), _p(_f32(c2w, 12)), _p(m))
    return m


def train_rays(K, c2w, H, W):
    ro = np.zeros((H * W, 3), np.float32)
    rd = np.zeros((H * W, 3), np.float32)
    lib().oracle_train_rays(_p(_f32(K, 9)), _p(_f32(c2w, 12)), H, W, _p(ro), _p(rd))
    return ro, rd


def train_tracing(ro, rd, imap, shape, smin, tile, K):
    ro, rd = _f32(ro, (-1, 3)), _f32(rd, (-1, 3))
    n = ro.shape[0]
    vis = np.zeros((n, K), np.int32)
    lib().oracle_train_tracing(_p(ro), _p(rd), n, _p(np.ascontiguousarray(imap, np.int32).reshape(-1)),
                               _p(np.ascontiguousarray(shape, np.int32)), _p(_f32(smin)), float(tile), K, _p(vis))
    return vis


def train_bgdepth(train_tile, visited, hits):
    vis = np.ascontiguousarray(visited, np.int32)
    n, K = vis.shape
    bg = np.zeros(n, np.float32)
    valid = np.zeros(n, np.int32)
    lib().oracle_train_bgdepth(int(train_tile), _p(vis), _p(_f32(hits)), n, K, _p(bg), _p(valid))
    return bg, valid


def gen_diffuse(origins, train_tile, ro, rd, hits, visited, images, depths, ms, H, W, bgdepth):
    """Returns diffuse [H*W,3]; bgdepth (float32 [H*W]) is updated in place."""
    vis = np.ascontiguousarray(visited, np.int32)
    K = vis.shape[1]
    nimg = int(np.asarray(ms).reshape(-1, 12).shape[0])
    out = np.zeros((H * W, 3), np.float32)
    assert bgdepth.dtype == np.float32 and bgdepth.flags.c_contiguous
    lib().oracle_gen_diffuse(_p(_f32(origins)), int(train_tile), _p(_f32(ro)), _p(_f32(rd)), _p(_f32(hits)), _p(vis),
                             _p(_f32(images)), _p(_f32(depths)), _p(_f32(ms)), K, nimg, H, W, _p(out), _p(bgdepth),
                             threads())
    return out


def sample_bg(ro, rd, bgz, ns, sample_range, center, tile, z):
    ro, rd = _f32(ro, (-1, 3)), _f32(rd, (-1, 3))
    assert z.dtype == np.float32 and z.flags.c_contiguous
    lib().oracle_sample_bg(_p(ro), _p(rd), _p(_f32(bgz)), ro.shape[0], int(ns), float(sample_range),
                           _p(_f32(center)), float(tile), _p(z))


def patch_rows(valid, H, W, P, ro, rd, bgdepth, gt, diffuse):
    half = P // 2
    cnt = lambda L: (L - P - half + P - 1) // P if L - P > half else 0
    rows = np.zeros((cnt(H) * cnt(W) * P * P, 14), np.float32)
    n = lib().oracle_patch_rows(_p(np.ascontiguousarray(valid, np.int32)), H, W, P, _p(_f32(ro)), _p(_f32(rd)),
                                _p(_f32(bgdepth)), _p(_f32(gt)), _p(_f32(diffuse)), _p(rows))
    return rows[:n * P * P].reshape(n, P * P, 14)
