"""The reference's own CUDA kernels, run on the GPU as parity checkers.

oracle/build_ref.py compiles the reference's kernel sources (read in place,
with the nvcc flags of the reference's torch CUDAExtension builds) into
sm_103a cubins under oracle/_ref/.  This module loads them through the CUDA
driver API (ctypes on libcuda) into the context torch uses and launches each
kernel with the launch shape, constant-memory symbols and argument list of
the reference's host wrapper for it (each wrapper below cites the one it
restates), on the current torch stream.

Before every launch the argument list is checked against the kernel's own
parameter table (cuFuncGetParamInfo: count and byte size of every
parameter).  Test infrastructure: only tests import it; the reference tree
itself is not read here.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")

_drv = None


def _cuda():
    global _drv
    if _drv is None:
        d = C.CDLL("libcuda.so.1")
        for name, args in (
                ("cuModuleLoad", [C.POINTER(C.c_void_p), C.c_char_p]),
                ("cuModuleUnload", [C.c_void_p]),
                ("cuModuleGetFunctionCount", [C.POINTER(C.c_uint), C.c_void_p]),
                ("cuModuleEnumerateFunctions", [C.POINTER(C.c_void_p), C.c_uint, C.c_void_p]),
                ("cuFuncGetName", [C.POINTER(C.c_char_p), C.c_void_p]),
                ("cuFuncGetParamInfo", [C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
                ("cuModuleGetGlobal_v2", [C.POINTER(C.c_uint64), C.POINTER(C.c_size_t), C.c_void_p, C.c_char_p]),
                ("cuMemcpyHtoD_v2", [C.c_uint64, C.c_void_p, C.c_size_t]),
                ("cuLaunchKernel", [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                    C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
                ("cuGetErrorString", [C.c_int, C.POINTER(C.c_char_p)])):
            f = getattr(d, name)
            f.restype = C.c_int
            f.argtypes = args
        _drv = d
    return _drv


def _check(rc: int, what: str):
    if rc != 0:
        s = C.c_char_p()
        _cuda().cuGetErrorString(rc, C.byref(s))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({(s.value or b'?').decode()})")


def cubin(name: str) -> str:
    return os.path.join(REF_DIR, name + ".cubin")


def available(*names: str) -> bool:
    return all(os.path.exists(cubin(n)) for n in names)


# ---------------------------------------------------------------------------
# argument helpers: one ctypes object per kernel parameter
# ---------------------------------------------------------------------------
def ptr(t):
    return C.c_void_p(t.data_ptr())


def f32(x):
    return C.c_float(float(x))


def i32(x):
    return C.c_int(int(x))


def b8(x):
    return C.c_bool(bool(x))


def f16(x):
    """A `half` passed by value: its 2-byte IEEE binary16 pattern."""
    return C.c_uint16(int(np.float16(x).view(np.uint16)))


def float3(a):
    return (C.c_float * 3)(*[float(v) for v in a])


class Module:
    """One cubin loaded into torch's current CUDA context."""

    def __init__(self, name: str):
        import torch
        torch.zeros(1, device="cuda")  # the primary context is current on this thread
        self.name = name
        self.mod = C.c_void_p()
        _check(_cuda().cuModuleLoad(C.byref(self.mod), cubin(name).encode()), f"load {name}.cubin")
        n = C.c_uint()
        _check(_cuda().cuModuleGetFunctionCount(C.byref(n), self.mod), "function count")
        fns = (C.c_void_p * n.value)()
        _check(_cuda().cuModuleEnumerateFunctions(fns, n.value, self.mod), "enumerate functions")
        self.functions = {}
        for f in fns:
            s = C.c_char_p()
            _check(_cuda().cuFuncGetName(C.byref(s), f), "function name")
            self.functions[s.value.decode()] = C.c_void_p(f)

    def function(self, base: str):
        """The free __global__ function `base` (Itanium name _Z<len><base>...)."""
        key = f"_Z{len(base)}{base}"
        hits = [v for k, v in self.functions.items() if k.startswith(key)]
        if len(hits) != 1:
            raise KeyError(f"{self.name}.cubin: {len(hits)} kernels named {base}")
        return hits[0]

    def set_const(self, name: str, values, dtype=np.float32):
        a = np.ascontiguousarray(np.asarray(values, dtype=dtype).reshape(-1))
        dptr, size = C.c_uint64(), C.c_size_t()
        _check(_cuda().cuModuleGetGlobal_v2(C.byref(dptr), C.byref(size), self.mod, name.encode()),
               f"{self.name}: symbol {name}")
        if size.value != a.nbytes:
            raise ValueError(f"{self.name}: symbol {name} holds {size.value} bytes, got {a.nbytes}")
        _check(_cuda().cuMemcpyHtoD_v2(dptr, a.ctypes.data, a.nbytes), f"{self.name}: set {name}")

    @staticmethod
    def param_sizes(fn):
        sizes = []
        while True:
            off, size = C.c_size_t(), C.c_size_t()
            if _cuda().cuFuncGetParamInfo(fn, len(sizes), C.byref(off), C.byref(size)) != 0:
                return sizes
            sizes.append(size.value)

    def launch(self, kernel: str, grid: int, block: int, args, smem: int = 0):
        import torch
        fn = self.function(kernel)
        sizes = self.param_sizes(fn)
        if len(sizes) != len(args) or any(C.sizeof(a) != s for a, s in zip(args, sizes)):
            raise TypeError(f"{kernel}: parameter sizes {sizes}, arguments {[C.sizeof(a) for a in args]}")
        if grid <= 0 or block <= 0:
            raise ValueError(f"{kernel}: empty launch")
        arr = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        _check(_cuda().cuLaunchKernel(fn, int(grid), 1, 1, int(block), 1, 1, int(smem), stream, arr, None), kernel)


_mods = {}


def module(name: str) -> Module:
    if name not in _mods:
        _mods[name] = Module(name)
    return _mods[name]


def _split_render(n: int, num_thread: int):
    """The render wrappers' job split: (grid, base_num, extra_num), e.g.
    rendering/src/compute_rays.cu:56-58."""
    nb = min(65535, (n + num_thread - 1) // num_thread)
    base = n // (nb * num_thread)
    return nb, base, n - base * nb * num_thread


def _split_train(n: int):
    """The training wrappers' split (512 threads): (grid, base_jobs, add_num),
    e.g. training/src/Sample_kernel.cu:415-419."""
    nb = min(65535, (n + 511) // 512)
    return nb, n // (nb * 512), n % (nb * 512)


# ---------------------------------------------------------------------------
# FASTRENDERING (rendering/src)
# ---------------------------------------------------------------------------
def compute_rays(intrinsic, c2w_rotation, num_thread, rays_d):
    """rendering/src/compute_rays.cu:46-69; intrinsic / rotation as numpy."""
    H, W = rays_d.shape[0], rays_d.shape[1]
    nb, base, extra = _split_render(H * W, num_thread)
    m = module("compute_rays")
    m.set_const("c_c2w", c2w_rotation)
    m.set_const("c_intrinsic", intrinsic)
    m.launch("compute_rays_kernel", nb, num_thread, [ptr(rays_d), i32(W), i32(extra), i32(base)])


def tracing_tiles(rays_d, IndexMap, origin, tile_shape, scene_min_corner, scene_size, tile_size, num_thread,
                  visitedTiles):
    """rendering/src/raytile_tracing.cu:63-94; origin .. scene_size as numpy."""
    H, W, K = visitedTiles.shape
    nb, base, extra = _split_render(H * W, num_thread)
    m = module("raytile_tracing")
    m.set_const("c_origin", origin)
    m.set_const("c_scene_min_corner", scene_min_corner)
    m.set_const("c_tile_shape", tile_shape, np.int32)
    m.set_const("c_scene_size", scene_size)
    m.launch("tracing_tiles_kernel", nb, num_thread,
             [ptr(rays_d), ptr(IndexMap), f32(tile_size), i32(K), ptr(visitedTiles), i32(extra), i32(base)])


def rendering_diffuse_octree_fp16(rays_d, visitedTiles, origin, groupMap, data_voxels, block_IndexMap,
                                  nodes_IndexMap, nodes_sampleFlag, voxels_start, centers, tile_size, voxel_size,
                                  sample_step, num_voxel, num_thread, trans_th, early_stop, soft_hit,
                                  frame_diffuse, inverse_near, netIdxs):
    """rendering/src/raydiffuse_render_octree_fp16.cu:238-287; origin as numpy."""
    assert num_voxel == 18
    K = visitedTiles.shape[-1]
    H, W = rays_d.shape[0], rays_d.shape[1]
    nb, base, extra = _split_render(H * W, num_thread)
    m = module("raydiffuse_render_octree_fp16")
    m.set_const("c_origin", origin)
    m.launch("rendering_diffuse_octree_fp16_kernel", nb, num_thread,
             [ptr(rays_d), ptr(visitedTiles), ptr(groupMap), ptr(data_voxels), ptr(block_IndexMap),
              ptr(nodes_IndexMap), ptr(nodes_sampleFlag), ptr(voxels_start), ptr(centers), f32(tile_size),
              f32(voxel_size), f32(sample_step), i32(K), i32(num_voxel), ptr(frame_diffuse), ptr(inverse_near),
              ptr(netIdxs), b8(soft_hit), f16(trans_th), f32(early_stop), i32(extra), i32(base)])


def inverse_z_sampling(origin, rays_d, inverse_near, inverse_bound, num_thread, offset, sample_per_ray,
                       sample_points, integrate_steps):
    """rendering/src/sampling.cu:48-80; origin as numpy."""
    H, W = inverse_near.shape[0], inverse_near.shape[1]
    n = H * W * sample_per_ray
    nb = min(65535, (n + num_thread - 1) // num_thread)
    base = n // (nb * num_thread)
    extra = n - base * nb * num_thread
    m = module("sampling")
    m.set_const("c_origin", origin)
    m.launch("inverse_z_sampling_kernel", nb, num_thread,
             [ptr(rays_d), ptr(inverse_near), ptr(inverse_bound), i32(offset), i32(sample_per_ray),
              ptr(sample_points), ptr(integrate_steps), i32(base), i32(extra)])


def integrate_points(sample_results, integrate_steps, num_thread, early_step, transparency, colors_buffer):
    """rendering/src/volume_rendering.cu:60-87 (16 samples per ray)."""
    H, W = colors_buffer.shape[0], colors_buffer.shape[1]
    nb, base, extra = _split_render(H * W, num_thread)
    module("volume_rendering").launch(
        "integrate_points_kernel", nb, num_thread,
        [ptr(sample_results), ptr(integrate_steps), ptr(transparency), f32(early_step), ptr(colors_buffer),
         i32(base), i32(extra)])


def assign_pixels(netIdxs, pixel_starts, block_starts, num_thread, new_netIdxs, new_pixel_starts):
    """rendering/src/reorder.cu:69-93."""
    nb, base, extra = _split_render(netIdxs.numel(), num_thread)
    module("reorder").launch("assign_pixels_kernel", nb, num_thread,
                             [ptr(netIdxs), ptr(pixel_starts), ptr(block_starts), ptr(new_netIdxs),
                              ptr(new_pixel_starts), i32(base), i32(extra)])


def inference_mlp(max_samples_per_ray, num_block, num_thread, inverse_far, trans_stop, netIdxs, transparency,
                  query_pixel_indices, pixel_starts, group_centers, samples, rays_d, params, sample_results):
    """rendering/src/rayreflection_render.cu:304-335 (44 KB of static shared
    memory per block for the network)."""
    module("rayreflection_render").launch(
        "inference_mlp_kernel", num_block, num_thread,
        [i32(max_samples_per_ray), f32(inverse_far), ptr(netIdxs), ptr(transparency), f32(trans_stop),
         ptr(query_pixel_indices), ptr(pixel_starts), ptr(group_centers), ptr(samples), ptr(rays_d), ptr(params),
         ptr(sample_results)])


# ---------------------------------------------------------------------------
# CUDA_EXT (training/src)
# ---------------------------------------------------------------------------
def Sample_sparse(rays_start, rays_dir, node_flags, cx, cy, cz, tile_size, num_voxel, z_vals, dists):
    """training/src/Sample_kernel.cu:397-434."""
    B, ns = z_vals.shape
    nb, base, add = _split_train(B)
    module("Sample_kernel").launch(
        "Sample_sparse_cuda_kernel", nb, 512,
        [ptr(rays_start), ptr(rays_dir), ptr(node_flags), float3((cx, cy, cz)), f32(tile_size), i32(ns),
         i32(num_voxel), ptr(z_vals), ptr(dists), i32(base), i32(add)])


def Sample_bg(rays_start, rays_dir, bg_zval, tile_center, tile_size, sample_range, z_vals):
    """training/src/Sample_kernel.cu:580-616."""
    B, ns = z_vals.shape
    nb, base, add = _split_train(B)
    module("Sample_kernel").launch(
        "Sample_bg_cuda_kernel", nb, 512,
        [ptr(rays_start), ptr(rays_dir), ptr(bg_zval), i32(ns), f32(sample_range), ptr(tile_center),
         f32(tile_size), ptr(z_vals), i32(base), i32(add)])


def transparency_statistic(rays_start, rays_dir, num_voxel, tile_center, tile_size, voxel_size, sample_step,
                           voxels, nodes, T_voxels):
    """training/src/Helper_kernel.cu:268-302."""
    nb, base, add = _split_train(rays_start.shape[0])
    module("Helper_kernel").launch(
        "transparency_statistic_cuda_kernel", nb, 512,
        [ptr(rays_start), ptr(rays_dir), i32(num_voxel), ptr(tile_center), f32(tile_size), f32(voxel_size),
         f32(sample_step), ptr(voxels), ptr(nodes), ptr(T_voxels), i32(base), i32(add)])


def dilate_boundary(nodes_flag, num_voxel):
    """training/src/Helper_kernel.cu:235-266: through a temporary, then copied back."""
    import torch
    total = int(num_voxel) ** 3
    nb, base, add = _split_train(total)
    tmp = torch.empty_like(nodes_flag)
    module("Helper_kernel").launch("dilate_boundary_cuda_kernel", nb, 512,
                                   [ptr(nodes_flag), ptr(tmp), i32(num_voxel), i32(base), i32(add)])
    nodes_flag.copy_(tmp)


# ---------------------------------------------------------------------------
# training-data preparation (training/src/cuda_func.cu), launched as
# get_trainData_v3 launches them (cuda_func.cu:1428-1439, 1500-1521): 512
# threads, one job per pixel (or per pixel x visited-tile slot)
# ---------------------------------------------------------------------------
def int3(a):
    return (C.c_int * 3)(*[int(v) for v in a])


def computing_rays(H, W, K, C2W, rays_o, rays_d):
    """cuda_func.cu:15-50; K [9], C2W [12] device arrays; rays [H*W, 3]."""
    nb, base, add = _split_train(H * W)
    module("cuda_func").launch("computing_rays_kernel", nb, 512,
                               [i32(H), i32(W), ptr(K), ptr(C2W), ptr(rays_o), ptr(rays_d), i32(add), i32(base)])


def tracing_tile(H, W, rays_o, rays_d, IndexMap, tile_shape, tile_size, K, visited, scene_min_corner):
    """cuda_func.cu:52-128; visited [H*W, K]."""
    nb, base, add = _split_train(H * W)
    module("cuda_func").launch("tracingTile_kernel", nb, 512,
                               [i32(H), i32(W), ptr(rays_o), ptr(rays_d), ptr(IndexMap), int3(tile_shape),
                                f32(tile_size), i32(K), ptr(visited), float3(scene_min_corner), i32(add), i32(base)])


def ray_double_hit_in_tile(H, W, rays_o, rays_d, vertices, faces, centers, BConFaceIdx, BConFaceNum, tile_size, K,
                           num_block, visited, double_hits):
    """cuda_func.cu:284-444; one job per (pixel, visited slot); double_hits [H*W, K, 2]."""
    nb, base, add = _split_train(H * W * K)
    module("cuda_func").launch("ray_doubleHit_inTile_kernel", nb, 512,
                               [i32(H), i32(W), ptr(rays_o), ptr(rays_d), ptr(vertices), ptr(faces), ptr(centers),
                                ptr(BConFaceIdx), ptr(BConFaceNum), f32(tile_size), i32(K), i32(num_block),
                                ptr(visited), ptr(double_hits), i32(add), i32(base)])


def get_train_data(train_tile, rays_o, rays_d, vertices, faces, visited, double_hits, K, bgdepth, valid):
    """cuda_func.cu:587-663; bgdepth / valid [H*W] (the host zeroes valid per view)."""
    nb, base, add = _split_train(valid.numel())
    module("cuda_func").launch("get_trainData_kernel", nb, 512,
                               [i32(train_tile), ptr(rays_o), ptr(rays_d), ptr(vertices), ptr(faces), ptr(visited),
                                ptr(double_hits), i32(K), ptr(bgdepth), ptr(valid), i32(add), i32(base)])


def gen_diffuse_in_tile(origins, train_tile, rays_o, rays_d, double_hits, visited, images, depths, ms, K, num_images,
                        H, W, diffuses, bgdepth):
    """cuda_func.cu:1197-1339; diffuses [H*W, 3]; bgdepth is read and updated."""
    nb, base, add = _split_train(H * W)
    module("cuda_func").launch("gen_diffuse_in_tile_kernel", nb, 512,
                               [ptr(origins), i32(train_tile), ptr(rays_o), ptr(rays_d), ptr(double_hits),
                                ptr(visited), ptr(images), ptr(depths), ptr(ms), i32(K), i32(num_images), i32(H),
                                i32(W), ptr(diffuses), ptr(bgdepth), i32(add), i32(base)])


def render_diffuse(train_tile, rays_o, rays_d, visited, sparse_to_group, K, tile_size, num_voxel, voxel_size,
                   sample_step, centers, voxels, nodes, diffuses, depths, valid):
    """cuda_func.cu:1687-1802 (the FP32 sparse-voxel renderer of the second
    training iteration); note its (base_jobs, add_num) parameter order."""
    n = valid.numel()
    nb, base, add = _split_train(n)
    module("cuda_func").launch("render_diffuse_kernel", nb, 512,
                               [i32(train_tile), ptr(rays_o), ptr(rays_d), ptr(visited), ptr(sparse_to_group), i32(K),
                                f32(tile_size), i32(num_voxel), f32(voxel_size), f32(sample_step), ptr(centers),
                                ptr(voxels), ptr(nodes), ptr(diffuses), ptr(depths), ptr(valid), i32(base), i32(add)])
