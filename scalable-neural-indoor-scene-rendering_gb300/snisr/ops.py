"""Reference-op mirrors: the FASTRENDERING (rendering/src/binding.cpp:13-27)
and CUDA_EXT (training/src/binding.cpp:4-12) entry points for this path, with
the reference's names, argument order and in-place outputs, implemented by
libsnisr's sm_103a kernels.

Inputs are checked like the reference's CHECK_INPUT (CUDA, contiguous) plus
dtype/shape checks; failures raise RuntimeError as TORCH_CHECK does.  The
`num_thread` arguments are accepted for signature compatibility; launch
shapes are chosen by the library.
"""
from __future__ import annotations

from . import _lib


def _check(t, name, dtype=None, dim=None):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise RuntimeError(f"{name} must be {dtype}, got {t.dtype}")
    if dim is not None and t.dim() != dim:
        raise RuntimeError(f"{name} must have {dim} dims, got {t.dim()}")


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def compute_rays(intrinsic, c2w_rotation, num_thread, rays_d):
    """rays_d[H,W,3] = R @ [(x-cx)/f, (y-cy)/f, 1] (rendering/src/compute_rays.cu:46-68)."""
    import torch
    _check(intrinsic, "intrinsic", torch.float32)
    _check(c2w_rotation, "c2w_rotation", torch.float32)
    _check(rays_d, "rays_d", torch.float32, 3)
    H, W = rays_d.shape[0], rays_d.shape[1]
    _lib.check(_lib.lib().snisr_op_compute_rays(intrinsic.data_ptr(), c2w_rotation.data_ptr(), H, W,
                                                rays_d.data_ptr(), _stream()))


def tracing_tiles(rays_d, IndexMap, origin, tile_shape, scene_min_corner, scene_size, tile_size, num_thread,
                  visitedTiles):
    """Visited non-empty tiles per pixel, -1 padded (rendering/src/raytile_tracing.cu:63-95)."""
    import torch
    _check(rays_d, "rays_d", torch.float32)
    _check(IndexMap, "IndexMap", torch.int32)
    _check(origin, "origin", torch.float32)
    _check(tile_shape, "tile_shape", torch.int32)
    _check(scene_min_corner, "scene_min_corner", torch.float32)
    _check(scene_size, "scene_size", torch.float32)
    _check(visitedTiles, "visitedTiles", torch.int32, 3)
    npix = visitedTiles.shape[0] * visitedTiles.shape[1]
    if rays_d.numel() != npix * 3:
        raise RuntimeError("rays_d and visitedTiles disagree on the pixel count")
    _lib.check(_lib.lib().snisr_op_tracing_tiles(rays_d.data_ptr(), npix, IndexMap.data_ptr(), origin.data_ptr(),
                                                 tile_shape.data_ptr(), scene_min_corner.data_ptr(),
                                                 scene_size.data_ptr(), float(tile_size), visitedTiles.shape[2],
                                                 visitedTiles.data_ptr(), _stream()))


def inverse_z_sampling(origin, rays_d, inverse_near, inverse_bound, num_thread, offset, sample_per_ray,
                       sample_points, integrate_steps):
    """1/z-uniform samples (rendering/src/sampling.cu:48-81)."""
    import torch
    for t, n in ((origin, "origin"), (rays_d, "rays_d"), (inverse_near, "inverse_near"),
                 (inverse_bound, "inverse_bound"), (sample_points, "sample_points"),
                 (integrate_steps, "integrate_steps")):
        _check(t, n, torch.float32)
    npix = inverse_near.numel()
    if rays_d.numel() != npix * 3 or inverse_bound.numel() != npix or sample_points.numel() != npix * sample_per_ray * 3:
        raise RuntimeError("inverse_z_sampling: inconsistent sizes")
    _lib.check(_lib.lib().snisr_op_inverse_z_sampling(rays_d.data_ptr(), origin.data_ptr(), inverse_near.data_ptr(),
                                                      inverse_bound.data_ptr(), npix, int(offset), int(sample_per_ray),
                                                      sample_points.data_ptr(), integrate_steps.data_ptr(),
                                                      _stream()))


def integrate_points(sample_results, integrate_steps, num_thread, early_step, transparency, colors_buffer):
    """Front-to-back compositing of 16 samples per pixel, transmittance carried
    across calls (rendering/src/volume_rendering.cu:60-87)."""
    import torch
    for t, n in ((sample_results, "sample_results"), (integrate_steps, "integrate_steps"),
                 (transparency, "transparency"), (colors_buffer, "colors_buffer")):
        _check(t, n, torch.float32)
    npix = transparency.numel()
    if sample_results.numel() != npix * 64 or integrate_steps.numel() != npix * 16 or colors_buffer.numel() != npix * 3:
        raise RuntimeError("integrate_points: expects 16 samples of (rgb, sigma) per pixel")
    _lib.check(_lib.lib().snisr_op_integrate_points(sample_results.data_ptr(), integrate_steps.data_ptr(), npix,
                                                    float(early_step), colors_buffer.data_ptr(),
                                                    transparency.data_ptr(), _stream()))


def Sample_sparse(rays_start, rays_dir, node_flags, cx, cy, cz, tile_size, num_voxel, z_vals, dists):
    """Samples only inside occupied voxels (training/src/Sample_kernel.cu:397-434).
    node_flags: int16 [N][N][N] x-major (1 = occupied)."""
    import torch
    _check(rays_start, "rays_start", torch.float32, 2)
    _check(rays_dir, "rays_dir", torch.float32, 2)
    _check(node_flags, "node_flags", torch.int16, 3)
    _check(z_vals, "z_vals", torch.float32, 2)
    _check(dists, "dists", torch.float32, 2)
    B, ns = z_vals.shape
    if rays_start.shape[0] != B or rays_dir.shape[0] != B or dists.shape != z_vals.shape:
        raise RuntimeError("Sample_sparse: inconsistent batch sizes")
    if node_flags.numel() != num_voxel ** 3:
        raise RuntimeError("Sample_sparse: node_flags must hold num_voxel^3 entries")
    _lib.check(_lib.lib().snisr_op_sample_sparse(rays_start.data_ptr(), rays_dir.data_ptr(), B, node_flags.data_ptr(),
                                                 float(cx), float(cy), float(cz), float(tile_size), int(num_voxel),
                                                 ns, z_vals.data_ptr(), dists.data_ptr(), _stream()))


def sparse_sampling(rays_o, rays_d, node_flags, num_voxel, center, size, nsamples):
    """training/scripts/utils.py:797-805: node_flags given as D x H x W (z,y,x),
    returns (z_vals, dists) pre-filled with -1."""
    import torch
    z = torch.full((rays_o.shape[0], nsamples), -1, dtype=torch.float32, device=rays_o.device)
    d = torch.full((rays_o.shape[0], nsamples), -1, dtype=torch.float32, device=rays_o.device)
    Sample_sparse(rays_o, rays_d, node_flags.permute(2, 1, 0).contiguous(), *center, size, num_voxel, z, d)
    return z, d


# ---------------------------------------------------------------------------
# Specular pass (the reference's reflection MLP and its batching by network)
# ---------------------------------------------------------------------------
_err_words = {}


def _err_word(device):
    import torch
    t = _err_words.get(device)
    if t is None:
        t = torch.zeros(1, dtype=torch.int32, device=device)
        _err_words[device] = t
    return t


def check_errors():
    """Synchronises and raises if an inference_mlp call's bounded device wait ran out."""
    import torch
    for dev, t in _err_words.items():
        torch.cuda.synchronize(dev)
        if int(t.item()) != 0:
            t.zero_()
            raise _lib.SnisrError(_lib.DEVICE_TIMEOUT, "inference_mlp: a bounded device wait ran out")


def sort_by_key(keys_tensor, values_tensor, starts_tensor):
    """Stable sort of (int16 keys, int32 values) in place, then unique_by_key
    over (keys, starts); returns the number of distinct keys
    (rendering/src/reorder.cu:10-22)."""
    import torch
    _check(keys_tensor, "keys", torch.int16)
    _check(values_tensor, "values", torch.int32)
    _check(starts_tensor, "starts", torch.int32)
    n = keys_tensor.numel()
    if values_tensor.numel() != n or starts_tensor.numel() != n:
        raise RuntimeError("sort_by_key: keys, values and starts must have the same length")
    import ctypes
    out = ctypes.c_int64()
    _lib.check(_lib.lib().snisr_op_sort_by_key(keys_tensor.data_ptr(), values_tensor.data_ptr(),
                                               starts_tensor.data_ptr(), n, ctypes.byref(out), _stream()))
    return int(out.value)


def assign_pixels(netIdxs, pixel_starts, block_starts, num_thread, new_netIdxs, new_pixel_starts):
    """Pixels of each network spread over its blocks (rendering/src/reorder.cu:24-94)."""
    import torch
    _check(netIdxs, "netIdxs", torch.int16)
    _check(pixel_starts, "pixel_starts", torch.int32)
    _check(block_starts, "block_starts", torch.int32)
    _check(new_netIdxs, "new_netIdxs", torch.int16)
    _check(new_pixel_starts, "new_pixel_starts", torch.int32)
    num_net = netIdxs.numel()
    if pixel_starts.numel() < num_net + 1 or block_starts.numel() < num_net + 1:
        raise RuntimeError("assign_pixels: pixel_starts and block_starts need num_net + 1 entries")
    _lib.check(_lib.lib().snisr_op_assign_pixels(netIdxs.data_ptr(), pixel_starts.data_ptr(), block_starts.data_ptr(),
                                                 num_net, new_netIdxs.data_ptr(), new_pixel_starts.data_ptr(),
                                                 _stream()))


def inference_mlp(max_samples_per_ray, num_block, num_thread, inverse_far, trans_stop, netIdxs, transparency,
                  query_pixel_indices, pixel_starts, group_centers, samples, rays_d, params, sample_results):
    """Per-group reflection MLP with SH colour (rendering/src/rayreflection_render.cu:111-301) on tcgen05.
    params: float16 [G, 22556] in the reference layout."""
    import torch
    _check(netIdxs, "netIdxs", torch.int16)
    _check(transparency, "transparency", torch.float32)
    _check(query_pixel_indices, "query_pixel_indices", torch.int32)
    _check(pixel_starts, "pixel_starts", torch.int32)
    _check(group_centers, "group_centers", torch.float32)
    _check(samples, "samples", torch.float32)
    _check(rays_d, "rays_d", torch.float32)
    _check(sample_results, "sample_results", torch.float32)
    if not params.is_cuda or not params.is_contiguous() or params.dtype != torch.float16:
        raise RuntimeError("params must be a contiguous CUDA float16 tensor")
    P = _lib.lib().snisr_op_inference_mlp_param_count()
    if params.numel() % P != 0:
        raise RuntimeError(f"params must hold a multiple of {P} values")
    npix = query_pixel_indices.numel()
    spr = int(max_samples_per_ray)
    if samples.numel() != npix * spr * 3 or sample_results.numel() != npix * spr * 4 or rays_d.numel() != npix * 3:
        raise RuntimeError("inference_mlp: samples / sample_results / rays_d sizes disagree with the pixel count")
    if pixel_starts.numel() < int(num_block) + 1 or netIdxs.numel() < int(num_block):
        raise RuntimeError("inference_mlp: netIdxs / pixel_starts shorter than num_block")
    err = _err_word(samples.device)
    _lib.check(_lib.lib().snisr_op_inference_mlp(spr, int(num_block), float(inverse_far), float(trans_stop),
                                                 netIdxs.data_ptr(), params.numel() // P, transparency.data_ptr(),
                                                 query_pixel_indices.data_ptr(), pixel_starts.data_ptr(),
                                                 group_centers.data_ptr(), samples.data_ptr(), rays_d.data_ptr(),
                                                 params.data_ptr(), sample_results.data_ptr(), err.data_ptr(),
                                                 _stream()))


def rendering_diffuse_octree_fp16(rays_d, visitedTiles, origin, groupMap, data_voxels, block_IndexMap,
                                  nodes_IndexMap, nodes_sampleFlag, voxels_start, centers, tile_size, voxel_size,
                                  sample_step, num_voxel, num_thread, trans_th, early_stop, soft_hit,
                                  frame_diffuse, inverse_near, netIdxs):
    """The reference's FP16 diffuse renderer on its octree scene format
    (rendering/src/raydiffuse_render_octree_fp16.cu:141-287); num_voxel is the
    dilated node side (18); outputs written in place."""
    import torch
    _check(rays_d, "rays_d", torch.float32)
    _check(visitedTiles, "visitedTiles", torch.int32)
    _check(origin, "origin", torch.float32)
    _check(groupMap, "groupMap", torch.int32)
    _check(block_IndexMap, "block_IndexMap", torch.int32)
    _check(nodes_IndexMap, "nodes_IndexMap", torch.int16)
    _check(voxels_start, "voxels_start", torch.int64)
    _check(centers, "centers", torch.float32)
    _check(frame_diffuse, "frame_diffuse", torch.float32)
    _check(inverse_near, "inverse_near", torch.float32)
    _check(netIdxs, "netIdxs", torch.int16)
    for t, n, dt in ((data_voxels, "data_voxels", torch.float16), (nodes_sampleFlag, "nodes_sampleFlag", torch.bool)):
        if not t.is_cuda or not t.is_contiguous() or t.dtype != dt:
            raise RuntimeError(f"{n} must be a contiguous CUDA {dt} tensor")
    npix = frame_diffuse.numel() // 3
    K = visitedTiles.shape[-1]
    if rays_d.numel() != npix * 3 or visitedTiles.numel() != npix * K or inverse_near.numel() != npix:
        raise RuntimeError("rendering_diffuse_octree_fp16: pixel counts disagree")
    _lib.check(_lib.lib().snisr_op_rendering_diffuse_octree(
        rays_d.data_ptr(), visitedTiles.data_ptr(), npix, K, origin.data_ptr(), groupMap.data_ptr(),
        data_voxels.data_ptr(), block_IndexMap.data_ptr(), nodes_IndexMap.data_ptr(), nodes_sampleFlag.data_ptr(),
        voxels_start.data_ptr(), centers.data_ptr(), centers.shape[0], float(tile_size), float(voxel_size),
        float(sample_step), int(num_voxel), float(trans_th), float(early_stop), int(bool(soft_hit)),
        frame_diffuse.data_ptr(),
        inverse_near.data_ptr(), netIdxs.data_ptr(),
        frame_diffuse.shape[1] if frame_diffuse.dim() == 3 else 0,  # an [H, W, 3] frame: its width
        _stream()))


# ---------------------------------------------------------------------------
# Pruning after a training epoch (CUDA_EXT helpers and the flag update of
# Tile.pruning), on dilated [x][y][z] grids of D = N + 2 cells per side
# ---------------------------------------------------------------------------
def transparency_statistic(rays_start, rays_dir, num_voxel, tile_center, tile_size, voxel_size, sample_step,
                           voxels, nodes, T_voxels):
    """training/src/Helper.cpp:29-56 / Helper_kernel.cu:108-172: T_voxels
    [D,D,D] max-combined in place with transmittance x trilinear weight at
    the samples of every ray in flagged (== 1) cells; num_voxel = D."""
    import torch
    _check(rays_start, "rays_start", torch.float32, 2)
    _check(rays_dir, "rays_dir", torch.float32, 2)
    _check(tile_center, "tile_center", torch.float32, 1)
    _check(voxels, "voxels", torch.float32, 3)
    _check(nodes, "nodes", torch.int16, 3)
    _check(T_voxels, "T_voxels", torch.float32, 3)
    D = int(num_voxel)
    for t, n in ((voxels, "voxels"), (nodes, "nodes"), (T_voxels, "T_voxels")):
        if tuple(t.shape) != (D, D, D):
            raise RuntimeError(f"transparency_statistic: {n} must be {D}^3")
    if rays_start.shape != rays_dir.shape or rays_start.shape[1] != 3:
        raise RuntimeError("transparency_statistic: rays must be [B,3]")
    _lib.check(_lib.lib().snisr_op_transparency_statistic(
        rays_start.data_ptr(), rays_dir.data_ptr(), rays_start.shape[0], D, tile_center.data_ptr(),
        float(tile_size), float(voxel_size), float(sample_step), voxels.data_ptr(), nodes.data_ptr(),
        T_voxels.data_ptr(), _stream()))


def dilate_boundary(nodes_flag, num_voxel):
    """training/src/Helper.cpp:6-13 / Helper_kernel.cu:174-270, in place."""
    import torch
    _check(nodes_flag, "nodes_flag", torch.int16, 3)
    if nodes_flag.numel() != int(num_voxel) ** 3:
        raise RuntimeError("dilate_boundary: nodes_flag must hold num_voxel^3 entries")
    _lib.check(_lib.lib().snisr_op_dilate_boundary(nodes_flag.data_ptr(), int(num_voxel), _stream()))


def prune_flags(T_voxels, voxel_sigma, init_flags, block, th, T_th, nodes_flag):
    """The flag update of Tile.pruning (training/scripts/tile/tile.py:337-372)
    after its model query: T_voxels [D,D,D], voxel_sigma [N,N,N] (density at
    the voxel centres), init_flags [N,N,N] int16 or None (all 1); nodes_flag
    [D,D,D] int16 is overwritten (D = N + 2)."""
    import torch
    _check(T_voxels, "T_voxels", torch.float32, 3)
    _check(voxel_sigma, "voxel_sigma", torch.float32, 3)
    _check(nodes_flag, "nodes_flag", torch.int16, 3)
    N = voxel_sigma.shape[0]
    if tuple(voxel_sigma.shape) != (N, N, N) or tuple(T_voxels.shape) != (N + 2,) * 3 or \
            tuple(nodes_flag.shape) != (N + 2,) * 3:
        raise RuntimeError("prune_flags: shapes must be N^3 (voxel_sigma, init_flags) and (N+2)^3")
    ip = None
    if init_flags is not None:
        _check(init_flags, "init_flags", torch.int16, 3)
        if tuple(init_flags.shape) != (N, N, N):
            raise RuntimeError("prune_flags: init_flags must be N^3")
        ip = init_flags.data_ptr()
    _lib.check(_lib.lib().snisr_op_prune_flags(T_voxels.data_ptr(), voxel_sigma.data_ptr(), ip, N, int(block),
                                               float(th), float(T_th), nodes_flag.data_ptr(), _stream()))


def pack_occupancy(nodes_flag):
    """Occupancy words (int64 view of this library's uint64 layout) and the
    number of occupied voxels (a 0-dim device tensor) of a [N+2]^3 flag grid."""
    import torch
    _check(nodes_flag, "nodes_flag", torch.int16, 3)
    N = nodes_flag.shape[0] - 2
    words = torch.empty((N ** 3 + 63) // 64, dtype=torch.int64, device=nodes_flag.device)
    count = torch.empty((), dtype=torch.int64, device=nodes_flag.device)
    _lib.check(_lib.lib().snisr_op_pack_occupancy(nodes_flag.data_ptr(), N, words.data_ptr(), count.data_ptr(),
                                                  _stream()))
    return words, count


# ---------------------------------------------------------------------------
# Training-ray preparation: background sampling (CUDA_EXT.Sample_bg)
# ---------------------------------------------------------------------------
def Sample_bg(rays_start, rays_dir, bg_zval, tile_center, tile_size, sample_range, z_vals):
    """training/src/Sample.cpp:81-105 / Sample_kernel.cu:481-542: z_vals
    [B,Ns] uniform over bg +- range/2 (behind the tile's exit if that range
    starts inside it); rows with bg == -1 are left as they are."""
    import torch
    _check(rays_start, "rays_start", torch.float32, 2)
    _check(rays_dir, "rays_dir", torch.float32, 2)
    _check(bg_zval, "bg_zval", torch.float32, 2)
    _check(tile_center, "tile_center", torch.float32, 1)
    _check(z_vals, "z_vals", torch.float32, 2)
    B, ns = z_vals.shape
    if rays_start.shape[0] != B or rays_dir.shape[0] != B or bg_zval.numel() != B:
        raise RuntimeError("Sample_bg: inconsistent batch sizes")
    _lib.check(_lib.lib().snisr_op_sample_bg(rays_start.data_ptr(), rays_dir.data_ptr(), bg_zval.data_ptr(), B, ns,
                                             float(sample_range), tile_center.data_ptr(), float(tile_size),
                                             z_vals.data_ptr(), _stream()))


def sampling_background(rays_o, rays_d, bgdepth, tile_center, tile_size, nsamples, sample_range):
    """training/scripts/utils.py:815-820: z_vals pre-filled with -1."""
    import torch
    z = torch.full((rays_o.shape[0], nsamples), -1, dtype=torch.float32, device=rays_o.device)
    Sample_bg(rays_o, rays_d, bgdepth, tile_center, tile_size, sample_range, z)
    return z
