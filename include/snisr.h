/*
 * snisr.h — C ABI of the GB300-native sparse-voxel tile renderer.
 *
 * One hot path from Scalable Neural Indoor Scene Rendering, rebuilt for
 * sm_103a: per ray, a tile-grid DDA and a voxel DDA over per-tile occupancy
 * bitfields, samples only inside occupied voxels, trilinear per-corner
 * features into a per-tile MLP, front-to-back compositing with early stop.
 *
 * Conventions shared by every entry point
 *   - Plain C types only; no exceptions cross this boundary.  Every call
 *     returns an snisr_status; snisr_last_error_string() describes the last
 *     failure of the calling thread.
 *   - Pointers named *_dev are device pointers (cudaMalloc / torch), *_host
 *     are host pointers.  `stream` is a cudaStream_t passed as void*
 *     (NULL = legacy default stream).  Calls enqueue work and return without
 *     synchronising unless the comment says otherwise.
 *   - The caller owns output buffers.  A scene owns its device copy of the
 *     scene data and a workspace sized at creation: rendering allocates no
 *     device memory after snisr_scene_create().
 *   - Index conventions follow the reference: dense grids are x-major,
 *     idx = (x*NY + y)*NZ + z (rendering/src/include/cuda_utils.h:137-140).
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   FASTRENDERING pybind module   rendering/src/binding.cpp:13-27
 *   CUDA_EXT pybind module        training/src/binding.cpp:4-12
 *   render_TileScene (C++ host)   training/src/cuda_func.cu:2395-2480
 */
#ifndef SNISR_H_
#define SNISR_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SNISR_ABI_VERSION 1

typedef enum snisr_status {
  SNISR_OK = 0,
  SNISR_INVALID_ARG = 1,     /* bad pointer, size, shape or enum            */
  SNISR_OOM = 2,             /* device or host allocation failed            */
  SNISR_CUDA_ERROR = 3,      /* a CUDA runtime call or launch failed        */
  SNISR_DEVICE_TIMEOUT = 4,  /* a bounded device wait ran out               */
  SNISR_CORRUPT_SCENE = 5,   /* scene data inconsistent (counts, indices)   */
  SNISR_OVERFLOW = 6,        /* a workspace bound was exceeded on device    */
  SNISR_UNSUPPORTED = 7      /* shape/configuration not supported by a form */
} snisr_status;

typedef enum snisr_dtype { SNISR_F32 = 0, SNISR_F16 = 1 } snisr_dtype;

/* Render forms.  PLAIN_FP32: one thread per ray, FP32 features, weights and
 * math on CUDA cores.  TC: batched form — traversal emits compacted samples,
 * grouped by tile, and the per-tile MLP runs as tcgen05 FP16 MMAs with FP32
 * accumulation in tensor memory. */
typedef enum snisr_form {
  SNISR_FORM_PLAIN_FP32 = 0, /* CUDA cores, FP32                                        */
  SNISR_FORM_TC = 1          /* tensor cores: render FP16 operands; training split BF16 */
} snisr_form;

/* ------------------------------------------------------------------------ */
/* Scene description (host arrays, borrowed for the duration of create).     */
/* ------------------------------------------------------------------------ */
typedef struct snisr_scene_desc {
  int32_t grid[3];            /* tiles along x, y, z                          */
  float scene_min[3];         /* world position of the grid's min corner      */
  float tile_size;            /* edge of a cubic tile (world units)           */
  int32_t res;                /* voxels per tile edge N (multiple of 4)       */
  int32_t num_tiles;          /* NT: tiles with an id in tile_index           */
  const int32_t* tile_index;  /* [grid x*y*z] dense tile -> sparse id or -1   */
  const uint64_t* occupancy;  /* [NT][N^3/64] bit (v&63) of word v>>6,
                                 v = (x*N + y)*N + z                          */
  int64_t num_voxels;         /* occupied voxels = total popcount             */
  const int32_t* voxel_corners; /* [num_voxels][8] vertex ids, voxels in
                                 (tile, v) order; corner k = dx*4+dy*2+dz     */
  int64_t num_vertices;       /* NV                                            */
  int32_t feat_dim;           /* F: 16 or 32                                   */
  snisr_dtype feat_type;      /* storage type of vertex_feat / vertex_density */
  const void* vertex_feat;    /* [NV][F]                                       */
  const void* vertex_density; /* [NV] density logits (softplus applied after
                                 trilinear interpolation)                     */
  /* per-tile MLP: in = F + 3 + 6*dir_freqs -> hidden x n_hidden -> 3        */
  int32_t dir_freqs;          /* view-direction encoding frequencies (4)      */
  int32_t mlp_hidden;         /* width: 32 or 64                               */
  int32_t mlp_layers;         /* hidden layers: 2 or 3                          */
  const float* mlp_params;    /* [NT][P]; per Linear: W[out][in] then b[out]   */
  /* proxy mesh (optional: num_triangles == 0 -> rays start at the AABB entry) */
  int64_t num_mesh_vertices;
  const float* mesh_vertices; /* [num_mesh_vertices][3]                        */
  int64_t num_triangles;
  const int32_t* mesh_faces;  /* [num_triangles][3]                            */
  /* marching parameters */
  float step_vox;             /* sample spacing in voxel lengths (0.5)        */
  float early_stop;           /* stop when transmittance < early_stop (1e-3)  */
  float start_offset_vox;     /* ray start = proxy hit - offset*voxel (2.0)   */
  /* workspace bound for the TC form: samples per pixel, on average         */
  int32_t max_samples_per_ray;
  int32_t max_pixels;         /* largest frame the workspace serves           */
} snisr_scene_desc;

typedef struct snisr_scene snisr_scene;

typedef struct snisr_scene_info {
  int64_t num_voxels, num_vertices, num_triangles, bvh_nodes;
  int32_t num_tiles, res, feat_dim, mlp_in, mlp_hidden, mlp_layers;
  int32_t params_per_tile;    /* P */
  int64_t device_bytes;       /* device memory the scene holds              */
  int64_t sample_capacity;    /* TC-form workspace in samples               */
} snisr_scene_info;

/* Pinhole camera, reference convention (rendering/src/compute_rays.cu:7-17):
 * x = (px - cx)*inv_focal, y = (py - cy)*inv_focal, d = R*[x, y, 1],
 * then normalised.  c2w is row-major 3x4 [R | origin]. */
typedef struct snisr_camera {
  int32_t width, height;
  float cx, cy, inv_focal;
  float c2w[12];
} snisr_camera;

/* Number of parameters of one tile's MLP for the given shape. */
int64_t snisr_mlp_param_count(int32_t feat_dim, int32_t dir_freqs,
                              int32_t hidden, int32_t layers);

/* Builds device-resident scene state on `device`: occupancy words with rank
 * prefixes, per-voxel 8-corner feature blocks (FP32 and FP16), per-tile MLP
 * images, the proxy-mesh BVH and the TC-form workspace.  Synchronous.
 * Replaces the scene-tensor setup of FRender (rendering/src/__init__.py:98-136). */
snisr_status snisr_scene_create(const snisr_scene_desc* desc, int32_t device,
                                snisr_scene** out);
snisr_status snisr_scene_destroy(snisr_scene* scene);
snisr_status snisr_scene_get_info(const snisr_scene* scene, snisr_scene_info* info);
/* Reads (and clears) the device-side error word of the scene: overflow of the
 * sample workspace or a bounded wait that ran out.  Synchronises `stream`. */
snisr_status snisr_scene_check(snisr_scene* scene, void* stream);
/* Replaces the per-tile MLP parameters ([NT][P] FP32, device pointer). */
snisr_status snisr_scene_set_mlp(snisr_scene* scene, const float* params_dev, void* stream);

/* ------------------------------------------------------------------------ */
/* Render: camera + scene -> colour/depth/opacity.                           */
/* Generalises render_TileScene (training/src/cuda_func.cu:2395-2480) and the */
/* per-frame op chain of FRender.render (rendering/src/__init__.py:246-341).  */
/* ------------------------------------------------------------------------ */
/* rgb_dev [H*W*3], depth_dev [H*W], opacity_dev [H*W] FP32 device buffers.
 * depth = sum_i w_i t_i (ray distance), opacity = 1 - final transmittance.
 * The tensor-core form takes at most 2^24 rays per call (SNISR_INVALID_ARG
 * beyond: its sample records hold a 24-bit pixel index). */
snisr_status snisr_render(snisr_scene* scene, const snisr_camera* cam, int32_t form,
                          float* rgb_dev, float* depth_dev, float* opacity_dev,
                          void* stream);
/* Same, with host output buffers (pinned for best speed): device->host copies
 * are enqueued on `stream` and the call synchronises it before returning. */
snisr_status snisr_render_host(snisr_scene* scene, const snisr_camera* cam, int32_t form,
                               float* rgb_host, float* depth_host, float* opacity_host,
                               void* stream);
/* Pipelined form for frame sequences: renders on `stream` into one of two
 * device staging slots and enqueues the device->host copies on a stream of
 * the scene, then returns without waiting, so that the copies of frame i
 * overlap the rendering of frame i+1.  The host buffers of a call are
 * complete after the second following call on the scene returns or after
 * snisr_render_host_wait; they must not be touched before. */
snisr_status snisr_render_host_async(snisr_scene* scene, const snisr_camera* cam, int32_t form,
                                     float* rgb_host, float* depth_host, float* opacity_host,
                                     void* stream);
/* Waits until every copy enqueued by snisr_render_host_async has landed. */
snisr_status snisr_render_host_wait(snisr_scene* scene);

/* Plain FP32 render of at most 32768 rays that allocates no device memory
 * (no counterpart in the reference).  For callers that may not call
 * cudaMalloc while rendering: hosts that own all device memory through a pool
 * of their own, and real-time frame loops that must not block on the
 * allocator.  Ray staging uses a 2 MiB file-scope __device__ array that every
 * GPU loading the library holds until exit; the first call on a device looks
 * up its address, so make that call before any stream capture.  The address
 * is tied to the device's CUDA context: after a cudaDeviceReset the next call
 * looks it up again (make that call before any capture as well).  All calls
 * share the array: calls that overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.  Results equal
 * snisr_render_rays(..., SNISR_FORM_PLAIN_FP32, ...); n > 32768 is rejected
 * with SNISR_INVALID_ARG. */
snisr_status snisr_render_rays_noalloc(snisr_scene* scene, const float* origins_dev,
                                       const float* dirs_dev, int64_t n, float* rgb_dev,
                                       float* depth_dev, float* opacity_dev, void* stream);

/* ------------------------------------------------------------------------ */
/* Per-stage entry points (parity harnesses and drop-in ops).               */
/* ------------------------------------------------------------------------ */
/* Normalised pinhole ray directions for a camera: dirs_dev [H*W*3]. */
snisr_status snisr_camera_rays(const snisr_camera* cam, float* dirs_dev, void* stream);

/* Proxy-mesh nearest hit through the BVH, FP32 Moller-Trumbore with an FP64
 * re-test in the near-degenerate band.  Replaces ray_firstHit_inTile_kernel
 * (training/src/cuda_func.cu:130-282).  t_dev [n] (-1 on miss), tri_dev [n]. */
snisr_status snisr_proxy_hit(snisr_scene* scene, const float* origins_dev,
                             const float* dirs_dev, int64_t n, float* t_dev,
                             int32_t* tri_dev, void* stream);

/* Occupied-voxel sequence of each ray (global voxel ids, in visit order,
 * -1 padded to K), ignoring transmittance; the start point honours the proxy
 * mesh when the scene has one.  count_dev [n] = number visited (may exceed K). */
snisr_status snisr_trace_voxels(snisr_scene* scene, const float* origins_dev,
                                const float* dirs_dev, int64_t n, int32_t K,
                                int32_t* visited_dev, int32_t* count_dev, void* stream);

/* Render arbitrary rays (rgb [n*3], depth [n], opacity [n]). */
snisr_status snisr_render_rays(snisr_scene* scene, const float* origins_dev,
                               const float* dirs_dev, int64_t n, int32_t form,
                               float* rgb_dev, float* depth_dev, float* opacity_dev,
                               void* stream);

/* ------------------------------------------------------------------------ */
/* Training: forward / hand-written adjoint (per-ray recomputation).         */
/* Replaces the autograd graph sparse_sampling + compute_voxels + query_voxel */
/* + volume_rendering (training/scripts/tile/tile.py:667-704,                */
/* training/scripts/utils.py:823-837).  Parameters are passed explicitly so  */
/* that an optimiser outside the library owns them.                          */
/* ------------------------------------------------------------------------ */
/* Ray segments: ray i is marched inside sparse tile ray_tile_dev[i] only
 * (rays split at tile faces, as per-tile training uses them); rays must be
 * grouped by tile (non-decreasing ids).  vfeat_dev [NV][F] FP32 features,
 * vdens_dev [NV] FP32 density logits, mlp_dev [NT][P] FP32 MLP parameters.
 * Rays normalised.  rgb_dev [n*3] out.  form PLAIN_FP32: FP32 CUDA-core MLP;
 * TC: tcgen05 MMAs with FP32 accumulation -- forward products with split
 * BF16 operands (hi + lo, ~16 significant bits), backward products with
 * BF16 operands.  Sample records are kept in
 * a per-scene training workspace (grown on the first call of a larger batch,
 * n * max_samples_per_ray records) for the backward call.  *generation_out
 * (may be NULL) receives a non-zero id of this forward's records; the next
 * forward on the scene replaces them and takes a new id. */
snisr_status snisr_train_forward(snisr_scene* scene, const float* vfeat_dev,
                                 const float* vdens_dev, const float* mlp_dev,
                                 const float* origins_dev, const float* dirs_dev,
                                 const int32_t* ray_tile_dev, int64_t n, int32_t form,
                                 float* rgb_dev, uint64_t* generation_out, void* stream);
/* Hand-written adjoint of a snisr_train_forward call on the same scene and
 * rays: per-ray reverse compositing with suffix sums, per-sample
 * recomputation of features and MLP activations.  `generation` is the id
 * that forward returned; if another forward ran on the scene since, its
 * records are gone and the call returns SNISR_INVALID_ARG (instead of
 * back-propagating through the other forward's samples).  grad_rgb_dev
 * [n*3] = dL/drgb; rgb_dev (the forward output) may be NULL.  Gradients are
 * ACCUMULATED (+=) into gvfeat_dev [NV][F] (16-byte aligned), gvdens_dev [NV],
 * gmlp_dev [NT][P]. */
snisr_status snisr_train_backward(snisr_scene* scene, const float* vfeat_dev,
                                  const float* vdens_dev, const float* mlp_dev,
                                  const float* origins_dev, const float* dirs_dev,
                                  const int32_t* ray_tile_dev, int64_t n, int32_t form,
                                  uint64_t generation, const float* rgb_dev,
                                  const float* grad_rgb_dev,
                                  float* gvfeat_dev, float* gvdens_dev, float* gmlp_dev,
                                  void* stream);

/* ------------------------------------------------------------------------ */
/* Reference-op drop-ins (argument meaning as in the reference; device ptrs) */
/* ------------------------------------------------------------------------ */
/* FASTRENDERING.compute_rays (rendering/src/compute_rays.cu:46-68):
 * intrinsic = [cx, cy, 1/f], c2w_rotation row-major 3x3, both device arrays;
 * rays_d [H][W][3] unnormalised. */
snisr_status snisr_op_compute_rays(const float* intrinsic_dev, const float* c2w_rot_dev,
                                   int32_t H, int32_t W, float* rays_d_dev, void* stream);
/* FASTRENDERING.tracing_tiles (rendering/src/raytile_tracing.cu:63-95):
 * origin[3], tile_shape[3] (int), scene_min_corner[3], scene_size[3] device
 * arrays; visited_dev [npix][K], -1 padded. */
snisr_status snisr_op_tracing_tiles(const float* rays_d_dev, int64_t npix,
                                    const int32_t* index_map_dev, const float* origin_dev,
                                    const int32_t* tile_shape_dev,
                                    const float* scene_min_dev, const float* scene_size_dev,
                                    float tile_size, int32_t K, int32_t* visited_dev,
                                    void* stream);
/* CUDA_EXT.Sample_sparse (training/src/Sample_kernel.cu:397-434): node_flags
 * [N][N][N] int16 (x-major, 1 = occupied), z_vals/dists [B][Nsamples], caller
 * pre-fills -1 as utils.sparse_sampling does (training/scripts/utils.py:797-805). */
snisr_status snisr_op_sample_sparse(const float* rays_o_dev, const float* rays_d_dev,
                                    int64_t B, const int16_t* node_flags_dev,
                                    float cx, float cy, float cz, float tile_size,
                                    int32_t num_voxel, int32_t nsamples,
                                    float* z_vals_dev, float* dists_dev, void* stream);
/* FASTRENDERING.inverse_z_sampling (rendering/src/sampling.cu:48-81):
 * origin[3], inverse_near [npix], inverse_bound [npix] (all device);
 * sample j of the call sits at z = 1/((offset+j)*inverse_bound + inverse_near);
 * points [npix][spr][3], steps [npix][spr] = max(z_{j+1} - z_j, 0). */
snisr_status snisr_op_inverse_z_sampling(const float* rays_d_dev, const float* origin_dev,
                                         const float* inverse_near_dev,
                                         const float* inverse_bound_dev, int64_t npix,
                                         int32_t offset, int32_t spr, float* points_dev,
                                         float* steps_dev, void* stream);
/* FASTRENDERING.integrate_points (rendering/src/volume_rendering.cu:60-87):
 * rgba [npix][16][4] (colour, sigma), z_dists [npix][16], frame [npix][3] and
 * transparency [npix] carried across calls. */
snisr_status snisr_op_integrate_points(const float* rgba_dev, const float* z_dists_dev,
                                       int64_t npix, float early_stop, float* frame_dev,
                                       float* transparency_dev, void* stream);

/* Specular pass (the reference's reflection MLP and its batching).        */
/* FASTRENDERING.sort_by_key (rendering/src/reorder.cu:10-22): stable sort of
 * (keys int16, values int32) by key in place, then unique_by_key over
 * (keys, starts): keys[k] = k-th distinct key, starts[k] = starts[first
 * position of its run] (positions past the run count keep the sorted keys and
 * the old starts).  *num_unique = number of distinct keys (host).  Uses
 * stream-ordered temporaries and synchronises `stream`. */
snisr_status snisr_op_sort_by_key(int16_t* keys_dev, int32_t* values_dev, int32_t* starts_dev,
                                  int64_t n, int64_t* num_unique, void* stream);
/* FASTRENDERING.assign_pixels (rendering/src/reorder.cu:24-94): network k's
 * pixels [pixel_starts[k], pixel_starts[k+1]) over blocks [block_starts[k],
 * block_starts[k+1]); the first (count mod blocks) blocks take one pixel more. */
snisr_status snisr_op_assign_pixels(const int16_t* net_dev, const int32_t* pixel_starts_dev,
                                    const int32_t* block_starts_dev, int64_t num_net,
                                    int16_t* new_net_dev, int32_t* new_pixel_starts_dev, void* stream);
/* Parameters per network of the reflection MLP (22556 FP16 values). */
int32_t snisr_op_inference_mlp_param_count(void);
/* FASTRENDERING.inference_mlp (rendering/src/rayreflection_render.cu:111-301):
 * block b evaluates network net[b] (int16, -1 = none; ids >= num_groups are
 * skipped) on the samples of pixels [pixel_starts[b], pixel_starts[b+1]) of
 * the sorted pixel list (query_pixel_indices maps them to frame pixels);
 * pixels with transparency < trans_stop are skipped and their results left
 * untouched.  MLP 63 -> 64 x 5 (LeakyReLU 0.01) -> 28 on the position
 * encoding of (sample - group centre) * inverse_far; colour = sigmoid(SH
 * degree 2 of the normalised ray direction), density = max(out[27], 0).
 * params: [num_groups][22556] FP16 bit patterns in the reference layout
 * (per layer bias[out] then W[in][out]); samples [npix][spr][3],
 * rays_d [npix][3], sample_results [npix][spr][4].  Runs on tcgen05 with
 * FP16 operands and FP32 accumulation (the reference accumulates in FP16).
 * err_dev (optional): the value 2 is OR-ed in if a bounded device wait ran out. */
snisr_status snisr_op_inference_mlp(int32_t samples_per_ray, int32_t num_block, float inverse_far,
                                    float trans_stop, const int16_t* net_dev, int32_t num_groups,
                                    const float* transparency_dev, const int32_t* query_pixel_indices_dev,
                                    const int32_t* pixel_starts_dev, const float* group_centers_dev,
                                    const float* samples_dev, const float* rays_d_dev,
                                    const uint16_t* params_dev, float* sample_results_dev,
                                    uint32_t* err_dev, void* stream);

/* FASTRENDERING.rendering_diffuse_octree_fp16
 * (rendering/src/raydiffuse_render_octree_fp16.cu:141-287) on the reference's
 * scene format: rays_d [npix][3], visited [npix][K] sparse tile ids (-1
 * padded, from snisr_op_tracing_tiles), origin [3] (device), group_map
 * [NT] (tile2group), data_voxels [Nv][4] FP16 bit patterns, block_map
 * [NT][64], node_map [Nn][D^3] int16, sample_flags [Nn][D^3] bytes (bool),
 * voxels_start [Nn] int64, centers [NT][3]; D = num_voxel / 4 + 2 (18).
 * Writes frame [npix][3]; inverse_near [npix] and net_idx [npix] only at
 * pixels with a first hit (transmittance below trans_th), as the reference;
 * with soft_hit != 0 a pixel without a first hit whose last examined tile has
 * a group takes that group and 1 / (the tile's exit distance).
 * FP16 trilinear and compositing with the CUDA half intrinsics; tile ids
 * outside [0, num_tiles) are skipped.  image_width > 0: the pixels are a
 * row-major image that wide, marched in 4 x 8-pixel warp tiles where it
 * divides into them (outputs identical); 0: pixel order. */
snisr_status snisr_op_rendering_diffuse_octree(
    const float* rays_d_dev, const int32_t* visited_dev, int64_t npix, int32_t K,
    const float* origin_dev, const int32_t* group_map_dev, const uint16_t* data_voxels_dev,
    const int32_t* block_map_dev, const int16_t* node_map_dev, const uint8_t* sample_flags_dev,
    const int64_t* voxels_start_dev, const float* centers_dev, int32_t num_tiles, float tile_size,
    float voxel_size, float sample_step, int32_t dilated_voxels, float trans_th, float early_stop,
    int32_t soft_hit, float* frame_dev, float* inverse_near_dev, int16_t* net_idx_dev, int32_t image_width,
    void* stream);

/* ------------------------------------------------------------------------ */
/* Training-ray preparation of one tile from posed views (get_trainData_v3,  */
/* training/src/cuda_func.cu:1341-1686).  All buffers are device memory.     */

/* computing_rays_kernel (cuda_func.cu:15-50, get_rays in
 * training/src/include/cuda_utils.h:143-155): K [9] row-major intrinsics,
 * c2w [12] row-major 3x4; pixel (x, y) -> rays_d = R ((x - K[2]) / K[0],
 * (y - K[5]) / K[4], 1) (not normalised), rays_o = t; [height*width][3]. */
snisr_status snisr_op_train_rays(const float* K_dev, const float* c2w_dev, int32_t height, int32_t width,
                                 float* rays_o_dev, float* rays_d_dev, void* stream);

/* tracingTile_kernel (cuda_func.cu:52-128): visited [n][K] sparse tile ids
 * (-1 padded) of the tile DDA of the normalised direction from the origin,
 * or from its entry into the scene box, clamped into the scene.  The
 * normalisation uses a correctly rounded 1/sqrt (the reference: rsqrtf). */
snisr_status snisr_op_train_tracing_tiles(const float* rays_o_dev, const float* rays_d_dev, int64_t n,
                                          const int32_t* index_map_dev, const int32_t tile_shape[3],
                                          const float scene_min_corner[3], float tile_size, int32_t K,
                                          int32_t* visited_dev, void* stream);

/* ray_doubleHit_inTile_kernel (cuda_func.cu:284-444) on the scene's proxy
 * BVH: double_hits [n][K][2] = the two nearest hits (t along rays_d, with
 * multiplicity) whose points lie in visited tile j (+-1e-5), -1 where
 * missing.  The reference walks per-block face lists; here the BVH is
 * clipped to the tile box (each triangle is counted once). */
snisr_status snisr_scene_double_hits(snisr_scene* scene, const float* rays_o_dev, const float* rays_d_dev,
                                     const int32_t* visited_dev, int64_t n, int32_t K, float* double_hits_dev,
                                     void* stream);

/* get_trainData_kernel (cuda_func.cu:587-663): valid [n] = 1 where the
 * training tile is visited at or before the first tile with a hit;
 * bgdepth [n] = the next hit then (-1 if none; -1 where not valid, where the
 * reference leaves the previous view's value). */
snisr_status snisr_op_train_bgdepth(int32_t train_tile, const int32_t* visited_dev, const float* double_hits_dev,
                                    int64_t n, int32_t K, float* bgdepth_dev, int32_t* valid_dev, void* stream);

/* gen_diffuse_in_tile_kernel (cuda_func.cu:1197-1339): for pixels with a
 * hit in the training tile, diffuse [H*W][3] = the (1 - cos)^2-weighted mean
 * of the bilinear colours of the hit point in the views that see it (depth
 * test 0.01); bgdepth set to -1 where no view sees the background point.
 * origins [num_images][3], images [num_images][H*W][3] float, depths
 * [num_images][H*W], proj [num_images][12] (compute_project_matrix). */
snisr_status snisr_op_gen_diffuse(const float* origins_dev, int32_t train_tile, const float* rays_o_dev,
                                  const float* rays_d_dev, const float* double_hits_dev, const int32_t* visited_dev,
                                  const float* images_dev, const float* depths_dev, const float* proj_dev, int32_t K,
                                  int32_t num_images, int32_t height, int32_t width, float* diffuse_dev,
                                  float* bgdepth_dev, void* stream);

/* CUDA_EXT.Sample_bg (training/src/Sample_kernel.cu:481-542): z_vals
 * [n][nsamples] uniform over bg +- range / 2, moved behind the tile's exit
 * when that interval starts inside the tile; rows with bg == -1 untouched. */
snisr_status snisr_op_sample_bg(const float* rays_o_dev, const float* rays_d_dev, const float* bg_zval_dev,
                                int64_t n, int32_t nsamples, float sample_range, const float* tile_center_dev,
                                float tile_size, float* z_vals_dev, void* stream);

/* Patch rows of get_trainData_v3 (cuda_func.cu:1545-1600): odd patch_size P,
 * patch centres (half + iP, half + jP) below (H - P, W - P); patches with a
 * valid pixel are written in order as P*P rows of 14 floats (rays_o, rays_d,
 * bgdepth, gt_rgb, diffuse, valid).  snisr_op_patch_capacity gives the
 * number of patch positions C (or -1): rows holds C*P*P*14 floats, scratch
 * 2*C int32; *num_patches_dev (int64) receives the count written. */
int64_t snisr_op_patch_capacity(int32_t height, int32_t width, int32_t patch_size);
snisr_status snisr_op_patch_rows(const int32_t* valid_dev, int32_t height, int32_t width, int32_t patch_size,
                                 const float* rays_o_dev, const float* rays_d_dev, const float* bgdepth_dev,
                                 const float* gt_rgb_dev, const float* diffuse_dev, int32_t* scratch_dev,
                                 float* rows_dev, int64_t* num_patches_dev, void* stream);

/* ------------------------------------------------------------------------ */
/* Pruning after a training epoch, on the reference's dilated per-tile grids  */
/* (D = N + 2 cells per side, [x][y][z] order, one cell of border).          */

/* CUDA_EXT.transparency_statistic (training/src/Helper_kernel.cu:108-172,
 * 272-303): rays_start/rays_dir [n][3]; tile_center [3] (device); voxels
 * [D^3] density per unit length; nodes [D^3] int16 flags (samples only where
 * 1); T_voxels [D^3] is max-combined in place with transmittance x trilinear
 * weight at the 8 corners of every sample.  num_voxel is D (<= 1024).  Flagged cells
 * on the grid border (where the reference asserts) contribute nothing. */
snisr_status snisr_op_transparency_statistic(const float* rays_start_dev, const float* rays_dir_dev, int64_t n,
                                             int32_t num_voxel, const float* tile_center_dev, float tile_size,
                                             float voxel_size, float sample_step, const float* voxels_dev,
                                             const int16_t* nodes_dev, float* T_voxels_dev, void* stream);

/* CUDA_EXT.dilate_boundary (training/src/Helper_kernel.cu:174-270): in
 * place on nodes_flag [D^3] int16 (num_voxel = D): -1 cells with a 1 cell in
 * their 3^3 neighbourhood become 0.  Allocates nothing. */
snisr_status snisr_op_dilate_boundary(int16_t* nodes_flag_dev, int32_t num_voxel, void* stream);

/* The flag update of Tile.pruning (training/scripts/tile/tile.py:337-372)
 * after the model query: nodes_flag [D^3] (D = num_voxel + 2) gets -1 on the
 * border; inside, init_flags [N^3] (NULL = all 1) with -1 where
 * exp(-max of voxel_sigma [N^3] over the voxel's block^3 block) > th or where
 * the 3^3 maximum of T_voxels [D^3] <= T_th; then dilate_boundary.
 * num_voxel must be a multiple of block. */
snisr_status snisr_op_prune_flags(const float* T_voxels_dev, const float* voxel_sigma_dev,
                                  const int16_t* init_flags_dev, int32_t num_voxel, int32_t block, float th,
                                  float T_th, int16_t* nodes_flag_dev, void* stream);

/* The 1 cells of nodes_flag's inner N^3 (N = num_voxel) as this library's
 * occupancy words (snisr_scene_desc.occupancy layout: voxel v = (x*N + y)*N
 * + z is bit v % 64 of word v / 64); words [ceil(N^3 / 64)], *count_dev =
 * number of set bits (device int64). */
snisr_status snisr_op_pack_occupancy(const int16_t* nodes_flag_dev, int32_t num_voxel, uint64_t* words_dev,
                                     int64_t* count_dev, void* stream);

/* ------------------------------------------------------------------------ */
/* Seeded synthetic scenes (input generation for tests and benchmarks).      */
/* ------------------------------------------------------------------------ */
typedef struct snisr_synth_params {
  int32_t kind;        /* 0 small room (1 tile), 1 room, 2 multi-room        */
  int32_t grid[3];
  float tile_size;
  int32_t res;
  int32_t feat_dim;
  snisr_dtype feat_type;
  int32_t mlp_hidden, mlp_layers, dir_freqs;
  int32_t num_boxes;
  float box_min, box_max;   /* box side range (world units)                */
  int32_t with_mesh;        /* build the proxy mesh                         */
  float mesh_cell;          /* target triangle-grid cell (world units)      */
  float density_mean, density_std, feat_std;
  uint64_t seed;            /* scene seed; tile weights use seed ^ tile     */
  int32_t round_weights_f16;/* store MLP weights rounded to FP16 values     */
} snisr_synth_params;

typedef struct snisr_synth_scene snisr_synth_scene;
/* Generates a scene; `desc` is filled with pointers owned by *out. */
snisr_status snisr_synth_create(const snisr_synth_params* p, snisr_synth_scene** out,
                                snisr_scene_desc* desc);
snisr_status snisr_synth_destroy(snisr_synth_scene* s);
/* Seeded interior camera pose (origin inside free space, random heading). */
snisr_status snisr_synth_camera(const snisr_synth_scene* s, uint64_t pose_seed,
                                int32_t width, int32_t height, float fov_x_deg,
                                snisr_camera* cam);

/* ------------------------------------------------------------------------ */
/* Launch shapes and their autotuner (no counterpart in the reference).      */
/* ------------------------------------------------------------------------ */
typedef struct snisr_tuning {
  int32_t traverse_threads;      /* TC render traversal block size: 32..256, multiple of 32 */
  int32_t scatter_blocks_per_sm; /* per-tile bucketing grid: 1..64 blocks per SM           */
  int32_t mlp_ctas_per_sm;       /* persistent MLP CTAs per SM: 0 = resident maximum, 1..8 */
  int32_t train_march_threads;   /* training march block size: 32..256, multiple of 32     */
  int32_t train_fwd_warps;       /* training TC forward warps per CTA: 4 or 8 (1 CTA / SM)  */
} snisr_tuning;
snisr_status snisr_scene_get_tuning(const snisr_scene* scene, snisr_tuning* out);
snisr_status snisr_scene_set_tuning(snisr_scene* scene, const snisr_tuning* tuning);
/* Times launch shapes of the TC render of `cam` (coordinate descent over the
 * knobs; each candidate: one warm-up frame, then `reps` frames timed with
 * CUDA events on `stream`), keeps the fastest in the scene and returns it
 * with its ms per frame.  Allocates temporary output buffers; synchronises. */
snisr_status snisr_scene_autotune_render(snisr_scene* scene, const snisr_camera* cam, int32_t reps,
                                         void* stream, snisr_tuning* out, float* best_ms);
/* Same for the TC training step (forward + backward with dL/drgb = 1) on the
 * given batch; gradient buffers are temporary.  Results do not depend on the
 * launch shapes beyond the summation order of atomics. */
snisr_status snisr_scene_autotune_train(snisr_scene* scene, const float* vfeat_dev,
                                        const float* vdens_dev, const float* mlp_dev,
                                        const float* origins_dev, const float* dirs_dev,
                                        const int32_t* ray_tile_dev, int64_t n, int32_t reps,
                                        void* stream, snisr_tuning* out, float* best_ms);

/* Stage timing: when enabled, render calls record CUDA events between
 * stages.  stage_times synchronises on the last frame and returns, in ms:
 * TC form [ray setup + proxy, traverse, scan, scatter, MLP, total];
 * plain form [ray setup + proxy, render, total]. */
snisr_status snisr_scene_set_profiling(snisr_scene* scene, int32_t enable);
snisr_status snisr_scene_stage_times(snisr_scene* scene, float* ms, int32_t cap, int32_t* n);
/* Counters of the last TC-form frame (synchronises `stream`): out[0] samples,
 * out[1] voxel DDA steps, out[2] sample slots reserved, out[3] MLP chunks. */
snisr_status snisr_scene_frame_stats(snisr_scene* scene, int64_t* out, void* stream);
/* Footprint of the last TC-form frame (profiling aid; synchronises `stream`):
 * out[0] distinct voxels whose samples the MLP stage read, out[1] distinct
 * vertices behind them (their trilinear corners). */
snisr_status snisr_scene_frame_footprint(snisr_scene* scene, int64_t* out, void* stream);

/* Diagnostics of the tcgen05 operand layouts.  mode 0: one 128 x N x 64 MMA
 * (N = 32 or 64) through the descriptors of the tensor-core MLP: A [128][64],
 * B [N][64] row-major FP16 (bf16 = 0) or BF16 (bf16 = 1) bit patterns,
 * D [128][N] FP32 = A * B^T.  mode 1/2 (N = 64): At [128][64], Bt [128][64]
 * stored sample-major and consumed as MN-major operands, D [128][64] with
 * D[m][n] = sum_k At[k][m] Bt[k][n] for m < 64 (two stride conventions).
 * mode 3: as mode 0 with A read from tensor memory (each row stored into
 * its lane by tcgen05.st).  Synchronises `stream`. */
snisr_status snisr_diag_mma(const uint16_t* A_dev, const uint16_t* B_dev, float* D_dev,
                            int32_t N, int32_t bf16, int32_t mode, void* stream);

/* The bounded-wait error path of the tensor-core kernels: one wait on an
 * mbarrier that nothing completes, given up after limit_ns (0 < limit_ns <=
 * 10 s) of the GPU's global timer.  Returns SNISR_DEVICE_TIMEOUT when the wait
 * ran out (the expected result), *waited_ns = the device time it waited.
 * Every kernel wait of this library has the same bound (2 s).  Synchronises
 * `stream`. */
snisr_status snisr_diag_wait_timeout(int64_t limit_ns, int64_t* waited_ns, void* stream);

/* The render march's own single-precision functions, elementwise on device
 * arrays (no counterpart in the reference; a check of the transmittance
 * arithmetic): fn 0 e^x for x <= 0, fn 1 log(1 + y) for y in [0, 1], fn 2
 * softplus.  The host restatement gives the same bits. */
snisr_status snisr_diag_march_math(int32_t fn, const float* x_dev, int64_t n, float* out_dev,
                                   void* stream);

/* The scene's per-tile 4^3-block distances, on the host (no GPU): mask
 * [(nb^3 + 31) / 32] bits of block occupancy (block (x, y, z) at bit
 * (x nb + y) nb + z), out [nb^3] = the Chebyshev distance, in blocks, to the
 * nearest occupied block (0 for an occupied one), at most 16.  The march
 * crosses the box of blocks within distance - 1 without occupancy loads. */
snisr_status snisr_diag_block_distance(const uint32_t* mask_host, int32_t nb, uint8_t* out_host);

const char* snisr_last_error_string(void);
const char* snisr_version(void);
int32_t snisr_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SNISR_H_ */
