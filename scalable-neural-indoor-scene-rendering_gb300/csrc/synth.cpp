// Seeded synthetic indoor scenes: tiles of sparse voxels around the surface
// of a room signed-distance field, per-vertex features, per-tile MLPs and the
// proxy triangle mesh of the same surface.
//
// Everything here is deterministic across x86-64 and AArch64: random numbers
// come from a counter hash (splitmix64 finaliser), normals are Irwin-Hall sums
// of twelve uniforms, and geometry uses only + - * / sqrt in double precision.
// Scenes therefore reproduce bit-for-bit on any host, which lets golden
// fixtures generated on one machine be checked on another.
//
// The reference builds its scenes from captured data (training/src/
// preparedata.cpp) that is not part of the reference tree; these scenes stand
// in for them with the shapes used by the benchmarks.
#include "snisr_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace snisr {

namespace {

inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline uint64_t hash3(uint64_t a, uint64_t b, uint64_t c) {
  return mix64(mix64(mix64(a) ^ b) ^ c);
}
inline double uniform01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }
// Irwin-Hall(12) - 6: mean 0, variance 1, support [-6, 6].
inline double normal_ih(uint64_t a, uint64_t b, uint64_t c) {
  double s = 0.0;
  uint64_t base = hash3(a, b, c);
  for (int i = 0; i < 12; ++i) s += uniform01(mix64(base + 0x632BE59BD9B4E019ull * (uint64_t)(i + 1)));
  return s - 6.0;
}

struct Rng {  // sequential stream for scene layout choices
  uint64_t state;
  explicit Rng(uint64_t s) : state(mix64(s ^ 0xA0761D6478BD642Full)) {}
  double uni() { state = mix64(state); return uniform01(state); }
  double uni(double lo, double hi) { return lo + (hi - lo) * uni(); }
};

struct Box { double lo[3], hi[3]; };
// Axis-aligned wall plane at coord[axis] = pos spanning [lo,hi] on the other
// two axes, with optional rectangular gaps (door openings).
struct Wall {
  int axis; double pos; double lo[3], hi[3];
  std::vector<Box> gaps;  // gap extents on the two in-plane axes
};

struct Surfaces {
  std::vector<Wall> walls;
  std::vector<Box> boxes;
};

// Unsigned distance to the surface of an axis-aligned box.
double box_surface_dist(const Box& b, const double p[3]) {
  double q[3], outside = 0.0, inside = -1e300;
  for (int i = 0; i < 3; ++i) {
    double c = 0.5 * (b.lo[i] + b.hi[i]), h = 0.5 * (b.hi[i] - b.lo[i]);
    q[i] = std::fabs(p[i] - c) - h;
    double m = q[i] > 0 ? q[i] : 0.0;
    outside += m * m;
    inside = std::max(inside, q[i]);
  }
  if (outside > 0) return std::sqrt(outside);
  return -inside;  // inside the box: distance to the nearest face
}

// Distance from a 2-D point to the complement of an axis-aligned rectangle
// (0 when outside it).
double dist_to_rect_outside(double u, double v, double u0, double u1, double v0, double v1) {
  if (u <= u0 || u >= u1 || v <= v0 || v >= v1) return 0.0;
  return std::min(std::min(u - u0, u1 - u), std::min(v - v0, v1 - v));
}

// Unsigned distance to a finite wall rectangle with gaps.
double wall_dist(const Wall& w, const double p[3]) {
  int a = w.axis, b = (a + 1) % 3, c = (a + 2) % 3;
  double d = p[a] - w.pos;
  // in-plane distance to the wall's rectangle
  double eb = std::max(std::max(w.lo[b] - p[b], p[b] - w.hi[b]), 0.0);
  double ec = std::max(std::max(w.lo[c] - p[c], p[c] - w.hi[c]), 0.0);
  double in_plane2 = eb * eb + ec * ec;
  if (in_plane2 == 0.0) {
    double g = 0.0;
    for (const Box& gap : w.gaps) g = std::max(g, dist_to_rect_outside(p[b], p[c], gap.lo[b], gap.hi[b], gap.lo[c], gap.hi[c]));
    in_plane2 = g * g;
  }
  return std::sqrt(d * d + in_plane2);
}

double surface_dist(const Surfaces& s, const double p[3]) {
  double best = 1e300;
  for (const Wall& w : s.walls) best = std::min(best, wall_dist(w, p));
  for (const Box& b : s.boxes) best = std::min(best, box_surface_dist(b, p));
  return best;
}

// Signed-ish free-space test used for camera placement: outside every box and
// at least `margin` from every surface.
bool in_free_space(const Surfaces& s, const double p[3], double margin) {
  for (const Box& b : s.boxes) {
    bool inside = true;
    for (int i = 0; i < 3; ++i) inside = inside && p[i] > b.lo[i] && p[i] < b.hi[i];
    if (inside) return false;
  }
  return surface_dist(s, p) > margin;
}

void build_surfaces(const snisr_synth_params& P, const double ext[3], Surfaces& S, Rng& rng) {
  auto add_wall = [&](int axis, double pos) {
    Wall w; w.axis = axis; w.pos = pos;
    for (int i = 0; i < 3; ++i) { w.lo[i] = 0.0; w.hi[i] = ext[i]; }
    S.walls.push_back(w);
  };
  if (P.kind == 0) {
    // one tile: floor and two walls on the tile's min faces
    add_wall(2, 0.0); add_wall(0, 0.0); add_wall(1, 0.0);
  } else {
    add_wall(2, 0.0); add_wall(2, ext[2]);
    add_wall(0, 0.0); add_wall(0, ext[0]);
    add_wall(1, 0.0); add_wall(1, ext[1]);
    if (P.kind == 2) {
      // interior walls every two tiles with one door gap per room span
      double room = 2.0 * P.tile_size;
      for (int axis = 0; axis < 2; ++axis) {
        int other = 1 - axis;
        for (double pos = room; pos < ext[axis] - 1e-9; pos += room) {
          Wall w; w.axis = axis; w.pos = pos;
          for (int i = 0; i < 3; ++i) { w.lo[i] = 0.0; w.hi[i] = ext[i]; }
          for (double seg = 0.0; seg < ext[other] - 1e-9; seg += room) {
            Box g;
            double width = 1.0, height = 2.2;
            double u0 = seg + rng.uni(0.3, room - width - 0.3);
            for (int i = 0; i < 3; ++i) { g.lo[i] = 0.0; g.hi[i] = 0.0; }
            g.lo[other] = u0; g.hi[other] = u0 + width;
            g.lo[2] = 0.0; g.hi[2] = height;
            w.gaps.push_back(g);
          }
          S.walls.push_back(w);
        }
      }
    }
  }
  for (int i = 0; i < P.num_boxes; ++i) {
    Box b;
    for (int a = 0; a < 3; ++a) {
      double side = rng.uni(P.box_min, P.box_max);
      double lo_lim = 0.05, hi_lim = ext[a] - 0.05 - side;
      double lo = rng.uni(lo_lim, std::max(lo_lim, hi_lim));
      if (a == 2 && rng.uni() < 0.6) lo = 0.0;  // most boxes rest on the floor
      b.lo[a] = lo; b.hi[a] = lo + side;
    }
    S.boxes.push_back(b);
  }
}

uint16_t f32_to_f16_bits(float f) {
  uint32_t x; std::memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  int32_t exp = (int32_t)((x >> 23) & 0xFF) - 127 + 15;
  uint32_t mant = x & 0x7FFFFFu;
  if (((x >> 23) & 0xFF) == 0xFF) return (uint16_t)(sign | 0x7C00u | (mant ? 0x200u : 0u));
  if (exp >= 31) return (uint16_t)(sign | 0x7C00u);
  if (exp <= 0) {
    if (exp < -10) return (uint16_t)sign;
    mant |= 0x800000u;
    int shift = 14 - exp;
    uint32_t half = mant >> shift;
    uint32_t rem = mant & ((1u << shift) - 1u), mid = 1u << (shift - 1);
    if (rem > mid || (rem == mid && (half & 1u))) ++half;
    return (uint16_t)(sign | half);
  }
  uint32_t half = sign | ((uint32_t)exp << 10) | (mant >> 13);
  uint32_t rem = mant & 0x1FFFu;
  if (rem > 0x1000u || (rem == 0x1000u && (half & 1u))) ++half;
  return (uint16_t)half;
}

}  // namespace

float f16_bits_to_f32(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t exp = (h >> 10) & 0x1F, mant = h & 0x3FFu, x;
  if (exp == 0) {
    if (mant == 0) x = sign;
    else {
      int e = -1;
      do { mant <<= 1; ++e; } while (!(mant & 0x400u));
      x = sign | ((uint32_t)(127 - 15 - e) << 23) | ((mant & 0x3FFu) << 13);
    }
  } else if (exp == 31) x = sign | 0x7F800000u | (mant << 13);
  else x = sign | ((exp - 15 + 127) << 23) | (mant << 13);
  float f; std::memcpy(&f, &x, 4); return f;
}
uint16_t f32_to_f16(float f) { return f32_to_f16_bits(f); }

}  // namespace snisr

using namespace snisr;

struct snisr_synth_scene {
  snisr_synth_params params;
  Surfaces surf;
  double ext[3];
  std::vector<int32_t> tile_index;
  std::vector<uint64_t> occupancy;
  std::vector<int32_t> voxel_corners;
  std::vector<float> vfeat32, vdens32;
  std::vector<uint16_t> vfeat16, vdens16;
  std::vector<float> mlp;
  std::vector<float> mesh_v;
  std::vector<int32_t> mesh_f;
};

namespace {

void add_rect_mesh(snisr_synth_scene* s, int axis, double pos, double u0, double u1, double v0, double v1,
                   double cell, const std::vector<Box>* gaps) {
  int b = (axis + 1) % 3, c = (axis + 2) % 3;
  int nu = std::max(1, (int)std::ceil((u1 - u0) / cell - 1e-9));
  int nv = std::max(1, (int)std::ceil((v1 - v0) / cell - 1e-9));
  int32_t base = (int32_t)(s->mesh_v.size() / 3);
  for (int j = 0; j <= nv; ++j)
    for (int i = 0; i <= nu; ++i) {
      double p[3];
      p[axis] = pos;
      p[b] = u0 + (u1 - u0) * i / nu;
      p[c] = v0 + (v1 - v0) * j / nv;
      for (int k = 0; k < 3; ++k) s->mesh_v.push_back((float)p[k]);
    }
  for (int j = 0; j < nv; ++j)
    for (int i = 0; i < nu; ++i) {
      if (gaps) {
        double cu = u0 + (u1 - u0) * (i + 0.5) / nu, cv = v0 + (v1 - v0) * (j + 0.5) / nv;
        bool skip = false;
        for (const Box& g : *gaps) skip = skip || (cu > g.lo[b] && cu < g.hi[b] && cv > g.lo[c] && cv < g.hi[c]);
        if (skip) continue;
      }
      int32_t a0 = base + j * (nu + 1) + i, a1 = a0 + 1, a2 = a0 + (nu + 1), a3 = a2 + 1;
      int32_t t[6] = {a0, a1, a3, a0, a3, a2};
      for (int k = 0; k < 6; ++k) s->mesh_f.push_back(t[k]);
    }
}

}  // namespace

extern "C" snisr_status snisr_synth_create(const snisr_synth_params* P, snisr_synth_scene** out,
                                           snisr_scene_desc* desc) {
  if (!P || !out || !desc) return set_error(SNISR_INVALID_ARG, "synth_create: null argument");
  if (P->res <= 0 || P->res % 4 != 0 || P->res > 1024) return set_error(SNISR_INVALID_ARG, "synth_create: res must be a positive multiple of 4 (<=1024)");
  if (P->feat_dim != 16 && P->feat_dim != 32) return set_error(SNISR_INVALID_ARG, "synth_create: feat_dim must be 16 or 32");
  if (P->grid[0] <= 0 || P->grid[1] <= 0 || P->grid[2] <= 0) return set_error(SNISR_INVALID_ARG, "synth_create: bad grid");
  if (!(P->tile_size > 0)) return set_error(SNISR_INVALID_ARG, "synth_create: bad tile size");
  snisr_synth_scene* s = new (std::nothrow) snisr_synth_scene();
  if (!s) return set_error(SNISR_OOM, "synth_create: host allocation failed");
  try {
    s->params = *P;
    const int N = P->res, F = P->feat_dim;
    const int GX = P->grid[0], GY = P->grid[1], GZ = P->grid[2];
    const double S = P->tile_size, v = S / N;
    s->ext[0] = S * GX; s->ext[1] = S * GY; s->ext[2] = S * GZ;
    Rng rng(P->seed);
    build_surfaces(*P, s->ext, s->surf, rng);

    // occupancy on the full scene voxel grid, stored per tile
    const int64_t words_per_tile = (int64_t)N * N * N / 64;
    const int64_t ntile_dense = (int64_t)GX * GY * GZ;
    std::vector<uint64_t> dense_occ((size_t)(ntile_dense * words_per_tile), 0ull);
    const int WX = GX * N, WY = GY * N, WZ = GZ * N;
    auto mark_region = [&](const double lo[3], const double hi[3], auto dist_fn) {
      int i0[3], i1[3];
      const int W[3] = {WX, WY, WZ};
      for (int a = 0; a < 3; ++a) {
        i0[a] = std::max(0, (int)std::floor((lo[a] - v) / v) - 1);
        i1[a] = std::min(W[a] - 1, (int)std::floor((hi[a] + v) / v) + 1);
      }
      for (int x = i0[0]; x <= i1[0]; ++x)
        for (int y = i0[1]; y <= i1[1]; ++y)
          for (int z = i0[2]; z <= i1[2]; ++z) {
            double p[3] = {(x + 0.5) * v, (y + 0.5) * v, (z + 0.5) * v};
            if (dist_fn(p) <= v) {
              int tx = x / N, ty = y / N, tz = z / N;
              int lx = x - tx * N, ly = y - ty * N, lz = z - tz * N;
              int64_t t = ((int64_t)tx * GY + ty) * GZ + tz;
              int64_t vid = ((int64_t)lx * N + ly) * N + lz;
              dense_occ[(size_t)(t * words_per_tile + (vid >> 6))] |= 1ull << (vid & 63);
            }
          }
    };
    for (const Wall& w : s->surf.walls) {
      double lo[3], hi[3];
      for (int a = 0; a < 3; ++a) { lo[a] = w.lo[a]; hi[a] = w.hi[a]; }
      lo[w.axis] = hi[w.axis] = w.pos;
      mark_region(lo, hi, [&](const double* p) { return wall_dist(w, p); });
    }
    for (const Box& b : s->surf.boxes)
      mark_region(b.lo, b.hi, [&](const double* p) { return box_surface_dist(b, p); });

    // sparse tile ids for tiles holding at least one occupied voxel
    s->tile_index.assign((size_t)ntile_dense, -1);
    int32_t nt = 0;
    for (int64_t t = 0; t < ntile_dense; ++t) {
      bool any = false;
      for (int64_t w = 0; w < words_per_tile && !any; ++w) any = dense_occ[(size_t)(t * words_per_tile + w)] != 0;
      if (any) s->tile_index[(size_t)t] = nt++;
    }
    s->occupancy.assign((size_t)(nt * words_per_tile), 0ull);
    std::vector<int64_t> tile_dense_of(nt);
    for (int64_t t = 0; t < ntile_dense; ++t)
      if (s->tile_index[(size_t)t] >= 0) {
        int32_t id = s->tile_index[(size_t)t];
        tile_dense_of[id] = t;
        std::memcpy(&s->occupancy[(size_t)(id * words_per_tile)], &dense_occ[(size_t)(t * words_per_tile)], (size_t)words_per_tile * 8);
      }
    dense_occ.clear(); dense_occ.shrink_to_fit();

    // vertices: shared within a tile, numbered by first touch in voxel order
    const int64_t NV1 = (int64_t)(N + 1);
    std::vector<int32_t> vmap((size_t)(NV1 * NV1 * NV1));
    int64_t nverts = 0;
    std::vector<int64_t> vert_key;  // (dense tile, vertex linear index) for feature hashing
    std::vector<int32_t> vert_tile;
    for (int32_t id = 0; id < nt; ++id) {
      std::fill(vmap.begin(), vmap.end(), -1);
      const uint64_t* occ = &s->occupancy[(size_t)(id * words_per_tile)];
      for (int64_t w = 0; w < words_per_tile; ++w) {
        uint64_t bits = occ[w];
        while (bits) {
          int bit = __builtin_ctzll(bits);
          bits &= bits - 1;
          int64_t vid = w * 64 + bit;
          int x = (int)(vid / ((int64_t)N * N)), y = (int)((vid / N) % N), z = (int)(vid % N);
          for (int k = 0; k < 8; ++k) {
            int dx = (k >> 2) & 1, dy = (k >> 1) & 1, dz = k & 1;
            int64_t lin = ((int64_t)(x + dx) * NV1 + (y + dy)) * NV1 + (z + dz);
            int32_t& slot = vmap[(size_t)lin];
            if (slot < 0) {
              slot = (int32_t)nverts++;
              vert_key.push_back(lin);
              vert_tile.push_back(id);
            }
            s->voxel_corners.push_back(slot);
          }
        }
      }
    }
    const int64_t nvox = (int64_t)s->voxel_corners.size() / 8;
    // features ~ N(0, feat_std), density logits ~ N(mean, std)
    s->vfeat32.resize((size_t)(nverts * F));
    s->vdens32.resize((size_t)nverts);
    for (int64_t i = 0; i < nverts; ++i) {
      uint64_t key = ((uint64_t)tile_dense_of[vert_tile[(size_t)i]] << 40) ^ (uint64_t)vert_key[(size_t)i];
      for (int c = 0; c < F; ++c)
        s->vfeat32[(size_t)(i * F + c)] = (float)(P->feat_std * normal_ih(P->seed ^ 0x1111ull, key, (uint64_t)c));
      s->vdens32[(size_t)i] = (float)(P->density_mean + P->density_std * normal_ih(P->seed ^ 0x2222ull, key, 0));
    }
    if (P->feat_type == SNISR_F16) {
      s->vfeat16.resize(s->vfeat32.size());
      s->vdens16.resize(s->vdens32.size());
      for (size_t i = 0; i < s->vfeat32.size(); ++i) s->vfeat16[i] = f32_to_f16(s->vfeat32[i]);
      for (size_t i = 0; i < s->vdens32.size(); ++i) s->vdens16[i] = f32_to_f16(s->vdens32[i]);
    }

    // per-tile MLP, Xavier-normal weights and zero biases (reference init_model
    // 'xavier', training/scripts/networks.py:55-58)
    const int in = F + 3 + 6 * P->dir_freqs, H = P->mlp_hidden, L = P->mlp_layers;
    const int64_t PP = snisr_mlp_param_count(F, P->dir_freqs, H, L);
    s->mlp.assign((size_t)(nt * PP), 0.0f);
    for (int32_t id = 0; id < nt; ++id) {
      float* p = &s->mlp[(size_t)(id * PP)];
      uint64_t tseed = P->seed ^ (0x5151ull + (uint64_t)tile_dense_of[id] * 0x9E37ull);
      int64_t off = 0;
      for (int l = 0; l <= L; ++l) {
        int fi = (l == 0) ? in : H, fo = (l == L) ? 3 : H;
        double std = std::sqrt(2.0 / (double)(fi + fo));
        for (int o = 0; o < fo; ++o)
          for (int i = 0; i < fi; ++i) {
            float wv = (float)(std * normal_ih(tseed, (uint64_t)l, (uint64_t)(o * fi + i)));
            if (P->round_weights_f16) wv = f16_bits_to_f32(f32_to_f16(wv));
            p[off++] = wv;
          }
        off += fo;  // biases stay zero
      }
    }

    // proxy mesh: subdivided wall rectangles and box faces
    if (P->with_mesh) {
      double cell = P->mesh_cell > 0 ? P->mesh_cell : 0.1;
      for (const Wall& w : s->surf.walls) {
        int b = (w.axis + 1) % 3, c = (w.axis + 2) % 3;
        add_rect_mesh(s, w.axis, w.pos, w.lo[b], w.hi[b], w.lo[c], w.hi[c], cell, w.gaps.empty() ? nullptr : &w.gaps);
      }
      for (const Box& bx : s->surf.boxes)
        for (int a = 0; a < 3; ++a) {
          int b = (a + 1) % 3, c = (a + 2) % 3;
          add_rect_mesh(s, a, bx.lo[a], bx.lo[b], bx.hi[b], bx.lo[c], bx.hi[c], cell, nullptr);
          add_rect_mesh(s, a, bx.hi[a], bx.lo[b], bx.hi[b], bx.lo[c], bx.hi[c], cell, nullptr);
        }
    }

    std::memset(desc, 0, sizeof(*desc));
    for (int a = 0; a < 3; ++a) { desc->grid[a] = P->grid[a]; desc->scene_min[a] = 0.0f; }
    desc->tile_size = (float)S;
    desc->res = N;
    desc->num_tiles = nt;
    desc->tile_index = s->tile_index.data();
    desc->occupancy = s->occupancy.data();
    desc->num_voxels = nvox;
    desc->voxel_corners = s->voxel_corners.data();
    desc->num_vertices = nverts;
    desc->feat_dim = F;
    desc->feat_type = P->feat_type;
    if (P->feat_type == SNISR_F16) { desc->vertex_feat = s->vfeat16.data(); desc->vertex_density = s->vdens16.data(); }
    else { desc->vertex_feat = s->vfeat32.data(); desc->vertex_density = s->vdens32.data(); }
    desc->dir_freqs = P->dir_freqs;
    desc->mlp_hidden = H;
    desc->mlp_layers = L;
    desc->mlp_params = s->mlp.data();
    desc->num_mesh_vertices = (int64_t)s->mesh_v.size() / 3;
    desc->mesh_vertices = s->mesh_v.empty() ? nullptr : s->mesh_v.data();
    desc->num_triangles = (int64_t)s->mesh_f.size() / 3;
    desc->mesh_faces = s->mesh_f.empty() ? nullptr : s->mesh_f.data();
    desc->step_vox = 0.5f;
    desc->early_stop = 1e-3f;
    desc->start_offset_vox = 2.0f;
    desc->max_samples_per_ray = 48;
    desc->max_pixels = 1920 * 1080;
    (void)v;
  } catch (const std::bad_alloc&) {
    delete s;
    return set_error(SNISR_OOM, "synth_create: host allocation failed");
  }
  *out = s;
  return SNISR_OK;
}

extern "C" snisr_status snisr_synth_destroy(snisr_synth_scene* s) {
  delete s;
  return SNISR_OK;
}

extern "C" snisr_status snisr_synth_camera(const snisr_synth_scene* s, uint64_t pose_seed, int32_t width,
                                           int32_t height, float fov_x_deg, snisr_camera* cam) {
  if (!s || !cam || width <= 0 || height <= 0) return set_error(SNISR_INVALID_ARG, "synth_camera: bad argument");
  // tan(fov/2) for the benchmark FOVs is tabulated so that cameras do not
  // depend on the host's libm.
  double t;
  if (fov_x_deg == 60.0f) t = 0.57735026918962576451;       // tan(30 deg) = 1/sqrt(3)
  else if (fov_x_deg == 75.0f) t = 0.76732698797896059164;  // tan(37.5 deg)
  else if (fov_x_deg == 90.0f) t = 1.0;
  else t = std::tan(fov_x_deg * 3.14159265358979323846 / 360.0);
  Rng rng(pose_seed * 0x9E3779B97F4A7C15ull + 17);
  const double margin = std::min(0.3, 0.1 * std::min(s->ext[0], std::min(s->ext[1], s->ext[2])));
  double o[3] = {0.5 * s->ext[0], 0.5 * s->ext[1], 0.5 * s->ext[2]};
  for (int it = 0; it < 10000; ++it) {
    double p[3];
    for (int a = 0; a < 3; ++a) p[a] = rng.uni(0.15 * s->ext[a], 0.85 * s->ext[a]);
    if (s->params.kind != 0) p[2] = rng.uni(0.3 * s->ext[2], 0.7 * s->ext[2]);
    if (in_free_space(s->surf, p, margin)) { for (int a = 0; a < 3; ++a) o[a] = p[a]; break; }
  }
  double f[3];
  for (;;) {
    f[0] = rng.uni(-1, 1); f[1] = rng.uni(-1, 1); f[2] = 0.35 * rng.uni(-1, 1);
    double n2 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    if (n2 > 0.05 && n2 <= 1.0) { double n = std::sqrt(n2); for (double& x : f) x /= n; break; }
  }
  // OpenCV-style axes: x right, y down, z forward; world z is up.
  double r[3] = {f[1] * 1.0 - f[2] * 0.0, f[2] * 0.0 - f[0] * 1.0, 0.0};
  double rn = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  for (double& x : r) x /= rn;
  double d[3] = {f[1] * r[2] - f[2] * r[1], f[2] * r[0] - f[0] * r[2], f[0] * r[1] - f[1] * r[0]};
  cam->width = width;
  cam->height = height;
  cam->cx = 0.5f * (float)width;
  cam->cy = 0.5f * (float)height;
  cam->inv_focal = (float)(t / (0.5 * width));
  const double R[3][3] = {{r[0], d[0], f[0]}, {r[1], d[1], f[1]}, {r[2], d[2], f[2]}};
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) cam->c2w[i * 4 + j] = (float)R[i][j];
    cam->c2w[i * 4 + 3] = (float)o[i];
  }
  return SNISR_OK;
}

extern "C" int64_t snisr_mlp_param_count(int32_t feat_dim, int32_t dir_freqs, int32_t hidden, int32_t layers) {
  int64_t in = feat_dim + 3 + 6 * dir_freqs, p = 0;
  for (int l = 0; l <= layers; ++l) {
    int64_t fi = l == 0 ? in : hidden, fo = l == layers ? 3 : hidden;
    p += fi * fo + fo;
  }
  return p;
}
