"""The five benchmark scenes: seeded synthetic stand-ins with the shapes,
sizes and value distributions of the benchmark configurations.

Seeds: scene_seed = 1000 + cfg, pose_seed = 2000 + 16*cfg + pose.
"""
from __future__ import annotations

from dataclasses import dataclass

from . import _lib


@dataclass(frozen=True)
class Config:
    name: str
    kind: int
    grid: tuple
    tile_size: float
    res: int
    feat_dim: int
    feat_type: int
    hidden: int
    layers: int
    num_boxes: int
    box_min: float
    box_max: float
    with_mesh: bool
    mesh_cell: float
    width: int
    height: int
    fov: float
    poses: int
    round_weights_f16: bool
    seed: int

    def synth_params(self) -> _lib.SynthParams:
        p = _lib.SynthParams()
        p.kind = self.kind
        for i in range(3):
            p.grid[i] = self.grid[i]
        p.tile_size = self.tile_size
        p.res = self.res
        p.feat_dim = self.feat_dim
        p.feat_type = self.feat_type
        p.mlp_hidden = self.hidden
        p.mlp_layers = self.layers
        p.dir_freqs = 4
        p.num_boxes = self.num_boxes
        p.box_min = self.box_min
        p.box_max = self.box_max
        p.with_mesh = 1 if self.with_mesh else 0
        p.mesh_cell = self.mesh_cell
        p.density_mean = 2.0
        p.density_std = 1.0
        p.feat_std = 0.1
        p.seed = self.seed
        p.round_weights_f16 = 1 if self.round_weights_f16 else 0
        return p

    def pose_seed(self, pose: int) -> int:
        cfg = int(self.name[3])
        return 2000 + 16 * cfg + pose

    def replace(self, **kw) -> "Config":
        d = dict(self.__dict__)
        d.update(kw)
        return Config(**d)


# 1: plain forward render, one 64^3 tile over 2 m, FP32 16-dim features,
#    MLP 43 -> 32 -> 32 -> 3, 256x256, no proxy mesh.
CFG1 = Config("cfg1_small", 0, (1, 1, 1), 2.0, 64, 16, _lib.F32, 32, 2, 3, 0.2, 0.6, False, 0.0,
              256, 256, 60.0, 8, False, 1001)
# Box sides are drawn U(box_min, box_max); the ranges below give the stated
# occupied fractions of the full-resolution scenes (voxels within one voxel of
# a surface): cfg2 5.1 %, cfg3 4.0 %, cfg4 5.0 %, cfg5 4.2 %.
#
# 2: full frame, 4x4x1 tiles of 128^3 over 3 m, FP16 32-dim features, per-tile
#    FP16 MLP 59 -> 64x3 -> 3, ~200k-triangle proxy mesh, 1280x720.
CFG2 = Config("cfg2_frame", 1, (4, 4, 1), 3.0, 128, 32, _lib.F16, 64, 3, 40, 0.5, 1.65, True, 0.085,
              1280, 720, 60.0, 8, True, 1002)
# 3: training, one 256^3 tile over 4 m, FP32 32-dim master features.
CFG3 = Config("cfg3_train", 1, (1, 1, 1), 4.0, 256, 32, _lib.F32, 64, 3, 12, 0.4, 1.4, False, 0.0,
              640, 480, 60.0, 8, False, 1003)
# 4: batched multi-tile training, 32 tiles of 128^3.
CFG4 = Config("cfg4_batched", 1, (4, 4, 2), 3.0, 128, 32, _lib.F32, 64, 3, 120, 0.5, 1.6, False, 0.0,
              640, 480, 60.0, 8, False, 1004)
# 5: large scene, 8x8x2 tiles of 128^3 over 24x24x6 m, multi-room, ~1M-tri mesh.
CFG5 = Config("cfg5_large", 2, (8, 8, 2), 3.0, 128, 32, _lib.F16, 64, 3, 300, 0.4, 1.5, True, 0.093,
              1920, 1080, 75.0, 16, True, 1005)

ALL = {c.name: c for c in (CFG1, CFG2, CFG3, CFG4, CFG5)}
