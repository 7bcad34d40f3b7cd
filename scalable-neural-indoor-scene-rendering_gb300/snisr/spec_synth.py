"""Seeded synthetic inputs for the specular pass ops (inputs for tests and
benchmarks; the reference's trained networks and captured scenes are not
distributed): per-group reflection MLPs in the reference's parameter layout
(rendering/src/rayreflection_render.cu:111-301), group centres, a downscaled
pixel grid of rays with their first-hit inverse depth, per-pixel network ids
(-1 = none) and transmittance."""
from __future__ import annotations

import numpy as np

P_SPEC = 22556  # 64 + 63*64 + 4*(64 + 64*64) + 28 + 64*28


def spec_params(G: int, rng) -> np.ndarray:
    """FP16 [G, 22556]: per layer bias[out] then W[in][out] (Xavier-uniform weights, small biases)."""
    out = np.zeros((G, P_SPEC), np.float16)
    for g in range(G):
        chunks = []
        for fi, fo in [(63, 64)] + [(64, 64)] * 4 + [(64, 28)]:
            a = np.sqrt(6.0 / (fi + fo))
            chunks.append(rng.normal(0, 0.05, fo))
            chunks.append(rng.uniform(-a, a, fi * fo))
        out[g] = np.concatenate(chunks).astype(np.float16)
    return out


def problem(seed: int = 0, G: int = 6, H: int = 48, W: int = 64, spr: int = 16):
    rng = np.random.default_rng(seed)
    npix = H * W
    params = spec_params(G, rng)
    centers = rng.uniform(-2, 2, (G, 3)).astype(np.float32)
    origin = np.array([0.3, -0.2, 1.1], np.float32)
    d = rng.normal(0, 1, (npix, 3)).astype(np.float32)
    d[:, 2] = np.abs(d[:, 2]) + 0.5  # unnormalised, as compute_rays returns them
    inv_near = (1.0 / rng.uniform(0.5, 4.0, npix)).astype(np.float32)
    net = rng.integers(-1, G, npix).astype(np.int16)
    transparency = rng.uniform(0, 1, npix).astype(np.float32)
    transparency[rng.random(npix) < 0.1] = 0.001  # below the stop: skipped
    far = 8.0
    return dict(G=G, H=H, W=W, spr=spr, npix=npix, params=params, centers=centers, origin=origin, rays_d=d,
                inv_near=inv_near, net=net, transparency=transparency, far=far, inverse_far=np.float32(1.0 / far),
                trans_stop=np.float32(0.01))
