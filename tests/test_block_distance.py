"""The per-tile 4^3-block distances that let the voxel march cross empty
space without occupancy loads (csrc/api.cpp block_distance, through
snisr_diag_block_distance; host code, no GPU): against a brute-force
Chebyshev distance on random masks of several densities and on edge cases
(empty, full, a single occupied block).  A distance too large would let the
march skip occupied voxels; the GPU tests of the visited voxel sequences
check that end to end."""
import ctypes as C

import numpy as np
import pytest

from snisr import _lib

CAP = 16  # distances are at most kBlkDistCap + 1


def _host(occ):
    nb = occ.shape[0]
    flat = occ.reshape(-1).astype(np.uint32)
    words = np.zeros((flat.size + 31) // 32, np.uint32)
    for k in np.nonzero(flat)[0]:
        words[k >> 5] |= np.uint32(1) << np.uint32(k & 31)
    out = np.zeros(flat.size, np.uint8)
    st = _lib.lib().snisr_diag_block_distance(words.ctypes.data_as(C.c_void_p), nb, out.ctypes.data_as(C.c_void_p))
    assert st == _lib.OK
    return out.reshape(occ.shape)


def _brute(occ):
    nb = occ.shape[0]
    pts = np.argwhere(occ)
    grid = np.stack(np.meshgrid(np.arange(nb), np.arange(nb), np.arange(nb), indexing="ij"), -1).reshape(-1, 3)
    if len(pts) == 0:
        return np.full(occ.shape, CAP, np.uint8)
    d = np.abs(grid[:, None, :] - pts[None, :, :]).max(-1).min(1)
    return np.minimum(d, CAP).astype(np.uint8).reshape(occ.shape)


@pytest.mark.parametrize("nb,density,seed", [(8, 0.02, 1), (12, 0.005, 2), (16, 0.001, 3), (10, 0.3, 4), (20, 0.0008, 5)])
def test_block_distance_matches_brute_force(nb, density, seed):
    occ = np.random.default_rng(seed).random((nb, nb, nb)) < density
    assert np.array_equal(_host(occ), _brute(occ))


def test_block_distance_edges():
    nb = 24
    assert (_host(np.zeros((nb,) * 3, bool)) == CAP).all()
    assert (_host(np.ones((nb,) * 3, bool)) == 0).all()
    one = np.zeros((nb,) * 3, bool)
    one[3, 20, 7] = True
    assert np.array_equal(_host(one), _brute(one))
    L = _lib.lib()
    out = np.zeros(8, np.uint8)
    assert L.snisr_diag_block_distance(None, 2, out.ctypes.data_as(C.c_void_p)) == _lib.INVALID_ARG
    assert L.snisr_diag_block_distance(out.ctypes.data_as(C.c_void_p), 0, out.ctypes.data_as(C.c_void_p)) == _lib.INVALID_ARG
