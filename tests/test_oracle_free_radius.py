"""The free-radius map of voxel-boundary stepping (the oracle's chamfer
transform, which the engine's Jacobi relaxation must reproduce for the
bit-identical parity tests to hold) against its definition, computed
independently: the largest r <= 31 such that every voxel of the grid within
Chebyshev distance r carries the voxel's label."""
import ctypes

import numpy as np
import pytest
from scipy import ndimage


def _oracle_map(oracle, labels):
    nz, ny, nx = labels.shape
    lab = np.ascontiguousarray(labels.astype(np.int16))
    out = np.zeros(labels.size, np.uint8)
    f = oracle.lib.oracle_free_radius
    f.argtypes = [ctypes.POINTER(ctypes.c_short), ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                  ctypes.POINTER(ctypes.c_ubyte)]
    f.restype = None
    f(lab.ctypes.data_as(ctypes.POINTER(ctypes.c_short)), nx, ny, nz, out.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)))
    return out.reshape(labels.shape)


def _definition(labels):
    """Chebyshev distance to the nearest voxel that has a differently
    labelled 26-neighbour inside the grid, capped at 31."""
    edge = np.zeros(labels.shape, bool)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sh = np.roll(labels, (dz, dy, dx), axis=(0, 1, 2))
                valid = np.ones(labels.shape, bool)
                for ax, d in ((0, dz), (1, dy), (2, dx)):
                    idx = [slice(None)] * 3
                    if d == 1:
                        idx[ax] = slice(0, 1)
                        valid[tuple(idx)] = False
                    elif d == -1:
                        idx[ax] = slice(-1, None)
                        valid[tuple(idx)] = False
                edge |= valid & (sh != labels)
    if not edge.any():
        return np.full(labels.shape, 31, np.uint8)
    d = ndimage.distance_transform_cdt(~edge, metric="chessboard")
    return np.minimum(d, 31).astype(np.uint8)


def _brute(labels, r_max=31):
    """The definition itself on a small grid: grow the cube while it holds
    the voxel's label only."""
    nz, ny, nx = labels.shape
    out = np.zeros(labels.shape, np.uint8)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                r = 0
                while r < r_max:
                    c = labels[max(z - r - 1, 0):z + r + 2, max(y - r - 1, 0):y + r + 2, max(x - r - 1, 0):x + r + 2]
                    if (c != labels[z, y, x]).any():
                        break
                    r += 1
                out[z, y, x] = r
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_free_radius_matches_its_definition(oracle, seed):
    rng = np.random.default_rng(seed)
    nz, ny, nx = 9, 13, 11
    lab = np.ones((nz, ny, nx), np.uint8)
    for _ in range(4):  # a few boxes of other labels
        z0, y0, x0 = rng.integers(0, [nz, ny, nx])
        lab[z0:z0 + rng.integers(1, 5), y0:y0 + rng.integers(1, 6), x0:x0 + rng.integers(1, 6)] = rng.integers(2, 5)
    got = _oracle_map(oracle, lab)
    assert np.array_equal(got, _brute(lab))
    assert np.array_equal(got, _definition(lab))


def test_free_radius_caps_and_large_grid(oracle):
    lab = np.ones((40, 90, 90), np.uint8)
    lab[20, 45, 45] = 2
    got = _oracle_map(oracle, lab)
    assert got.max() == 31 and got[20, 45, 45] == 0 and got[20, 45, 46] == 0 and got[20, 45, 47] == 1
    assert np.array_equal(got, _definition(lab))
    assert np.all(_oracle_map(oracle, np.ones((5, 6, 7), np.uint8)) == 31)
