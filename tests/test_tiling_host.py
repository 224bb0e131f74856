"""Host side of the tiled layout: brick ordering and tile cuts (CPU)."""
import numpy as np

from probabilistic_peridynamics_gb300 import lattice
from probabilistic_peridynamics_gb300.tiling import (TILE_NODES_MAX,
                                                     brick_order,
                                                     split_tiles)


def _check(perm, tile_start, n, max_nodes=TILE_NODES_MAX):
    assert np.array_equal(np.sort(perm), np.arange(n))
    assert tile_start[0] == 0 and tile_start[-1] == n
    sizes = np.diff(tile_start)
    assert np.all(sizes >= 1) and np.all(sizes <= max_nodes)


def test_lattice_bricks_are_compact():
    coords = lattice.lattice_coords(40, 30, 10, 0.005)
    perm, ts = brick_order(coords)
    _check(perm, ts, coords.shape[0])
    # 125-node target on a lattice: 5 x 5 x 5 bricks
    sizes = np.diff(ts)
    assert np.median(sizes) == 125
    for t in range(0, sizes.size, 7):
        c = coords[perm[ts[t]:ts[t + 1]]]
        ext = (c.max(axis=0) - c.min(axis=0)) / 0.005
        assert np.all(ext <= 4 + 1e-9)
    # reference order inside a brick (stable sort)
    for t in range(sizes.size):
        assert np.all(np.diff(perm[ts[t]:ts[t + 1]]) > 0)


def test_segments_never_share_a_brick():
    a = lattice.lattice_coords(12, 9, 5, 0.005)
    coords = np.concatenate([a, a, a[:300]])  # instances overlap in space
    seg = np.repeat([0, 1, 2], [a.shape[0], a.shape[0], 300])
    perm, ts = brick_order(coords, seg)
    _check(perm, ts, coords.shape[0])
    # each segment's nodes are contiguous in internal order
    s = seg[perm]
    assert np.all(np.diff(s) >= 0)


def test_large_bricks_split_and_degenerate_sets():
    rng = np.random.default_rng(0)
    pts = rng.random((5000, 3)) * [1.0, 1.0, 0.0]  # flat: one live dim less
    perm, ts = brick_order(pts, target=400, max_nodes=128)
    _check(perm, ts, 5000)
    perm, ts = brick_order(np.zeros((300, 3)))  # all coincident
    _check(perm, ts, 300)
    perm, ts = brick_order(np.zeros((0, 3)))
    assert perm.size == 0 and list(ts) == [0]
    perm, ts = brick_order(np.ones((1, 3)))
    _check(perm, ts, 1)


def test_split_tiles_halves():
    ts = np.array([0, 100, 228, 229], dtype=np.int32)
    out = split_tiles(ts, [0, 1, 2])
    assert list(out) == [0, 50, 100, 164, 228, 229]
