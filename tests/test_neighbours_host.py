"""Binning grid of the GPU neighbour search (host side, no GPU)."""
import numpy as np
import pytest

from probabilistic_peridynamics_gb300.neighbours import grid


def test_grid_covers_points_with_cells_wider_than_horizon():
    rng = np.random.default_rng(0)
    pts = rng.uniform(-1.0, 2.0, size=(500, 3)) * [1.0, 0.5, 0.1]
    lo, cell, dims = grid(pts, 0.07)
    assert cell >= 0.07 * (1 + 1e-6)
    c = np.floor((pts - lo) / cell).astype(np.int64)
    assert np.all(c >= 0) and np.all(c < dims)


def test_grid_widens_cells_to_bound_their_number():
    pts = np.array([[0.0, 0.0, 0.0], [100.0, 100.0, 100.0]])
    lo, cell, dims = grid(pts, 0.01, max_cells=1000)
    assert int(np.prod(dims.astype(np.int64))) <= 1000
    assert cell > 0.01


def test_grid_degenerate_and_invalid():
    lo, cell, dims = grid(np.zeros((5, 3)), 0.0)
    assert tuple(dims) == (1, 1, 1) and cell > 0
    with pytest.raises(ValueError):
        grid(np.array([[0.0, 0.0, np.nan]]), 1.0)
