"""Neighbour families built on the GPU (pp_neighbour_cells/_rows).

Bar: identical to the host search (scipy cKDTree pairs assembled by
``model.build_family``, the layout PeriPy's ``Model`` produces) on regular
lattices, Poisson-disk sets, random sets with coincident points and the
2113-node plate, whose sets also equal the reference's own connectivity
golden; identical to a binary64 brute force with the same
distance formula where pairs lie exactly at the horizon; edge cases (no
node, one node, all nodes coincident, a coarse grid).
"""
import numpy as np
import pytest

from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


def _host(coords, horizon, pow2=True):
    from probabilistic_peridynamics_gb300.model import (build_family,
                                                        neighbour_pairs)
    return build_family(coords.shape[0], neighbour_pairs(coords, horizon),
                        pow2=pow2)


def _brute(coords, horizon):
    """Binary64 brute force: (dx*dx + dy*dy) + dz*dz <= horizon**2."""
    d = coords[None, :, :] - coords[:, None, :]
    d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    hit = d2 <= horizon * horizon
    np.fill_diagonal(hit, False)
    return hit


def _same(got, want):
    for g, w in zip(got, want):
        assert np.array_equal(np.asarray(g), np.asarray(w))


def _gpu(*args, **kw):
    from probabilistic_peridynamics_gb300.neighbours import neighbour_family
    return neighbour_family(*args, **kw)


@pytest.mark.parametrize("pow2", [True, False])
def test_lattice_matches_host(pow2):
    from probabilistic_peridynamics_gb300 import lattice
    coords = lattice.lattice_coords(20, 20, 5, 0.05)
    got = _gpu(coords, 3.015 * 0.05, pow2=pow2)
    _same(got, _host(coords, 3.015 * 0.05, pow2))
    assert int(got[0].sum()) == 166_508


def test_poisson_disk_matches_host():
    from probabilistic_peridynamics_gb300.pointset import poisson_disk
    coords = poisson_disk((0, 0, 0), (0.16, 0.08, 0.04), 0.004, 2500, 2)
    _same(_gpu(coords, 0.012), _host(coords, 0.012))


def test_random_points_with_duplicates_match_host_and_brute_force():
    rng = np.random.default_rng(3)
    coords = rng.uniform(0.0, 1.0, size=(3000, 3))
    coords[100:120] = coords[7]  # coincident points are neighbours
    fam, nl, width = _gpu(coords, 0.08)
    _same((fam, nl, width), _host(coords, 0.08))
    hit = _brute(coords, 0.08)
    assert np.array_equal(fam, hit.sum(1))


def test_pairs_exactly_at_the_horizon_follow_the_formula():
    from probabilistic_peridynamics_gb300 import lattice
    coords = lattice.lattice_coords(9, 8, 7, 0.1)
    horizon = 0.3  # lattice distances of exactly 3 dx
    fam, nl, _ = _gpu(coords, horizon)
    hit = _brute(coords, horizon)
    assert np.array_equal(fam, hit.sum(1))
    for i in range(coords.shape[0]):
        assert np.array_equal(nl[i, :fam[i]], np.nonzero(hit[i])[0])
        assert np.all(nl[i, fam[i]:] == -1)


def test_coarse_grid_gives_the_same_rows():
    from probabilistic_peridynamics_gb300.pointset import poisson_disk
    coords = poisson_disk((0, 0, 0), (0.16, 0.08, 0.04), 0.004, 2500, 5)
    _same(_gpu(coords, 0.012, max_cells=8), _gpu(coords, 0.012))


def test_plate_mesh_matches_host_and_reference_connectivity(golden):
    """The 2113-node plate: the reference's own connectivity (sklearn
    KD-tree, ``expected_connectivity_basic.npz``) as sets, the host search
    row for row."""
    from tests.plate_setup import HORIZON
    coords = golden["points"]
    fam, nl, width = _gpu(coords, HORIZON)
    _same((fam, nl, width), _host(coords, HORIZON))
    ref_nl, ref_n = golden["nlist_basic"], golden["n_neigh_basic"]
    assert np.array_equal(fam, ref_n)
    for i in range(coords.shape[0]):
        assert np.array_equal(nl[i, :fam[i]], np.sort(ref_nl[i, :ref_n[i]]))


def test_edge_cases():
    fam, nl, width = _gpu(np.zeros((0, 3)), 1.0)
    assert fam.shape == (0,) and nl.shape[0] == 0
    fam, nl, width = _gpu(np.zeros((1, 3)), 1.0)
    assert fam.tolist() == [0] and nl.tolist() == [[-1]] and width == 1
    fam, nl, width = _gpu(np.ones((50, 3)), 0.0)
    assert np.all(fam == 49) and width == 64
    assert np.array_equal(nl[3, :49], np.delete(np.arange(50), 3))
