"""Poisson-disk point sets and the composite workload (host, no GPU)."""
import numpy as np
import pytest

from probabilistic_peridynamics_gb300.pointset import (composite,
                                                       nlinear_tables,
                                                       poisson_disk,
                                                       trilinear)


def test_poisson_disk_spacing_count_and_seed():
    from scipy.spatial import cKDTree
    box = (0.2, 0.1, 0.05)
    p = poisson_disk((0, 0, 0), box, 0.004, 5000, seed=3)
    assert p.shape == (5000, 3)
    assert np.all(p >= 0) and np.all(p < np.array(box))
    d, _ = cKDTree(p).query(p, k=2)
    assert d[:, 1].min() > 0.004
    assert np.array_equal(p, poisson_disk((0, 0, 0), box, 0.004, 5000, 3))
    assert not np.array_equal(p, poisson_disk((0, 0, 0), box, 0.004, 5000, 4))


def test_poisson_disk_matches_one_by_one_addition():
    """Batched acceptance equals testing the candidate stream one by one."""
    lo, hi, r, count, seed = (0, 0, 0), (0.03, 0.02, 0.02), 0.004, 60, 9
    batched = poisson_disk(lo, hi, r, count, seed, batch=1000)
    rng = np.random.default_rng(seed)
    ext = np.asarray(hi, dtype=np.float64)
    pts = []
    m = int(min(1000, max(1000, 4 * count)))
    while len(pts) < count:
        for c in rng.random((m, 3)) * ext:
            if all(np.sum((q - c) ** 2) > r * r for q in pts):
                pts.append(c)
                if len(pts) == count:
                    break
        m = int(min(1000, max(1000, 4 * (count - len(pts)))))
    assert np.array_equal(batched, np.array(pts))


def test_poisson_disk_jammed_box_raises():
    with pytest.raises(ValueError):
        poisson_disk((0, 0, 0), (0.01, 0.01, 0.01), 0.004, 1000, seed=1)


def test_nlinear_tables_continuous_force():
    k, s, c = nlinear_tables(*trilinear(2.0, 0.004, 0.006, 0.01))
    assert k.shape == s.shape == c.shape == (1, 3)
    for r in range(1, 3):
        x = s[0, r - 1]
        assert np.isclose(k[0, r - 1] * x + c[0, r - 1], k[0, r] * x + c[0, r])
    # force vanishes at the breaking stretch
    assert abs(k[0, 2] * s[0, 2] + c[0, 2]) < 1e-12


def test_composite_types_and_tables():
    w = composite(count=2500, box=(0.16, 0.08, 0.04), split=0.08, seed=2)
    n = w["coords"].shape[0]
    nl, bt = w["nlist"], w["bond_types"]
    valid = nl != -1
    assert w["max_neigh"] == nl.shape[1] and w["max_neigh"] & (w["max_neigh"] - 1) == 0
    assert np.array_equal(valid.sum(1), w["family"])
    left = w["coords"][:, 0] < 0.08
    i = np.broadcast_to(np.arange(n)[:, None], nl.shape)[valid]
    j = nl[valid]
    want = np.where(left[i] & left[j], 0, np.where(~left[i] & ~left[j], 1, 2))
    assert np.array_equal(bt[valid], want)
    assert set(np.unique(want)) == {0, 1, 2}
    # symmetric types, interface micro-modulus = harmonic mean
    k = w["bond_stiffness"]
    assert np.isclose(k[2, 0], 2 * k[0, 0] * k[1, 0] / (k[0, 0] + k[1, 0]))
    assert np.isclose(k[1, 0], 3 * k[0, 0])
    assert w["nregimes"] == 3 and w["nbond_types"] == 3
    assert np.all(w["critical_stretch"] == [0.004, 0.006, 0.01])
    assert np.isclose(w["volume"].sum(), 0.16 * 0.08 * 0.04)
    assert w["bc_types"][:, 0].sum() > 0
    assert np.all(w["bc_values"][left & (w["bc_types"][:, 0] == 1), 0] == -1)
