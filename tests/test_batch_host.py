"""Host logic of batched instances (no GPU)."""
import numpy as np
import pytest

from probabilistic_peridynamics_gb300 import batch
from probabilistic_peridynamics_gb300.lattice import lattice_family


def test_pair_noise_symmetric_and_in_range():
    _, nlist, _ = lattice_family(6, 5, 3, 3.015)
    z = batch.pair_noise(nlist, 0.9, 1.1, seed=11)
    valid = nlist >= 0
    assert np.all((z[valid] >= 0.9) & (z[valid] < 1.1))
    assert np.all(z[~valid] == 1.0)
    for i in range(nlist.shape[0]):
        for s in np.nonzero(valid[i])[0]:
            j = nlist[i, s]
            k = np.nonzero(nlist[j] == i)[0][0]
            assert z[i, s] == z[j, k]
    # a different seed gives different noise
    assert not np.array_equal(z, batch.pair_noise(nlist, 0.9, 1.1, seed=12))


def test_concatenate_split_round_trip():
    inst = batch.uq_instances(count=4, nx_range=(5, 8), ny_range=(5, 7),
                              nz=3)
    b = batch.concatenate(inst)
    assert b.nnodes == sum(i.nnodes for i in inst)
    assert b.bonds == sum(int(i.family.sum()) for i in inst)
    assert list(np.bincount(b.node_instance)) == [i.nnodes for i in inst]
    for part, i in zip(b.split(b.nlist, "nlist"), inst):
        assert np.array_equal(part, i.nlist)
    for part, i in zip(b.split(b.coords), inst):
        assert np.array_equal(part, i.coords)
    # bonds never cross instances
    for k in range(len(inst)):
        a, e = b.offsets[k], b.offsets[k + 1]
        rows = b.nlist[a:e]
        assert np.all((rows == -1) | ((rows >= a) & (rows < e)))


def test_uq_critical_stretch_distribution():
    inst = batch.uq_instances(count=64, nx_range=(3, 4), ny_range=(3, 4),
                              nz=3)
    s0 = np.array([i.critical_stretch for i in inst])
    # lognormal with mean 0.005: the sample mean is within 10%
    assert abs(s0.mean() - 0.005) < 0.0005
    assert np.all(s0 > 0)


def test_too_many_instances_rejected():
    inst = batch.uq_instances(count=1, nx_range=(3, 3), ny_range=(3, 3),
                              nz=3)
    with pytest.raises(ValueError):
        batch.concatenate(inst * 257)
