"""Batched independent instances on the GPU vs the oracle per instance.

Five uneven lattices with per-instance critical stretch and symmetric
per-bond stiffness noise, Euler-Cromer, load-induced breaking.  Bars: the
binary64 fused step bit-identical to the oracle run on each instance alone;
the mixed step within 1e-5 with the same broken-bond mask; every tile shape
of the mixed kernel gives identical results.
"""
import numpy as np
import pytest

from oracle import cref
from tests.conftest import cuda_available
from tests.gpu_helpers import rel_err

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]

K = 0.01
STEPS = 60
MAGS = 3e-3 * np.arange(1, STEPS + 1)


def _instances():
    from probabilistic_peridynamics_gb300 import batch
    return batch.uq_instances(count=5, seed=5, nx_range=(6, 10),
                              ny_range=(5, 8), nz=3, dx=1.0, s0_mean=0.02,
                              s0_sigma=0.2, density=50.0)


def _run(precision, variant=None):
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300 import batch
    b = batch.concatenate(_instances())
    integ = pp.EulerCromerCUDA(0.5, dt=1.0, precision=precision,
                               autotune=variant is None)
    sim = batch.BatchedSimulation(b, integ, K)
    if variant is not None:
        integ._fargs.variant = variant
    sim.run(STEPS, MAGS)
    return b, sim.results()


def _oracle(inst):
    n = inst.nnodes
    st = cref.Stepper("euler_cromer", 1.0, inst.coords, inst.volume,
                      inst.family, inst.nlist, inst.bc_types, inst.bc_values,
                      np.zeros((n, 3), dtype=np.intc), np.zeros((n, 3)), K,
                      inst.critical_stretch, damping=0.5,
                      densities=inst.densities,
                      stiffness_corrections=inst.stiffness_corrections)
    for k in range(STEPS):
        st.step(MAGS[k], 0.0)
    return st.write()


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_batch_matches_oracle_per_instance(precision):
    b, res = _run(precision)
    broken = 0
    for inst, (u, ud, damage, nlist, n_neigh) in zip(b.instances, res):
        ref = _oracle(inst)
        broken += int((inst.nlist != -1).sum() - (ref[6] != -1).sum())
        assert np.array_equal(nlist, ref[6])
        assert np.array_equal(n_neigh, ref[7])
        if precision == "float64":
            assert np.array_equal(u, ref[0])
            assert np.array_equal(ud, ref[1])
            assert np.array_equal(damage, ref[5])
        else:
            assert rel_err(u, ref[0]) < 1e-5
    assert broken > 0


def test_tile_shapes_agree():
    from probabilistic_peridynamics_gb300 import _lib
    outs = [_run("mixed", v)[1] for v in range(_lib.PP_MIXED_VARIANTS)]
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            for x, y in zip(a, b):
                assert np.array_equal(x, y)
