"""Edge cases of the time step against the oracle.

* a node with no neighbours (family 0): no bond force, and damage
  ``1 - 0/0`` = NaN, as the reference's damage kernel computes it
  (``peripy/cl/peridynamics.cl:606-608``);
* a model of one node;
* rows of width 1, 2 and 4 (a chain of nodes), below the warp width;
* every bond of a node broken within the run.

Bars as in the parity tests: FP64 paths bit-identical to the oracle (NaN
where the oracle has NaN), mixed within 1e-5 with the same broken-bond
mask.
"""
import numpy as np
import pytest

from tests.conftest import cuda_available
from tests.gpu_helpers import lattice, pull_bcs, rel_err, run_integrator, \
    run_oracle

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]

KINDS = {"euler": "EulerCUDA", "euler_cromer": "EulerCromerCUDA",
         "velocity_verlet": "VelocityVerletCUDA"}
MODES = ["plain", "fused64", "mixed"]


def _setup(coords, volume, family, nlist, kind, k=0.01, s0=0.02):
    n = coords.shape[0]
    bc_types, bc_values = pull_bcs(coords, 0)
    return dict(coords=coords, volume=volume, family=family, nlist=nlist,
                n_neigh=family.copy(), bc_types=bc_types,
                bc_values=bc_values,
                force_bc_types=np.zeros((n, 3), dtype=np.intc),
                force_bc_values=np.zeros((n, 3)),
                densities=None if kind == "euler" else np.full((n, 3), 50.0),
                nnodes=n, max_neigh=nlist.shape[1], k=k, s0=s0,
                dt=0.5 if kind == "euler" else 1.0)


def _run_both(kind, mode, setup, steps, mags):
    import probabilistic_peridynamics_gb300 as pp
    cls = getattr(pp, KINDS[kind])
    kw = dict(fused=mode != "plain",
              precision="mixed" if mode == "mixed" else "float64")
    integ = (cls(dt=setup["dt"], **kw) if kind == "euler"
             else cls(damping=0.5, dt=setup["dt"], **kw))
    with np.errstate(invalid="ignore", divide="ignore"):
        out = run_integrator(integ, setup, steps, mags)
        ref = run_oracle(kind, setup, steps, mags,
                         damping=0.0 if kind == "euler" else 0.5)
    return out, ref


def _check(mode, out, ref):
    if mode == "mixed":
        assert np.array_equal(out[6], ref[6])
        assert rel_err(out[0], ref[0]) < 1e-5
        assert np.array_equal(out[5], ref[5], equal_nan=True)
        return
    for got, want in zip(out, ref):
        assert np.array_equal(got, want, equal_nan=True)


def _with_isolated_node():
    coords, volume, _, family, nlist, _ = lattice(6, 5, 4, 1.0)
    coords = np.vstack([coords, [[40.0, 40.0, 40.0]]])
    volume = np.append(volume, 1.0)
    family = np.append(family, 0).astype(np.intc)
    nlist = np.vstack([nlist, np.full((1, nlist.shape[1]), -1,
                                      dtype=np.intc)])
    return coords, volume, family, nlist


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("mode", MODES)
def test_isolated_node(kind, mode):
    coords, volume, family, nlist = _with_isolated_node()
    setup = _setup(coords, volume, family, nlist, kind)
    steps = 20
    out, ref = _run_both(kind, mode, setup, steps,
                         3e-3 * np.arange(1, steps + 1))
    assert np.isnan(ref[5][-1]) and np.isnan(out[5][-1])
    assert np.all(np.isfinite(out[5][:-1]))
    _check(mode, out, ref)


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("mode", MODES)
def test_single_node(kind, mode):
    setup = _setup(np.zeros((1, 3)), np.ones(1), np.zeros(1, dtype=np.intc),
                   np.full((1, 1), -1, dtype=np.intc), kind)
    out, ref = _run_both(kind, mode, setup, 5, 1e-3 * np.arange(1, 6))
    _check(mode, out, ref)


@pytest.mark.parametrize("width", [1, 2, 4])
@pytest.mark.parametrize("mode", MODES)
def test_narrow_rows(width, mode):
    """A chain x = 0, 1, 2, ...: horizon 1 gives rows of 2 slots, horizon
    2 of 4; width 1 keeps only the right-hand neighbour (the last node has
    none)."""
    from probabilistic_peridynamics_gb300.model import (build_family,
                                                        neighbour_pairs)
    n = 40
    coords = np.zeros((n, 3))
    coords[:, 0] = np.arange(n, dtype=np.float64)
    if width == 1:
        nlist = np.append(np.arange(1, n), -1).astype(np.intc)[:, None]
        family = (nlist[:, 0] != -1).astype(np.intc)
    else:
        family, nlist, _ = build_family(
            n, neighbour_pairs(coords, {2: 1.0, 4: 2.0}[width]))
    assert nlist.shape[1] == width
    setup = _setup(coords, np.ones(n), family, nlist, "velocity_verlet")
    steps = 30
    out, ref = _run_both("velocity_verlet", mode, setup, steps,
                         5e-3 * np.arange(1, steps + 1))
    _check(mode, out, ref)


@pytest.mark.parametrize("mode", MODES)
def test_node_losing_every_bond(mode):
    """One node is pulled far out of its family by a displacement boundary
    condition; all its bonds break and its damage reaches 1."""
    coords, volume, _, family, nlist, _ = lattice(6, 5, 4, 1.0)
    setup = _setup(coords, volume, family, nlist, "euler_cromer")
    centre = int(np.argmin(np.sum((coords - coords.mean(0)) ** 2, axis=1)))
    setup["bc_types"][centre] = 1
    setup["bc_values"][centre] = (0.0, 0.0, 1.0)
    steps = 15
    out, ref = _run_both("euler_cromer", mode, setup, steps,
                         0.7 * np.arange(1, steps + 1))
    assert ref[5][centre] == 1.0 and np.all(ref[6][centre] == -1)
    _check(mode, out, ref)
