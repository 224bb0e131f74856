"""The C restatement and the compiled reference against the NumPy oracle.

* ``oracle/pp_oracle.c`` must be bit-identical to ``oracle/cl_step.py`` on
  the plate goldens, on load-induced breaking and on the n-linear,
  bond-type and stiffness-correction variants (bond_force1..4).
* The reference's own Cython step (``peripy/peridynamics.pyx``, compiled by
  ``oracle/build_ref.py``), called as ``Euler.__call__`` does
  (``peripy/integrators.py:330-349``), must reproduce the plate goldens and
  agree with the oracle to 1e-11; it forms ``r = r0 + u`` before
  differencing, so agreement is to rounding, not bit for bit.
"""
import numpy as np
import pytest

from oracle import build_ref, cl_step, cref
from tests.gpu_helpers import lattice, pull_bcs
from tests.plate_setup import (BOND_STIFFNESS, CRITICAL_STRETCH, DISP_MAGS,
                               DT, STEPS)


def _steppers(kind, setup, **kw):
    args = (kind, setup["dt"], setup["coords"], setup["volume"],
            setup["family"], setup["nlist"], setup["bc_types"],
            setup["bc_values"], setup["force_bc_types"],
            setup["force_bc_values"], kw.pop("k", setup.get("k")),
            kw.pop("s0", setup.get("s0")))
    return cl_step.Stepper(*args, **kw), cref.Stepper(*args, **kw)


def _compare(kind, setup, steps, mags, **kw):
    a, b = _steppers(kind, setup, **kw)
    for k in range(steps):
        a.step(mags[k], 0.0)
        b.step(mags[k], 0.0)
    for x, y in zip(a.write(), b.write()):
        assert np.array_equal(x, y)
    return a


@pytest.mark.parametrize("kind", ["euler", "euler_cromer",
                                  "velocity_verlet"])
def test_c_oracle_plate(plate, kind):
    setup = dict(plate, k=BOND_STIFFNESS, s0=CRITICAL_STRETCH, dt=DT)
    dens = None if kind == "euler" else plate["densities"]
    _compare(kind, setup, STEPS, DISP_MAGS, densities=dens)


def _lattice_setup():
    coords, volume, _, family, nlist, n_neigh = lattice(8, 6, 4, 1.0)
    n = coords.shape[0]
    bc_types, bc_values = pull_bcs(coords, 0)
    return dict(coords=coords, volume=volume, family=family, nlist=nlist,
                n_neigh=n_neigh, bc_types=bc_types, bc_values=bc_values,
                force_bc_types=np.zeros((n, 3), dtype=np.intc),
                force_bc_values=np.zeros((n, 3)), dt=0.5, k=0.01, s0=0.02)


def test_c_oracle_breaking():
    setup = _lattice_setup()
    mags = 3e-3 * np.arange(1, 61)
    st = _compare("euler", setup, 60, mags)
    assert (st.nlist != -1).sum() < (setup["nlist"] != -1).sum()


@pytest.mark.parametrize("corrections", [False, True])
def test_c_oracle_nlinear(corrections):
    from probabilistic_peridynamics_gb300.model import Model
    setup = _lattice_setup()
    nlist = setup["nlist"]
    n, mn = nlist.shape
    valid = nlist != -1
    left = setup["coords"][:, 0] < 3.5
    jj = np.where(valid, nlist, 0)
    bt = np.where(left[:, None] & left[jj], 0, 1)
    bt = np.where(valid, bt, 0).astype(np.intc)
    ks = np.array([[0.01, 0.005, -0.0025], [0.02, 0.01, -0.005]])
    ss = np.array([[0.010, 0.016, 0.024], [0.008, 0.014, 0.022]])
    k_tab, s_tab, c_tab, nbt, nreg = Model._set_damage_model(None, ks, ss)
    sc = None
    if corrections:
        sc = np.where(valid, np.random.default_rng(3).uniform(
            0.9, 1.1, (n, mn)), 0.0)
    mags = 3e-3 * np.arange(1, 51)
    st = _compare("velocity_verlet", setup, 50, mags, k=k_tab, s0=s_tab,
                  bond_types=bt, plus_cs=c_tab, nregimes=int(nreg),
                  stiffness_corrections=sc, damping=0.5,
                  densities=np.full((n, 3), 50.0))
    assert np.any(st.regimes[st.nlist != -1] > 0)


@pytest.fixture(scope="module")
def ref_module():
    if not build_ref.build(quiet=True):
        pytest.skip("reference checkout absent and no generated C")
    return build_ref.load()


def test_reference_cython_plate(plate, golden, ref_module):
    """The reference CPU step reproduces the goldens and the oracle."""
    coords = np.ascontiguousarray(plate["coords"])
    width = int(plate["family"].max())
    nlist = np.ascontiguousarray(plate["nlist"][:, :width]).astype(np.intc)
    nlist[nlist == -1] = 0
    n_neigh = plate["n_neigh"].astype(np.intc).copy()
    u = np.zeros_like(coords)
    for k in range(STEPS):
        ref_module.break_bonds(coords + u, coords, nlist, n_neigh,
                               CRITICAL_STRETCH)
        force = ref_module.bond_force(
            coords + u, coords, nlist, n_neigh, plate["volume"],
            BOND_STIFFNESS, plate["force_bc_values"],
            plate["force_bc_types"], 0.0)
        ref_module.update_displacement(u, plate["bc_values"],
                                       plate["bc_types"], force,
                                       DISP_MAGS[k], DT)
    assert np.allclose(u, golden["euler_u"])
    assert np.max(np.abs(u - golden["euler_u"])) / np.max(
        np.abs(golden["euler_u"])) < 1e-11
    st, _ = _steppers("euler", dict(plate, k=BOND_STIFFNESS,
                                    s0=CRITICAL_STRETCH, dt=DT))
    for k in range(STEPS):
        st.step(DISP_MAGS[k], 0.0)
    assert np.max(np.abs(u - st.u)) / np.max(np.abs(st.u)) < 1e-11
    assert np.max(np.abs(force - st.force)) / np.max(
        np.abs(st.force)) < 1e-10
    assert np.array_equal(n_neigh, golden["euler_n_neigh"])


def test_reference_cython_layout_goldens(golden, ref_module):
    from tests.cython_setup import cython_plate, run_reference_euler
    """The Cython integrator's regression (test_integrators.py:150-195) on
    its own layout: the golden connectivity after the crack and 10 steps is
    reproduced exactly, the displacements and forces to 1e-11."""
    setup = cython_plate(golden)
    u, force, damage, nlist, n_neigh = run_reference_euler(
        ref_module, setup, STEPS, DISP_MAGS, DT, BOND_STIFFNESS,
        CRITICAL_STRETCH)
    assert np.array_equal(nlist, golden["cy_nlist_crack"])
    assert np.array_equal(n_neigh, golden["cy_n_neigh_crack"])
    for got, want in ((u, golden["euler_u"]), (force, golden["euler_force"])):
        assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < 1e-11
    assert np.allclose(damage, golden["euler_damage"])
