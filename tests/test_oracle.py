"""The oracle pinned against the reference's golden vectors (CPU only).

The oracle (``oracle/cl_step.py``) must reproduce, before anything is
compared with it:

* the reference's kernel known answers (``tests/known_answers.py``);
* the 2113-node plate regression goldens of EulerCL, EulerCromerCL and
  VelocityVerletCL after 10 steps (``peripy/test/test_integrators.py``
  ``test_call``), within the reference test's own ``np.allclose`` and,
  tighter, 1e-9 relative on u, ud, udd and force, exact on nlist and
  n_neigh, exact on damage (Euler: within one ulp, see below).

Measured: Euler u 1.2e-12, force 9.1e-12 relative (the Euler goldens come
from the Cython integrator, which forms r = r0 + u before differencing);
Euler-Cromer and Velocity-Verlet u 4.7e-16, force 7.3e-14.
"""
import numpy as np
import pytest

from oracle import cl_step
from tests import known_answers
from tests.plate_setup import (BOND_STIFFNESS, CRITICAL_STRETCH, DISP_MAGS,
                               DT, STEPS)


@pytest.mark.parametrize("name", list(known_answers.bond_force_cases()))
def test_bond_force_known_answers(name):
    case = known_answers.bond_force_cases()[name]
    n = case["r0"].shape[0]
    nlist = case["nlist"].copy()
    force, body = cl_step.bond_force(
        case["u"], case["r0"], case["vols"], nlist,
        np.zeros((n, 3), dtype=np.intc), np.zeros((n, 3)), 1.0, case["k"],
        case["s0"], stiffness_corrections=case["sc"])
    if case["force"] is not None:
        assert np.allclose(force, case["force"])
        assert np.array_equal(force, body)
    if "nlist_out" in case:
        assert np.array_equal(nlist, case["nlist_out"])
        n_neigh, damage = cl_step.damage(nlist, case["family"])
        assert np.array_equal(n_neigh, case["n_neigh_out"])
        assert np.allclose(damage, case["damage_out"])


def test_force_directions():
    """Restorative force signs (peripy/test/test_model.py:1604-1626)."""
    case = known_answers.bond_force_cases()["force"]
    force, _ = cl_step.bond_force(
        case["u"], case["r0"], case["vols"], case["nlist"].copy(),
        np.zeros((3, 3), dtype=np.intc), np.zeros((3, 3)), 1.0, case["k"],
        case["s0"])
    assert force[0, 0] > 0 and force[1, 0] < 0
    assert force[1, 1] > 0 and force[2, 1] < 0
    assert np.all(force[0, 1:] == 0)
    assert force[1, 2] == 0
    assert np.all(force[2, [0, 2]] == 0)


@pytest.mark.parametrize("idx", range(len(known_answers.update_cases())))
def test_update_known_answers(idx):
    kind, inp, exp = known_answers.update_cases()[idx]
    u = inp["u"].copy()
    if kind == "euler":
        cl_step.update_euler(inp["force"], u, inp["bc_types"],
                             inp["bc_values"], inp["bc_scale"], inp["dt"])
        assert np.array_equal(u, exp["u"])
        return
    ud = inp["ud"].copy()
    udd = inp["udd"].copy()
    fn = (cl_step.update_euler_cromer if kind == "euler_cromer"
          else cl_step.update_velocity_verlet)
    fn(inp["force"], u, ud, udd, inp["bc_types"], inp["bc_values"],
       inp["densities"], inp["bc_scale"], inp["damping"], inp["dt"])
    assert np.array_equal(u, exp["u"])
    assert np.array_equal(ud, exp["ud"])
    assert np.array_equal(udd, exp["udd"])


def test_tree_sum_order():
    """The tree order is the work-group order, not a sequential sum."""
    a = np.array([[1e16, 1.0, -1e16, 1.0]])
    # ((1e16 + -1e16) + (1.0 + 1.0)) = 2.0, a left fold would give 1.0
    assert cl_step.tree_sum(a)[0] == 2.0
    with pytest.raises(ValueError):
        cl_step.tree_sum(np.zeros((1, 3)))


def test_crack_connectivity(plate, golden):
    """The reference crack applied to the basic CL connectivity."""
    assert np.array_equal(plate["nlist"], golden["euler_nlist"])
    assert np.array_equal(plate["n_neigh"], golden["euler_n_neigh"])


def _run_plate(plate, integrator):
    st = cl_step.Stepper(
        integrator, DT, plate["coords"], plate["volume"], plate["family"],
        plate["nlist"], plate["bc_types"], plate["bc_values"],
        plate["force_bc_types"], plate["force_bc_values"], BOND_STIFFNESS,
        CRITICAL_STRETCH, damping=0.0,
        densities=None if integrator == "euler" else plate["densities"])
    for k in range(STEPS):
        st.step(DISP_MAGS[k], 0.0)
    return st.write()


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("integrator,prefix", [
    ("euler", "euler"), ("euler_cromer", "ec"), ("velocity_verlet", "vv")])
def test_oracle_plate_goldens(plate, golden, integrator, prefix):
    u, ud, udd, force, body, damage, nlist, n_neigh = _run_plate(
        plate, integrator)
    assert np.allclose(u, golden[f"{prefix}_u"])
    assert np.allclose(force, golden[f"{prefix}_force"])
    assert _rel(u, golden[f"{prefix}_u"]) < 1e-9
    assert _rel(force, golden[f"{prefix}_force"]) < 1e-9
    if prefix in ("ec", "vv"):
        assert _rel(ud, golden[f"{prefix}_ud"]) < 1e-9
    if prefix == "vv":
        assert _rel(udd, golden["vv_udd"]) < 1e-9
    assert np.array_equal(nlist, golden[f"{prefix}_nlist"])
    assert np.array_equal(n_neigh, golden[f"{prefix}_n_neigh"])
    if prefix == "euler":
        # The Euler goldens are shared with the Cython integrator, whose
        # damage is (family - n_neigh)/family (peripy/peridynamics.pyx:29);
        # the CL formula 1 - n_neigh/family differs by at most one ulp.
        fam = plate["family"].astype(np.float64)
        assert np.array_equal((fam - n_neigh) / fam, golden["euler_damage"])
        assert np.max(np.abs(damage - golden["euler_damage"])) <= 1.2e-16
    else:
        assert np.array_equal(damage, golden[f"{prefix}_damage"])
