"""Known-answer cases of the reference's kernel tests.

Inputs and expected outputs restate the hand-built cases of
``peripy/test/test_cl_peridynamics.py`` (bond_force1: 43-234 zero and
directional force, 236-376 bond breaking and damage; bond_force2: 379-585
stiffness corrections) and the single-node integrator cases of
``test_cl_euler.py:38-190``, ``test_cl_euler_cromer.py:38-269`` and
``test_cl_velocity_verlet.py:38-272``.  The same cases are run against the
oracle (CPU) and against the CUDA kernels through the C ABI (GPU).
"""
import numpy as np

FORCE_VALUE = 0.00229417

_R0_5 = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0],
                  [2.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
_NLIST_5 = np.array([[1, 2, 4, -1], [0, 3, -1, -1], [0, -1, -1, -1],
                     [1, -1, -1, -1], [0, -1, -1, -1]], dtype=np.intc)
_R0_3 = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [1.0, 1.0, 0.0]])
_U_3 = np.array([[0.0, 0.0, 0.0], [0.05, 0.0, 0.0], [0.05, 0.05, 0.0]])
_NLIST_3 = np.array([[1, -1, -1, -1], [0, 2, -1, -1], [1, -1, -1, -1]],
                    dtype=np.intc)
_K_3 = 18.0 * 0.05 / (np.pi * 1.01 ** 4)
_F3 = np.array([[FORCE_VALUE, 0.0, 0.0], [-FORCE_VALUE, FORCE_VALUE, 0.0],
                [0.0, -FORCE_VALUE, 0.0]])


def bond_force_cases():
    """name -> dict(inputs..., expected outputs)."""
    cases = {}
    cases["initial_force"] = dict(
        r0=_R0_5, u=np.zeros((5, 3)), vols=np.ones(5), nlist=_NLIST_5,
        k=1.0, s0=1000.0, sc=None, force=np.zeros((5, 3)))
    cases["force"] = dict(
        r0=_R0_3, u=_U_3, vols=np.full(3, 0.16666667), nlist=_NLIST_3,
        k=_K_3, s0=1000.0, sc=None, force=_F3)
    cases["force_unit_corrections"] = dict(
        r0=_R0_3, u=_U_3, vols=np.full(3, 0.16666667), nlist=_NLIST_3,
        k=_K_3, s0=1000.0, sc=np.ones((3, 4)), force=_F3)
    cases["stiffness_correction"] = dict(
        r0=_R0_3, u=_U_3, vols=np.full(3, 0.16666667), nlist=_NLIST_3,
        k=_K_3, s0=1000.0,
        sc=np.array([[4.0, 1.0, 1.0, 1.0], [4.0, 2.0, 1.0, 1.0],
                     [2.0, 1.0, 1.0, 1.0]]),
        force=np.array([[4.0 * FORCE_VALUE, 0.0, 0.0],
                        [-4.0 * FORCE_VALUE, 2.0 * FORCE_VALUE, 0.0],
                        [0.0, -2.0 * FORCE_VALUE, 0.0]]))
    cases["break_bonds"] = dict(
        r0=_R0_5,
        u=np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 0.0],
                    [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]]),
        vols=np.full(5, 0.16666667), nlist=_NLIST_5,
        k=18.0 * 0.05 / (np.pi * 1.1 ** 4), s0=1.0, sc=None, force=None,
        family=np.array([3, 2, 1, 1, 1], dtype=np.intc),
        nlist_out=np.array([[-1, 2, -1, -1], [-1, 3, -1, -1],
                            [0, -1, -1, -1], [1, -1, -1, -1],
                            [-1, -1, -1, -1]], dtype=np.intc),
        n_neigh_out=np.array([1, 1, 1, 1, 0]),
        damage_out=np.array([2. / 3, 1. / 2, 0.0, 0.0, 1.0]))
    return cases


def update_cases():
    """(integrator, inputs, expected) with exact (==) expected values."""
    f = np.array([1.0, 2.0, 3.0])
    z = np.zeros(3)
    free = np.array([0, 0, 0], dtype=np.intc)
    bc110 = np.array([1, 1, 0], dtype=np.intc)
    out = []
    # Euler (test_cl_euler.py)
    out.append(("euler", dict(u=z, force=f, bc_types=free, bc_values=z,
                              bc_scale=0.0, dt=1.0), dict(u=f)))
    out.append(("euler", dict(u=z, force=f, bc_types=free, bc_values=z,
                              bc_scale=0.0, dt=2.0), dict(u=2.0 * f)))
    out.append(("euler", dict(u=z, force=f, bc_types=bc110, bc_values=z,
                              bc_scale=1.0, dt=2.0),
                dict(u=np.array([0.0, 0.0, 6.0]))))
    out.append(("euler", dict(u=z, force=f, bc_types=bc110,
                              bc_values=np.array([2.0, 2.0, 0.0]),
                              bc_scale=0.5, dt=2.0),
                dict(u=np.array([1.0, 1.0, 6.0]))))
    # Euler-Cromer (test_cl_euler_cromer.py)
    one = np.ones(3)
    out.append(("euler_cromer",
                dict(u=z, ud=z, udd=z, densities=one, force=f,
                     bc_types=free, bc_values=z, bc_scale=0.0, dt=1.0,
                     damping=1.0), dict(u=f, ud=f, udd=f)))
    out.append(("euler_cromer",
                dict(u=z, ud=z, udd=z, densities=one, force=f,
                     bc_types=free, bc_values=z, bc_scale=0.0, dt=2.0,
                     damping=1.0), dict(u=4.0 * f, ud=2.0 * f, udd=f)))
    out.append(("euler_cromer",
                dict(u=z, ud=one, udd=z, densities=one, force=f,
                     bc_types=bc110, bc_values=z, bc_scale=1.0, dt=2.0,
                     damping=2.0),
                dict(u=np.array([0.0, 0.0, 6.0]),
                     ud=np.array([-1.0, 1.0, 3.0]),
                     udd=np.array([-1.0, 0.0, 1.0]))))
    out.append(("euler_cromer",
                dict(u=z, ud=z, udd=z, densities=one, force=f,
                     bc_types=bc110, bc_values=np.array([2.0, 2.0, 0.0]),
                     bc_scale=0.5, dt=2.0, damping=1.0),
                dict(u=np.array([1.0, 1.0, 12.0]),
                     ud=np.array([2.0, 4.0, 6.0]), udd=f)))
    # Velocity-Verlet (test_cl_velocity_verlet.py)
    out.append(("velocity_verlet",
                dict(u=z, ud=z, udd=z, densities=one, force=f,
                     bc_types=free, bc_values=z, bc_scale=0.0, dt=1.0,
                     damping=1.0), dict(u=f, ud=f / 2, udd=f)))
    out.append(("velocity_verlet",
                dict(u=z, ud=z, udd=one, densities=one, force=f,
                     bc_types=free, bc_values=z, bc_scale=0.0, dt=2.0,
                     damping=0.0),
                dict(u=np.array([6.0, 10.0, 14.0]),
                     ud=np.array([2.0, 3.0, 4.0]),
                     udd=np.array([1.0, 2.0, 3.0]))))
    out.append(("velocity_verlet",
                dict(u=z, ud=one, udd=z, densities=one, force=f,
                     bc_types=bc110, bc_values=z, bc_scale=1.0, dt=2.0,
                     damping=2.0),
                dict(u=np.array([0.0, 0.0, 6.0]),
                     ud=np.array([0.0, 1.0, 2.0]),
                     udd=np.array([-1.0, 0.0, 1.0]))))
    out.append(("velocity_verlet",
                dict(u=z, ud=z, udd=z, densities=one, force=f,
                     bc_types=bc110, bc_values=np.array([2.0, 2.0, 0.0]),
                     bc_scale=0.5, dt=2.0, damping=1.0),
                dict(u=np.array([1.0, 1.0, 12.0]), ud=f, udd=f)))
    return out
