"""The reference regression setup in the layout of PeriPy's CPU integrator
``Euler`` (compact rows, 0-padded), and that integrator's step run with the
reference's own compiled functions (``oracle/_ref``): the checker of the
GPU ``Euler`` (``test_gpu_euler_cython.py``), pinned to the Cython-layout
goldens by ``test_oracle_c.py``.
"""
import numpy as np


def cython_plate(golden):
    """The reference regression setup in the Cython integrator's compact
    layout: the golden basic connectivity (KD-tree row order, width 68)
    with the crack cut by ``create_crack`` as ``Model`` cuts it."""
    from probabilistic_peridynamics_gb300.model import create_crack
    from tests.plate_setup import crack_pairs, plate_inputs
    base = plate_inputs(golden)
    nlist = golden["cy_nlist_basic"].astype(np.intc).copy()
    n_neigh = golden["cy_n_neigh_basic"].astype(np.intc).copy()
    family = n_neigh.copy()
    create_crack(np.array(crack_pairs(base["coords"], nlist, n_neigh)),
                 nlist, n_neigh)
    return dict(base, nlist=nlist, n_neigh=n_neigh, family=family,
                densities=None)


def run_reference_euler(ref, setup, steps, mags, dt, k, s0, fmags=None):
    """``Euler.__call__`` (integrators.py:330-349) with the reference's own
    compiled functions, on copies of the setup's arrays."""
    coords = np.ascontiguousarray(setup["coords"], dtype=np.float64)
    nlist = setup["nlist"].astype(np.intc).copy()
    n_neigh = setup["n_neigh"].astype(np.intc).copy()
    u = np.zeros_like(coords)
    force = np.zeros_like(coords)
    for t in range(steps):
        ref.break_bonds(coords + u, coords, nlist, n_neigh, s0)
        force = ref.bond_force(
            coords + u, coords, nlist, n_neigh, setup["volume"], k,
            setup["force_bc_values"], setup["force_bc_types"],
            0.0 if fmags is None else fmags[t])
        ref.update_displacement(u, setup["bc_values"], setup["bc_types"],
                                force, mags[t], dt)
    damage = ref.damage(n_neigh, setup["family"].astype(np.intc))
    return u, force, damage, nlist, n_neigh
