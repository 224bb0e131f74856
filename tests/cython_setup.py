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


def breaking_lattice():
    """A jittered 9x8x5 lattice in the compact layout with shuffled rows,
    node volumes that differ, pulled x faces and a loaded top face (force
    boundary condition), where bonds break in tension and in compression."""
    from probabilistic_peridynamics_gb300.model import (build_family,
                                                        neighbour_pairs)
    from tests.gpu_helpers import pull_bcs
    rng = np.random.default_rng(11)
    nx, ny, nz = 9, 8, 5
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                             indexing="ij")
    coords = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], 1).astype(float)
    coords += rng.uniform(-0.05, 0.05, coords.shape)
    n = coords.shape[0]
    family, nlist, _ = build_family(n, neighbour_pairs(coords, 2.2),
                                    pow2=False)
    # shuffle each row (the KD-tree order of the reference is not sorted)
    for i in range(n):
        nlist[i, :family[i]] = rng.permutation(nlist[i, :family[i]])
    bc_types, bc_values = pull_bcs(coords, 0, width=0.1)
    fct = np.zeros((n, 3), dtype=np.intc)
    fcv = np.zeros((n, 3))
    top = coords[:, 2] > nz - 1.2
    fct[top, 2] = 1
    fcv[top, 2] = -1.0 / max(int(top.sum()), 1)
    return dict(coords=coords, volume=rng.uniform(0.8, 1.2, n),
                family=family, nlist=nlist, n_neigh=family.copy(),
                bc_types=bc_types, bc_values=bc_values, force_bc_types=fct,
                force_bc_values=fcv)


def run_gpu_euler(setup, steps, mags, dt, k, s0, fmags=None, fused=True):
    """The same run through the GPU ``Euler`` (needs a GPU)."""
    import probabilistic_peridynamics_gb300 as pp
    n = setup["coords"].shape[0]
    integ = pp.Euler(dt, fused=fused)
    assert integ.context is None
    integ.build(n, 3, setup["nlist"].shape[1], setup["coords"],
                setup["volume"], setup["family"], setup["bc_types"],
                setup["bc_values"], setup["force_bc_types"],
                setup["force_bc_values"], None, None, None)
    z = lambda: np.zeros((n, 3))  # noqa: E731
    integ.create_buffers(setup["nlist"].astype(np.intc).copy(),
                         setup["n_neigh"].astype(np.intc).copy(), k, s0,
                         None, z(), z(), z(), z(), z(), np.zeros(n), None, 1,
                         1)
    for t in range(steps):
        integ(mags[t], 0.0 if fmags is None else fmags[t])
    u, _, _, force, _, damage, nlist, n_neigh = integ.write(
        None, None, None, None, None, None, None, None)
    return u, force, damage, nlist, n_neigh
