"""Inputs of the reference's 2113-node plate regression tests.

Restates the setup of ``peripy/test/conftest.py:23-63`` and
``peripy/test/test_integrators.py:10-104``: the mesh, volume and basic CL
connectivity come from the golden fixture; the crack is the pairs selected
by the reference's ``is_crack`` predicate, removed with ``create_crack``;
the displacement boundary pulls ``x < 0.15`` by -1 and ``x > 0.85`` by +1
along x with y and z clamped; horizon 0.1, ``k = 18*0.05/(pi*0.1**4)``,
``s0 = 0.005``, ``dt = 1e-3`` and ``disp_mag[n] = 5e-6*(n+1)``.
"""
import numpy as np

HORIZON = 0.1
BOND_STIFFNESS = 18.0 * 0.05 / (np.pi * 0.1 ** 4)
CRITICAL_STRETCH = 0.005
DT = 1e-3
STEPS = 10
DISP_MAGS = 0.00001 / 2 * np.linspace(1, 10, 10)


def is_crack(x, y):
    """The reference regression crack predicate (conftest.py:43-63)."""
    crack_length = 0.3
    output = 0
    p1 = x
    p2 = y
    if x[0] > y[0]:
        p2 = x
        p1 = y
    if p1[0] < 0.5 + 1e-6 and p2[0] > 0.5 + 1e-6:
        m = (p2[1] - p1[1]) / (p2[0] - p1[0])
        c = p1[1] - m * p1[0]
        height = m * 0.5 + c
        if (height > 0.5 * (1 - crack_length)
                and height < 0.5 * (1 + crack_length)):
            output = 1
    return output


def is_displacement_boundary(x):
    """The reference regression displacement boundary (conftest.py:26-39)."""
    bnd = [None, None, None]
    if x[0] < 1.5 * 0.1:
        bnd[0] = -1
        bnd[1] = 0
        bnd[2] = 0
    elif x[0] > 1.0 - 1.5 * 0.1:
        bnd[0] = 1
        bnd[1] = 0
        bnd[2] = 0
    return bnd


def is_density(x):
    """Unit density (test_integrators.py:35-37)."""
    return 1.0


def crack_pairs(coords, nlist, n_neigh):
    """Pairs (i < j) crossing the crack, in row order."""
    out = []
    for i in range(nlist.shape[0]):
        for j in nlist[i][:n_neigh[i]]:
            if i < j and is_crack(coords[i], coords[j]):
                out.append((i, int(j)))
    return out


def plate_inputs(golden):
    from probabilistic_peridynamics_gb300.model import create_crack
    coords = golden["points"]
    nnodes = coords.shape[0]
    nlist = golden["nlist_basic"].astype(np.intc).copy()
    n_neigh = golden["n_neigh_basic"].astype(np.intc).copy()
    family = n_neigh.copy()
    create_crack(np.array(crack_pairs(coords, nlist, n_neigh)), nlist,
                 n_neigh)
    bc_types = np.zeros((nnodes, 3), dtype=np.intc)
    bc_values = np.zeros((nnodes, 3))
    for i in range(nnodes):
        for d, v in enumerate(is_displacement_boundary(coords[i])):
            if v is not None:
                bc_types[i, d] = 1
                bc_values[i, d] = v
    return dict(coords=coords, volume=golden["volume"], family=family,
                nlist=nlist, n_neigh=n_neigh, bc_types=bc_types,
                bc_values=bc_values,
                force_bc_types=np.zeros((nnodes, 3), dtype=np.intc),
                force_bc_values=np.zeros((nnodes, 3)),
                densities=np.ones((nnodes, 3)), nnodes=nnodes,
                max_neigh=nlist.shape[1])
