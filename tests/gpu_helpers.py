"""Helpers shared by the GPU tests: synthetic lattices and runners."""
import numpy as np

from oracle import cl_step


def lattice(nx, ny, nz, dx, horizon_factor=3.015):
    """Regular lattice r0 = dx*(i, j, k), z fastest; volume dx**3.

    Returns coords, volume, horizon, family, nlist (CL layout) and n_neigh.
    """
    from probabilistic_peridynamics_gb300.model import (build_family,
                                                        neighbour_pairs)
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                             indexing="ij")
    coords = dx * np.stack([ii.ravel(), jj.ravel(), kk.ravel()],
                           axis=1).astype(np.float64)
    horizon = horizon_factor * dx
    pairs = neighbour_pairs(coords, horizon)
    family, nlist, _ = build_family(coords.shape[0], pairs, pow2=True)
    volume = np.full(coords.shape[0], dx ** 3)
    return coords, volume, horizon, family, nlist, family.copy()


def pull_bcs(coords, axis=0, width=None):
    """Pull the min face by -1 and the max face by +1 along ``axis``."""
    n = coords.shape[0]
    lo, hi = coords[:, axis].min(), coords[:, axis].max()
    if width is None:
        width = 1e-9
    bc_types = np.zeros((n, 3), dtype=np.intc)
    bc_values = np.zeros((n, 3))
    left = coords[:, axis] <= lo + width
    right = coords[:, axis] >= hi - width
    bc_types[left, axis] = 1
    bc_values[left, axis] = -1.0
    bc_types[right, axis] = 1
    bc_values[right, axis] = 1.0
    return bc_types, bc_values


def run_integrator(integ, setup, steps, disp_mags, force_mags=None,
                   use_run=False, bond_stiffness=None, critical_stretch=None,
                   plus_cs=None, nregimes=1, nbond_types=1, regimes=None):
    """build + create_buffers + steps + write through the Integrator API."""
    n = setup["nnodes"]
    integ.build(n, 3, setup["max_neigh"], setup["coords"], setup["volume"],
                setup["family"], setup["bc_types"], setup["bc_values"],
                setup["force_bc_types"], setup["force_bc_values"],
                setup.get("stiffness_corrections"), setup.get("bond_types"),
                setup.get("densities"))
    z = lambda: np.zeros((n, 3))  # noqa: E731
    u, ud, udd, force, body = z(), z(), z(), z(), z()
    damage = np.zeros(n)
    nlist = setup["nlist"].copy()
    n_neigh = setup["n_neigh"].copy()
    integ.create_buffers(
        nlist, n_neigh,
        setup["k"] if bond_stiffness is None else bond_stiffness,
        setup["s0"] if critical_stretch is None else critical_stretch,
        plus_cs, u, ud, udd, force, body, damage, regimes, nregimes,
        nbond_types)
    if force_mags is None:
        force_mags = np.zeros(steps)
    if use_run:
        integ._run(disp_mags, force_mags, 0, steps)
    else:
        for k in range(steps):
            integ(disp_mags[k], force_mags[k])
    return integ.write(u, ud, udd, force, body, damage, nlist, n_neigh)


def run_oracle(kind, setup, steps, disp_mags, force_mags=None, damping=0.0,
               dt=None, bond_stiffness=None, critical_stretch=None,
               plus_cs=None, nregimes=1):
    st = cl_step.Stepper(
        kind, setup["dt"] if dt is None else dt, setup["coords"],
        setup["volume"], setup["family"], setup["nlist"], setup["bc_types"],
        setup["bc_values"], setup["force_bc_types"],
        setup["force_bc_values"],
        setup["k"] if bond_stiffness is None else bond_stiffness,
        setup["s0"] if critical_stretch is None else critical_stretch,
        damping=damping,
        densities=None if kind == "euler" else setup["densities"],
        stiffness_corrections=setup.get("stiffness_corrections"),
        bond_types=setup.get("bond_types"), plus_cs=plus_cs,
        nregimes=nregimes)
    if force_mags is None:
        force_mags = np.zeros(steps)
    for k in range(steps):
        st.step(disp_mags[k], force_mags[k])
    return st.write()


def rel_err(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def breaking_setup(kind, nx=10, ny=8, nz=4):
    """A lattice whose pulled faces break bonds within tens of steps
    (k 0.01, s0 0.02; densities 50 for the dynamic integrators)."""
    coords, volume, horizon, family, nlist, n_neigh = lattice(nx, ny, nz,
                                                              1.0)
    bc_types, bc_values = pull_bcs(coords, 0)
    n = coords.shape[0]
    return dict(coords=coords, volume=volume, family=family, nlist=nlist,
                n_neigh=n_neigh, bc_types=bc_types, bc_values=bc_values,
                force_bc_types=np.zeros((n, 3), dtype=np.intc),
                force_bc_values=np.zeros((n, 3)),
                densities=None if kind == "euler" else np.full((n, 3), 50.0),
                nnodes=n, max_neigh=nlist.shape[1], k=0.01, s0=0.02,
                dt=0.5 if kind == "euler" else 1.0)
