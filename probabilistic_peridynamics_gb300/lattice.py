"""Synthetic regular lattices, plane cracks and face boundary conditions.

Fast, vectorised set-up of the model arrays for regular lattices, in the
layouts ``Model`` builds (``peripy/model.py:536-597``): the neighbour list
of a lattice is the set of stencil offsets within the horizon, which gives
exactly the neighbour sets of a radius search (distance <= horizon) without
a KD-tree.  Rows are in ascending node order, padded with -1 to the next
power of two (the device-integrator layout).
"""
import numpy as np


def lattice_coords(nx, ny, nz, dx, centered=True):
    """Node coordinates, index ``(ix*ny + iy)*nz + iz`` (z fastest).

    With ``centered`` the nodes sit at cell centres ``(i + 0.5)*dx``.
    """
    off = 0.5 if centered else 0.0
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                             indexing="ij")
    coords = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1)
    return (coords + off) * dx


def stencil(horizon_cells):
    """Integer offsets (a, b, c) != 0 with a^2 + b^2 + c^2 <= h^2."""
    r = int(np.floor(horizon_cells))
    a, b, c = np.meshgrid(np.arange(-r, r + 1), np.arange(-r, r + 1),
                          np.arange(-r, r + 1), indexing="ij")
    off = np.stack([a.ravel(), b.ravel(), c.ravel()], axis=1)
    d2 = np.sum(off * off, axis=1)
    keep = (d2 > 0) & (d2 <= horizon_cells * horizon_cells * (1 + 1e-12))
    return off[keep]


def lattice_family(nx, ny, nz, horizon_cells, pow2=True):
    """Family and neighbour list of a regular lattice.

    :returns: ``(family, nlist, max_neighbours)``; ``nlist`` is
        (n, max_neighbours) int32, rows ascending, padded with -1.
    """
    off = stencil(horizon_cells)
    lin = off[:, 0] * (ny * nz) + off[:, 1] * nz + off[:, 2]
    order = np.argsort(lin, kind="stable")
    off, lin = off[order], lin[order]
    n = nx * ny * nz
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                             indexing="ij")
    ix, iy, iz = ix.ravel(), iy.ravel(), iz.ravel()
    ok = np.ones((n, off.shape[0]), dtype=bool)
    for d, (idx, size) in enumerate(((ix, nx), (iy, ny), (iz, nz))):
        p = idx[:, None] + off[None, :, d]
        ok &= (p >= 0) & (p < size)
    family = ok.sum(axis=1).astype(np.intc)
    fmax = int(family.max())
    width = 1 << (fmax - 1).bit_length() if pow2 else fmax
    nlist = np.full((n, width), -1 if pow2 else 0, dtype=np.intc)
    # compact each row's valid offsets to the front, keeping ascending order
    col = np.cumsum(ok, axis=1) - 1
    rows = np.nonzero(ok)
    nlist[rows[0], col[rows]] = (np.arange(n)[:, None] + lin[None, :])[rows]
    return family, nlist, np.intc(width)


def plane_crack_pairs(coords, nlist, n_neigh, x0, y_max, axis=0,
                      along=1):
    """Bond pairs (i < j) whose segment crosses ``coord[axis] == x0`` at
    ``coord[along] < y_max``.
    """
    n = nlist.shape[0]
    cols = np.arange(nlist.shape[1])[None, :]
    valid = (cols < n_neigh[:, None]) & (nlist != -1)
    i = np.broadcast_to(np.arange(n)[:, None], nlist.shape)[valid]
    j = nlist[valid]
    keep = i < j
    i, j = i[keep], j[keep]
    xi, xj = coords[i, axis], coords[j, axis]
    crosses = (xi - x0) * (xj - x0) < 0
    i, j, xi, xj = i[crosses], j[crosses], xi[crosses], xj[crosses]
    t = (x0 - xi) / (xj - xi)
    yc = coords[i, along] + t * (coords[j, along] - coords[i, along])
    sel = yc < y_max
    return np.stack([i[sel], j[sel]], axis=1)


def remove_pairs(pairs, nlist, n_neigh, context=None):
    """``create_crack`` for many pairs: on the GPU of ``context`` when one
    is given (:func:`.neighbours.create_crack`), else on the host.

    Both produce the neighbour list of applying ``peripy/create_crack.pyx``
    pair by pair: each row is compacted with the swap-remove rule in pair
    order.
    """
    if context:
        from .neighbours import create_crack as crack_on_gpu
        crack_on_gpu(pairs, nlist, n_neigh, context)
    else:
        from .model import create_crack
        create_crack(pairs, nlist, n_neigh)


def face_bcs(coords, axis=0, tol=None):
    """Pull the min face by -1 and the max face by +1 along ``axis``.

    :returns: ``(bc_types, bc_values)`` (n, 3).
    """
    n = coords.shape[0]
    lo, hi = coords[:, axis].min(), coords[:, axis].max()
    if tol is None:
        tol = 1e-9 * max(1.0, abs(hi - lo))
    bc_types = np.zeros((n, 3), dtype=np.intc)
    bc_values = np.zeros((n, 3))
    for mask, v in ((coords[:, axis] <= lo + tol, -1.0),
                    (coords[:, axis] >= hi - tol, 1.0)):
        bc_types[mask, axis] = 1
        bc_values[mask, axis] = v
    return bc_types, bc_values


def bond_stiffness_pmb(bulk_modulus, horizon):
    """Micro-modulus ``c = 18 K / (pi delta^4)`` of 3-D PMB."""
    return 18.0 * bulk_modulus / (np.pi * horizon ** 4)
