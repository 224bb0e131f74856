"""Seeded crack lists for the ``create_crack`` parity tests.

Each case is ``(crack, nlist, n_neigh)`` on a small lattice in the CL
layout (ascending rows, ``-1`` padding to a power of two), with a crack
list that exercises the sequential semantics of
``peripy/create_crack.pyx:1-43``: many removals in one row (the row's
order after a swap-remove decides where later removals land), repeated
and reversed pairs, pairs that are not bonded, ``i == j``, negative
indices (the reference's memoryviews count the row from the end but look
for the other index as given, so such a pair removes nothing) and every
bond of some nodes.
"""
import numpy as np


def lattice_rows(nx, ny, nz, horizon_cells):
    from probabilistic_peridynamics_gb300 import lattice
    family, nlist, _ = lattice.lattice_family(nx, ny, nz, horizon_cells,
                                              pow2=True)
    return nlist.astype(np.intc), family.astype(np.intc).copy()


def _bonds(nlist, n_neigh):
    n = nlist.shape[0]
    cols = np.arange(nlist.shape[1])[None, :]
    valid = cols < n_neigh[:, None]
    i = np.broadcast_to(np.arange(n)[:, None], nlist.shape)[valid]
    return np.stack([i, nlist[valid]], axis=1)


def crack_cases(case):
    rng = np.random.default_rng(1000 + case)
    dims = [(8, 7, 6, 2.2), (10, 9, 4, 3.015), (6, 6, 6, 1.5),
            (12, 5, 5, 2.6), (9, 9, 3, 3.015), (5, 5, 5, 2.2)][case % 6]
    nlist, n_neigh = lattice_rows(*dims)
    n = nlist.shape[0]
    bonds = _bonds(nlist, n_neigh)
    pick = bonds[rng.choice(len(bonds), size=len(bonds) // 5,
                            replace=False)]
    parts = [pick]
    parts.append(pick[rng.choice(len(pick), size=40)][:, ::-1])  # reversed
    parts.append(pick[rng.choice(len(pick), size=40)])          # repeated
    parts.append(rng.integers(0, n, size=(60, 2)))              # unbonded
    same = rng.integers(0, n, size=12)
    parts.append(np.stack([same, same], axis=1))                # i == j
    neg = bonds[rng.choice(len(bonds), size=30)]
    parts.append(neg - n)                                       # negative
    for node in rng.choice(n, size=3, replace=False):           # all bonds
        row = nlist[node, :n_neigh[node]]
        parts.append(np.stack([np.full(row.size, node), row], axis=1))
    crack = np.concatenate(parts)
    crack = crack[rng.permutation(len(crack))]
    return (np.ascontiguousarray(crack, dtype=np.intc), nlist.copy(),
            n_neigh.copy())
