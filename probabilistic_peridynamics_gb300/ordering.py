"""Node orderings for gather locality.

The fused step gathers each neighbour's position and displacement; nodes
that are close in space should be close in memory so that a CTA's
neighbourhoods share L1 lines.  A Morton (Z-order) key on a uniform grid
gives that for any point set; numbering nodes by it changes no arithmetic of
the step (each node still sums its own bonds in slot order).
"""
import numpy as np


def _spread3(v):
    """Spread the low 21 bits of ``v`` so that bit k lands at bit 3k."""
    v = v.astype(np.uint64) & np.uint64(0x1FFFFF)
    v = (v | (v << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
    v = (v | (v << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
    v = (v | (v << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
    v = (v | (v << np.uint64(2))) & np.uint64(0x1249249249249249)
    return v


def morton_keys(coords, cell):
    """Z-order keys of ``coords`` on a grid of spacing ``cell``."""
    coords = np.asarray(coords, dtype=np.float64)
    q = np.floor((coords - coords.min(axis=0)) / cell).astype(np.int64)
    if q.size and q.max() >= 1 << 21:
        raise ValueError("grid too fine for 21-bit Morton keys")
    return (_spread3(q[:, 0]) << np.uint64(2)) | \
        (_spread3(q[:, 1]) << np.uint64(1)) | _spread3(q[:, 2])


def morton_order(coords, cell=None, groups=None):
    """Permutation ``order`` (new -> old) that numbers nodes along a Z-order
    curve; ``coords[order]`` are the renumbered positions.

    :arg cell: grid spacing (default: the extent / 2**20 of the widest axis,
        fine enough that few nodes share a cell).
    :arg groups: optional integer label per node (e.g. the instance of a
        batched model); nodes are kept grouped by it, in ascending label
        order, and ordered along the curve within each group.
    """
    coords = np.asarray(coords, dtype=np.float64)
    n = coords.shape[0]
    if n == 0:
        return np.zeros(0, dtype=np.int64)
    if cell is None:
        ext = float(np.max(coords.max(axis=0) - coords.min(axis=0)))
        cell = ext / (1 << 20) if ext > 0 else 1.0
    keys = morton_keys(coords, cell)
    if groups is None:
        return np.argsort(keys, kind="stable")
    return np.lexsort((keys, np.asarray(groups)))


def inverse(order):
    """Inverse permutation (old -> new)."""
    inv = np.empty_like(order)
    inv[order] = np.arange(order.size, dtype=order.dtype)
    return inv


def permute_nlist(nlist, order, inv):
    """Rows of ``nlist`` in the new numbering: row r is old row order[r]
    with every neighbour index relabelled old -> new; -1 stays -1 and the
    slot order within each row is kept."""
    rows = nlist[order]
    return np.where(rows >= 0, inv[np.where(rows >= 0, rows, 0)],
                    rows).astype(nlist.dtype)
