"""Irregular point sets and the two-material composite workload.

PeriPy reads its irregular meshes from files (``peripy/model.py:481-503``);
for synthetic runs this module draws a seeded Poisson-disk point set
(random sequential addition: candidates uniform in the box, each accepted
when it lies farther than the minimum spacing from every point accepted
before it) and builds the bond families, bond types and n-linear damage
tables of a two-material plate on it.
"""
import numpy as np

from .model import build_family, neighbour_pairs


def _cell_offsets(reach):
    """Offsets (d0, d1, d2) of grid cells that can hold a point closer than
    the spacing, for cells of edge spacing/sqrt(3): along an axis two such
    cells are at least (|d| - 1) * cell apart."""
    r = np.arange(-reach, reach + 1)
    d = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    gap = np.maximum(np.abs(d) - 1, 0)
    return d[(gap * gap).sum(1) < 3]


def poisson_disk(lo, hi, spacing, count, seed, batch=200_000):
    """``count`` points in the box ``[lo, hi)`` with pairwise distances
    greater than ``spacing``: random sequential addition of uniform
    candidates, deterministic for a given ``seed``.

    Candidates come in batches; a candidate is kept when no earlier point
    (accepted in a previous batch, or kept earlier in its own batch) lies
    within ``spacing``.  The result is the same as testing the candidate
    stream one by one.

    :raises ValueError: when ``count`` points do not fit (the box is close
        to jammed: acceptance fell below 1e-3).
    """
    from scipy.spatial import cKDTree
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    ext = hi - lo
    rng = np.random.default_rng(seed)
    cell = spacing / np.sqrt(3.0)  # a cell holds at most one point
    dims = np.maximum(np.ceil(ext / cell).astype(np.int64), 1)
    grid = np.full(int(dims.prod()), -1, dtype=np.int32)
    strides = np.array([dims[1] * dims[2], dims[2], 1], dtype=np.int64)
    offsets = _cell_offsets(2)
    pts = np.empty((count, 3))
    n = 0
    r2 = spacing * spacing
    while n < count:
        m = int(min(batch, max(1000, 4 * (count - n))))
        cand = lo + rng.random((m, 3)) * ext
        c = np.minimum(((cand - lo) / cell).astype(np.int64), dims - 1)
        ok = np.ones(m, dtype=bool)
        for off in offsets:
            nb = c + off
            inside = np.all((nb >= 0) & (nb < dims), axis=1)
            owner = np.full(m, -1, dtype=np.int64)
            owner[inside] = grid[nb[inside] @ strides]
            has = owner >= 0
            d = pts[owner[has]] - cand[has]
            clash = np.zeros(m, dtype=bool)
            clash[has] = (d * d).sum(1) <= r2
            ok &= ~clash
        cand, c = cand[ok], c[ok]
        keep = np.ones(len(cand), dtype=bool)
        if len(cand) > 1:
            pairs = cKDTree(cand).query_pairs(spacing, output_type="ndarray")
            if len(pairs):
                pairs = pairs[np.lexsort((pairs[:, 0], pairs[:, 1]))]
                for a, b in pairs:  # a < b: a's fate is settled first
                    if keep[a]:
                        keep[b] = False
        cand, c = cand[keep][:count - n], c[keep][:count - n]
        if len(cand) < 1e-3 * m and n + len(cand) < count:
            raise ValueError("only {} points with spacing {} fit".format(
                n + len(cand), spacing))
        grid[c @ strides] = np.arange(n, n + len(cand), dtype=np.int32)
        pts[n:n + len(cand)] = cand
        n += len(cand)
    return pts


def nlinear_tables(bond_stiffness, critical_stretch):
    """``(k, s, plus_cs)`` tables of shape (nbond_types, nregimes) for an
    n-linear damage model: ``plus_cs[t, r] = plus_cs[t, r-1] +
    k[t, r-1] s[t, r-1] - k[t, r] s[t, r-1]`` so that the bond force
    ``k s + plus_cs`` is continuous across regimes
    (``peripy/model.py:1056-1069``)."""
    k = np.atleast_2d(np.asarray(bond_stiffness, dtype=np.float64))
    s = np.atleast_2d(np.asarray(critical_stretch, dtype=np.float64))
    if k.shape != s.shape:
        raise ValueError("bond_stiffness and critical_stretch differ in shape")
    c = np.zeros_like(k)
    for r in range(1, k.shape[1]):
        c[:, r] = (c[:, r - 1] + k[:, r - 1] * s[:, r - 1]
                   - k[:, r] * s[:, r - 1])
    return k, s, c


def trilinear(c, s0, s1, sc):
    """Stiffness and stretch rows of a trilinear softening bond: linear up
    to ``s0``, constant force ``c s0`` up to ``s1``, then linear decay to
    zero at ``sc`` where the bond breaks."""
    return [c, 0.0, -c * s0 / (sc - s1)], [s0, s1, sc]


def composite(count=1_000_000, box=(2.0, 1.0, 0.1), spacing=0.004,
              horizon_factor=3.0, split=1.0, bulk_moduli=(1e9, 3e9),
              stretches=(0.004, 0.006, 0.01), density=2400.0, seed=5,
              context=None):
    """The irregular composite plate: ``count`` Poisson-disk points in
    ``box``, numbered along a Z-order curve, horizon ``horizon_factor *
    spacing``, node volume box/count.

    Bond types: 0 when both ends lie at x < ``split`` (bulk modulus
    ``bulk_moduli[0]``), 1 when both lie at x >= ``split``
    (``bulk_moduli[1]``), 2 across the interface (micro-modulus the
    harmonic mean of the two).  Every type has the trilinear damage of
    :func:`trilinear` with ``stretches``.  The faces x < horizon and
    x > box_x - horizon carry displacement BCs -1 and +1 along x.  With a
    :class:`~.integrators.CUDAContext` the families are built on its GPU.

    :returns: dict of the arrays ``Integrator.build``/``create_buffers``
        take (``coords``, ``volume``, ``family``, ``nlist``, ``n_neigh``,
        ``max_neigh``, ``bond_types``, ``bond_stiffness``,
        ``critical_stretch``, ``plus_cs``, ``nregimes``, ``nbond_types``,
        ``bc_types``, ``bc_values``, ``densities``, ``horizon``).
    """
    horizon = horizon_factor * spacing
    coords = poisson_disk((0.0, 0.0, 0.0), box, spacing, count, seed)
    # number the points along a Z-order curve (random sequential addition
    # leaves them in random order; a mesher numbers nodes coherently)
    from .ordering import morton_order
    coords = coords[morton_order(coords, cell=spacing)]
    n = coords.shape[0]
    if context is not None:
        from .neighbours import neighbour_family
        family, nlist, max_neigh = neighbour_family(coords, horizon, context)
    else:
        family, nlist, max_neigh = build_family(
            n, neighbour_pairs(coords, horizon))
    valid = nlist != -1
    j = np.where(valid, nlist, 0)
    left_i = coords[:, 0] < split
    left_j = left_i[j]
    bond_types = np.where(left_i[:, None] & left_j, 0,
                          np.where(~left_i[:, None] & ~left_j, 1, 2))
    bond_types = np.where(valid, bond_types, 0).astype(np.intc)
    c0 = 18.0 * bulk_moduli[0] / (np.pi * horizon ** 4)
    c1 = 18.0 * bulk_moduli[1] / (np.pi * horizon ** 4)
    c2 = 2.0 * c0 * c1 / (c0 + c1)
    rows = [trilinear(cc, *stretches) for cc in (c0, c1, c2)]
    k, s, plus_cs = nlinear_tables([r[0] for r in rows], [r[1] for r in rows])
    bc_types = np.zeros((n, 3), dtype=np.intc)
    bc_values = np.zeros((n, 3))
    for mask, v in ((coords[:, 0] < horizon, -1.0),
                    (coords[:, 0] > box[0] - horizon, 1.0)):
        bc_types[mask, 0] = 1
        bc_values[mask, 0] = v
    return dict(
        coords=coords, volume=np.full(n, np.prod(box) / n), family=family,
        nlist=nlist, n_neigh=family.copy(), max_neigh=int(max_neigh),
        bond_types=bond_types, bond_stiffness=k, critical_stretch=s,
        plus_cs=plus_cs, nregimes=np.intc(k.shape[1]),
        nbond_types=np.intc(k.shape[0]), bc_types=bc_types,
        bc_values=bc_values, densities=np.full((n, 3), density),
        horizon=horizon)
