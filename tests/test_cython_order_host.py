"""The two ordering rules the GPU ``Euler`` rests on, checked on the host
against the reference's own compiled functions (``oracle/_ref``), without
the GPU.

* ``break_bonds`` (``peripy/peridynamics.pyx:102-156``) runs over the nodes
  in ascending order, yet the final state of row i is that of (1) the
  removals made by its lower neighbours k < i, in ascending k, then (2) its
  own scan, because whether a bond breaks depends only on positions.
* ``bond_force`` (``peridynamics.pyx:34-99``) gives node i the sequential
  sum from 0 of -f vol[k] over its lower neighbours in ascending k, then
  +f vol[j] over its upper neighbours in row order, then the force
  boundary condition.

Both rules are restated here row by row / node by node in Python floats
(IEEE binary64, ``math.sqrt`` correctly rounded) and must give the
reference's results bit for bit on a lattice where many bonds break in
tension and in compression.
"""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref():
    from oracle import build_ref
    if not build_ref.available():
        build_ref.build(quiet=True)
    if not build_ref.available():
        pytest.skip("reference checkout absent and no generated C")
    return build_ref.load()


def ceuclid(r1, r2):
    d = [(r2[k] - r1[k]) * (r2[k] - r1[k]) for k in range(3)]
    return math.sqrt((d[0] + d[1]) + d[2])


def strain(r, r0, lo, hi):
    l0 = ceuclid(r0[lo], r0[hi])
    return (ceuclid(r[lo], r[hi]) - l0) / l0


def break_rows(r, r0, nlist, n_neigh, s0):
    """Row-local restatement of break_bonds."""
    nl, nn = nlist.copy(), n_neigh.copy()
    for i in range(nl.shape[0]):
        row = list(nl[i])
        cnt = int(nn[i])
        cnt0 = cnt

        def broken(j):
            lo, hi = min(i, j), max(i, j)
            return not (abs(strain(r, r0, lo, hi)) < s0)
        # (1) removals by the lower neighbours, ascending
        for k in sorted(j for j in row[:cnt] if j < i and broken(j)):
            p = row[:cnt].index(k)
            row[p] = row[cnt - 1]
            cnt -= 1
        # (2) the row's own scan
        p = 0
        while p < cnt:
            j = row[p]
            if j > i and broken(j):
                row[p] = row[cnt - 1]
                cnt -= 1
            else:
                p += 1
        nl[i, :cnt0] = row[:cnt0]
        nn[i] = cnt
    return nl, nn


def forces(r, r0, nlist, n_neigh, vol, k, fcv, fct, scale):
    """Node-local restatement of bond_force."""
    n = nlist.shape[0]
    out = np.zeros((n, 3))
    for i in range(n):
        row = [int(j) for j in nlist[i, :n_neigh[i]]]
        order = sorted(j for j in row if j < i) + [j for j in row if j > i]
        acc = [0.0, 0.0, 0.0]
        for j in order:
            lo, hi = min(i, j), max(i, j)
            l = ceuclid(r[lo], r[hi])
            l0 = ceuclid(r0[lo], r0[hi])
            fn = ((l - l0) / l0 * k) / l
            for d in range(3):
                f = fn * (r[hi][d] - r[lo][d])
                acc[d] = acc[d] - f * vol[lo] if j < i else acc[d] + f * vol[j]
        for d in range(3):
            if fct[i, d] != 0:
                acc[d] = acc[d] + scale * fcv[i, d]
        out[i] = acc
    return out


def test_row_and_node_orders_reproduce_the_reference(ref):
    from tests.cython_setup import breaking_lattice
    setup = breaking_lattice()
    coords = setup["coords"]
    nlist = setup["nlist"].astype(np.intc)
    n_neigh = setup["n_neigh"].astype(np.intc)
    rng = np.random.default_rng(4)
    # a displaced state that breaks many bonds, in tension and compression
    u = rng.normal(0.0, 0.02, coords.shape)
    u[:, 0] += 0.03 * coords[:, 0]
    r = coords + u
    s0 = 0.01
    want_nl, want_nn = nlist.copy(), n_neigh.copy()
    ref.break_bonds(r, coords, want_nl, want_nn, s0)
    got_nl, got_nn = break_rows(r, coords, nlist, n_neigh, s0)
    assert int(n_neigh.sum() - want_nn.sum()) > 500
    assert np.array_equal(got_nl, want_nl) and np.array_equal(got_nn, want_nn)
    k = 0.05
    want_f = ref.bond_force(r, coords, want_nl, want_nn, setup["volume"], k,
                            setup["force_bc_values"], setup["force_bc_types"],
                            0.7)
    got_f = forces(r, coords, want_nl, want_nn, setup["volume"], k,
                   setup["force_bc_values"], setup["force_bc_types"], 0.7)
    assert np.array_equal(got_f, want_f)
