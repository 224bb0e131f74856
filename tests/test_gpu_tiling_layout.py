"""The tiled layout built on the device, against a NumPy construction of
the same layout (GPU).  Integer and index work: every array must be equal.

From the reference neighbour list, a node order and a cut into tiles, the
layout is fully determined (pp_gb300.h, pp_tiling): per tile the ascending
set of its nodes and of every valid neighbour of them (internal indices),
the halo index of its first node, its reference point (the middle of its
nodes' fixed-point bounding box); per node a row of its valid slots in slot
order, rounded up to 16 entries, entry p = 16m + 8h + l stored at 16m + 2l
+ h, holding 16 x the neighbour's halo index (padding: the node's own),
the reference slot (padding 0xFF), and the bond type, regime and
correction of the slot.  After bonds are broken on the device, export
writes -1 exactly at the broken slots.
"""
import ctypes

import numpy as np
import pytest

from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


def _expected(nlist, perm, tile_start, q, extra):
    n, L = nlist.shape
    inv = np.empty(n, dtype=np.int64)
    inv[perm] = np.arange(n)
    halos, own, refs = [], [], []
    for t in range(len(tile_start) - 1):
        a, b = tile_start[t], tile_start[t + 1]
        nodes = set(range(a, b))
        for i in range(a, b):
            row = nlist[perm[i]]
            nodes |= set(inv[row[(row >= 0) & (row < n)]].tolist())
        h = np.array(sorted(nodes), dtype=np.int64)
        halos.append(h)
        own.append(int(np.searchsorted(h, a)))
        qq = q[perm[a:b]]
        refs.append(((qq.min(axis=0).astype(np.int64) +
                      qq.max(axis=0)) >> 1))
    counts = np.array([np.count_nonzero((nlist[perm[i]] >= 0) &
                                        (nlist[perm[i]] < n))
                       for i in range(n)])
    row_off = np.r_[0, np.cumsum((counts + 15) // 16)]
    size = 16 * row_off[-1]
    entry = np.zeros(size, dtype=np.int64)
    slot = np.zeros(size, dtype=np.int64)
    cols = {k: np.zeros(size, dtype=v.dtype) for k, v in extra.items()}
    tile_of = np.searchsorted(tile_start, np.arange(n), side="right") - 1
    for i in range(n):
        t = tile_of[i]
        self_e = 16 * (own[t] + i - tile_start[t])
        row = nlist[perm[i]]
        valid = np.flatnonzero((row >= 0) & (row < n))
        base = 16 * row_off[i]
        for p in range(16 * (row_off[i + 1] - row_off[i])):
            pos = base + 16 * (p >> 4) + 2 * (p & 7) + ((p >> 3) & 1)
            if p < len(valid):
                s = valid[p]
                entry[pos] = 16 * np.searchsorted(halos[t], inv[row[s]])
                slot[pos] = s
                for k, v in extra.items():
                    cols[k][pos] = v[perm[i], s]
            else:
                entry[pos] = self_e
                slot[pos] = 0xFF
    return halos, own, refs, row_off, entry, slot, cols


def _build(w, tiled_cls_args, corrections=None, types=False, order=None):
    import probabilistic_peridynamics_gb300 as pp
    cls, args = tiled_cls_args
    integ = cls(*args, precision="mixed", autotune=False)
    n = w["nnodes"]
    integ.build(n, 3, w["max_neigh"], w["coords"], w["volume"], w["family"],
                w["bc_types"], w["bc_values"], w["force_bc_types"],
                w["force_bc_values"], corrections,
                w.get("bond_types") if types else None, w.get("densities"))
    if order is not None:
        integ._order = order
    z = np.zeros((n, 3))
    if types:
        integ.create_buffers(w["nlist"], w["n_neigh"], w["bond_stiffness"],
                             w["critical_stretch"], w["plus_cs"], z, z, z, z,
                             z, np.zeros(n), w["regimes"], w["nregimes"],
                             w["nbond_types"])
    else:
        integ.create_buffers(w["nlist"], w["n_neigh"], w["k"], w["s0"], None,
                             z, z, z, z, z, np.zeros(n), None, 1, 1)
    return integ


def _check(integ, w, extra):
    t = integ.tiling
    perm = t.perm.astype(np.int64)
    ts = t.tile_start.astype(np.int64)
    n = w["nnodes"]
    # fixed-point positions as pp_mixed_pack forms them
    q = np.rint((w["coords"] - np.asarray(integ.pos_origin)) /
                integ.pos_scale).astype(np.int64)
    halos, own, refs, row_off, entry, slot, cols = _expected(
        w["nlist"], perm, ts, q, extra)
    cap = t.halo_cap
    hd = t.halo_d.cpu().numpy().reshape(-1, cap)
    hc = t.halo_count_d.cpu().numpy()
    for k, h in enumerate(halos):
        assert hc[k] == len(h)
        assert np.array_equal(hd[k, :len(h)], h)
    assert np.array_equal(t.own_off_d.cpu().numpy()[:len(own)], own)
    refd = t.tile_ref_d.cpu().numpy().reshape(-1, 4)
    assert np.array_equal(refd[:len(refs), :3], np.array(refs))
    assert np.array_equal(t.row_off_d.cpu().numpy(), row_off)
    e = t.entry_d.cpu().numpy().view(np.uint16)[:len(entry)]
    assert np.array_equal(e, entry)
    sl = t.slot_d.cpu().numpy()[:len(slot)]
    assert np.array_equal(sl, slot)
    if "bond_types" in cols:
        assert np.array_equal(t.bond_type_d.cpu().numpy()[:len(slot)],
                              cols["bond_types"])
        assert np.array_equal(t.regime_d.cpu().numpy()[:len(slot)],
                              cols["regimes"])
    if "corrections" in cols:
        assert np.array_equal(t.correction_d.cpu().numpy()[:len(slot)],
                              cols["corrections"].astype(np.float32))
    counts = [np.count_nonzero(w["nlist"][perm[i]] >= 0) for i in range(n)]
    assert np.array_equal(t.n_neigh_d.cpu().numpy()[:n], counts)
    return entry, slot, row_off, own, perm, ts


def test_lattice_layout_and_export():
    """A lattice with stiffness corrections, the brick order; then bonds
    broken by the step: export writes -1 exactly where the entries now
    hold the node's own entry."""
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300 import batch
    from tests.gpu_helpers import breaking_setup
    w = breaking_setup("velocity_verlet", 12, 10, 6)
    corr = batch.pair_noise(w["nlist"], 0.9, 1.1, 7)
    cls = (pp.VelocityVerletCUDA, (0.5, 1.0))
    integ = _build(w, cls, corrections=corr)
    entry, slot, row_off, own, perm, ts = _check(
        integ, w, {"corrections": corr})
    steps = 40
    integ._run(3e-3 * np.arange(1, steps + 1), np.zeros(steps), 0, steps)
    n = w["nnodes"]
    z = [np.zeros((n, 3)) for _ in range(5)]
    out = integ.write(*z, np.zeros(n), w["nlist"].copy(),
                      w["n_neigh"].copy())
    e_now = integ.tiling.entry_d.cpu().numpy().view(np.uint16)
    want = w["nlist"].copy()
    tile_of = np.searchsorted(ts, np.arange(n), side="right") - 1
    for i in range(n):
        self_e = 16 * (own[tile_of[i]] + i - ts[tile_of[i]])
        lo, hi = 16 * row_off[i], 16 * row_off[i + 1]
        for pos in range(lo, hi):
            if slot[pos] != 0xFF and e_now[pos] == self_e:
                want[perm[i], slot[pos]] = -1
    assert np.array_equal(out[6], want)
    assert np.count_nonzero(want == -1) > np.count_nonzero(w["nlist"] == -1)


def test_composite_layout_with_types_and_a_random_order():
    """Bond types and regimes (nonzero regimes given), a random node order
    and tiles of 1 to 37 nodes."""
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300.pointset import composite
    w = composite(count=1500, box=(0.16, 0.08, 0.04), split=0.08, seed=3)
    n = w["coords"].shape[0]
    rng = np.random.default_rng(1)
    regimes = np.where(w["nlist"] >= 0, rng.integers(0, 3, w["nlist"].shape),
                       0).astype(np.intc)
    w.update(nnodes=n, force_bc_types=np.zeros((n, 3), dtype=np.intc),
             force_bc_values=np.zeros((n, 3)), regimes=regimes)
    perm = rng.permutation(n).astype(np.int32)
    cuts = np.unique(np.r_[0, np.cumsum(rng.integers(1, 38, n)), n])
    ts = cuts[cuts <= n].astype(np.int32)
    cls = (pp.VelocityVerletCUDA, (2.5e6, 1e-6))
    integ = _build(w, cls, types=True, order=(perm, ts))
    _check(integ, w, {"bond_types": w["bond_types"], "regimes": regimes})
