"""Tiled layout of the mixed-precision step (``pp_tiling`` in the C ABI).

The mixed step gathers, for every bond, the record (position, weight,
displacement) of the neighbour.  On the tiled layout a CTA copies the
records of a whole tile's neighbourhood (its *halo*) into shared memory once
and gathers every bond of the tile from there; rows hold 16-bit indices into
the halo.  The nodes are renumbered internally for this: :func:`brick_order`
sorts them into spatial bricks of about ``target`` nodes and cuts the order
into tiles of at most ``PP_TILE_NODES_MAX`` nodes.  Results do not depend on
the ordering (each node still sums its own bonds in slot order); the
ordering only decides how large the halos are.

:class:`DeviceTiling` holds the device arrays of one tiling and builds them
from the reference neighbour list (``pp_tile_halos``, ``pp_tile_rows``),
splitting any tile whose halo exceeds the capacity.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib

TILE_NODES_MAX = 128
#: Halo capacity per tile: 32 bytes of shared memory per record, 24 KB per
#: CTA, so that eight CTAs of 128 threads fit on an SM (a tile whose halo is
#: longer is split).
HALO_CAP = 768


def brick_order(coords, segments=None, target=125, max_nodes=TILE_NODES_MAX):
    """Internal node order and tile boundaries.

    Nodes are binned into cubic bricks whose edge gives ``target`` nodes at
    the mean density (per segment: nodes of different segments, e.g. the
    instances of a batch, never share a brick), sorted brick by brick
    (stable: reference order within a brick), and cut into tiles of whole
    bricks while they fit ``max_nodes``; a larger brick is split evenly.

    :returns: ``(perm, tile_start)``: ``perm[i]`` is the reference node of
        internal node ``i``; tile ``t`` is ``[tile_start[t],
        tile_start[t+1])``.
    """
    coords = np.asarray(coords, dtype=np.float64)
    n = coords.shape[0]
    if n == 0:
        return np.zeros(0, dtype=np.int32), np.zeros(1, dtype=np.int32)
    seg = (np.zeros(n, dtype=np.int64) if segments is None
           else np.asarray(segments, dtype=np.int64))
    _, seg = np.unique(seg, return_inverse=True)
    nseg = int(seg.max()) + 1
    lo = np.full((nseg, 3), np.inf)
    hi = np.full((nseg, 3), -np.inf)
    np.minimum.at(lo, seg, coords)
    np.maximum.at(hi, seg, coords)
    ext = hi - lo
    # brick edge from the mean density over the dimensions that have extent
    scale = max(float(ext.max()), 1e-300)
    live = ext.max(axis=0) > 1e-9 * scale
    d = int(live.sum())
    if d == 0:
        edge = 1.0
        spacing = 1.0
    else:
        # each node fills about one spacing: the bounding boxes grown by a
        # spacing per live dimension (a few fixed-point rounds)
        spacing = 0.0
        for _ in range(4):
            vol = float(np.sum(np.prod(np.where(live, ext + spacing, 1.0),
                                       axis=1)))
            spacing = (vol / n) ** (1.0 / d)
        edge = (target * vol / n) ** (1.0 / d)
    # half a spacing of offset keeps lattice nodes away from brick faces
    rel = (coords - lo[seg] + 0.5 * spacing) / edge
    b = np.floor(rel).astype(np.int64)
    b[:, ~live] = 0
    dims = b.max(axis=0) + 1
    key = ((seg * dims[0] + b[:, 0]) * dims[1] + b[:, 1]) * dims[2] + b[:, 2]
    perm = np.argsort(key, kind="stable")
    sorted_key = key[perm]
    starts = np.flatnonzero(np.r_[True, sorted_key[1:] != sorted_key[:-1]])
    counts = np.diff(np.r_[starts, n])
    bounds = [0]
    acc = 0
    for c in counts.tolist():
        if c > max_nodes:
            if acc:
                bounds.append(bounds[-1] + acc)
                acc = 0
            parts = -(-c // max_nodes)
            base = bounds[-1]
            for k in range(1, parts + 1):
                bounds.append(base + (c * k) // parts)
        elif acc + c > max_nodes:
            bounds.append(bounds[-1] + acc)
            acc = c
        else:
            acc += c
    if acc:
        bounds.append(bounds[-1] + acc)
    return perm.astype(np.int32), np.asarray(bounds, dtype=np.int32)


def split_tiles(tile_start, tiles):
    """Halve each tile of ``tiles`` (indices into ``tile_start``)."""
    ts = tile_start.astype(np.int64)
    mids = [(ts[t] + ts[t + 1]) // 2 for t in tiles if ts[t + 1] - ts[t] > 1]
    return np.unique(np.r_[ts, mids]).astype(np.int32)


class DeviceTiling:
    """Device arrays of one tiling (see ``pp_tiling``).

    :arg perm, tile_start: from :func:`brick_order`.
    :arg device: torch device.
    """

    def __init__(self, perm, tile_start, device, halo_cap=None):
        import torch
        self._torch = torch
        self.device = device
        self.halo_cap = int(HALO_CAP if halo_cap is None else halo_cap)
        self.perm = np.ascontiguousarray(perm, dtype=np.int32)
        self.tile_start = np.ascontiguousarray(tile_start, dtype=np.int32)
        n = self.perm.size
        inv = np.empty(n, dtype=np.int32)
        inv[self.perm] = np.arange(n, dtype=np.int32)
        self.perm_d = torch.from_numpy(self.perm).to(device)
        self.inv_d = torch.from_numpy(inv).to(device)
        self.struct = _lib.Tiling()
        self.splits = 0

    def _t(self, shape, dtype):
        return self._torch.empty(shape, dtype=dtype, device=self.device)

    def build(self, fargs, stream, corrections=False, types=False,
              instances=False, max_rounds=12):
        """Fill the tiling from the reference arrays of ``fargs`` (a
        ``FusedArgs`` with nnodes, max_neigh, nlist, r0, bc_values,
        fc_values and, as present, bond_types/regimes,
        stiffness_corrections, node_instance set); the step is queued on
        ``stream`` (a handle) and the call waits for it."""
        torch = self._torch
        n = int(fargs.nnodes)
        s = self.struct
        i32 = torch.int32
        for _ in range(max_rounds):
            nt = self.tile_start.size - 1
            self.tile_start_d = torch.from_numpy(self.tile_start).to(
                self.device)
            self.halo_d = self._t((max(nt, 1) * self.halo_cap,), i32)
            self.halo_count_d = self._t((max(nt, 1),), i32)
            self.own_off_d = self._t((max(nt, 1),), i32)
            self.tile_ref_d = self._t((max(nt, 1) * 4,), i32)
            self.row_off_d = self._t((n + 1,), i32)
            self.n_neigh_d = self._t((max(n, 1),), i32)
            self.sched_d = torch.zeros(2, dtype=i32, device=self.device)
            self.r0_d = self._t((max(n, 1), 3), torch.float64)
            self.bc_values_d = self._t((max(n, 1), 3), torch.float64)
            self.fc_values_d = self._t((max(n, 1), 3), torch.float64)
            self.node_instance_d = (self._t((max(n, 1),), i32) if instances
                                    else None)
            s.ntiles = nt
            s.halo_cap = self.halo_cap
            s.perm = self.perm_d.data_ptr()
            s.inv = self.inv_d.data_ptr()
            s.tile_start = self.tile_start_d.data_ptr()
            s.halo = self.halo_d.data_ptr()
            s.halo_count = self.halo_count_d.data_ptr()
            s.own_off = self.own_off_d.data_ptr()
            s.tile_ref = self.tile_ref_d.data_ptr()
            s.row_off = self.row_off_d.data_ptr()
            s.n_neigh = self.n_neigh_d.data_ptr()
            s.sched = self.sched_d.data_ptr()
            s.r0 = self.r0_d.data_ptr()
            s.bc_values = self.bc_values_d.data_ptr()
            s.fc_values = self.fc_values_d.data_ptr()
            s.node_instance = (self.node_instance_d.data_ptr()
                               if instances else None)
            check(lib().pp_tile_halos(ctypes.byref(fargs), ctypes.byref(s),
                                      stream), "pp_tile_halos")
            counts = self.halo_count_d.cpu().numpy()[:nt]
            over = np.flatnonzero(counts > self.halo_cap)
            if over.size == 0:
                break
            self.tile_start = split_tiles(self.tile_start, over)
            self.splits += int(over.size)
        else:
            raise _lib.LibraryError(
                "tiling: halos still exceed the capacity after splitting")
        blocks = int(self.row_off_d[n].item()) if n else 0
        if blocks < 0:
            raise _lib.LibraryError("tiling: too many neighbour entries")
        entries = 16 * max(blocks, 1)
        self.entry_d = self._t((entries,), torch.int16)
        self.slot_d = self._t((entries,), torch.uint8)
        self.bond_type_d = (self._t((entries,), torch.uint8) if types
                            else None)
        self.regime_d = self._t((entries,), torch.uint8) if types else None
        self.correction_d = (self._t((entries,), torch.float32)
                             if corrections else None)
        s.entry = self.entry_d.data_ptr()
        s.slot = self.slot_d.data_ptr()
        s.bond_type = (self.bond_type_d.data_ptr() if types else None)
        s.regime = self.regime_d.data_ptr() if types else None
        s.correction = (self.correction_d.data_ptr() if corrections
                        else None)
        check(lib().pp_tile_rows(ctypes.byref(fargs), ctypes.byref(s),
                                 stream), "pp_tile_rows")
        self.entries = 16 * blocks
        self.halo_counts = counts
        return self

    def stats(self):
        """Tile and halo sizes (for reports)."""
        sizes = np.diff(self.tile_start)
        h = self.halo_counts
        return {"tiles": int(sizes.size),
                "nodes_per_tile_mean": float(sizes.mean()) if sizes.size
                else 0.0,
                "halo_mean": float(h.mean()) if h.size else 0.0,
                "halo_max": int(h.max()) if h.size else 0,
                "entries": int(self.entries), "splits": self.splits}
