"""Neighbour families on the GPU (model set-up).

PeriPy builds the bond families on the host with a KD-tree
(``peripy/model.py:536-597``, sklearn ``KDTree.query_radius``); for large
models (1M points) that search and the row assembly take seconds to
minutes.  :func:`neighbour_family` builds the same families on the device
(``pp_neighbour_cells`` / ``pp_neighbour_rows``): the nodes are binned into
cubic cells a little wider than the horizon and one warp per node tests the
27 surrounding cells.  The result is the layout ``Model`` hands to
``Integrator.build``: rows in ascending node order, ``-1``-padded to a
power-of-two width for the device integrators, or ``family.max()`` wide and
``0``-padded otherwise (``peripy/model.py:575-585``).
"""
import ctypes

import numpy as np

from ._lib import LibraryError, check, lib

#: Most cells of the binning grid; the cell edge grows beyond the horizon
#: when the bounding box would need more.
MAX_CELLS = 1 << 26


def grid(coords, horizon, max_cells=MAX_CELLS):
    """Corner, cell edge and cell counts of the binning grid.

    The edge is at least ``horizon * (1 + 1e-6)`` (neighbours then lie in
    the 27 cells around a node's own, with room for the rounding of the
    cell coordinates) and is widened until the grid has at most
    ``max_cells`` cells.
    """
    coords = np.asarray(coords, dtype=np.float64)
    lo = coords.min(axis=0)
    ext = coords.max(axis=0) - lo
    cell = max(float(horizon) * (1.0 + 1e-6), 1e-300)
    if not np.all(np.isfinite(ext)) or not np.isfinite(cell):
        raise ValueError("coordinates and horizon must be finite")
    while True:
        dims = np.floor(ext / cell).astype(np.int64) + 1
        if int(np.prod(dims)) <= max_cells:
            return lo, cell, dims.astype(np.int32)
        cell *= 1.26


def neighbour_family(coords, horizon, context=None, pow2=True,
                     max_cells=MAX_CELLS):
    """``(family, nlist, max_neighbours)`` of every node pair closer than
    ``horizon``, built on the GPU.

    Same result as ``model.build_family(n, model.neighbour_pairs(coords,
    horizon), pow2)``: a pair is a neighbour pair when ``(dx*dx + dy*dy) +
    dz*dz <= horizon**2`` in binary64.

    :arg context: a :class:`~.integrators.CUDAContext` (default: device 0).
    :arg bool pow2: ``-1``-padded power-of-two width (device integrators);
        else ``family.max()`` wide, ``0``-padded.
    :arg int max_cells: bound on the binning grid (see :func:`grid`).
    """
    import torch
    from .integrators import CUDAContext
    ctx = context if context is not None else CUDAContext(0)
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    n = coords.shape[0]
    if n == 0:
        width = 1 if pow2 else 0
        return (np.zeros(0, dtype=np.intc),
                np.full((0, width), -1 if pow2 else 0, dtype=np.intc),
                np.intc(width))
    if n > np.iinfo(np.int32).max:
        raise ValueError("too many nodes")
    lo, cell, dims = grid(coords, horizon, max_cells)
    ncells = int(np.prod(dims.astype(np.int64)))
    lo_c = (ctypes.c_double * 3)(*lo)
    dims_c = (ctypes.c_int32 * 3)(*dims)
    dev = ctx.device
    with ctx.on_stream():
        r = torch.as_tensor(coords, device=dev)
        cs = torch.empty(ncells + 1, dtype=torch.int32, device=dev)
        order = torch.empty(n, dtype=torch.int32, device=dev)
        family = torch.empty(n, dtype=torch.int32, device=dev)
        overflow = torch.zeros(1, dtype=torch.int32, device=dev)
        st = ctx.stream_handle
        check(lib().pp_neighbour_cells(r.data_ptr(), n, lo_c, cell, dims_c,
                                       cs.data_ptr(), order.data_ptr(), st),
              "pp_neighbour_cells")
        check(lib().pp_neighbour_rows(r.data_ptr(), n, float(horizon), lo_c,
                                      cell, dims_c, cs.data_ptr(),
                                      order.data_ptr(), 0, None,
                                      family.data_ptr(), None, st),
              "pp_neighbour_rows")
        fmax = int(family.max().item())
        width = 1 << (max(fmax, 1) - 1).bit_length()
        if width > 1024:
            raise LibraryError(
                f"a node has {fmax} neighbours; at most 1024 are supported")
        nlist = torch.empty((n, width), dtype=torch.int32, device=dev)
        check(lib().pp_neighbour_rows(r.data_ptr(), n, float(horizon), lo_c,
                                      cell, dims_c, cs.data_ptr(),
                                      order.data_ptr(), width,
                                      nlist.data_ptr(), family.data_ptr(),
                                      overflow.data_ptr(), st),
              "pp_neighbour_rows")
        if int(overflow.item()) != 0:
            raise LibraryError("neighbour rows overflowed their width")
        family_h = family.cpu().numpy().astype(np.intc)
        nlist_h = nlist.cpu().numpy().astype(np.intc)
    if pow2:
        return family_h, nlist_h, np.intc(width)
    compact = np.ascontiguousarray(nlist_h[:, :fmax])
    compact[compact == -1] = 0
    return family_h, compact, np.intc(fmax)


def crack_device(crack, nlist, n_neigh, context):
    """Apply ``pp_create_crack`` to device tensors in place.

    :arg crack: ``(npairs, 2)`` int32 tensor of node indices in
        ``[-nnodes, nnodes)`` on the context's device (see
        :func:`create_crack` for negative ones).
    :arg nlist: ``(nnodes, max_neigh)`` int32 device tensor, in/out.
    :arg n_neigh: ``(nnodes,)`` int32 device tensor, in/out.
    :raises IndexError: a node index is out of range (nothing is changed).
    """
    import torch
    npairs = int(crack.shape[0])
    if npairs == 0:
        return
    n, width = nlist.shape
    for t in (crack, nlist, n_neigh):
        if t.dtype != torch.int32 or not t.is_contiguous():
            raise TypeError("crack, nlist and n_neigh must be contiguous "
                            "int32 tensors")
    dev = context.device
    with context.on_stream():
        scratch = torch.empty(n + 1 + 4 * npairs, dtype=torch.int32,
                              device=dev)
        bad = torch.empty(1, dtype=torch.int32, device=dev)
        check(lib().pp_create_crack(crack.data_ptr(), npairs, n, width,
                                    nlist.data_ptr(), n_neigh.data_ptr(),
                                    scratch.data_ptr(), bad.data_ptr(),
                                    context.stream_handle),
              "pp_create_crack")
        if int(bad.item()) != 0:
            raise IndexError("crack node index out of range")


def create_crack(crack, nlist, n_neigh, context=None):
    """``peripy.create_crack.create_crack`` on the GPU: remove the bond pairs
    in ``crack`` from the host arrays ``nlist`` and ``n_neigh`` in place.

    Same result as the sequential loop of ``peripy/create_crack.pyx:1-43``:
    for each pair ``(i, j)`` in order, ``j`` is removed from row ``i`` and
    then ``i`` from row ``j``; a removed entry takes the row's last entry,
    whose slot becomes ``-1``.  As with the reference's memoryviews, a
    negative index selects the row counted from the end, but the node
    looked for in the other row is the index as given, which no row holds.
    At the first pair with an index outside ``[-nnodes, nnodes)`` the pairs
    before it are applied and :class:`IndexError` is raised, as the
    reference's bounds check does.

    :arg crack: ``(npairs, 2)`` node indices.
    :arg nlist: ``(nnodes, max_neigh)`` int32 C-contiguous host array.
    :arg n_neigh: ``(nnodes,)`` int32 host array.
    :arg context: a :class:`~.integrators.CUDAContext` (default: device 0).
    """
    import torch
    from .integrators import CUDAContext
    for name, a, nd in (("nlist", nlist, 2), ("n_neigh", n_neigh, 1)):
        if (not isinstance(a, np.ndarray) or a.dtype != np.intc
                or a.ndim != nd or not a.flags.c_contiguous
                or not a.flags.writeable):
            raise TypeError(f"{name} must be a writeable C-contiguous "
                            f"int32 array of {nd} dimensions")
    crack = np.asarray(crack, dtype=np.int64).reshape(-1, 2)
    n = nlist.shape[0]
    if n_neigh.shape[0] != n:
        raise ValueError("nlist and n_neigh disagree on the number of nodes")
    bad = np.nonzero(((crack < -n) | (crack >= n)).any(axis=1))[0]
    stop = int(bad[0]) if bad.size else len(crack)
    if stop:
        ctx = context if context is not None else CUDAContext(0)
        dev = ctx.device
        with ctx.on_stream():
            c = torch.as_tensor(
                np.ascontiguousarray(crack[:stop], dtype=np.int32),
                device=dev)
            nl = torch.as_tensor(nlist, device=dev)
            nn = torch.as_tensor(n_neigh, device=dev)
            crack_device(c, nl, nn, ctx)
            nlist[...] = nl.cpu().numpy()
            n_neigh[...] = nn.cpu().numpy()
    if bad.size:
        raise IndexError("Out of bounds on buffer access (axis 0)")
