"""Write-step sums on the GPU.

At every write step PeriPy's ``Model.simulate`` copies all eight state
arrays back to the host (``Integrator.write``, ``peripy/integrators.py:
285-300``), writes a mesh file with the displacements and damage, and
records NumPy sums of the state (``peripy/model.py:1320-1366``): ``np.sum``
of ``u``, ``ud``, ``udd``, ``force * volume[:, None]``, ``body_force *
volume[:, None]`` and ``damage``, and per tip type the running sums of the
same quantities over its ``(node, dof)`` list.

:class:`WriteSums` computes those numbers on the device with
``pp_write_sums``, in NumPy's own summation order, so they are bit-identical
to the reference's; a write then needs only ``u`` and ``damage`` on the host
(the mesh file's fields) instead of all eight arrays, among them the
``(nnodes, max_neighbours)`` neighbour list.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib

#: Keys of a tip type's record, in the order of the tip sums.
TIP_KEYS = ("displacement", "velocity", "acceleration", "force",
            "body_force")


def pairwise_plan(n):
    """The summation tree of NumPy's float64 sum of ``n`` contiguous
    elements (``pp_pairwise_plan``), as an int32 array.

    Header ``[leaves, inner, heights, n]``, then the leaves' first elements
    and lengths, the inner nodes' left and right value indices (leaves
    first, inner nodes after them in height order) and the height offsets.
    """
    L = lib()
    need = L.pp_pairwise_plan(int(n), None, 0)
    if need < 0:
        raise ValueError(f"no pairwise plan for {n} elements")
    plan = np.empty(need, dtype=np.int32)
    got = L.pp_pairwise_plan(int(n), plan.ctypes.data_as(ctypes.c_void_p),
                             need)
    if got != need:
        raise _lib.LibraryError("pp_pairwise_plan changed its length")
    return plan


def evaluate_plan(plan, values):
    """Sum ``values`` on the host by following ``plan`` (a checker of the
    plan: it equals ``np.sum(values)`` bit for bit)."""
    values = np.ascontiguousarray(values, dtype=np.float64).ravel()
    leaves, inner, heights, n = (int(v) for v in plan[:4])
    if n != values.size:
        raise ValueError("plan and values disagree on the length")
    if leaves == 0:
        return 0.0
    lo = plan[4:4 + leaves]
    ln = plan[4 + leaves:4 + 2 * leaves]
    left = plan[4 + 2 * leaves:4 + 2 * leaves + inner]
    right = plan[4 + 2 * leaves + inner:4 + 2 * leaves + 2 * inner]
    val = np.zeros(leaves + inner)
    for t in range(leaves):
        a = values[lo[t]:lo[t] + ln[t]]
        if a.size < 8:
            r = np.float64(0.0)
            for x in a:
                r = r + x
            val[t] = r
            continue
        body = a.size - a.size % 8
        acc = a[:8].copy()
        for i in range(8, body, 8):
            acc = acc + a[i:i + 8]
        r = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + \
            ((acc[4] + acc[5]) + (acc[6] + acc[7]))
        for x in a[body:]:
            r = r + x
        val[t] = r
    for k in range(inner):  # height order: children come first
        val[leaves + k] = val[left[k]] + val[right[k]]
    return np.float64(0.0) + val[leaves + inner - 1 if inner else 0]


def tip_entries(tip_types):
    """``(offsets, entries)`` of ``Model.tip_types`` in its dict order."""
    offsets = [0]
    entries = []
    for node_list in tip_types.values():
        entries.extend((int(i), int(j)) for i, j in node_list)
        offsets.append(len(entries))
    return (np.asarray(offsets, dtype=np.int32),
            np.asarray(entries, dtype=np.int32).reshape(-1, 2))


class WriteSums:
    """The write-step sums of one model on one device.

    :arg context: the integrator's :class:`~.integrators.CUDAContext`.
    :arg int nnodes: number of nodes.
    :arg volume: ``(nnodes,)`` float64 device tensor (the integrator's
        node volumes, the ``Model.volume`` the reference scales by).
    :arg dict tip_types: ``Model.tip_types`` (name -> ``(node, dof)`` list).
    """

    def __init__(self, context, nnodes, volume, tip_types):
        import torch
        self.context = context
        self.nnodes = int(nnodes)
        self.tip_names = list(tip_types)
        dev = context.device
        p3 = pairwise_plan(3 * self.nnodes)
        p1 = pairwise_plan(self.nnodes)
        offsets, entries = tip_entries(tip_types)
        if entries.size and (entries[:, 0].min() < 0
                             or entries[:, 0].max() >= self.nnodes
                             or entries[:, 1].min() < 0
                             or entries[:, 1].max() > 2):
            raise ValueError("tip entries outside (nnodes, 3)")
        a = _lib.WriteSumsArgs()
        a.nnodes = self.nnodes
        a.ntips = len(self.tip_names)
        a.leaves3, a.values3 = int(p3[0]), int(p3[0] + p3[1])
        a.leaves1, a.values1 = int(p1[0]), int(p1[0] + p1[1])
        with context.on_stream():
            self._keep = [torch.as_tensor(p3, device=dev),
                          torch.as_tensor(p1, device=dev),
                          torch.as_tensor(offsets, device=dev),
                          torch.as_tensor(entries.reshape(-1), device=dev)
                          if entries.size else
                          torch.zeros(2, dtype=torch.int32, device=dev),
                          torch.empty(max(5 * a.values3 + a.values1, 1),
                                      dtype=torch.float64, device=dev),
                          torch.empty(6 + 5 * a.ntips, dtype=torch.float64,
                                      device=dev)]
        self._volume = volume
        (a.plan3, a.plan1, a.tip_offsets, a.tip_entries, a.scratch,
         a.sums) = [t.data_ptr() for t in self._keep]
        a.volume = volume.data_ptr()
        self._args = a
        self._host = torch.empty(6 + 5 * a.ntips, dtype=torch.float64,
                                 pin_memory=True)

    def __call__(self, u, ud, udd, force, body_force, damage):
        """The sums of the given device arrays (``None`` counts as zeros).

        :returns: float64 array: the six model sums (``u``, ``ud``,
            ``udd``, ``force * volume``, ``body_force * volume``,
            ``damage``), then five per tip type (:data:`TIP_KEYS`).
        """
        a = self._args

        def ptr(t):
            if t is None:
                return None
            if t.dtype.itemsize != 8 or not t.is_contiguous():
                raise TypeError("write sums need contiguous float64 arrays")
            return t.data_ptr()

        a.u, a.ud, a.udd = ptr(u), ptr(ud), ptr(udd)
        a.force, a.body_force = ptr(force), ptr(body_force)
        a.damage = ptr(damage)
        with self.context.on_stream():
            check(lib().pp_write_sums(ctypes.byref(a),
                                      self.context.stream_handle),
                  "pp_write_sums")
            self._host.copy_(self._keep[5], non_blocking=True)
            self.context.stream.synchronize()
        return self._host.numpy().copy()
