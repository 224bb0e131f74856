"""Stiffness correction factors on the GPU (model set-up).

PeriPy's ``Model`` can scale every bond's stiffness by a micromodulus
function, a partial-volume correction and a surface correction
(``peripy/correction.pyx:5-277``, applied by ``peripy/model.py:349-375``).
:func:`stiffness_corrections` computes the same factors with
``pp_stiffness_corrections`` and returns the ``(nnodes, max_neighbours)``
array the integrators take as ``stiffness_corrections``.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib


def stiffness_corrections(coords, volume, nlist, n_neigh, horizon,
                          micromodulus_function=None,
                          volume_correction=None, surface_correction=None,
                          node_radius=None, dimensions=3,
                          search_horizon=None, context=None):
    """The correction factors ``Model.__init__`` builds from its flags.

    :arg horizon: the peridynamic horizon as given to ``Model``.
    :arg search_horizon: the horizon of the neighbour search (``horizon +
        node_radius`` when a volume correction is applied, as ``Model``
        sets it); sets the bulk family volume of the surface correction.
    :arg micromodulus_function: ``0`` (conical) or ``None``.
    :arg volume_correction: ``0`` (partial volume) or ``None``; needs
        ``node_radius``.
    :arg surface_correction: ``1`` (actual volumes), ``0`` (average volume)
        or ``None``.

    The partial-volume factors are those of the reference's call
    ``self._set_volume_corrections(volume_correction, stiffness_corrections,
    node_radius, horizon)`` (``model.py:363-365``), whose last two
    arguments are in the opposite order to its signature (``model.py:823``):
    the factor is 1 within ``node_radius - horizon``, ``(node_radius +
    horizon - l0) / (2 horizon)`` up to ``node_radius + horizon``, 0 beyond.
    Reproduced as the reference computes it.

    :returns: the factors, or None when no flag is set (the reference then
        applies no correction).
    """
    for name, value, allowed in (
            ("micromodulus_function", micromodulus_function, (0,)),
            ("volume_correction", volume_correction, (0,)),
            ("surface_correction", surface_correction, (0, 1))):
        if value is not None and value not in allowed:
            raise ValueError(
                "{} value is wrong (expected {} or None, got {})".format(
                    name, " or ".join(map(str, allowed)), value))
    if (micromodulus_function is None and volume_correction is None
            and surface_correction is None):
        return None
    if volume_correction is not None and node_radius is None:
        raise TypeError("volume_correction needs node_radius")
    import torch
    from .integrators import CUDAContext
    ctx = context if context is not None else CUDAContext(0)
    nlist = np.ascontiguousarray(nlist, dtype=np.intc)
    n, width = nlist.shape
    h_search = horizon if search_horizon is None else search_horizon
    if dimensions == 2:
        bulk = np.pi * np.power(h_search, 2)
    else:
        bulk = (4. / 3) * np.pi * np.power(h_search, 3)
    a = _lib.CorrectionsArgs()
    a.nnodes, a.max_neigh = n, width
    a.micromodulus_function = -1 if micromodulus_function is None else 0
    a.volume_correction = -1 if volume_correction is None else 0
    a.surface_correction = (-1 if surface_correction is None
                            else int(surface_correction))
    a.micromodulus_horizon = float(horizon)
    if volume_correction is not None:
        a.vc_horizon = float(node_radius)
        a.vc_node_radius = float(horizon)
    a.family_volume_bulk = float(bulk)
    volume = np.asarray(volume, dtype=np.float64)
    a.average_volume = float(np.sum(volume) / n) if n else 0.0
    dev = ctx.device
    with ctx.on_stream():
        keep = [torch.as_tensor(np.ascontiguousarray(coords, np.float64),
                                device=dev),
                torch.as_tensor(volume, device=dev),
                torch.as_tensor(nlist, device=dev),
                torch.as_tensor(np.ascontiguousarray(n_neigh, np.intc),
                                device=dev),
                torch.ones((n, width), dtype=torch.float64, device=dev),
                torch.empty(max(n, 1), dtype=torch.float64, device=dev)]
        (a.r0, a.volume, a.nlist, a.n_neigh, a.corrections,
         a.family_volume) = [t.data_ptr() for t in keep]
        check(lib().pp_stiffness_corrections(ctypes.byref(a),
                                             ctx.stream_handle),
              "pp_stiffness_corrections")
        return keep[4].cpu().numpy()
