"""Integrators: the drop-in boundary of the time step.

Mirrors PeriPy's ``Integrator`` API (``peripy/integrators.py:11-300``):
``build`` (called once by ``Model.__init__``), ``create_buffers`` (called at
the start of every ``Model.simulate``), ``__call__`` (one time step) and
``write`` (device to host), with the same argument names, order, meaning
and ``ValueError`` checks.  The OpenCL integrators ``EulerCL``,
``EulerCromerCL`` and ``VelocityVerletCL`` (``integrators.py:462-764``) are
replaced by :class:`EulerCUDA`, :class:`EulerCromerCUDA` and
:class:`VelocityVerletCUDA`, which run hand-written sm_103a kernels through
the C ABI of ``include/pp_gb300.h``; the old names are kept as aliases so a
script only changes its import line.

Each CUDA integrator takes two extra keyword arguments:

``fused`` (default True)
    True: one fused kernel per step (stretch, break, force, reduction,
    boundary conditions, intact count, update).  False: the
    reference-structured "plain" sequence of separate bond-force and update
    kernels (``peripy/integrators.py:266-283, 530-541``).
``precision`` (default ``"float64"``)
    ``"float64"``: binary64 throughout, bit-identical to the reference
    arithmetic.  ``"mixed"``: FP32 bond arithmetic, the break/regime test
    decided exactly as binary64 would on the same state, and double-float
    node state (fused only).

Device memory is owned by the integrator as torch tensors; all work is
queued on the context's CUDA stream and is asynchronous until ``write``.
"""
from abc import ABC, abstractmethod
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib


class ContextError(Exception):
    """No suitable CUDA device was found by :func:`get_context`."""

    def __init__(self):
        """Exception constructor (``peripy/integrators.py:767-775``)."""
        message = ("No suitable context was found. You can manually specify "
                   "the context by passing a CUDAContext to the integrator "
                   "with the 'context' argument.")
        super().__init__(message)


class CUDAContext:
    """A CUDA device and the stream all of an integrator's work runs on.

    Replaces the pyopencl context and in-order queue the reference creates
    in ``Integrator.__init__`` (``peripy/integrators.py:38-58``).  It is
    truthy, which is what makes ``Model`` choose the power-of-two, ``-1``
    padded neighbour-list layout (``peripy/model.py:575-585``).
    """

    def __init__(self, device=0, stream=None):
        import torch
        if not torch.cuda.is_available():
            raise ContextError()
        self.device = torch.device("cuda", device)
        # A dedicated (capturable) stream unless the caller gives one; all
        # of an integrator's torch copies and kernels are ordered on it.
        self.stream = (stream if stream is not None
                       else torch.cuda.Stream(self.device))

    def on_stream(self):
        """Context manager that makes this stream torch's current one."""
        import torch
        return torch.cuda.stream(self.stream)

    @property
    def stream_handle(self):
        return ctypes.c_void_p(self.stream.cuda_stream)

    def __bool__(self):
        return True

    def __repr__(self):
        return f"CUDAContext({self.device})"


def get_context():
    """Return a :class:`CUDAContext` on device 0, or None without a GPU.

    Counterpart of ``peripy/cl/utilities.py:28-44``.
    """
    try:
        import torch
    except ImportError:  # pragma: no cover - torch is a hard dependency
        return None
    if not torch.cuda.is_available():
        return None
    return CUDAContext(0)


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


#: Host arrays of at least this size are page-locked while a write fills
#: them from the device.
_REGISTER_BYTES = 4 << 20


def _pos_frame(coords, extent):
    """Origin and power-of-two step of the fixed-point positions.

    Positions become int32 ``q = rint((r0 - origin) / step)``.  The step is
    the smallest power of two with ``extent / step <= 2**21``, where
    ``extent`` is the largest bond component length, so every bond's
    ``|q[j] - q[i]| < 2**22`` converts to float exactly; it is coarsened if
    the domain would not fit ``|q| < 2**30``.
    """
    lo = coords.min(axis=0)
    hi = coords.max(axis=0)
    origin = (lo + hi) / 2
    half = float(np.max(hi - lo) / 2)
    ext = float(extent) if extent > 0 else max(half, 1.0)
    k = int(np.ceil(np.log2(ext))) - 21
    if half > 0:
        k = max(k, int(np.ceil(np.log2(half))) - 29)
    return origin.astype(np.float64), 2.0 ** k


class Integrator(ABC):
    """Base class for integrators (``peripy/integrators.py:11-300``).

    Concrete integrators define ``__init__``, ``__call__``,
    ``_build_special`` and ``_create_special_buffers``.
    """

    @abstractmethod
    def __init__(self, dt, context=None):
        """Create an :class:`Integrator` on a CUDA device.

        :arg float dt: The length of time (in seconds [s]) of one time-step.
        :arg context: Optional :class:`CUDAContext`; default is device 0.
        :raises ContextError: when no CUDA device is available.
        :raises TypeError: when ``context`` is not a :class:`CUDAContext`.
        """
        self.dt = dt
        if context is None:
            self.context = get_context()
            if not isinstance(self.context, CUDAContext):
                raise ContextError()
        else:
            if not isinstance(context, CUDAContext):
                raise TypeError("context must be a CUDAContext object")
            self.context = context
        lib()  # fail loudly now if the CUDA library is missing

    @abstractmethod
    def __call__(self):
        """Conduct one iteration of the integrator."""

    @abstractmethod
    def _build_special(self):
        """Build what is special to the chosen integrator."""

    @abstractmethod
    def _create_special_buffers(self):
        """Create buffers that are special to the chosen integrator."""


class _CUDAIntegrator(Integrator):
    """Shared implementation of the CUDA integrators."""

    _kind = None          # PP_EULER / PP_EULER_CROMER / PP_VELOCITY_VERLET
    _dynamic = False      # needs densities, ud, udd

    def __init__(self, dt, context=None, fused=True, precision="float64",
                 compensated=False, nodes_per_block=0, use_graph=True,
                 autotune=True, tiled=True):
        super().__init__(dt, context)
        if precision not in ("float64", "mixed"):
            raise ValueError("precision must be 'float64' or 'mixed' "
                             f"(got {precision!r})")
        if precision == "mixed" and not fused:
            raise ValueError("precision='mixed' is implemented by the fused "
                             "kernel only; use fused=True")
        if compensated and precision != "mixed":
            raise ValueError("compensated=True applies to the FP32 force sums "
                             "of precision='mixed'")
        self.fused = bool(fused)
        self.precision = precision
        self.compensated = bool(compensated)
        self.nodes_per_block = int(nodes_per_block)
        self.use_graph = bool(use_graph)
        self.autotune = bool(autotune)
        # mixed precision: gather neighbour records from shared memory on
        # the tiled layout (False: the untiled kernel, from L1/L2)
        self.tiled = bool(tiled) and precision == "mixed"
        self.tiling = None
        self.tile_target = 125  # nodes per brick of the internal order
        self._order = None
        self.tuning = None
        self.damping = 0.0
        self._parity = 0
        self._fargs = None
        self._instances = None

    def set_instances(self, node_instance, instance_critical_stretch):
        """Step many independent models at once (see :mod:`.batch`).

        Node ``i`` breaks its bonds at
        ``instance_critical_stretch[node_instance[i]]`` instead of the
        scalar critical stretch.  Fused integrators and the PMB damage model
        only; call before :meth:`build`.
        """
        if not self.fused:
            raise ValueError("instances need a fused integrator")
        node_instance = np.ascontiguousarray(node_instance, dtype=np.intc)
        s0 = np.ascontiguousarray(instance_critical_stretch,
                                  dtype=np.float64).ravel()
        if not 1 <= s0.size <= 256:
            raise ValueError("between 1 and 256 instances are supported")
        if node_instance.size and (node_instance.min() < 0
                                   or node_instance.max() >= s0.size):
            raise ValueError("node_instance out of range")
        self._instances = (node_instance, s0)

    # -------------------------------------------------------------- helpers
    def _dev(self, array, dtype):
        import torch
        t = torch.as_tensor(np.ascontiguousarray(array, dtype=dtype))
        return t.to(self.context.device, non_blocking=False)

    def _empty(self, shape, dtype):
        import torch
        return torch.empty(shape, dtype=dtype, device=self.context.device)

    def _zeros(self, shape, dtype):
        import torch
        return torch.zeros(shape, dtype=dtype, device=self.context.device)

    @property
    def _stream(self):
        return self.context.stream_handle

    # ---------------------------------------------------------------- build
    def build(self, nnodes, degrees_freedom, max_neighbours, coords, volume,
              family, bc_types, bc_values, force_bc_types, force_bc_values,
              stiffness_corrections, bond_types, densities):
        """Copy the simulate-independent arrays to the device.

        Same arguments as ``peripy/integrators.py:84-188``.
        """
        with self.context.on_stream():
            self._build(nnodes, degrees_freedom, max_neighbours, coords,
                        volume, family, bc_types, bc_values, force_bc_types,
                        force_bc_values, stiffness_corrections, bond_types,
                        densities)

    def _build(self, nnodes, degrees_freedom, max_neighbours, coords, volume,
               family, bc_types, bc_values, force_bc_types, force_bc_values,
               stiffness_corrections, bond_types, densities):
        import torch
        self.nnodes = int(nnodes)
        self.degrees_freedom = int(degrees_freedom)
        self.max_neighbours = int(max_neighbours)
        self.densities = densities
        mn = self.max_neighbours
        if mn < 1 or mn > 1024 or (mn & (mn - 1)):
            raise ValueError(
                "max_neighbours must be a power of two in [1, 1024] for CUDA "
                f"integrators (got {mn})")
        if self.degrees_freedom != 3:
            raise ValueError("degrees_freedom must be 3 "
                             f"(got {self.degrees_freedom})")
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.r0_d = self._dev(self.coords, np.float64)
        self.vols_d = self._dev(volume, np.float64)
        self.family_d = self._dev(family, np.int32)
        self.bc_types_d = self._dev(bc_types, np.int32)
        self.bc_values_d = self._dev(bc_values, np.float64)
        self.force_bc_types_d = self._dev(force_bc_types, np.int32)
        self.force_bc_values_d = self._dev(force_bc_values, np.float64)
        self.stiffness_corrections_d = (
            None if stiffness_corrections is None
            else self._dev(stiffness_corrections, np.float64))
        self.bond_types_d = (None if bond_types is None
                             else self._dev(bond_types, np.int32))
        if self._instances is not None:
            if bond_types is not None:
                raise ValueError("instances support the PMB damage model "
                                 "only (no bond types)")
            if self._instances[0].shape != (self.nnodes,):
                raise ValueError("node_instance must have nnodes entries")
            self.node_instance_d = self._dev(self._instances[0], np.int32)
            self.instance_s0_d = self._dev(self._instances[1], np.float64)
        else:
            self.node_instance_d = self.instance_s0_d = None
        if self.bond_types_d is not None and (
                tuple(self.bond_types_d.shape) != (self.nnodes, mn)):
            raise ValueError("bond_types shape must be (nnodes, "
                             "max_neighbours)")
        self._torch = torch
        if self.tiled:
            from .tiling import brick_order
            self._order = brick_order(
                self.coords, None if self._instances is None
                else self._instances[0], target=self.tile_target)
        self._build_special()

    def _check_densities(self):
        if self._dynamic:
            if self.densities is None:
                raise ValueError(
                    "densities must be supplied when using {} integrator "
                    "(got {}). This integrator is dynamic and requires the "
                    "density or is_density argument to be supplied to "
                    ":class:Model, alternatively, use a static integrator, "
                    "such as EulerCUDA.".format(type(self).__name__,
                                                type(self.densities)))
            self.densities_d = self._dev(self.densities, np.float64)
        else:
            if self.densities is not None:
                raise ValueError(
                    "densities are not supported by this integrator "
                    "(expected {}, got {}). This integrator neglects "
                    "inertial effects. Do not supply a density or is_density "
                    "argument or, alternatively, use a dynamic integrator, "
                    "such as EulerCromerCUDA.".format(type(None),
                                                      type(self.densities)))
            self.densities_d = None

    def _build_special(self):
        """Check and upload the densities (``integrators.py:505-524``)."""
        self._check_densities()

    def _create_special_buffers(self):
        """There are no integrator-specific buffers."""

    # ------------------------------------------------------- create_buffers
    def create_buffers(self, nlist, n_neigh, bond_stiffness,
                       critical_stretch, plus_cs, u, ud, udd, force,
                       body_force, damage, regimes, nregimes, nbond_types):
        """Copy the simulate-dependent state to the device.

        Same arguments as ``peripy/integrators.py:190-254``: with one bond
        type and one regime the stiffness and critical stretch are kept as
        ``np.float64`` scalars, else as device tables.
        """
        with self.context.on_stream():
            self._create_buffers(nlist, n_neigh, bond_stiffness,
                                 critical_stretch, plus_cs, u, ud, udd,
                                 regimes, nregimes, nbond_types)

    def _create_buffers(self, nlist, n_neigh, bond_stiffness,
                        critical_stretch, plus_cs, u, ud, udd, regimes,
                        nregimes, nbond_types):
        n, mn = self.nnodes, self.max_neighbours
        if self._instances is not None and (nbond_types != 1 or nregimes != 1):
            raise ValueError("instances support the PMB damage model only")
        if (nbond_types == 1) and (nregimes == 1):
            self.bond_stiffness_d = np.float64(bond_stiffness)
            self.critical_stretch_d = np.float64(critical_stretch)
            self.plus_cs_d = None
            self.regimes_d = None
        else:
            self.bond_stiffness_d = self._dev(
                np.asarray(bond_stiffness).ravel(), np.float64)
            self.critical_stretch_d = self._dev(
                np.asarray(critical_stretch).ravel(), np.float64)
            self.plus_cs_d = self._dev(np.asarray(plus_cs).ravel(),
                                       np.float64)
            self.regimes_d = self._dev(
                np.zeros((n, mn)) if regimes is None else regimes, np.int32)
            if self.bond_types_d is None:
                self.bond_types_d = self._zeros((n, mn), self._torch.int32)
        self.nregimes = np.intc(nregimes)
        self.nbond_types = np.intc(nbond_types)
        if self.bond_types_d is not None and self.plus_cs_d is None:
            # Bond types with a single regime and type: one-entry tables.
            self.plus_cs_d = self._dev(np.zeros(1), np.float64)
            self.bond_stiffness_tab_d = self._dev(
                np.atleast_1d(np.float64(bond_stiffness)), np.float64)
            self.critical_stretch_tab_d = self._dev(
                np.atleast_1d(np.float64(critical_stretch)), np.float64)
            self.regimes_d = self._dev(
                np.zeros((n, mn)) if regimes is None else regimes, np.int32)
        elif self.plus_cs_d is not None:
            self.bond_stiffness_tab_d = self.bond_stiffness_d
            self.critical_stretch_tab_d = self.critical_stretch_d
        else:
            self.bond_stiffness_tab_d = None
            self.critical_stretch_tab_d = None

        torch = self._torch
        self.nlist_d = self._dev(nlist, np.int32)
        if tuple(self.nlist_d.shape) != (n, mn):
            raise ValueError("nlist shape must be (nnodes, max_neighbours) = "
                             f"{(n, mn)}, got {tuple(self.nlist_d.shape)}")
        self.n_neigh_d = self._dev(n_neigh, np.int32)
        self.u_d = [self._dev(u, np.float64).reshape(n, 3),
                    self._empty((n, 3), torch.float64)]
        self.ud_d = self._dev(ud, np.float64).reshape(n, 3)
        self.udd_d = self._dev(udd, np.float64).reshape(n, 3)
        self.force_d = self._zeros((n, 3), torch.float64)
        self.body_force_d = self._zeros((n, 3), torch.float64)
        self.damage_d = self._zeros((n,), torch.float64)
        self._parity = 0
        if self.precision == "mixed":
            self._create_mixed_buffers()
        self.bond_length_d = None
        if self.fused and self.precision == "float64":
            # |xi| per slot, read by the fused binary64 step instead of a
            # square root per bond and step (the same binary64 value)
            self.bond_length_d = torch.empty(
                (n, self.max_neighbours), dtype=torch.float64,
                device=self.context.device)
            check(lib().pp_bond_lengths(
                _ptr(self.r0_d), _ptr(self.nlist_d), n, self.max_neighbours,
                _ptr(self.bond_length_d), self._stream), "pp_bond_lengths")
        self._fargs = self._make_fused_args() if self.fused else None
        if self.precision == "mixed":
            if self.tiled:
                from .tiling import DeviceTiling
                self.tiling = DeviceTiling(*self._order, self.context.device)
                self.tiling.build(
                    self._fargs, self._stream,
                    corrections=self.stiffness_corrections_d is not None,
                    types=self.bond_types_d is not None,
                    instances=self.node_instance_d is not None)
                self._fargs.tiling = ctypes.addressof(self.tiling.struct)
            check(lib().pp_mixed_pack(ctypes.byref(self._fargs), 0,
                                      self._stream), "pp_mixed_pack")
            if self.autotune:
                from .autotune import tune_mixed
                self.tuning = tune_mixed(self)
        self._create_special_buffers()

    def _drop_tiling(self):
        """Switch a mixed-precision integrator set up tiled to the untiled
        kernel (the autotuner found it faster): repack the state in the
        reference node order.  Only at create_buffers, before any step."""
        torch = self._torch
        n, mn = self.nnodes, self.max_neighbours
        self.tiled = False
        self.tiling = None
        if self.stiffness_corrections_d is not None:
            self.sc32_d = self._empty((n, mn), torch.float32)
        a = self._fargs
        a.tiling = None
        a.sc32 = _ptr(self.sc32_d)
        check(lib().pp_mixed_pack(ctypes.byref(a), self._parity,
                                  self._stream), "pp_mixed_pack")

    def _create_mixed_buffers(self):
        torch = self._torch
        n, mn = self.nnodes, self.max_neighbours
        # 32-byte node records {q, w; u, max|u|} (pp_fused_args.rec)
        self.rec_d = [self._zeros((n, 8), torch.float32) for _ in range(2)]
        self.ulo_d = [self._zeros((n, 4), torch.float32) for _ in range(2)]
        self.frc_d = self._zeros((n, 8), torch.float32)
        if self._dynamic:
            self.vel_d = self._zeros((n, 8), torch.float32)
            self.acc_d = self._zeros((n, 4), torch.float32)
            self.rho32_d = self._zeros((n, 4), torch.float32)
        else:
            self.vel_d = self.acc_d = self.rho32_d = None
        self.sc32_d = (None if self.stiffness_corrections_d is None
                       or self.tiled
                       else self._empty((n, mn), torch.float32))
        self.nflags_d = self._empty((n,), torch.int32)
        self.umax_d = self._zeros((1,), torch.float32)
        self.status_d = self._zeros((1,), torch.int32)
        ext = self._zeros((2,), torch.float64)
        check(lib().pp_bond_extent(_ptr(self.nlist_d), _ptr(self.r0_d), n, mn,
                                   _ptr(ext), self._stream), "pp_bond_extent")
        ext = ext.cpu().numpy()
        self.bond_extent = float(ext[0])
        self.min_bond = float(ext[1]) if ext[1] < 1e300 else 0.0
        self.pos_origin, self.pos_scale = _pos_frame(self.coords,
                                                     self.bond_extent)

    def _make_fused_args(self):
        a = _lib.FusedArgs()
        a.nnodes = self.nnodes
        a.max_neigh = self.max_neighbours
        a.integrator = self._kind
        a.precision = (_lib.PP_MIXED if self.precision == "mixed"
                       else _lib.PP_FLOAT64)
        a.nregimes = int(self.nregimes)
        a.nbond_types = int(self.nbond_types)
        a.flags = _lib.PP_FLAG_COMPENSATED if self.compensated else 0
        a.nodes_per_block = self.nodes_per_block
        a.dt = float(self.dt)
        a.damping = float(self.damping)
        if isinstance(self.bond_stiffness_d, np.float64):
            a.bond_stiffness = float(self.bond_stiffness_d)
            a.critical_stretch = float(self.critical_stretch_d)
        a.bond_stiffness_table = _ptr(self.bond_stiffness_tab_d)
        a.critical_stretch_table = _ptr(self.critical_stretch_tab_d)
        a.plus_cs = _ptr(self.plus_cs_d)
        a.r0 = _ptr(self.r0_d)
        a.vols = _ptr(self.vols_d)
        a.family = _ptr(self.family_d)
        a.bc_types = _ptr(self.bc_types_d)
        a.bc_values = _ptr(self.bc_values_d)
        a.fc_types = _ptr(self.force_bc_types_d)
        a.fc_values = _ptr(self.force_bc_values_d)
        a.densities = _ptr(self.densities_d)
        a.stiffness_corrections = _ptr(self.stiffness_corrections_d)
        a.bond_types = _ptr(self.bond_types_d)
        a.bond_length = _ptr(getattr(self, "bond_length_d", None))
        if self.node_instance_d is not None:
            a.node_instance = _ptr(self.node_instance_d)
            a.instance_s0 = _ptr(self.instance_s0_d)
            a.ninstances = int(self.instance_s0_d.numel())
        a.nlist = _ptr(self.nlist_d)
        a.regimes = _ptr(self.regimes_d)
        a.u[0] = self.u_d[0].data_ptr()
        a.u[1] = self.u_d[1].data_ptr()
        a.ud = _ptr(self.ud_d)
        a.udd = _ptr(self.udd_d)
        a.force = _ptr(self.force_d)
        a.body_force = _ptr(self.body_force_d)
        a.n_neigh = _ptr(self.n_neigh_d)
        a.damage = _ptr(self.damage_d)
        if self.precision == "mixed":
            a.rec[0] = self.rec_d[0].data_ptr()
            a.rec[1] = self.rec_d[1].data_ptr()
            a.ulo[0] = self.ulo_d[0].data_ptr()
            a.ulo[1] = self.ulo_d[1].data_ptr()
            a.vel = _ptr(self.vel_d)
            a.acc = _ptr(self.acc_d)
            a.frc = _ptr(self.frc_d)
            a.rho32 = _ptr(self.rho32_d)
            a.sc32 = _ptr(self.sc32_d)
            a.nflags = _ptr(self.nflags_d)
            a.umax = _ptr(self.umax_d)
            a.status = _ptr(self.status_d)
            a.min_bond = float(self.min_bond)
            a.pos_scale = float(self.pos_scale)
            for k in range(3):
                a.pos_origin[k] = float(self.pos_origin[k])
        return a

    # ----------------------------------------------------------------- step
    def __call__(self, displacement_bc_magnitude, force_bc_magnitude):
        """Conduct one iteration of the integrator.

        :arg float displacement_bc_magnitude: the magnitude applied to the
             displacement boundary conditions for the current time-step.
        :arg float force_bc_magnitude: the magnitude applied to the force
            boundary conditions for the current time-step.
        """
        if self.fused:
            check(lib().pp_fused_step(
                ctypes.byref(self._fargs), self._parity,
                float(displacement_bc_magnitude), float(force_bc_magnitude),
                self._stream), "pp_fused_step")
            self._parity ^= 1
        else:
            self._bond_force(force_bc_magnitude)
            self._update_displacement(displacement_bc_magnitude)

    def _run(self, displacement_bc_magnitudes, force_bc_magnitudes, first,
             steps):
        """Run ``steps`` steps with magnitudes ``mags[first .. first+steps)``.

        Equivalent to ``steps`` calls of ``__call__``; the fused path queues
        them from C (optionally as a replayed CUDA graph), so Python adds no
        per-step overhead.
        """
        if steps <= 0:
            return
        if not self.fused:
            for k in range(first, first + steps):
                self(displacement_bc_magnitudes[k], force_bc_magnitudes[k])
            return
        with self.context.on_stream():
            self._run_fused(displacement_bc_magnitudes, force_bc_magnitudes,
                            first, steps)

    def _run_fused(self, displacement_bc_magnitudes, force_bc_magnitudes,
                   first, steps):
        dm = self._dev(np.asarray(displacement_bc_magnitudes)[
            first:first + steps], np.float64)
        fm = self._dev(np.asarray(force_bc_magnitudes)[
            first:first + steps], np.float64)
        self._run_device(dm, fm, 0, steps)
        # keep the magnitude arrays alive until the queued work has run
        self._pending = (dm, fm)

    def _run_device(self, dm, fm, first, steps):
        """Queue ``steps`` fused steps reading ``dm[first + k]`` and
        ``fm[first + k]`` from device float64 tensors (no host copies)."""
        if not hasattr(self, "_step_base_d"):
            with self.context.on_stream():
                self._step_base_d = self._zeros((1,), self._torch.int64)
        check(lib().pp_fused_run(
            ctypes.byref(self._fargs), self._parity, steps, _ptr(dm),
            _ptr(fm), first, int(self.use_graph), 16,
            _ptr(self._step_base_d), self._stream), "pp_fused_run")
        self._parity ^= steps & 1

    def _bond_force(self, force_bc_magnitude):
        """Plain bond-force launch (``integrators.py:266-283``)."""
        a = _lib.BondForceArgs()
        a.nnodes = self.nnodes
        a.max_neigh = self.max_neighbours
        a.nregimes = int(self.nregimes)
        a.nbond_types = int(self.nbond_types)
        a.u = _ptr(self.u_d[0])
        a.force = _ptr(self.force_d)
        a.body_force = _ptr(self.body_force_d)
        a.r0 = _ptr(self.r0_d)
        a.vols = _ptr(self.vols_d)
        a.nlist = _ptr(self.nlist_d)
        a.fc_types = _ptr(self.force_bc_types_d)
        a.fc_values = _ptr(self.force_bc_values_d)
        a.stiffness_corrections = _ptr(self.stiffness_corrections_d)
        a.bond_types = _ptr(self.bond_types_d)
        a.regimes = _ptr(self.regimes_d)
        a.plus_cs = _ptr(self.plus_cs_d)
        a.bond_stiffness_table = _ptr(self.bond_stiffness_tab_d)
        a.critical_stretch_table = _ptr(self.critical_stretch_tab_d)
        if isinstance(self.bond_stiffness_d, np.float64):
            a.bond_stiffness = float(self.bond_stiffness_d)
            a.critical_stretch = float(self.critical_stretch_d)
        a.fc_scale = float(force_bc_magnitude)
        check(lib().pp_bond_force(ctypes.byref(a), self._stream),
              "pp_bond_force")

    def _update_displacement(self, displacement_bc_magnitude):
        raise NotImplementedError

    # ---------------------------------------------------------------- write
    def _sync_state(self):
        """Bring the current state to the reference layouts on the device."""
        L = lib()
        if self.precision == "mixed":
            check(L.pp_mixed_export(ctypes.byref(self._fargs), self._parity,
                                    self._stream), "pp_mixed_export")
        check(L.pp_damage(_ptr(self.nlist_d), _ptr(self.family_d),
                          _ptr(self.n_neigh_d), _ptr(self.damage_d),
                          self.nnodes, self.max_neighbours, self._stream),
              "pp_damage")

    def write(self, u, ud, udd, force, body_force, damage, nlist, n_neigh):
        """Copy the state variables from device memory to host memory.

        Computes the damage first, then fills the given host arrays in place
        and returns them (``peripy/integrators.py:285-300``).
        """
        with self.context.on_stream():
            return self._write(u, ud, udd, force, body_force, damage, nlist,
                               n_neigh)

    def _synced(self):
        """Export the state and damage, and check the device status."""
        self._sync_state()
        self.context.stream.synchronize()
        if self.precision == "mixed":
            status = int(self.status_d.cpu().item())
            if status != _lib.PP_STATUS_OK:
                raise _lib.LibraryError(
                    f"a mixed-precision step reported device status {status} "
                    "(PP_STATUS_*): the state is invalid")

    @staticmethod
    def _put(host, dev):
        """Fill ``host`` with ``dev`` (as ``cl.enqueue_copy`` fills it).

        A C-contiguous, writeable host array of the device dtype and size
        receives the copy directly (the DMA writes its pages; a fresh
        staging array would be page-faulted in first, several times
        slower); anything else goes through a host copy.
        """
        import torch
        if host is None:
            return dev.cpu().numpy()
        np_dtype = {torch.float64: np.float64, torch.float32: np.float32,
                    torch.int32: np.int32,
                    torch.int64: np.int64}.get(dev.dtype)
        if (isinstance(host, np.ndarray) and host.flags.c_contiguous
                and host.flags.writeable and host.size == dev.numel()
                and host.dtype == np_dtype):
            # A large array is page-locked for the copy, so that the DMA
            # writes it directly instead of through the driver's staging
            # buffers (on the GPU machine: ~130 against ~20 GB/s into fresh
            # pages); if it cannot be registered it is copied as it is.
            # Memory that is pinned already (a view of a pinned tensor) is
            # left as it is: registering it again would fail.
            # The registration goes through the library, whose own CUDA
            # runtime keeps (and clears) the error of a failed attempt,
            # e.g. when only part of the array is registered already.
            target = torch.from_numpy(host.reshape(-1))
            registered = False
            if host.nbytes >= _REGISTER_BYTES and not target.is_pinned():
                registered = lib().pp_host_register(
                    host.ctypes.data, host.nbytes) == _lib.PP_SUCCESS
            try:
                target.copy_(dev.reshape(-1))
            finally:
                if registered:
                    lib().pp_host_unregister(host.ctypes.data)
            return host
        src = dev.cpu().numpy()
        flat = host.reshape(-1)
        flat[:src.size] = src.reshape(-1)[:flat.size]
        return host

    def write_sums(self, u, damage, sums):
        """A write step that brings back only ``u`` and ``damage``.

        Computes the damage, copies displacements and damage into the given
        host arrays (as :meth:`write` does) and evaluates the write-step
        sums of the whole state on the device.

        :arg sums: a :class:`~.writes.WriteSums` of this model.
        :returns: ``(u, damage, values)``, ``values`` as
            :meth:`.writes.WriteSums.__call__` returns them.
        """
        with self.context.on_stream():
            self._synced()
            values = sums(self.u_d[self._parity], self.ud_d, self.udd_d,
                          self.force_d, self.body_force_d, self.damage_d)
            return (self._put(u, self.u_d[self._parity]),
                    self._put(damage, self.damage_d), values)

    def _write(self, u, ud, udd, force, body_force, damage, nlist, n_neigh):
        self._synced()
        cur = self.u_d[self._parity]
        put = self._put
        u = put(u, cur)
        ud = put(ud, self.ud_d)
        udd = put(udd, self.udd_d)
        force = put(force, self.force_d)
        body_force = put(body_force, self.body_force_d)
        damage = put(damage, self.damage_d)
        nlist = put(nlist, self.nlist_d)
        n_neigh = put(n_neigh, self.n_neigh_d)
        return (u, ud, udd, force, body_force, damage, nlist, n_neigh)


class Euler(Integrator):
    r"""PeriPy's CPU integrator ``Euler`` (``peripy/integrators.py:303-459``)
    on the GPU.

    Same arithmetic and the same sequential semantics as the Cython step it
    replaces (``peripy/peridynamics.pyx``), bit for bit: bonds break when
    ``|strain| >= critical_stretch`` (tension or compression) and are
    swap-removed from both rows; each bond pair's force is applied to both
    nodes; ``u(t + dt) = u(t) + dt f(t)``.  As in the reference, the
    ``context`` attribute is None, so :class:`~.model.Model` builds the
    compact, 0-padded neighbour list this step works on; the kernels run on
    a :class:`CUDAContext` of their own (``device_context``, device 0 by
    default).  Bond types, n-linear damage, stiffness corrections and
    densities are rejected as the reference rejects them.  The neighbour
    list must be symmetric (j among the valid entries of row i exactly when
    i is among those of row j), as every list Model builds is:
    :meth:`create_buffers` raises ValueError otherwise.
    """

    def __init__(self, dt, device_context=None, fused=True):
        """Create an :class:`Euler` integrator object.

        :arg float dt: The length of time (in seconds [s]) of one time-step.
        :arg device_context: Optional :class:`CUDAContext` for the kernels.
        :arg bool fused: True: bond breaking and bond forces in one kernel
            (``pp_cy_break_and_force``, each bond's strain computed once,
            reference lengths cached per entry); False: one kernel per
            Cython function.  Same results.
        """
        if device_context is not None and not isinstance(device_context,
                                                         CUDAContext):
            raise TypeError("device_context must be a CUDAContext object")
        self.dt = dt
        self.fused = bool(fused)
        # Not a device-layout integrator: Model builds the compact layout
        self.context = None
        self._device = device_context
        lib()  # fail loudly now if the CUDA library is missing

    @property
    def device_context(self):
        if self._device is None:
            self._device = CUDAContext(0)
        return self._device

    def _dev(self, array, dtype, shape=None):
        import torch
        a = np.ascontiguousarray(array, dtype=dtype)
        if shape is not None:
            a = a.reshape(shape)
        return torch.as_tensor(a, device=self.device_context.device).clone()

    def build(self, nnodes, degrees_freedom, max_neighbours, coords, volume,
              family, bc_types, bc_values, force_bc_types, force_bc_values,
              stiffness_corrections, bond_types, densities):
        """Initiate integrator arrays (``peripy/integrators.py:371-412``)."""
        if bond_types is not None:
            raise ValueError("bond_types are not supported by this "
                             "integrator (expected {}, got {}), please use "
                             "EulerCL instead".format(type(None),
                                                      type(bond_types)))
        if stiffness_corrections is not None:
            raise ValueError("stiffness_corrections are not supported by this "
                             "integrator (expected {}, got {}), please use "
                             "EulerCL instead".format(
                                 type(None), type(stiffness_corrections)))
        if densities is not None:
            raise ValueError("densities are not supported by this "
                             "integrator (expected {}, got {}). This "
                             " integrator neglects inertial effects. Do not "
                             "supply a density or is_density argument or, "
                             "alternatively, please use a dynamic integrator, "
                             "such as EulerCromerCL.".format(type(None),
                                                             type(densities)))
        n = int(nnodes)
        self.nnodes = n
        self.coords = coords
        self.family = family
        self.volume = volume
        self.bc_types = bc_types
        self.bc_values = bc_values
        self.force_bc_types = force_bc_types
        self.force_bc_values = force_bc_values
        with self.device_context.on_stream():
            self._coords_d = self._dev(coords, np.float64, (n, 3))
            self._volume_d = self._dev(volume, np.float64, (n,))
            self._family_d = self._dev(family, np.int32, (n,))
            self._bc_types_d = self._dev(bc_types, np.int32, (n, 3))
            self._bc_values_d = self._dev(bc_values, np.float64, (n, 3))
            self._fc_types_d = self._dev(force_bc_types, np.int32, (n, 3))
            self._fc_values_d = self._dev(force_bc_values, np.float64, (n, 3))

    def create_buffers(self, nlist, n_neigh, bond_stiffness, critical_stretch,
                       plus_cs, u, ud, udd, force, body_force, damage, regimes,
                       nregimes, nbond_types):
        """Initiate the simulation arrays (``peripy/integrators.py:351-369``).
        """
        if nregimes != 1:
            raise ValueError("n-linear damage model's are not supported by "
                             "this integrator. Please supply just one "
                             "bond_stiffness.")
        if nbond_types != 1:
            raise ValueError("n-material composite models are not supported by"
                             " this integrator. Please supply just one "
                             "material type and bond_stiffness.")
        import torch
        self.nlist = nlist
        self.n_neigh = n_neigh
        self.bond_stiffness = bond_stiffness
        self.critical_stretch = critical_stretch
        self.u = u
        self.ud = ud
        self.udd = udd
        self.force = force
        self.body_force = body_force
        n = self.nnodes
        width = int(np.shape(nlist)[1]) if np.ndim(nlist) == 2 else 0
        if width > 1024:
            raise ValueError("the neighbour list is wider than 1024 (got "
                             f"{width})")
        self._width = width
        with self.device_context.on_stream():
            nlist_d = self._dev(nlist, np.int32, (n, width))
            n_neigh_d = self._dev(n_neigh, np.int32, (n,))
            if not self._symmetric(nlist_d, n_neigh_d, width):
                raise ValueError(
                    "the GPU Euler integrator needs a symmetric neighbour "
                    "list (j among the first n_neigh[i] entries of row i "
                    "exactly when i is among those of row j), as Model "
                    "builds it; this list is not")
            self._nlist_d, self._n_neigh_d = nlist_d, n_neigh_d
            self._u_d = self._dev(u, np.float64, (n, 3))
            self._force_d = self._dev(force, np.float64, (n, 3))
            self._damage_d = torch.empty(n, dtype=torch.float64,
                                         device=self.device_context.device)
            self._l0_d = None
            if self.fused and width > 0 and n > 0:
                # reference length of every entry (the same value the step
                # would compute), kept in entry order by the fused kernel
                self._l0_d = torch.empty((n, width), dtype=torch.float64,
                                         device=self.device_context.device)
                check(lib().pp_bond_lengths(
                    _ptr(self._coords_d), _ptr(self._nlist_d), n, width,
                    _ptr(self._l0_d), self.device_context.stream_handle),
                    "pp_bond_lengths")

    def _symmetric(self, nlist_d, n_neigh_d, width):
        """Is j an entry of row i exactly as often as i is one of row j?
        (``pp_cy_check_symmetric``: one warp per row on the device.)"""
        import torch
        bad = torch.empty(1, dtype=torch.int32,
                          device=self.device_context.device)
        check(lib().pp_cy_check_symmetric(
            _ptr(nlist_d), _ptr(n_neigh_d), self.nnodes, width, _ptr(bad),
            self.device_context.stream_handle), "pp_cy_check_symmetric")
        return int(bad.cpu().item()) == 0

    def __call__(self, displacement_bc_magnitude, force_bc_magnitude):
        """One step: break bonds, bond forces, Euler update
        (``peripy/integrators.py:330-349``)."""
        ctx = self.device_context
        st = ctx.stream_handle
        L = lib()
        n, w = self.nnodes, self._width
        with ctx.on_stream():
            if self.fused:
                check(L.pp_cy_break_and_force(
                    _ptr(self._coords_d), _ptr(self._u_d),
                    _ptr(self._nlist_d), _ptr(self._n_neigh_d),
                    _ptr(self._volume_d), float(self.bond_stiffness),
                    float(self.critical_stretch), _ptr(self._fc_values_d),
                    _ptr(self._fc_types_d), float(force_bc_magnitude), n, w,
                    _ptr(self._force_d), _ptr(self._l0_d), st),
                    "pp_cy_break_and_force")
            else:
                self._break_and_force(L, n, w, force_bc_magnitude, st)
            check(L.pp_cy_update_displacement(
                _ptr(self._u_d), _ptr(self._bc_values_d),
                _ptr(self._bc_types_d), _ptr(self._force_d),
                float(displacement_bc_magnitude), float(self.dt), n, st),
                "pp_cy_update_displacement")

    def _break_and_force(self, L, n, w, force_bc_magnitude, st):
        """break_bonds and bond_force as two kernels."""
        check(L.pp_cy_break_bonds(
            _ptr(self._coords_d), _ptr(self._u_d), _ptr(self._nlist_d),
            _ptr(self._n_neigh_d), n, w, float(self.critical_stretch), st),
            "pp_cy_break_bonds")
        check(L.pp_cy_bond_force(
            _ptr(self._coords_d), _ptr(self._u_d), _ptr(self._nlist_d),
            _ptr(self._n_neigh_d), _ptr(self._volume_d),
            float(self.bond_stiffness), _ptr(self._fc_values_d),
            _ptr(self._fc_types_d), float(force_bc_magnitude), n, w,
            _ptr(self._force_d), st), "pp_cy_bond_force")

    def write(self, damage, u, ud, udd, force, body_force, nlist, n_neigh):
        """Return the state variable arrays (``peripy/integrators.py:
        452-459``): the arrays given to :meth:`create_buffers`, filled from
        the device, and a new damage array.  The arguments are ignored, as
        the reference ignores them."""
        ctx = self.device_context
        put = _CUDAIntegrator._put
        with ctx.on_stream():
            check(lib().pp_cy_damage(_ptr(self._n_neigh_d),
                                     _ptr(self._family_d), self.nnodes,
                                     _ptr(self._damage_d), ctx.stream_handle),
                  "pp_cy_damage")
            ctx.stream.synchronize()
            self.u = put(self.u, self._u_d)
            self.force = put(self.force, self._force_d)
            self.nlist = put(self.nlist, self._nlist_d)
            self.n_neigh = put(self.n_neigh, self._n_neigh_d)
            damage = self._damage_d.cpu().numpy()
        return (self.u, self.ud, self.udd, self.force, self.body_force, damage,
                self.nlist, self.n_neigh)

    def _create_special_buffers(self):
        """Create buffers that are special to the Euler integrator."""
        # There are none

    def _build_special(self):
        """Build programs that are special to the Euler integrator."""
        # There are none


class EulerCUDA(_CUDAIntegrator):
    r"""Euler integrator on CUDA (replaces ``EulerCL``, integrators.py:462).

    .. math::
        u(t + \delta t) = u(t) + \delta t f(t)
    """

    _kind = _lib.PP_EULER
    _dynamic = False

    def __init__(self, *args, **kwargs):
        """Create an :class:`EulerCUDA` integrator object."""
        super().__init__(*args, **kwargs)

    def _update_displacement(self, displacement_bc_magnitude):
        check(lib().pp_update_displacement_euler(
            _ptr(self.force_d), _ptr(self.u_d[0]), _ptr(self.bc_types_d),
            _ptr(self.bc_values_d), float(displacement_bc_magnitude),
            float(self.dt), 3 * self.nnodes, self._stream),
            "pp_update_displacement_euler")


class EulerCromerCUDA(_CUDAIntegrator):
    r"""Euler-Cromer integrator on CUDA (replaces ``EulerCromerCL``).

    .. math::
        \ddot{u}(t) = \frac{f(t) - \eta \dot{u}(t)}{\rho},\quad
        \dot{u}(t + \delta t) = \dot{u}(t) + \delta t \ddot{u}(t),\quad
        u(t + \delta t) = u(t) + \delta t \dot{u}(t + \delta t)
    """

    _kind = _lib.PP_EULER_CROMER
    _dynamic = True

    def __init__(self, damping, *args, **kwargs):
        """Create an :class:`EulerCromerCUDA` integrator object.

        :arg float damping: The dynamic relaxation damping constant with
            units [kg/(m^3 s)]
        """
        super().__init__(*args, **kwargs)
        self.damping = damping

    def _update_displacement(self, displacement_bc_magnitude):
        check(lib().pp_update_displacement_euler_cromer(
            _ptr(self.force_d), _ptr(self.u_d[0]), _ptr(self.ud_d),
            _ptr(self.udd_d), _ptr(self.bc_types_d), _ptr(self.bc_values_d),
            _ptr(self.densities_d), float(displacement_bc_magnitude),
            float(self.damping), float(self.dt), 3 * self.nnodes,
            self._stream), "pp_update_displacement_euler_cromer")


class VelocityVerletCUDA(_CUDAIntegrator):
    r"""Velocity-Verlet integrator on CUDA (replaces ``VelocityVerletCL``).

    Uses the reference's own update (``peripy/cl/velocity_verlet.cl:90-94``):
    the displacement advances by ``dt * (ud + dt/2 * udd)`` with the new
    full-step velocity ``ud`` and acceleration ``udd``.
    """

    _kind = _lib.PP_VELOCITY_VERLET
    _dynamic = True

    def __init__(self, damping, *args, **kwargs):
        """Create a :class:`VelocityVerletCUDA` integrator object.

        :arg float damping: The dynamic relaxation damping constant with
            units [kg/(m^3 s)]
        """
        super().__init__(*args, **kwargs)
        self.damping = damping

    def _update_displacement(self, displacement_bc_magnitude):
        check(lib().pp_update_displacement_velocity_verlet(
            _ptr(self.force_d), _ptr(self.u_d[0]), _ptr(self.ud_d),
            _ptr(self.udd_d), _ptr(self.bc_types_d), _ptr(self.bc_values_d),
            _ptr(self.densities_d), float(displacement_bc_magnitude),
            float(self.damping), float(self.dt), 3 * self.nnodes,
            self._stream), "pp_update_displacement_velocity_verlet")


# Drop-in names of the reference's device integrators.
EulerCL = EulerCUDA
EulerCromerCL = EulerCromerCUDA
VelocityVerletCL = VelocityVerletCUDA
