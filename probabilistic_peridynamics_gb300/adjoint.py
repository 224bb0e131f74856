"""Gradients of a displacement loss through an Euler rollout.

:class:`AdjointProblem` holds a model (the arrays ``Integrator.build``
takes) whose per-bond stiffness ``k_b`` is a parameter; :func:`rollout`
runs ``steps`` Euler steps from rest and returns the final displacement as
a differentiable function of ``k_b`` (``torch.autograd``).

Forward: the binary64 fused step (``pp_fused_step``, per-bond stiffness as
stiffness corrections with unit bond stiffness, ``peripy/cl/peridynamics.cl
:214`` semantics, breaking at the given critical stretch); after each step
the first step at which every bond is seen broken is recorded
(``pp_mark_breaks``), and the state is kept every ``checkpoint_every`` steps.

Backward: for each checkpoint segment, last first, the states of the segment
are recomputed from its checkpoint with the bond set of each step frozen
(``pp_bonds_at_step``, no new breaks), then ``pp_adjoint_backward`` runs the
reverse steps.  Memory is one checkpoint per segment plus the states of one
segment, so long rollouts fit in device memory.  The break pattern is
frozen in the backward pass: the loss is piecewise constant in the critical
stretch, whose gradient is therefore zero.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib
from .integrators import CUDAContext

INT32_MAX = 2 ** 31 - 1


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class AdjointProblem:
    """A model with a per-bond stiffness parameter, stepped with Euler.

    :arg coords, volume, nlist, bc_types, bc_values: as ``Integrator.build``
        / ``create_buffers`` take them (CL layout: ``-1`` padded, power-of-
        two width).
    :arg displacement_bc_magnitudes: magnitude of the displacement boundary
        condition at each step (len >= steps).
    :arg float dt: time step.
    """

    def __init__(self, coords, volume, nlist, bc_types, bc_values,
                 displacement_bc_magnitudes, dt, context=None):
        import torch
        self.torch = torch
        self.context = context if context is not None else CUDAContext(0)
        dev = self.context.device
        nlist = np.ascontiguousarray(nlist, dtype=np.intc)
        self.nnodes, self.max_neigh = nlist.shape
        mn = self.max_neigh
        if mn < 1 or mn > 1024 or (mn & (mn - 1)):
            raise ValueError("max_neigh must be a power of two <= 1024")
        n = self.nnodes
        self.dt = float(dt)
        self.mags = np.asarray(displacement_bc_magnitudes, dtype=np.float64)

        def dev_t(a, dtype):
            return torch.as_tensor(np.ascontiguousarray(a, dtype=dtype)).to(
                dev)

        with self.context.on_stream():
            self.r0 = dev_t(coords, np.float64).reshape(n, 3)
            self.vols = dev_t(volume, np.float64)
            self.nlist0 = dev_t(nlist, np.int32)
            self.bc_types = dev_t(bc_types, np.int32).reshape(n, 3)
            self.bc_values = dev_t(bc_values, np.float64).reshape(n, 3)
            self.family = (self.nlist0 != -1).sum(dim=1).to(torch.int32)
            self.zeros_i = torch.zeros((n, 3), dtype=torch.int32, device=dev)
            self.zeros_d = torch.zeros((n, 3), dtype=torch.float64,
                                       device=dev)
            self.partner = torch.empty_like(self.nlist0)
            self.force = torch.empty((n, 3), dtype=torch.float64, device=dev)
            self.body = torch.empty_like(self.force)
            self.n_neigh = torch.empty(n, dtype=torch.int32, device=dev)
            self.damage = torch.empty(n, dtype=torch.float64, device=dev)
            check(lib().pp_partner_slots(_p(self.nlist0), n, mn,
                                         _p(self.partner), self._stream),
                  "pp_partner_slots")
            # reference bond lengths for the binary64 forward step (read
            # instead of a square root per bond and step; same values)
            self.bond_length = torch.empty((n, mn), dtype=torch.float64,
                                           device=dev)
            check(lib().pp_bond_lengths(_p(self.r0), _p(self.nlist0), n, mn,
                                        _p(self.bond_length), self._stream),
                  "pp_bond_lengths")

    @property
    def _stream(self):
        return self.context.stream_handle

    def step(self, u, k, t, nlist, critical_stretch):
        """One binary64 Euler step from ``u``; returns the new state.

        ``nlist`` (device, mutated where bonds break) and the per-bond
        stiffness ``k`` (device float64) define the bonds.
        """
        torch = self.torch
        out = torch.empty_like(u)
        a = _lib.FusedArgs()
        a.nnodes, a.max_neigh = self.nnodes, self.max_neigh
        a.integrator, a.precision = _lib.PP_EULER, _lib.PP_FLOAT64
        a.dt = self.dt
        a.bond_stiffness = 1.0
        a.critical_stretch = float(critical_stretch)
        a.r0, a.vols, a.family = _p(self.r0), _p(self.vols), _p(self.family)
        a.bc_types, a.bc_values = _p(self.bc_types), _p(self.bc_values)
        a.fc_types, a.fc_values = _p(self.zeros_i), _p(self.zeros_d)
        a.stiffness_corrections = _p(k)
        a.bond_length = _p(self.bond_length)
        a.nlist = _p(nlist)
        a.u[0], a.u[1] = u.data_ptr(), out.data_ptr()
        a.force, a.body_force = _p(self.force), _p(self.body)
        a.n_neigh, a.damage = _p(self.n_neigh), _p(self.damage)
        check(lib().pp_fused_step(ctypes.byref(a), 0, float(self.mags[t]),
                                  0.0, self._stream), "pp_fused_step")
        return out

    def bonds_at_step(self, break_step, t, out):
        check(lib().pp_bonds_at_step(_p(self.nlist0), _p(break_step),
                                     self.nlist0.numel(), t, _p(out),
                                     self._stream), "pp_bonds_at_step")
        return out

    def backward_step(self, u, lam_next, grad_k, k, nlist):
        torch = self.torch
        lam = torch.empty_like(lam_next)
        a = _lib.AdjointArgs()
        a.nnodes, a.max_neigh, a.dt = self.nnodes, self.max_neigh, self.dt
        a.r0, a.vols = _p(self.r0), _p(self.vols)
        a.nlist, a.partner = _p(nlist), _p(self.partner)
        a.bc_types, a.stiffness = _p(self.bc_types), _p(k)
        check(lib().pp_adjoint_backward(ctypes.byref(a), _p(u),
                                        _p(lam_next), _p(lam), _p(grad_k),
                                        self._stream), "pp_adjoint_backward")
        return lam


def _rollout_function():
    import torch

    class Rollout(torch.autograd.Function):
        """u_T(k) of an Euler rollout; gradients by the adjoint kernel."""

        @staticmethod
        def forward(ctx, stiffness, critical_stretch, problem, steps,
                    checkpoint_every):
            caller = torch.cuda.current_stream(problem.context.device)
            problem.context.stream.wait_stream(caller)
            with problem.context.on_stream():
                k = stiffness.detach().to(torch.float64).contiguous()
                s0 = float(critical_stretch)
                nl = problem.nlist0.clone()
                breaks = torch.full_like(nl, INT32_MAX)
                u = torch.zeros((problem.nnodes, 3), dtype=torch.float64,
                                device=k.device)
                checkpoints = []
                for t in range(steps):
                    if t % checkpoint_every == 0:
                        checkpoints.append(u)
                    u = problem.step(u, k, t, nl, s0)
                    check(lib().pp_mark_breaks(_p(nl), _p(breaks), nl.numel(),
                                               t, problem._stream),
                          "pp_mark_breaks")
            # the caller's stream may use u only after the rollout
            caller.wait_stream(problem.context.stream)
            u.record_stream(caller)
            ctx.problem = problem
            ctx.steps = steps
            ctx.every = checkpoint_every
            ctx.checkpoints = checkpoints
            ctx.breaks = breaks
            ctx.k = k
            ctx.param_dtype = stiffness.dtype
            ctx.s0_like = torch.as_tensor(critical_stretch)
            return u

        @staticmethod
        def backward(ctx, grad_u):
            problem = ctx.problem
            caller = torch.cuda.current_stream(problem.context.device)
            problem.context.stream.wait_stream(caller)
            with problem.context.on_stream():
                lam = grad_u.detach().to(torch.float64).contiguous()
                grad_k = torch.zeros_like(ctx.k)
                nl_t = torch.empty_like(problem.nlist0)
                for seg in reversed(range(len(ctx.checkpoints))):
                    t0 = seg * ctx.every
                    t1 = min(t0 + ctx.every, ctx.steps)
                    states = [ctx.checkpoints[seg]]
                    for t in range(t0, t1 - 1):
                        problem.bonds_at_step(ctx.breaks, t, nl_t)
                        states.append(problem.step(states[-1], ctx.k, t, nl_t,
                                                   float("inf")))
                    for t in range(t1 - 1, t0 - 1, -1):
                        problem.bonds_at_step(ctx.breaks, t, nl_t)
                        lam = problem.backward_step(states[t - t0], lam,
                                                    grad_k, ctx.k, nl_t)
                # frozen breaks: the loss does not depend on the critical
                # stretch between breaks
                grad_s0 = (torch.zeros_like(ctx.s0_like, dtype=torch.float64)
                           if ctx.needs_input_grad[1] else None)
                grad_k = grad_k.to(ctx.param_dtype)
            caller.wait_stream(problem.context.stream)
            grad_k.record_stream(caller)
            return (grad_k, grad_s0, None, None, None)

    return Rollout


_ROLLOUT = None


def rollout(stiffness, critical_stretch, problem, steps, checkpoint_every=50):
    """Final displacement (nnodes, 3) float64 after ``steps`` Euler steps
    from rest, differentiable in ``stiffness`` ((nnodes, max_neigh) tensor,
    any float dtype) and ``critical_stretch`` (gradient zero: frozen
    breaks)."""
    global _ROLLOUT
    if _ROLLOUT is None:
        _ROLLOUT = _rollout_function()
    return _ROLLOUT.apply(stiffness, critical_stretch, problem, steps,
                          checkpoint_every)
