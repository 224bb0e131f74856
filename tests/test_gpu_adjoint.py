"""Adjoint of the Euler rollout (GPU).

* Central finite differences on 32 random bonds of the 50x50x5 lattice
  after 500 Euler steps, loss = sum of squared displacements of 100 seeded
  probe nodes, checkpoint every 50 steps, in two set-ups:
  - as the adjoint workload states it: float32 stiffness parameter, pull
    1e-9 per step, relative step 1e-4; agreement better than 1e-2;
  - well conditioned: float64 stiffness, pull 1e-5 per step, relative step
    1e-3; agreement better than 1e-6.
  The difference quotient is limited by rounding, not truncation: the
  stretch (|p| - |xi|)/|xi| loses log10(1/s) digits to cancellation, so the
  quotient's error grows as the strain or the step shrinks (measured on 8
  bonds: at a pull of 1e-9 per step the error is up to 1e-4 at step 1e-3,
  1e-3 at 1e-4 and 6e-3 at 1e-5; at 1e-5 per step up to 1e-8 at step 1e-3
  and 4e-5 at 1e-6).  Bonds are drawn among those whose gradient is at
  least 1e-2 of the largest.
* An FP64 torch-autograd restatement of the same forward (breaking included,
  the break pattern frozen as the adjoint freezes it) on a smaller lattice
  whose bonds break: gradients agree to 1e-9 relative.
* The gradient with respect to the critical stretch is zero, and so is its
  finite difference while no bond breaks.
* Gradients do not depend on the checkpoint interval (bit for bit).
"""
import numpy as np
import pytest

from tests.conftest import cuda_available
from tests.gpu_helpers import lattice, pull_bcs

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]

DT = 0.5
K0 = 0.01


@pytest.fixture(scope="module")
def torch():
    import torch as _torch
    return _torch


def _problem(nx, ny, nz, steps, rate):
    from probabilistic_peridynamics_gb300.adjoint import AdjointProblem
    coords, volume, _, family, nlist, _ = lattice(nx, ny, nz, 1.0)
    bc_types, bc_values = pull_bcs(coords, 0)
    mags = rate * np.arange(1, steps + 1)
    prob = AdjointProblem(coords, volume, nlist, bc_types, bc_values, mags,
                          DT)
    return prob, coords, volume, nlist, bc_types, bc_values, mags


def _stiffness(nlist, seed, torch):
    rng = np.random.default_rng(seed)
    k = np.where(nlist != -1, K0 * rng.uniform(0.9, 1.1, nlist.shape), 0.0)
    return torch.tensor(k, dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("rate,eps,tol,param", [
    (1e-9, 1e-4, 1e-2, "float32"),
    (1e-5, 1e-3, 1e-6, "float64")], ids=["stated", "conditioned"])
def test_adjoint_vs_central_differences(torch, rate, eps, tol, param):
    from probabilistic_peridynamics_gb300.adjoint import rollout
    steps, every = 500, 50
    prob, coords, _, nlist, *_ = _problem(50, 50, 5, steps, rate)
    rng = np.random.default_rng(4)
    probes = torch.tensor(rng.choice(coords.shape[0], 100, replace=False),
                          device="cuda")
    dtype = getattr(torch, param)
    k = _stiffness(nlist, 1, torch).to(dtype).requires_grad_(True)
    s0 = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)

    def loss(kk):
        u = rollout(kk, s0, prob, steps, every)
        return (u[probes] ** 2).sum()

    L = loss(k)
    L.backward()
    assert k.grad.dtype == dtype
    grad = k.grad.detach().double().cpu().numpy()
    # Central differences resolve a bond's gradient only above the rounding
    # noise of the loss: draw the 32 random bonds among those whose
    # gradient is at least 1e-2 of the largest.
    significant = np.argwhere((nlist != -1) &
                              (np.abs(grad) >= 1e-2 * np.abs(grad).max()))
    assert len(significant) >= 32
    picks = significant[rng.choice(len(significant), 32, replace=False)]
    with torch.no_grad():
        for i, s in picks:
            kp = k.detach().clone()
            kp[i, s] *= 1 + eps
            km = k.detach().clone()
            km[i, s] *= 1 - eps
            # the step actually taken, after rounding to the parameter type
            h2 = float(kp[i, s].double() - km[i, s].double())
            fd = (float(loss(kp)) - float(loss(km))) / h2
            g = grad[i, s]
            assert abs(fd - g) <= tol * abs(fd), (i, s, fd, g)
    # critical stretch: frozen breaks, zero gradient and zero FD (nothing
    # breaks at s0 = 1 in this elastic run)
    assert float(s0.grad) == 0.0
    with torch.no_grad():
        l1 = float(loss(k.detach()))
        s0.data.fill_(2.0)
        l2 = float(loss(k.detach()))
    assert l1 == l2


def _torch_reference(torch, k, coords, volume, nlist, bc_types, bc_values,
                     mags, steps, s0):
    """FP64 autograd restatement of the breaking Euler rollout."""
    dev = "cuda"
    r0 = torch.tensor(coords, dtype=torch.float64, device=dev)
    vol = torch.tensor(volume, dtype=torch.float64, device=dev)
    nl = torch.tensor(nlist, dtype=torch.int64, device=dev)
    bct = torch.tensor(bc_types, device=dev) != 0
    bcv = torch.tensor(bc_values, dtype=torch.float64, device=dev)
    n = r0.shape[0]
    ii = torch.arange(n, device=dev)[:, None].expand_as(nl)
    valid = nl != -1
    jj = torch.where(valid, nl, (ii + 1) % n)  # finite stand-in for padding
    xi_v = r0[jj] - r0[ii]
    xi = torch.sqrt((xi_v * xi_v).sum(-1))
    u = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    for t in range(steps):
        p = xi_v + u[jj] - u[ii]
        y = torch.sqrt((p * p).sum(-1))
        s = (y - xi) / xi
        with torch.no_grad():
            valid = valid & (s < s0)
        f = torch.where(valid, s * k * vol[jj], torch.zeros_like(s))
        force = (f[..., None] * p / y[..., None]).sum(1)
        u = torch.where(bct, float(mags[t]) * bcv, u + DT * force)
    return u, valid


def test_adjoint_vs_fp64_autograd_with_breaks(torch):
    from probabilistic_peridynamics_gb300.adjoint import rollout
    steps, s0 = 40, 0.02
    prob, coords, volume, nlist, bct, bcv, mags = _problem(9, 7, 4, steps,
                                                           3e-3)
    k_ref = _stiffness(nlist, 2, torch).requires_grad_(True)
    u_ref, valid = _torch_reference(torch, k_ref, coords, volume, nlist, bct,
                                    bcv, mags, steps, s0)
    assert int(valid.sum()) < int((torch.tensor(nlist) != -1).sum())
    w = torch.linspace(0.5, 1.5, u_ref.numel(), dtype=torch.float64,
                       device="cuda").reshape(u_ref.shape)
    (w * u_ref ** 2).sum().backward()
    k = k_ref.detach().clone().requires_grad_(True)
    u = rollout(k, s0, prob, steps, checkpoint_every=7)
    (w * u ** 2).sum().backward()
    scale = float(k_ref.grad.abs().max())
    assert float((u - u_ref).detach().abs().max()) <= \
        1e-12 * float(u_ref.detach().abs().max())
    assert float((k.grad - k_ref.grad).abs().max()) <= 1e-9 * scale


def test_checkpoint_interval_does_not_change_gradients(torch):
    from probabilistic_peridynamics_gb300.adjoint import rollout
    steps = 30
    prob, _, _, nlist, *_ = _problem(8, 6, 4, steps, 3e-3)
    grads = []
    for every in (1, 7, 30):
        k = _stiffness(nlist, 3, torch).to(torch.float32).requires_grad_(True)
        u = rollout(k, 0.02, prob, steps, checkpoint_every=every)
        (u ** 2).sum().backward()
        assert k.grad.dtype == torch.float32
        grads.append(k.grad.detach().cpu().numpy())
    assert np.array_equal(grads[0], grads[1])
    assert np.array_equal(grads[0], grads[2])
