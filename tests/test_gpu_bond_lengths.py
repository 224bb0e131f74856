"""Cached reference bond lengths of the fused binary64 step.

``pp_bond_lengths`` writes ``|r0[j] - r0[i]|`` per slot with the bond
body's own binary64 operations (``peripy/cl/peridynamics.cl:65-73``); the
fused FP64 step reads it instead of a square root per bond and step.  Bar:
the lengths equal NumPy's ``sqrt((x*x + y*y) + z*z)`` bit for bit, and the
fused step with the cache is bit-identical to the step without it (and so
to the oracle, which the parity tests check with the cache in place) for
every integrator, with breaks, bond types and corrections.
"""
import ctypes

import numpy as np
import pytest

from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


def test_lengths_match_numpy():
    import torch
    from probabilistic_peridynamics_gb300 import _lib, lattice
    from probabilistic_peridynamics_gb300.integrators import CUDAContext
    rng = np.random.default_rng(5)
    coords = lattice.lattice_coords(12, 9, 7, 0.013)
    coords = coords + rng.uniform(-3e-3, 3e-3, coords.shape)
    family, nlist, width = lattice.lattice_family(12, 9, 7, 2.6)
    nlist = nlist.copy()
    nlist[rng.uniform(size=nlist.shape) < 0.1] = -1  # broken bonds
    n = coords.shape[0]
    ctx = CUDAContext(0)
    dev = ctx.device
    r0 = torch.as_tensor(coords, device=dev)
    nl = torch.as_tensor(nlist, device=dev)
    out = torch.full((n, int(width)), np.nan, dtype=torch.float64, device=dev)
    with ctx.on_stream():
        assert _lib.lib().pp_bond_lengths(
            ctypes.c_void_p(r0.data_ptr()), ctypes.c_void_p(nl.data_ptr()), n,
            int(width), ctypes.c_void_p(out.data_ptr()),
            ctx.stream_handle) == 0
    got = out.cpu().numpy()
    j = np.where(nlist >= 0, nlist, 0)
    d = coords[j] - coords[:, None, :]
    want = np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1])
                   + d[..., 2] * d[..., 2])
    want[nlist < 0] = 0.0
    assert np.array_equal(got, want)


@pytest.mark.parametrize("kind", ["euler", "euler_cromer", "velocity_verlet"])
def test_fused_step_with_and_without_cache(kind):
    import probabilistic_peridynamics_gb300 as pp
    from tests.gpu_helpers import run_integrator
    from tests.gpu_helpers import breaking_setup
    setup = breaking_setup(kind)
    cls = {"euler": pp.EulerCUDA, "euler_cromer": pp.EulerCromerCUDA,
           "velocity_verlet": pp.VelocityVerletCUDA}[kind]
    steps = 60
    mags = 3e-3 * np.arange(1, steps + 1)
    outs = []
    for cached in (True, False):
        integ = (cls(dt=setup["dt"]) if kind == "euler"
                 else cls(0.5, dt=setup["dt"]))
        if not cached:
            orig = integ._make_fused_args

            def no_cache(orig=orig):
                a = orig()
                a.bond_length = None
                return a
            integ._make_fused_args = no_cache
        outs.append(run_integrator(integ, setup, steps, mags))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    assert np.any(outs[0][6] == -1)  # bonds broke
