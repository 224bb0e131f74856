"""The entry point that allocates nothing, against the existing one (GPU).

``pp_fused_run_static`` is for callers that cannot allocate device memory
themselves (for example code handed a fixed set of device arrays by its
host runtime): it takes the boundary-condition magnitude schedule in host
memory and keeps every scratch word in a device array the library owns.
Here it is called through the C ABI for two calls in a row and must give
exactly the results of ``pp_fused_run`` (device-side schedule, caller
scratch) -- the bar of the other parity tests for these paths is bit
equality -- for the binary64 and the mixed-precision step.  It must also
reject more steps than its array holds.

This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from tests.conftest import cuda_available
from tests.gpu_helpers import lattice, pull_bcs

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


def _setup():
    coords, volume, _, family, nlist, n_neigh = lattice(10, 8, 4, 1.0)
    n = coords.shape[0]
    bc_types, bc_values = pull_bcs(coords, 0)
    return dict(coords=coords, volume=volume, family=family, nlist=nlist,
                n_neigh=n_neigh, bc_types=bc_types, bc_values=bc_values,
                force_bc_types=np.zeros((n, 3), dtype=np.intc),
                force_bc_values=np.zeros((n, 3)),
                densities=np.full((n, 3), 50.0), nnodes=n,
                max_neigh=nlist.shape[1])


def _integrator(setup, precision):
    import probabilistic_peridynamics_gb300 as pp
    integ = pp.VelocityVerletCUDA(0.5, dt=1.0, precision=precision)
    n = setup["nnodes"]
    integ.build(n, 3, setup["max_neigh"], setup["coords"], setup["volume"],
                setup["family"], setup["bc_types"], setup["bc_values"],
                setup["force_bc_types"], setup["force_bc_values"], None,
                None, setup["densities"])
    z = np.zeros((n, 3))
    integ.create_buffers(setup["nlist"], setup["n_neigh"], 0.01, 0.02, None,
                         z, z, z, z, z, np.zeros(n), None, 1, 1)
    return integ


def _state(integ, setup):
    n = setup["nnodes"]
    z = lambda: np.zeros((n, 3))  # noqa: E731
    return integ.write(z(), z(), z(), z(), z(), np.zeros(n),
                       setup["nlist"].copy(), setup["n_neigh"].copy())


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_static_run_matches_fused_run(precision):
    from probabilistic_peridynamics_gb300 import _lib
    L = _lib.lib()
    setup = _setup()
    steps = 40
    disp = np.ascontiguousarray(3e-3 * np.arange(1, 2 * steps + 1))
    force = np.zeros(2 * steps)
    ref = _integrator(setup, precision)
    new = _integrator(setup, precision)
    broke = False
    for first in (0, steps):  # two calls in a row
        ref._run(disp, force, first, steps)
        rc = L.pp_fused_run_static(
            ctypes.byref(new._fargs), new._parity, steps,
            disp[first:].ctypes.data_as(ctypes.c_void_p),
            force[first:].ctypes.data_as(ctypes.c_void_p), new._stream)
        assert rc == _lib.PP_SUCCESS, L.pp_status_string(rc)
        new._parity ^= steps & 1
        status = ctypes.c_int32(-1)
        assert L.pp_static_status(ctypes.byref(status), new._stream) == 0
        assert status.value == _lib.PP_STATUS_OK
        got, want = _state(new, setup), _state(ref, setup)
        for a, b in zip(got, want):
            assert np.array_equal(a, b)
        broke = broke or bool(np.any(got[6] != setup["nlist"]))
    assert broke  # the run exercises load-induced breaking


def test_static_run_rejects_too_many_steps():
    from probabilistic_peridynamics_gb300 import _lib
    L = _lib.lib()
    setup = _setup()
    integ = _integrator(setup, "float64")
    n = _lib.PP_STATIC_MAX_STEPS + 1
    mags = np.zeros(n)
    ptr = mags.ctypes.data_as(ctypes.c_void_p)
    rc = L.pp_fused_run_static(ctypes.byref(integ._fargs), 0, n, ptr, ptr,
                               integ._stream)
    assert rc == _lib.PP_ERROR_TOO_LARGE
    assert b"PP_STATIC_MAX_STEPS" in L.pp_status_string(rc)


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_static_run_leaves_device_memory_unchanged(precision):
    """Free device memory (cudaMemGetInfo) is the same before and after the
    first ``pp_fused_run_static`` call and after a second one.

    The CUDA runtime loads a library's module lazily, at its first use in a
    context; that load places the module's code and its file-scope array
    (the 1 MB schedule buffer) in device memory, where they stay until the
    process exits.  ``pp_static_status`` is called first so that this load
    happens before the measurement: what is measured is the call itself.
    """
    import torch
    from probabilistic_peridynamics_gb300 import _lib
    L = _lib.lib()
    setup = _setup()
    steps = 40
    disp = np.ascontiguousarray(3e-3 * np.arange(1, 2 * steps + 1))
    force = np.zeros(2 * steps)
    ref = _integrator(setup, precision)
    ref._run(disp, force, 0, steps)  # loads the step kernels' modules
    integ = _integrator(setup, precision)
    status = ctypes.c_int32(-1)
    assert L.pp_static_status(ctypes.byref(status), integ._stream) == 0
    torch.cuda.synchronize()
    free = [torch.cuda.mem_get_info()[0]]
    for first in (0, steps):
        rc = L.pp_fused_run_static(
            ctypes.byref(integ._fargs), integ._parity, steps,
            disp[first:].ctypes.data_as(ctypes.c_void_p),
            force[first:].ctypes.data_as(ctypes.c_void_p), integ._stream)
        assert rc == _lib.PP_SUCCESS, L.pp_status_string(rc)
        integ._parity ^= steps & 1
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
    assert free[1] == free[0] and free[2] == free[0], free
