"""Write-step sums on the GPU (``pp_write_sums``) and ``Model.simulate``
with intermediate writes.

Bar: bit-identical to the reference's NumPy reductions
(``peripy/model.py:1320-1366``) on the same arrays -- ``np.sum`` of the
state arrays, of ``force * volume[:, None]`` and of damage, and the
sequential tip sums -- at odd lengths and at the 400k-node size; and a
``simulate`` with ``write=`` and tips gives the same ``data``, mesh files
and returned state as the host path that copies every array back.
"""
import numpy as np
import pytest

from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


def _host_sums(u, ud, udd, force, body_force, damage, volume, tip_types):
    """The reference's reductions (model.py:1329-1362) on host arrays."""
    model = [np.sum(u), np.sum(ud), np.sum(udd),
             np.sum(force * volume[:, np.newaxis]),
             np.sum(body_force * volume[:, np.newaxis]), np.sum(damage)]
    tips = []
    for node_list in tip_types.values():
        acc = np.zeros(5)
        for i, j in node_list:
            acc[0] += u[i, j]
            acc[1] += ud[i, j]
            acc[2] += udd[i, j]
            acc[3] += force[i, j] * volume[i]
            acc[4] += body_force[i, j] * volume[i]
        tips.extend(acc)
    return np.array(model + tips)


@pytest.mark.parametrize("n", [1, 2, 3, 43, 129, 1000, 33_333, 400_000])
def test_sums_match_numpy(n):
    import torch
    from probabilistic_peridynamics_gb300.integrators import CUDAContext
    from probabilistic_peridynamics_gb300.writes import WriteSums
    rng = np.random.default_rng(n)
    arrays = [rng.standard_normal((n, 3)) * 10.0 ** rng.integers(-9, 3)
              for _ in range(5)]
    damage = rng.uniform(0, 1, size=n) * (rng.uniform(size=n) < 0.3)
    volume = rng.uniform(0.5, 2.0, size=n) * 1e-7
    tips = {"a": [(int(i), int(j)) for i, j in
                  zip(rng.integers(0, n, 50), rng.integers(0, 3, 50))],
            "empty": [], "b": [(n - 1, 2), (0, 0)]}
    ctx = CUDAContext(0)
    dev = ctx.device
    vol_d = torch.as_tensor(volume, device=dev)
    sums = WriteSums(ctx, n, vol_d, tips)
    got = sums(*[torch.as_tensor(a, device=dev) for a in arrays],
               torch.as_tensor(damage, device=dev))
    want = _host_sums(*arrays, damage, volume, tips)
    assert got.shape == want.shape
    assert np.array_equal(got, want), np.nonzero(got != want)
    # missing arrays count as zeros
    got = sums(torch.as_tensor(arrays[0], device=dev), None, None, None,
               None, torch.as_tensor(damage, device=dev))
    zeros = np.zeros_like(arrays[0])
    want = _host_sums(arrays[0], zeros, zeros, zeros, zeros, damage, volume,
                      tips)
    assert np.array_equal(got, want)


def test_signed_zeros_and_no_nodes():
    import torch
    from probabilistic_peridynamics_gb300.integrators import CUDAContext
    from probabilistic_peridynamics_gb300.writes import WriteSums
    ctx = CUDAContext(0)
    dev = ctx.device
    n = 700
    neg = torch.full((n, 3), -0.0, dtype=torch.float64, device=dev)
    sums = WriteSums(ctx, n, torch.ones(n, dtype=torch.float64, device=dev),
                     {"t": [(3, 1)]})
    got = sums(neg, neg, neg, neg, neg, neg[:, 0].contiguous())
    want = np.sum(np.full((n, 3), -0.0))
    assert np.all(got[:6] == want) and not np.any(np.signbit(got[:6]))
    empty = torch.zeros((0, 3), dtype=torch.float64, device=dev)
    sums0 = WriteSums(ctx, 0, torch.zeros(0, dtype=torch.float64, device=dev),
                      {})
    got = sums0(empty, empty, empty, empty, empty,
                torch.zeros(0, dtype=torch.float64, device=dev))
    assert got.tolist() == [0.0] * 6


def _unit(x):
    return 1.0


def _tip(x):
    """Three tip types, one node in two of them."""
    if x[0] > 0.9:
        return ["right", None, ("right", "edge")]
    if x[1] < 0.05:
        return [None, "bottom", None]
    return [None, None, None]


@pytest.mark.parametrize("kind,precision", [
    ("euler", "float64"), ("euler_cromer", "float64"),
    ("velocity_verlet", "float64"), ("velocity_verlet", "mixed")])
def test_simulate_with_writes_matches_host_path(kind, precision, golden,
                                                tmp_path):
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300.mesh import write_vtk
    from tests.plate_setup import (BOND_STIFFNESS, CRITICAL_STRETCH,
                                   is_crack, is_displacement_boundary)
    cls = {"euler": pp.EulerCUDA, "euler_cromer": pp.EulerCromerCUDA,
           "velocity_verlet": pp.VelocityVerletCUDA}[kind]

    class HostWrites(cls):
        write_sums = None  # the host path: every array copied back

    mesh = tmp_path / "plate.vtk"
    write_vtk(mesh, golden["points"], [("triangle", golden["cells_triangle"]),
                                       ("line", golden["cells_line"])])
    steps = 40
    mags = 2e-4 * np.arange(1, steps + 1)  # loads that break bonds
    out = {}
    for name, c in (("device", cls), ("host", HostWrites)):
        integ = (c(dt=1e-3, precision=precision) if kind == "euler" else
                 c(0.5, dt=1e-3, precision=precision))
        model = pp.Model(mesh, integrator=integ, horizon=0.1,
                         critical_stretch=CRITICAL_STRETCH,
                         bond_stiffness=BOND_STIFFNESS,
                         initial_crack=pp.initial_crack_helper(is_crack),
                         is_displacement_boundary=is_displacement_boundary,
                         is_tip=_tip,
                         is_density=None if kind == "euler" else _unit)
        path = tmp_path / name
        path.mkdir()
        res = model.simulate(steps=steps, displacement_bc_magnitudes=mags,
                             write=7, write_path=path)
        out[name] = (res, path)
    (dev_res, dev_path), (host_res, host_path) = out["device"], out["host"]
    dev_data, host_data = dev_res[5], host_res[5]
    assert set(dev_data) == set(host_data) == {"model", "right", "edge",
                                               "bottom"}
    for key in host_data:
        for field in host_data[key]:
            assert np.array_equal(dev_data[key][field],
                                  host_data[key][field]), (key, field)
    assert host_data["model"]["damage_sum"][-1] > 0  # bonds broke
    for a, b in zip((dev_res[0], dev_res[1], dev_res[3], dev_res[4]),
                    (host_res[0], host_res[1], host_res[3], host_res[4])):
        assert np.array_equal(a, b)
    assert np.array_equal(dev_res[2][0], host_res[2][0])
    for step in (7, 14, 21, 28, 35):
        name = f"U_{step}.vtk"
        assert (dev_path / name).read_bytes() == \
            (host_path / name).read_bytes()


def test_write_into_registered_and_pinned_arrays(monkeypatch):
    """Integrator.write page-locks large host arrays for the copy (every
    array here, with the size threshold at 0) and leaves memory that is
    pinned already alone; the values are those of an ordinary copy and no
    CUDA error is left behind, also when part of a target array was
    registered beforehand, so that registering the whole array fails."""
    import torch
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300 import integrators
    from tests.gpu_helpers import breaking_setup
    setup = breaking_setup("velocity_verlet")
    n = setup["nnodes"]
    outs = []
    partial = None
    for mode in ("plain", "registered", "pinned", "partly_registered"):
        monkeypatch.setattr(integrators, "_REGISTER_BYTES",
                            1 << 40 if mode == "plain" else 0)
        integ = pp.VelocityVerletCUDA(0.5, dt=setup["dt"])
        integ.build(n, 3, setup["max_neigh"], setup["coords"],
                    setup["volume"], setup["family"], setup["bc_types"],
                    setup["bc_values"], setup["force_bc_types"],
                    setup["force_bc_values"], None, None,
                    setup["densities"])
        z = np.zeros((n, 3))
        integ.create_buffers(setup["nlist"].copy(), setup["n_neigh"].copy(),
                             setup["k"], setup["s0"], None, z, z, z, z, z,
                             np.zeros(n), None, 1, 1)
        for t in range(20):
            integ(3e-3 * (t + 1), 0.0)
        if mode == "pinned":
            bufs = [torch.zeros(n * 3, dtype=torch.float64,
                                pin_memory=True) for _ in range(5)]
            host = [b.numpy().reshape(n, 3) for b in bufs]
            nl = torch.zeros(setup["nlist"].size, dtype=torch.int32,
                             pin_memory=True).numpy().reshape(
                                 setup["nlist"].shape)
        else:
            host = [np.zeros((n, 3)) for _ in range(5)]
            nl = np.zeros_like(setup["nlist"])
        if mode == "partly_registered":
            # whole pages inside the neighbour-list target are registered
            # beforehand: registering the whole array then fails
            # (cudaErrorHostMemoryAlreadyRegistered), the copy goes ahead
            # unregistered and no error may reach torch's next launch
            page = 4096
            lo = -(-nl.ctypes.data // page) * page
            hi = (nl.ctypes.data + nl.nbytes) // page * page
            assert hi > lo
            cudart = torch.cuda.cudart()
            assert int(cudart.cudaHostRegister(lo, hi - lo, 0)) == 0
            partial = lo
        try:
            out = integ.write(*host, np.zeros(n), nl,
                              np.zeros(n, dtype=np.intc))
            y = torch.ones(4, device="cuda") * 3  # a launch right after
            torch.cuda.synchronize()
            assert float(y.sum()) == 12.0
        finally:
            if partial is not None:
                torch.cuda.cudart().cudaHostUnregister(partial)
                partial = None
        outs.append([np.array(a, copy=True) for a in out])
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)
    x = torch.ones(4, device="cuda") * 2  # a launch after the writes
    torch.cuda.synchronize()
    assert float(x.sum()) == 8.0
